"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Tolerances (stated per test): the FP32 form must stay within 1e-3 rad of the
FP64 oracle in phase, the FP64 form within 1e-10 rad.  Phase errors are
measured on pixels whose filtered magnitude is not negligible (where the
phase is defined)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_PHASE_TOL = 1e-3
F64_PHASE_TOL = 1e-10


def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def wff_gpu(glsu, f, prec, params, method=None):
    torch = _torch()
    dt = np.complex64 if prec == "f32" else np.complex128
    t = torch.from_numpy(np.ascontiguousarray(f, dt)).cuda()
    out = torch.empty_like(t)
    w = glsu.WFF2(f.shape[1], f.shape[0], prec, params)
    if method is not None:
        w.set_method(method)
    ms = w.run(t.data_ptr(), out.data_ptr())
    thr = w.threshold
    w.close()
    return out.cpu().numpy(), thr, ms


def field(shape, seed, noise=0.1):
    rng = np.random.default_rng(seed)
    H, W = shape
    y, x = np.mgrid[0:H, 0:W]
    phi = 0.05 * x + 0.03 * y + 2.0 * np.sin(x / 17.0) * np.cos(y / 23.0)
    return np.exp(1j * phi) * (1 + noise * rng.standard_normal(shape)) + noise * (
        rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def compare(out, ref, mask_frac=0.05):
    mag = np.abs(ref)
    m = mag > mask_frac * mag.max()
    perr = np.abs(np.angle(out[m] * np.conj(ref[m]))).max()
    rel = np.abs(out - ref).max() / mag.max()
    return perr, rel


WFF_CASES = [
    # (shape, params: sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, thr)
    ((64, 80), (4.0, -1.0, 1.0, 0.25, 4.0, -1.0, 1.0, 0.25, 0.5)),         # half-size 12
    ((37, 44), (3.0, -1.0, 1.0, 0.25, 4.0, -0.8, 0.8, 0.2, 0.5)),          # odd size, sigx != sigy
    ((96, 130), (6.5, -0.8, 0.8, 0.4, 6.5, -0.8, 0.8, 0.4, 1.0)),          # half-size 20
    ((128, 128), (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)),       # the 21x21 sweep, half 30
    ((140, 100), (15.0, -0.6, 0.6, 0.2, 15.0, -0.6, 0.6, 0.2, 0.3)),       # half-size 45
    ((150, 170), (20.0, -0.15, 0.15, 0.05, 20.0, -0.15, 0.15, 0.05, 15)),  # DPRA defaults, half 60
    ((64, 64), (4.0, 0.3, 0.3, 0.1, 4.0, -0.2, -0.2, 0.1, 0.3)),          # single frequency
    ((72, 90), (5.0, -1.0, 1.0, 0.4, 5.0, -1.0, 1.0, 0.4, -1.0)),          # automatic threshold
    ((5, 7), (2.0, -1.0, 1.0, 0.5, 2.0, -1.0, 1.0, 0.5, 0.1)),             # tiny image
]


@pytest.mark.parametrize("method", ["direct", "fft"])
@pytest.mark.parametrize("case", range(len(WFF_CASES)))
def test_wff_f32_matches_oracle(glsu, oracle, case, method):
    """Both column-sweep methods (direct convolution, shared-memory FFT)."""
    shape, p = WFF_CASES[case]
    f = field(shape, case)
    ref, rthr = oracle.wff2(f.astype(np.complex64).astype(np.complex128), *p)
    m = glsu.METHOD_DIRECT if method == "direct" else glsu.METHOD_FFT
    out, thr, _ = wff_gpu(glsu, f, "f32", glsu.WffParams(*p), m)
    perr, rel = compare(out, ref)
    print("wff f32 %s case %d: phase err %.3g rad, rel err %.3g" % (method, case, perr, rel))
    assert abs(thr - rthr) <= 1e-5 * rthr
    assert perr < F32_PHASE_TOL and rel < 1e-4


@pytest.mark.parametrize("case", [0, 1, 3, 5, 6, 7])
def test_wff_f64_matches_oracle(glsu, oracle, case):
    shape, p = WFF_CASES[case]
    f = field(shape, case)
    ref, rthr = oracle.wff2(f, *p)
    out, thr, _ = wff_gpu(glsu, f, "f64", glsu.WffParams(*p))
    perr, rel = compare(out, ref)
    print("wff f64 case %d: phase err %.3g rad, rel err %.3g" % (case, perr, rel))
    assert abs(thr - rthr) <= 1e-12 * rthr
    assert perr < F64_PHASE_TOL and rel < 1e-11


def test_column_method_switch(glsu):
    w = glsu.WFF2(64, 64, "f64", glsu.WffParams(4.0, -1, 1, 0.5, 4.0, -1, 1, 0.5, 0.1))
    with pytest.raises(glsu.GlsuError) as e:
        w.set_method(glsu.METHOD_FFT)
    assert e.value.code == glsu.ERR_UNSUPPORTED
    w.set_method(glsu.METHOD_DIRECT)
    with pytest.raises(glsu.GlsuError):
        w.set_method(7)
    w.close()


@pytest.mark.parametrize("case", [0, 2, 4])
def test_wff_fft_plans_match_oracle(glsu, oracle, case):
    """Every compiled FFT plan that fits the shape -- each transform length
    >= H + 2s, at both compiled CTA widths -- within the FP32 tolerance of
    the oracle; radix orders other than 0 are rejected."""
    shape, p = WFF_CASES[case]
    f = field(shape, case)
    ref, _ = oracle.wff2(f.astype(np.complex64).astype(np.complex128), *p)
    torch = _torch()
    t = torch.from_numpy(np.ascontiguousarray(f, np.complex64)).cuda()
    out = torch.empty_like(t)
    w = glsu.WFF2(shape[1], shape[0], "f32", glsu.WffParams(*p))
    w.set_method(glsu.METHOD_FFT)
    ran = 0
    lengths = w.fft_lengths(16)
    assert len(lengths) >= 10
    for L in lengths:
        w.set_fft_length(L)
        nc0 = w.tuning()["fft_columns"]
        for nc in (nc0, 2 * nc0):
            try:
                w.set_fft_plan(nc, 0)
            except glsu.GlsuError as e:
                assert e.code == glsu.ERR_UNSUPPORTED
                continue
            w.run(t.data_ptr(), out.data_ptr())
            perr, rel = compare(out.cpu().numpy(), ref)
            print("fft plan case %d L %d nc %d: phase err %.3g, rel %.3g" % (case, L, nc, perr, rel))
            assert perr < F32_PHASE_TOL and rel < 1e-4
            ran += 1
        with pytest.raises(glsu.GlsuError):
            w.set_fft_plan(nc0, 1)
    w.close()
    assert ran >= len(lengths)


def test_autotuner_choices(glsu, oracle):
    """METHOD_AUTO (the default) resolves from the shape by the cost model,
    with no timing: with the reference's DPRA WFF parameters (sigma 20, 7x7
    frequencies) and with sigma 10 and 21x21 frequencies it is the FFT sweep,
    for a narrow window on a small frame the direct kernel, in each case bit
    for bit the output of a handle with that method set explicitly.
    METHOD_TIMED times the candidates once per shape and process and picks
    the FFT sweep for the DPRA defaults (about 3x faster there)."""
    import os
    torch = _torch()
    dp = glsu.dpra_default_params()
    f = field((512, 512), 3)
    w = glsu.WFF2(512, 512, "f32", dp)
    tu = w.tuning()
    print("model choice, DPRA defaults 512^2:", tu)
    assert tu["tuned"] == 2 and tu["method"] == glsu.METHOD_FFT and 0 < tu["ms_fft"] < tu["ms_direct"]
    t = torch.from_numpy(np.ascontiguousarray(f, np.complex64)).cuda()
    out = torch.empty_like(t)
    w.run(t.data_ptr(), out.data_ptr())
    w2 = glsu.WFF2(512, 512, "f32", dp)  # the same shape: the same choice
    assert w2.tuning() == tu
    w2.close()
    ref, _ = oracle.wff2(f.astype(np.complex64).astype(np.complex128), *dp.tuple())
    perr, rel = compare(out.cpu().numpy(), ref)
    assert perr < F32_PHASE_TOL and rel < 1e-4

    w.set_method(glsu.METHOD_TIMED)
    tt = w.tuning()
    print("timed choice, DPRA defaults 512^2:", tt)
    assert tt["tuned"] == 1 and tt["method"] == glsu.METHOD_FFT and 0 < tt["ms_fft"] < tt["ms_direct"]
    out2 = torch.empty_like(t)
    w.run(t.data_ptr(), out2.data_ptr())
    perr, rel = compare(out2.cpu().numpy(), ref)
    assert perr < F32_PHASE_TOL and rel < 1e-4
    w.set_method(glsu.METHOD_AUTO)  # back to the model's choice and plan
    assert w.tuning() == tu
    w.close()

    p10 = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    f = field((256, 256), 4)
    a, _, _ = wff_gpu(glsu, f, "f32", p10)
    b, _, _ = wff_gpu(glsu, f, "f32", p10, glsu.METHOD_FFT)
    w = glsu.WFF2(256, 256, "f32", p10)
    tu = w.tuning()
    w.close()
    print("model choice, sigma 10 21x21 256^2:", tu)
    assert tu["method"] == glsu.METHOD_FFT and tu["tuned"] == 2
    assert np.array_equal(a, b)

    # a narrow window (half-size 12) on a small frame: the direct kernel,
    # bit for bit an explicit METHOD_DIRECT handle's output
    p4 = glsu.WffParams(4.0, -1.0, 1.0, 0.25, 4.0, -1.0, 1.0, 0.25, 0.5)
    f = field((64, 80), 5)
    a, _, _ = wff_gpu(glsu, f, "f32", p4)
    b, _, _ = wff_gpu(glsu, f, "f32", p4, glsu.METHOD_DIRECT)
    w = glsu.WFF2(80, 64, "f32", p4)
    tu = w.tuning()
    w.close()
    print("model choice, sigma 4 9x9 64x80:", tu)
    assert tu["method"] == glsu.METHOD_DIRECT and tu["tuned"] == 2
    assert np.array_equal(a, b)

    # GLSU_AUTOTUNE=0: AUTO is the direct kernel
    os.environ["GLSU_AUTOTUNE"] = "0"
    try:
        d = glsu.DPRA(np.zeros((200, 136), np.float32), 1, 1, "f32", dp)
        tu = d.tuning()
        d.close()
    finally:
        del os.environ["GLSU_AUTOTUNE"]
    assert tu["method"] == glsu.METHOD_DIRECT and tu["ms_direct"] == 0 and tu["ms_fft"] == 0


_TWO_PROC = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import glsu
from glsu import synth
frames, phi0, _ = synth.sequence(1024, 1024, 3, seed=1)
wp = glsu.WffParams(*[float(v) for v in sys.argv[3].split(",")])
d = glsu.DPRA(phi0.astype(np.float32), 1, 3, "f32", wp)
out = [d.per_frame(f)[0] for f in frames[1:]]
np.save(sys.argv[2], np.stack(out))
print(d.tuning())
d.close()
"""


@pytest.mark.parametrize("wp", ["10,-1,1,0.1,10,-1,1,0.1,0.2", "20,-0.15,0.15,0.05,20,-0.15,0.15,0.05,15"])
def test_two_processes_give_identical_bits(glsu, tmp_path, wp):
    """The default (AUTO) column sweep is decided without timing, so two fresh
    processes give the same dphi bits for the same frames: the bench's 1024^2
    shape (direct kernel) and the reference's DPRA defaults (FFT sweep)."""
    import subprocess
    import sys
    res = []
    for k in range(2):
        path = str(tmp_path / ("dphi%d.npy" % k))
        r = subprocess.run([sys.executable, "-c", _TWO_PROC, glsu.PKG_ROOT, path, wp], capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        print(r.stdout.strip())
        res.append(np.load(path))
    assert np.array_equal(res[0], res[1])


def test_wff_threshold_is_kept_after_first_call(glsu, oracle):
    torch = _torch()
    p = glsu.WffParams(4.0, -1, 1, 0.5, 4.0, -1, 1, 0.5, -1)
    f1, f2 = field((40, 40), 1), 3 * field((40, 40), 2)
    w = glsu.WFF2(40, 40, "f64", p)
    a, b = torch.from_numpy(f1).cuda(), torch.from_numpy(f2).cuda()
    out = torch.empty_like(a)
    w.run(a.data_ptr(), out.data_ptr())
    t1 = w.threshold
    w.run(b.data_ptr(), out.data_ptr())
    assert w.threshold == t1  # cached like the reference's m_rThr
    ref, _ = oracle.wff2(f2, 4.0, -1, 1, 0.5, 4.0, -1, 1, 0.5, t1)
    assert compare(out.cpu().numpy(), ref)[1] < 1e-11
    w.close()


@pytest.mark.parametrize("prec,r,img,ls", [("f32", 1, "u8", 0), ("f32", 3, "f32", 0), ("f32", 4, "f32", 0),
                                           ("f32", 3, "u8", 0), ("f32", 1, "u8", 1), ("f32", 3, "f32", 1),
                                           ("f64", 2, "f32", 0), ("f64", 3, "f64", 0), ("f64", 1, "u8", 0),
                                           # the largest windows (radius up to 8, 17x17)
                                           ("f32", 5, "f32", 0), ("f32", 8, "u8", 0), ("f32", 8, "f32", 1),
                                           ("f64", 6, "u8", 0), ("f64", 8, "f32", 0)])
def test_dpra_least_squares_matches_oracle(glsu, oracle, synth, prec, r, img, ls):
    """FP32 form in both arithmetics (ls 0: float-float, 1: FP64 sums); FP64 form."""
    H, W = 61, 75
    frames, phi0, _ = synth.sequence(H, W, 3, seed=r)
    fr = frames[2]
    if img == "u8":
        fr = np.clip(np.round(fr * 255), 0, 255).astype(np.uint8)
    elif img == "f64":
        fr = fr.astype(np.float64)
    phi_in = phi0.astype(np.float32 if prec == "f32" else np.float64)
    d = glsu.DPRA(phi_in, 1, r, prec, glsu.WffParams(3.0, -0.5, 0.5, 0.5, 3.0, -0.5, 0.5, 0.5, 0.1))
    if prec == "f32":
        d.set_ls_method(ls)
    d.per_frame(fr)
    z = d.get_lsq()
    zr = oracle.dpra_ls(fr.astype(np.float64), phi_in.astype(np.float64), r)
    err = np.abs(np.angle(z * np.conj(zr)))
    kap = oracle.dpra_kappa(phi_in.astype(np.float64), r)
    print("dpra LS %s r=%d %s ls=%d: max %.3g rad, rms %.3g, min kappa %.2g" % (prec, r, img, ls, err.max(),
                                                                                np.sqrt(np.mean(err ** 2)),
                                                                                kap.min()))
    if prec == "f32":
        assert err.max() < 1e-4  # FP32 output rounding; the sums and the solve run in FP64
    else:
        assert err.max() < 1e-10
    d.close()


@pytest.mark.parametrize("tile", [(32, 8), (32, 32)])
@pytest.mark.parametrize("r,img", [(1, "u8"), (3, "f32"), (8, "f32")])
def test_dpra_ls_tiles_match_oracle(glsu, oracle, synth, tile, r, img):
    """The float-float least squares with the other output tiles (the DPRA
    tile-shape knob) against the oracle, on a ragged frame, within the same
    bound as the default tile; and within float-float rounding of it."""
    H, W = 61, 75
    frames, phi0, _ = synth.sequence(H, W, 3, seed=r)
    fr = frames[2] if img == "f32" else np.clip(np.round(frames[2] * 255), 0, 255).astype(np.uint8)
    phi_in = phi0.astype(np.float32)
    wp = glsu.WffParams(3.0, -0.5, 0.5, 0.5, 3.0, -0.5, 0.5, 0.5, 0.1)
    if tile == (32, 32) and r == 8:
        # 246 KB of shared memory: above the per-block limit, refused up front
        d = glsu.DPRA(phi_in, 1, r, "f32", wp)
        with pytest.raises(glsu.GlsuError) as e:
            d.set_ls_tile(*tile)
        assert e.value.code == glsu.ERR_UNSUPPORTED and d.ls_tile() == (32, 16)
        d.per_frame(fr)  # the handle is still usable
        d.close()
        return
    out = []
    for t in ((32, 16), tile):
        d = glsu.DPRA(phi_in, 1, r, "f32", wp)
        d.set_ls_tile(*t)
        assert d.ls_tile() == t
        d.per_frame(fr)
        out.append(d.get_lsq())
        d.close()
    zr = oracle.dpra_ls(fr.astype(np.float64), phi_in.astype(np.float64), r)
    err = np.abs(np.angle(out[1] * np.conj(zr)))
    dif = np.abs(np.angle(out[1] * np.conj(out[0])))
    print("LS tile %s r=%d %s: max %.3g rad against the oracle, %.3g against 32x16" % (tile, r, img, err.max(),
                                                                                      dif.max()))
    assert err.max() < 1e-4 and dif.max() < 1e-4


def test_dpra_ls_tile_tuning(glsu, synth):
    frames, phi0, _ = synth.sequence(512, 512, 2, seed=5)
    d = glsu.DPRA(phi0.astype(np.float32), 1, 3, "f32", glsu.WffParams(10.0, -1, 1, 0.1, 10.0, -1, 1, 0.1, 0.2))
    assert d.ls_tile() == (32, 16)
    ms = d.tune_ls_tile()
    tiles = [(32, 16), (32, 8), (32, 32)]
    print("LS tile times (ms):", dict(zip(tiles, ms)), "chosen", d.ls_tile())
    assert all(m > 0 for m in ms) and d.ls_tile() == tiles[int(np.argmin(ms))]
    with pytest.raises(glsu.GlsuError):
        d.set_ls_tile(16, 16)
    d.per_frame(frames[1])  # runs with the chosen tile
    assert np.isfinite(d.get(glsu.PHI_CURR)).all()
    d.close()
    # at r = 8 the 32 x 32 tile does not fit in shared memory: not a candidate
    d = glsu.DPRA(phi0.astype(np.float32), 1, 8, "f32", glsu.WffParams(10.0, -1, 1, 0.1, 10.0, -1, 1, 0.1, 0.2))
    ms = d.tune_ls_tile()
    print("LS tile times at r = 8 (ms):", dict(zip(tiles, ms)), "chosen", d.ls_tile())
    assert ms[2] < 0 and ms[0] > 0 and ms[1] > 0 and d.ls_tile() == tiles[int(np.argmin(ms[:2]))]
    d.per_frame(frames[1])
    assert np.isfinite(d.get(glsu.PHI_CURR)).all()
    d.close()


MASK_MAG = 0.1  # phase compared where |filtered| >= 0.1 (unit-modulus input; median ~0.9)


def teacher_forced(glsu, oracle, frames, phi0, r, wp, prec, rr=1):
    """Run the GPU sequence and, for every frame, the oracle on the GPU's own
    reference state (teacher forcing).  Returns per-frame error stats."""
    dt = np.float32 if prec == "f32" else np.float64
    d = glsu.DPRA(phi0.astype(dt), rr, r, prec, wp)
    stats = []
    for i, fr in enumerate(frames):
        pref = d.get(glsu.PHI_REF).astype(np.float64)
        dref = d.get(glsu.DPHI_REF).astype(np.float64)
        dphi, _ = d.per_frame(fr)
        pc = d.get(glsu.PHI_CURR)
        opc, odp, _, ofilt = oracle.glsu_frame(fr.astype(np.float64), pref, dref, r, oracle.WffParams(*wp.tuple()))
        m = np.abs(ofilt) >= MASK_MAG
        e_pc = np.abs(np.angle(np.exp(1j * (pc.astype(np.float64) - opc))))
        e_dp = np.abs(dphi.astype(np.float64) - odp)
        stats.append({"frame": i, "kept": m.mean(), "pc_max": e_pc[m].max(), "dp_max": e_dp[m].max(),
                      "pc_rms_all": np.sqrt(np.mean(e_pc ** 2)), "pc_max_all": e_pc.max()})
        if i % rr == 0:
            d.update_ref_phi()
    d.close()
    return stats


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_glsu_sequence_256_matches_oracle(glsu, oracle, synth, prec):
    """The FP64 reference path's workload: 256x256, DPRA 7x7, WFF2 sigma 10,
    21x21 frequencies, threshold 0.2; first 4 frames, teacher-forced."""
    frames, phi0, _ = synth.sequence(256, 256, 4, seed=0)
    wp = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    dt = np.float32 if prec == "f32" else np.float64
    st = teacher_forced(glsu, oracle, frames.astype(dt), phi0, 3, wp, prec)
    for s_ in st:
        print("sequence %s frame %d: kept %.4f, phi max %.3g, dphi max %.3g, phi rms(all) %.3g, max(all) %.3g"
              % (prec, s_["frame"], s_["kept"], s_["pc_max"], s_["dp_max"], s_["pc_rms_all"], s_["pc_max_all"]))
    tol = F32_PHASE_TOL if prec == "f32" else F64_PHASE_TOL
    assert all(s_["pc_max"] < tol and s_["dp_max"] < tol and s_["pc_rms_all"] < tol for s_ in st)


_FREE_RUN = {}


def _oracle_free_run(oracle, frames, phi0, owp):
    """The oracle's own free-running recursion from phi0 (dphi per frame)."""
    key = phi0.tobytes()
    if key not in _FREE_RUN:
        pref, dref = phi0.astype(np.float64), np.zeros(phi0.shape)
        out = []
        for fr in frames:
            opc, odp, _, _ = oracle.glsu_frame(fr.astype(np.float64), pref, dref, 3, owp)
            out.append(odp)
            pref, dref = opc, odp
        _FREE_RUN[key] = np.stack(out)
    return _FREE_RUN[key]


def _drift(a, b):
    """Per-frame RMS of the wrapped difference (all pixels)."""
    e = np.angle(np.exp(1j * (a - b)))
    return np.sqrt(np.mean(e ** 2, axis=(1, 2)))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_glsu_sequence_256_free_running_drift(glsu, oracle, synth, prec):
    """The whole 20-frame 256x256 sequence of the FP64 reference workload
    (DPRA 7x7, WFF2 sigma 10, 21x21 frequencies, threshold 0.2, reference
    update every frame), free running on the GPU and in the oracle.

    The recursion feeds each frame's phase back as the next reference, and
    on this generator it amplifies any perturbation about 2.5x per frame
    (a 1e-9 rad perturbation of phi0 alone reaches 0.3 rad RMS after 20
    frames in the oracle itself).  So the drift is judged against the
    oracle's own sensitivity: FP64 within 10x of what a 4e-16 relative
    perturbation of phi0 causes in the oracle; FP32, started from the FP32
    phi0 that the reference's float interface passes, no more than what
    that rounding of phi0 alone causes in the oracle.  The first frame meets
    the per-frame tolerances (1e-10 / 1e-3 rad)."""
    frames, phi0, _ = synth.sequence(256, 256, 20, seed=0)
    wp = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    owp = oracle.WffParams(*wp.tuple())
    dt = np.float32 if prec == "f32" else np.float64
    d = glsu.DPRA(phi0.astype(dt), 1, 3, prec, wp)
    gpu, _ = d.sequence(frames.astype(dt))
    d.close()
    gpu = gpu.astype(np.float64)
    base = _oracle_free_run(oracle, frames, phi0, owp)
    fmt = lambda c: " ".join("%.2g" % v for v in c)
    if prec == "f64":
        rng = np.random.default_rng(1)
        pert = _oracle_free_run(oracle, frames, phi0 * (1 + 4e-16 * rng.standard_normal(phi0.shape)), owp)
        got, sens = _drift(gpu, base), _drift(pert, base)
        print("free-running f64 drift vs oracle: %s\n  oracle, phi0 perturbed 4e-16: %s" % (fmt(got), fmt(sens)))
        assert got[0] < F64_PHASE_TOL
        assert np.all(got <= 10 * sens + 1e-13)
    else:
        o32 = _oracle_free_run(oracle, frames, phi0.astype(np.float32).astype(np.float64), owp)
        got, sens = _drift(gpu, o32), _drift(o32, base)
        print("free-running f32 drift vs oracle from the same phi0: %s\n  oracle, phi0 rounded to FP32: %s\n"
              "  f32 vs oracle from the FP64 phi0: %s" % (fmt(got), fmt(sens), fmt(_drift(gpu, base))))
        assert got[0] < F32_PHASE_TOL
        assert np.all(got <= sens)


def test_reference_update_rate_semantics(glsu, oracle, synth):
    frames, phi0, _ = synth.sequence(48, 40, 5, seed=9)
    wp = glsu.WffParams(3.0, -0.5, 0.5, 0.25, 3.0, -0.5, 0.5, 0.25, 0.1)
    st = teacher_forced(glsu, oracle, frames.astype(np.float64), phi0, 2, wp, "f64", rr=2)
    assert all(s_["dp_max"] < F64_PHASE_TOL for s_ in st)
    d = glsu.DPRA(phi0, 2, 2, "f64", wp)
    dps, _ = d.sequence(frames.astype(np.float64))
    d.close()
    d = glsu.DPRA(phi0, 2, 2, "f64", wp)
    ref = []
    for i, fr in enumerate(frames.astype(np.float64)):
        ref.append(d.per_frame(fr)[0])
        if i % 2 == 0:
            d.update_ref_phi()
    d.close()
    assert np.array_equal(dps, np.stack(ref))


@pytest.mark.parametrize("prec,rr,img", [("f32", 1, "f32"), ("f32", 3, "u8"), ("f64", 2, "f64")])
def test_pipelined_sequence_equals_frame_loop(glsu, synth, prec, rr, img):
    """Pinned host buffers take the copy-overlapped sequence path; it must give
    the per-frame loop's results bit for bit (same kernels, same order)."""
    torch = _torch()
    frames, phi0, _ = synth.sequence(96, 128, 7, seed=5)
    wp = glsu.WffParams(6.0, -1.0, 1.0, 0.25, 6.0, -1.0, 1.0, 0.25, -1)
    dt = np.float32 if prec == "f32" else np.float64
    if img == "u8":
        fr = np.clip(np.round(frames * 255), 0, 255).astype(np.uint8)
    else:
        fr = frames.astype(np.float32 if img == "f32" else np.float64)
    d = glsu.DPRA(phi0.astype(dt), rr, 3, prec, wp)
    ref = []
    for i, f in enumerate(fr):
        ref.append(d.per_frame(f)[0])
        if i % rr == 0:
            d.update_ref_phi()
    ref_state = d.get(glsu.PHI_REF)
    d.close()
    tf = torch.from_numpy(fr).pin_memory()
    out = torch.empty((fr.shape[0],) + fr.shape[1:], dtype=torch.float32 if prec == "f32" else torch.float64)
    out = out.pin_memory()
    d = glsu.DPRA(phi0.astype(dt), rr, 3, prec, wp)
    itype = {"u8": glsu.U8, "f32": glsu.F32, "f64": glsu.F64}[img]
    ms = d.sequence_ptr(fr.shape[0], tf.data_ptr(), itype, out.data_ptr())
    assert ms > 0
    assert np.array_equal(out.numpy(), np.stack(ref))
    assert np.array_equal(d.get(glsu.PHI_REF), ref_state)
    # a second sequence on the same handle continues from the updated state
    ms2 = d.sequence_ptr(2, tf.data_ptr(), itype, out.data_ptr())
    d.close()
    d = glsu.DPRA(phi0.astype(dt), rr, 3, prec, wp)
    seq_np, _ = d.sequence(fr)
    more, _ = d.sequence(np.ascontiguousarray(fr[:2]))
    d.close()
    assert ms2 > 0 and np.array_equal(out.numpy()[:2], more)
    assert np.array_equal(seq_np, np.stack(ref))


@pytest.mark.parametrize("rr", [1, 3])
def test_graph_mode_equals_eager_fp64(glsu, synth, rr):
    """The FP64 handle (DPRA_CUDA) replayed from graphs: the eager phases bit
    for bit, f64 and u8 frames, across reference updates."""
    frames, phi0, _ = synth.sequence(72, 96, 6, seed=13)
    wp = glsu.WffParams(4.0, -0.5, 0.5, 0.25, 4.0, -0.5, 0.5, 0.25, 0.2)
    out = []
    for graph in (False, True):
        d = glsu.DPRA(phi0.astype(np.float64), rr, 2, "f64", wp)
        d.set_graph(graph)
        res = []
        for k, f in enumerate(frames):
            img = f.astype(np.float64) if k % 2 else np.clip(f * 255, 0, 255).astype(np.uint8)
            dphi, _ = d.per_frame(img)
            res.append((dphi.copy(), d.get(glsu.PHI_CURR).copy()))
            if k % rr == 0:
                d.update_ref_phi()
        d.close()
        out.append(res)
    for (a1, b1), (a2, b2) in zip(*out):
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


def test_graph_mode_on_the_legacy_stream_runs_eagerly(glsu, synth):
    """The legacy default stream cannot be captured: a handle moved onto it
    keeps graph mode on but runs its frames eagerly, with the same results;
    the batched form refuses such a handle."""
    frames, phi0, _ = synth.sequence(64, 80, 4, seed=12)
    wp = glsu.WffParams(4.0, -0.5, 0.5, 0.25, 4.0, -0.5, 0.5, 0.25, 0.2)
    out = []
    for legacy in (False, True):
        d = glsu.DPRA(phi0.astype(np.float32), 1, 2, "f32", wp)
        d.set_graph(True)
        if legacy:
            d.set_stream(0)
        res, _ = d.sequence(frames)
        out.append(res)
        if legacy:
            torch = _torch()
            t = torch.from_numpy(frames).cuda()
            with pytest.raises(glsu.GlsuError) as e:
                glsu.dpra_batch_step([d], [t[0].data_ptr()], glsu.F32)
            assert e.value.code == glsu.ERR_INVALID
        d.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("graph", [False, True])
def test_batched_uneven_sequences_equal_sequential(glsu, synth, graph):
    """The batched form: sequences of uneven sizes, window radii 2..4,
    reference rates 1..3 and lengths, one frame of each per step, each on
    its handle's stream and in flight together (ended sequences pass no
    frame), give every sequence's phases bit for bit as its own
    glsu_dpra_sequence does; FP32, u8 frames; plain and surrogate handles."""
    torch = _torch()
    from glsu import train_surrogate as T
    wp = glsu.WffParams(6.0, -1.0, 1.0, 0.25, 6.0, -1.0, 1.0, 0.25, 0.2)
    specs = [((64, 48), 2, 1, 5), ((96, 80), 3, 2, 3), ((128, 128), 4, 3, 6), ((80, 120), 3, 1, 4),
             ((128, 128), 2, 1, 2), ((72, 100), 4, 2, 5)]
    params = T.init_params(3, scale_last=1.0)
    seqs, handles, ref = [], [], []
    for k, ((H, W), r, rr, nf) in enumerate(specs):
        frames, phi0, _ = synth.sequence(H, W, nf, seed=40 + k)
        u8 = np.clip(np.round(frames * 255), 0, 255).astype(np.uint8)
        d = glsu.DPRA(phi0.astype(np.float32), rr, r, "f32", wp)
        if k == 2:
            d.set_surrogate(params, [1, 2, 4, 8, 16, 8, 4, 1], 64, 8, 0.1)
        out, _ = d.sequence(u8)
        ref.append((out, d.get(glsu.PHI_REF).copy()))
        d.close()
        d = glsu.DPRA(phi0.astype(np.float32), rr, r, "f32", wp)
        if k == 2:
            d.set_surrogate(params, [1, 2, 4, 8, 16, 8, 4, 1], 64, 8, 0.1)
        d.set_graph(graph)
        handles.append(d)
        seqs.append(torch.from_numpy(u8).cuda())
    dphi = [[] for _ in specs]
    for step in range(max(s[3] for s in specs)):
        ptrs = [seqs[k][step].data_ptr() if step < specs[k][3] else None for k in range(len(specs))]
        glsu.dpra_batch_step(handles, ptrs, glsu.U8)
        glsu.dpra_batch_wait(handles)
        for k in range(len(specs)):
            if step < specs[k][3]:
                dphi[k].append(handles[k].get(glsu.DPHI).copy())
    for k, d in enumerate(handles):
        assert np.array_equal(np.stack(dphi[k]), ref[k][0]), k
        assert np.array_equal(d.get(glsu.PHI_REF), ref[k][1]), k
        d.close()
    with pytest.raises(glsu.GlsuError):
        h = glsu.DPRA(np.zeros((16, 16), np.float32), 1, 1, "f32", wp)
        try:
            glsu.dpra_batch_step([h, h], [seqs[0][0].data_ptr()] * 2, glsu.U8)
        finally:
            h.close()


@pytest.mark.parametrize("graph", [False, True])
def test_staged_batch_equals_sequential(glsu, synth, graph):
    """The staged batch (glsu_dpra_batch_*): sequences of uneven sizes,
    window radii 2..4, reference rates 1..3, WFF parameters with different
    column sweeps (FFT sweeps of three transform lengths batched per length,
    and a narrow window on the direct sweep), ended sequences passing no
    frame: every sequence's phases bit for bit as its own glsu_dpra_sequence
    gives them; FP32, u8 and f32 frames."""
    torch = _torch()
    w21 = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)   # FFT sweep (model)
    w11 = glsu.WffParams(10.0, -1.0, 1.0, 0.2, 10.0, -1.0, 1.0, 0.2, 0.2)   # direct sweep at 96x80
    w4 = glsu.WffParams(4.0, -1.0, 1.0, 0.25, 4.0, -1.0, 1.0, 0.25, 0.3)    # direct sweep
    specs = [((128, 128), 2, 1, 5, w21), ((96, 80), 3, 2, 3, w11), ((256, 256), 4, 3, 6, w21),
             ((128, 128), 3, 1, 4, w21), ((384, 512), 2, 1, 3, w21), ((64, 80), 3, 2, 4, w4)]
    for img in ("u8", "f32"):
        seqs, handles, ref, methods = [], [], [], []
        for k, ((H, W), r, rr, nf, wp) in enumerate(specs):
            frames, phi0, _ = synth.sequence(H, W, nf, seed=70 + k)
            fr = np.clip(np.round(frames * 255), 0, 255).astype(np.uint8) if img == "u8" else frames
            d = glsu.DPRA(phi0.astype(np.float32), rr, r, "f32", wp)
            out, _ = d.sequence(fr)
            ref.append((out, d.get(glsu.PHI_REF).copy()))
            d.close()
            d = glsu.DPRA(phi0.astype(np.float32), rr, r, "f32", wp)
            methods.append((d.tuning()["method"], d.tuning()["fft_length"]))
            handles.append(d)
            seqs.append(torch.from_numpy(fr).cuda())
        assert {m for m, _ in methods} == {glsu.METHOD_FFT, glsu.METHOD_DIRECT}, methods
        assert len({L for m, L in methods if m == glsu.METHOD_FFT}) >= 2, methods
        b = glsu.DpraBatch(handles, graph=graph)
        dphi = [[] for _ in specs]
        for step in range(max(s[3] for s in specs)):
            ptrs = [seqs[k][step].data_ptr() if step < specs[k][3] else None for k in range(len(specs))]
            b.run(ptrs, glsu.U8 if img == "u8" else glsu.F32)
            b.sync()
            for k in range(len(specs)):
                if step < specs[k][3]:
                    dphi[k].append(handles[k].get(glsu.DPHI).copy())
        b.close()
        for k, d in enumerate(handles):
            assert np.array_equal(np.stack(dphi[k]), ref[k][0]), (img, k, methods[k])
            assert np.array_equal(d.get(glsu.PHI_REF), ref[k][1]), (img, k)
            d.close()
    print("methods (sweep, length):", methods)
    h = glsu.DPRA(np.zeros((16, 16)), 1, 1, "f64", w4)
    with pytest.raises(glsu.GlsuError) as e:
        glsu.DpraBatch([h])
    assert e.value.code == glsu.ERR_UNSUPPORTED
    h.close()


def test_aia_reference_bmp_frames(glsu, oracle):
    """AIA on the reference's own test frames Test/{1,2,3}.bmp with the
    deltas of its tests (uint8 path, as AIA_CUDAF receives cv::Mat CV_8UC1)."""
    import os
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "aia_bmp.npz"))
    frames = g["frames"]
    d0 = g["deltas0"]
    a = glsu.AIA(3, 256, 256)
    phi, d, ms, it, err = a.run(list(frames), d0, max_iter=20, max_err=1e-4)
    ophi, od, oit, oerr = oracle.aia(frames.astype(np.float64), d0.astype(np.float64), 20, 1e-4)
    e_phi = np.abs(np.angle(np.exp(1j * (phi - ophi)))).max()
    print("aia bmp: iters %d/%d, delta err %.3g, phi err %.3g" % (it, oit, np.abs(d - od).max(), e_phi))
    assert it == oit
    assert np.abs(d - od).max() < 1e-4 and e_phi < 1e-3
    a.close()


@pytest.mark.parametrize("M", [3, 5, 32])
def test_aia_synthetic_matches_oracle(glsu, oracle, synth, M):
    """AIA from the fewest frames it accepts (3) to the most (32)."""
    frames, _, _ = synth.aia_frames(200, 180, M, seed=4)
    d0 = glsu.random_deltas(M, 11)
    a = glsu.AIA(M, 180, 200)
    phi, d, ms, it, err = a.run(list(frames), None, max_iter=30, max_err=1e-4, seed=11)
    ophi, od, oit, oerr = oracle.aia(frames.astype(np.float64), d0.astype(np.float64), 30, 1e-4)
    e_phi = np.abs(np.angle(np.exp(1j * (phi - ophi)))).max()
    print("aia synthetic M=%d: iters %d/%d, delta err %.3g, phi err %.3g" % (M, it, oit, np.abs(d - od).max(), e_phi))
    assert it == oit and np.abs(d - od).max() < 1e-4 and e_phi < 1e-3
    a.close()


@pytest.mark.parametrize("M", [5, 8])
def test_aia_relative_convergence_matches_oracle(glsu, oracle, synth, M):
    """With the convergence measure of AIA_CUDAF_YC2 (the change of the shifts
    relative to the first) the GPU stops where the oracle stops, well before
    the cap, with the oracle's shifts and phase."""
    frames, _, _ = synth.aia_frames(200, 180, M, seed=1000)
    d0 = glsu.random_deltas(M, 7)
    a = glsu.AIA(M, 180, 200)
    a.set_convergence(True)
    phi, d, ms, it, err = a.run(list(frames), None, max_iter=30, max_err=1e-4, seed=7)
    a.close()
    ophi, od, oit, oerr = oracle.aia(frames.astype(np.float64), d0.astype(np.float64), 30, 1e-4, relative=True)
    e_phi = np.abs(np.angle(np.exp(1j * (phi - ophi)))).max()
    print("aia relative M=%d: iters %d/%d, err %.3g, delta err %.3g, phi err %.3g"
          % (M, it, oit, err, np.abs(d - od).max(), e_phi))
    assert it == oit and it < 30 and err <= 1e-4
    assert np.abs(d - od).max() < 1e-4 and e_phi < 1e-3


def test_wff_phase_equivariance_full_size(glsu):
    """Size-independent property at 1024x1024: WFF2(e^{ja} f) = e^{ja} WFF2(f)."""
    torch = _torch()
    f = field((1024, 1024), 3)
    p = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    a = torch.from_numpy(f.astype(np.complex64)).cuda()
    b = a * np.exp(1j * 1.234)
    oa, ob = torch.empty_like(a), torch.empty_like(a)
    w = glsu.WFF2(1024, 1024, "f32", p)
    w.run(a.data_ptr(), oa.data_ptr())
    w.run(b.data_ptr(), ob.data_ptr())
    oa = oa.cpu().numpy() * np.exp(1j * 1.234)
    perr, rel = compare(ob.cpu().numpy(), oa)
    assert perr < 1e-4 and rel < 1e-4
    w.close()


def test_large_workload_shape_2048(glsu, oracle, synth):
    """The large streaming workload's shape: 2048x2048 FP32, DPRA 9x9, WFF2
    sigma 15 with 31x31 frequencies on [-1.5, 1.5], 8 Gaussians, noise 0.05.
    One frame end to end; its least squares against the oracle (a local
    stage, so the full frame is checked); the WFF2 stage through the
    size-independent phase equivariance WFF2(e^{ja} z) = e^{ja} WFF2(z) at this
    size (its kernels, half size 45, meet the oracle at small sizes in
    test_wff_f32_matches_oracle)."""
    torch = _torch()
    H = W = 2048
    frames, phi0, _ = synth.sequence(H, W, 2, seed=4, noise=0.05, n_gauss=8)
    wp = glsu.WffParams(15.0, -1.5, 1.5, 0.1, 15.0, -1.5, 1.5, 0.1, 0.2)
    d = glsu.DPRA(phi0.astype(np.float32), 1, 4, "f32", wp)
    print("tuning 2048^2 sigma 15 31x31:", d.tuning())
    fr = torch.from_numpy(frames[1]).cuda()
    d.per_frame_device(fr.data_ptr(), glsu.F32)
    z = d.get_lsq()
    pc = d.get(glsu.PHI_CURR)
    d.close()
    assert np.isfinite(pc).all()
    zr = oracle.dpra_ls(frames[1].astype(np.float64), phi0.astype(np.float32).astype(np.float64), 4)
    e = np.abs(np.angle(z * np.conj(zr)))
    print("2048^2 LS r=4: max %.3g rad, rms %.3g" % (e.max(), np.sqrt(np.mean(e ** 2))))
    assert e.max() < F32_PHASE_TOL
    a = torch.from_numpy(z).cuda()
    b = a * np.exp(1j * 0.77)
    oa, ob = torch.empty_like(a), torch.empty_like(a)
    w = glsu.WFF2(W, H, "f32", wp)
    ms = w.run(a.data_ptr(), oa.data_ptr())
    w.run(b.data_ptr(), ob.data_ptr())
    w.close()
    perr, rel = compare(ob.cpu().numpy(), oa.cpu().numpy() * np.exp(1j * 0.77))
    print("2048^2 WFF2 (961 frequencies): %.1f ms; equivariance phase %.3g rel %.3g" % (ms, perr, rel))
    assert perr < 1e-4 and rel < 1e-4


def test_glsu_frame_1024_matches_oracle(glsu, oracle, synth):
    """One full-size frame (1024x1024, DPRA 7x7, 441 frequencies) against the oracle."""
    frames, phi0, _ = synth.sequence(1024, 1024, 2, seed=1)
    wp = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    st = teacher_forced(glsu, oracle, frames[1:], phi0, 3, wp, "f32")[0]
    print("1024 frame f32: kept %.4f, phi max %.3g, dphi max %.3g, rms(all) %.3g, max(all) %.3g"
          % (st["kept"], st["pc_max"], st["dp_max"], st["pc_rms_all"], st["pc_max_all"]))
    assert st["pc_max"] < F32_PHASE_TOL and st["pc_rms_all"] < F32_PHASE_TOL


def test_error_codes_on_device(glsu):
    with pytest.raises(glsu.GlsuError) as e:
        glsu.WFF2(64, 64, "f32", glsu.WffParams(), wft_type=glsu.WFT_WFR)
    assert e.value.code == glsu.ERR_UNSUPPORTED
    with pytest.raises(glsu.GlsuError) as e:
        glsu.WFF2(4090, 8, "f32", glsu.WffParams())
    assert e.value.code == glsu.ERR_PADDING
    d = glsu.DPRA(np.zeros((16, 16), np.float32), 1, 1, "f32", glsu.WffParams(2.0, -1, 1, 1, 2.0, -1, 1, 1, 0.1))
    with pytest.raises((TypeError, glsu.GlsuError)):
        d.per_frame(np.zeros((16, 16), np.int16))
    d.close()


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("shape,start", [((64, 80), (-1, -1)), ((37, 300), (19, 19)), ((1, 50), (0, 49)),
                                         ((200, 1), (5, 0)), ((512, 384), (0, 383))])
def test_unwrap_matches_oracle(glsu, oracle, prec, shape, start):
    torch = _torch()
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    true = 0.5 * x - 0.35 * y + 3 * np.sin(x / 11.0) * np.cos(y / 13.0) + 0.3 * rng.standard_normal(shape)
    w = np.angle(np.exp(1j * true))
    dt = np.float32 if prec == "f32" else np.float64
    t = torch.from_numpy(w.astype(dt)).cuda()
    glsu.unwrap2_device(prec, t.data_ptr(), shape[1], shape[0], *start)
    torch.cuda.synchronize()
    got = t.cpu().numpy().astype(np.float64)
    sr, sc = start
    ref = oracle.unwrap2(w.astype(dt).astype(np.float64), None if sr < 0 else sr, None if sc < 0 else sc)
    k = np.round((got - ref) / (2 * np.pi))
    print("unwrap %s %s: 2pi-count mismatches %d, max diff %.3g" % (prec, shape, int((k != 0).sum()),
                                                                   np.abs(got - ref).max()))
    assert (k == 0).all()
    assert np.abs(got - ref).max() < (1e-4 if prec == "f32" else 1e-10) * max(1, np.abs(ref).max())


def test_dpra_with_unwrapping_matches_matlab_semantics(glsu, oracle, synth):
    """dphi = dphi_ref + unwrap(angle(filtered)) (MatLab/fp_ls3u.m:104)."""
    frames, phi0, _ = synth.sequence(64, 72, 3, seed=8)
    wp = glsu.WffParams(4.0, -1.0, 1.0, 0.5, 4.0, -1.0, 1.0, 0.5, 0.3)
    d = glsu.DPRA(phi0, 1, 2, "f64", wp)
    d.set_unwrap(True, 19, 19)
    for fr in frames[1:]:
        pref = d.get(glsu.PHI_REF)
        dref = d.get(glsu.DPHI_REF)
        dphi, _ = d.per_frame(fr.astype(np.float64))
        _, _, _, filt = oracle.glsu_frame(fr.astype(np.float64), pref, dref, 2, oracle.WffParams(*wp.tuple()))
        ref = dref + oracle.unwrap2(np.angle(filt), 19, 19)
        assert np.abs(dphi - ref).max() < 1e-9
        d.update_ref_phi()
    d.close()


@pytest.mark.gpu
@pytest.mark.parametrize("surrogate", [False, True])
@pytest.mark.parametrize("rr", [1, 2])
def test_graph_mode_equals_eager(glsu, synth, surrogate, rr):
    """Frames replayed from captured CUDA graphs (host frames, device frames at
    arbitrary addresses, u8 and f32) give the eager path's phases bit for bit,
    across reference updates and a configuration change."""
    import torch
    from glsu import train_surrogate as T
    H, W = 96, 136
    frames, phi0, _ = synth.sequence(H, W, 7, seed=8)
    wp = glsu.WffParams(4.0, -0.5, 0.5, 0.25, 4.0, -0.5, 0.5, 0.25, 0.2)
    params, dil = T.init_params(3, scale_last=1.0), [1, 2, 4, 8, 16, 8, 4, 1]
    out = []
    for graph in (False, True):
        d = glsu.DPRA(phi0.astype(np.float32), rr, 2, "f32", wp)
        if surrogate:
            d.set_surrogate(params, dil, 64, 8, 0.1)
        d.set_graph(graph)
        res = []
        dev = torch.from_numpy(frames.astype(np.float32)).cuda()
        for k, f in enumerate(frames[1:], start=1):
            if k == 4:
                d.set_ls_method(glsu.LS_FP64_SUMS)  # drops the captured graphs
            if k % 3 == 0:
                dphi, _ = d.per_frame(np.clip(f * 255, 0, 255).astype(np.uint8))
            elif k % 3 == 1:
                dphi, _ = d.per_frame(f.astype(np.float32))
            else:
                d.per_frame_device(dev[k].data_ptr(), glsu.F32)
                dphi = d.get(glsu.DPHI)
            res.append((dphi.copy(), d.get(glsu.PHI_CURR).copy()))
            if k % rr == 0:
                d.update_ref_phi()
        # the sequence API: pageable (per frame) and page-locked (pipelined,
        # two input slots) buffers
        seq, _ = d.sequence(frames[1:4].astype(np.float32))
        res.append((seq, d.get(glsu.PHI_REF).copy()))
        pin_in = torch.from_numpy(frames[1:5].astype(np.float32)).pin_memory()
        pin_out = torch.empty((4, H, W), dtype=torch.float32).pin_memory()
        d.sequence_ptr(4, pin_in.data_ptr(), glsu.F32, pin_out.data_ptr())
        res.append((pin_out.numpy().copy(), d.get(glsu.PHI_REF).copy()))
        if surrogate:
            res.append((np.asarray(d.surrogate_stats()), np.zeros(1)))
        d.close()
        out.append(res)
    for (a1, b1), (a2, b2) in zip(*out):
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)


# ---- parity against the reference's own CPU classes (tests/golden/ref_golden.npz) ----
def _ref_gold():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz"))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_wff_matches_reference_wft2_cpu(glsu, prec):
    """WFF2 on the GPU against the reference's WFT2_cpu (compiled from its
    sources): config-0 parameters, DPRA's hard-wired ones, and an automatic
    threshold on a ragged size."""
    g = _ref_gold()
    for k in range(3):
        f, ref = g["wff%d_in" % k], g["wff%d_out" % k]
        p = g["wff%d_params" % k]
        counts = [(glsu.wff_count(p[1 + o], p[2 + o], p[3 + o], glsu.F32),
                   glsu.wff_count(p[1 + o], p[2 + o], p[3 + o], glsu.F64)) for o in (0, 4)]
        if prec == "f32" and any(a != b for a, b in counts):
            # the reference counts frequencies in the class's precision: the
            # float class sweeps another grid than the double class's fixture
            print("f32 case %d skipped: frequency counts (float, double) %s" % (k, counts))
            continue
        out, thr, _ = wff_gpu(glsu, f, prec, glsu.WffParams(*p))
        perr, rel = compare(out, ref, 1e-3)
        print("%s case %d: phase %.3g rad, rel %.3g, thr %.9g / %.9g" % (prec, k, perr, rel, thr, g["wff%d_thr" % k]))
        if prec == "f64":
            assert perr < F64_PHASE_TOL and rel < 1e-12
            assert abs(thr - g["wff%d_thr" % k]) <= 1e-12 * abs(thr)
        else:
            assert perr < F32_PHASE_TOL and rel < 1e-4


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_dpra_ls_matches_reference_dpra_cpu_by_conditioning(glsu, oracle, prec):
    """The DPRA least squares (3x3 window, 8-bit frames) against the
    reference DPRA_CPU's LAPACKE_dsysv solves, teacher-forced on its phases,
    per conditioning bucket kappa = det/trace^2 of the reduced normal
    matrix: FP64 within 1e-9 rad where kappa > 1e-3 and 1e-6 where
    1e-4 < kappa <= 1e-3; FP32 within its 1e-3 bar in both; numerically
    singular windows (kappa <= 1e-4) are reported, not bounded."""
    g = _ref_gold()
    u8, pc = g["dpra_frames"], g["dpra_phi_curr"]
    pref = g["dpra_phi0"]
    wp = glsu.WffParams(20.0, -0.15, 0.15, 0.05, 20.0, -0.15, 0.15, 0.05, 15.0)
    bars = {"f64": (1e-9, 1e-6), "f32": (F32_PHASE_TOL, F32_PHASE_TOL)}[prec]
    for k in range(u8.shape[0]):
        d = glsu.DPRA(pref.astype(np.float64 if prec == "f64" else np.float32), 1, 1, prec, wp)
        d.per_frame(u8[k])
        z = d.get_lsq()
        d.close()
        kap = oracle.dpra_kappa(pref, 1)
        e = np.abs(np.angle(z * np.conj(g["dpra_lsq"][k])))
        for (lo, hi), bar in (((1e-3, 1.0), bars[0]), ((1e-4, 1e-3), bars[1]), ((-1.0, 1e-4), None)):
            m = (kap > lo) & (kap <= hi)
            emax = float(e[m].max()) if m.any() else 0.0
            print("%s frame %d kappa (%g, %g]: %d px, max %.3g rad" % (prec, k, lo, hi, int(m.sum()), emax))
            if bar is not None:
                assert emax <= bar
        pref = pc[k]


def test_wff_and_update_on_reference_lsq_match_reference_phases(glsu):
    """FP64 WFF2 on the GPU of the reference's own least-squares output, then
    the phase update: the reference's phi_curr to its float rounding of the
    angle (DPRA/dpra_cpu.cpp:246, at most 2^-24 pi)."""
    torch = _torch()
    g = _ref_gold()
    pref = g["dpra_phi0"]
    H, W = pref.shape
    w = glsu.WFF2(W, H, "f64", glsu.WffParams(20.0, -0.15, 0.15, 0.05, 20.0, -0.15, 0.15, 0.05, 15.0))
    for k in range(g["dpra_frames"].shape[0]):
        a = torch.from_numpy(np.ascontiguousarray(g["dpra_lsq"][k])).cuda()
        out = torch.empty_like(a)
        w.run(a.data_ptr(), out.data_ptr())
        t = np.angle(out.cpu().numpy())
        pc = np.angle(np.exp(1j * (t + pref)))
        e = np.abs(np.angle(np.exp(1j * (pc - g["dpra_phi_curr"][k]))))
        print("frame %d: phi_curr max %.3g rad" % (k, e.max()))
        assert e.max() <= 2.0 ** -24 * np.pi * 1.01
        pref = g["dpra_phi_curr"][k]
    w.close()
