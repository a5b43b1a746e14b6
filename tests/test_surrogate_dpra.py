"""The surrogate form of the DPRA frame (network -> sparse exact WFF2 probes
-> per-tile plain-WFF2 fallback -> phase update), on the GPU.

Bit-exact checks: a tile recomputed by the plain WFF2 runs the same kernels
on the same data as the plain path, with the same column sweep (direct
kernel or shared-memory FFT sweep, whichever the handle uses), so its phases
equal that path's bit for bit; a tile left to the network equals the
network-only run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIL = [1, 2, 4, 8, 16, 8, 4, 1]
H, W, TILE, PATCH = 200, 300, 64, 8
WP = (6.0, -1.0, 1.0, 0.25, 6.0, -1.0, 1.0, 0.25, 0.2)
# a wide window with few frequencies, where the cost model picks the FFT
# column sweep (half-size 45: 4 x 4 probe patches)
WIDE = dict(H=512, W=512, TILE=128, PATCH=4, WP=(15.0, -0.75, 0.75, 0.25, 15.0, -0.75, 0.75, 0.25, 0.2))
NARROW = dict(H=H, W=W, TILE=TILE, PATCH=PATCH, WP=WP)


def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _params(glsu, seed=3):
    from glsu import train_surrogate as T
    return T.init_params(seed, scale_last=1.0)


def _run(glsu, synth, params, tol, nframes=3, seed=11, method=None, case=None, tuning=None):
    c = case or NARROW
    h, w, tile, patch = c["H"], c["W"], c["TILE"], c["PATCH"]
    frames, phi0, _ = synth.sequence(h, w, nframes, seed=seed)
    d = glsu.DPRA(phi0.astype(np.float32), 1, 3, "f32", glsu.WffParams(*c["WP"]))
    if method is not None:
        d.set_method(method)
    if tuning is not None:
        tuning.append(d.tuning())
    if params is not None:
        d.set_surrogate(params, DIL, tile, patch, tol)
    ntiles = ((h + tile - 1) // tile) * ((w + tile - 1) // tile)
    out, stats, lsq = [], [], []
    for f in frames[1:]:
        dphi, _ = d.per_frame(f)
        out.append((dphi, d.get(glsu.PHI_CURR)))
        lsq.append(d.get_lsq())
        if params is not None and tol > 0:
            stats.append(d.surrogate_stats(ntiles))
        d.update_ref_phi()
    d.close()
    return out, stats, lsq


def _tiles(case=None):
    c = case or NARROW
    for ty in range(0, c["H"], c["TILE"]):
        for tx in range(0, c["W"], c["TILE"]):
            yield (slice(ty, min(c["H"], ty + c["TILE"])), slice(tx, min(c["W"], tx + c["TILE"])))


@pytest.mark.parametrize("which", ["direct", "fft", "auto_wide"])
def test_all_flagged_tiles_equal_the_plain_path(glsu, synth, which):
    """With a zero-width tolerance every probed tile is recomputed by the
    plain WFF2 and must equal the plain frame bit for bit, whichever column
    sweep the handle runs: the direct kernel, the FFT sweep, or the default
    (AUTO) on a shape where it is the FFT sweep."""
    method = {"direct": glsu.METHOD_DIRECT, "fft": glsu.METHOD_FFT, "auto_wide": None}[which]
    case = WIDE if which == "auto_wide" else NARROW
    tu = []
    plain, _, _ = _run(glsu, synth, None, 0, method=method, case=case, tuning=tu)
    if which == "auto_wide":
        assert tu[0]["method"] == glsu.METHOD_FFT and tu[0]["tuned"] == 2, tu[0]
    sur, stats, _ = _run(glsu, synth, _params(glsu), 1e-12, method=method, case=case)
    for k, ((pd, pc), (sd, sc), st) in enumerate(zip(plain, sur, stats)):
        resid = st[2]
        n_checked = 0
        for t, (ys, xs) in enumerate(_tiles(case)):
            if resid[t] > 1e-12:
                assert np.array_equal(sd[ys, xs], pd[ys, xs]), (k, t)
                assert np.array_equal(sc[ys, xs], pc[ys, xs]), (k, t)
                n_checked += 1
        assert n_checked >= len(resid) - 1
    print("%s: probed/flagged %s" % (which, stats[-1][:2]))


def test_probe_residual_matches_host_recomputation(glsu, synth):
    """The device probe's exact WFF2 patch against a full-frame WFF2 of the same LS output."""
    torch = _torch()
    p = _params(glsu)
    _, stats, lsq = _run(glsu, synth, p, 1e9, nframes=2)
    _, _, resid, sites = stats[0]
    z = torch.from_numpy(lsq[0]).cuda()
    exact = torch.empty_like(z)
    w = glsu.WFF2(W, H, "f32", glsu.WffParams(*WP))
    w.run(z.data_ptr(), exact.data_ptr())
    w.close()
    net = glsu.Surrogate(1, W, H, DIL)
    net.params = p
    so = torch.empty_like(z)
    net.forward(z.data_ptr(), so.data_ptr())
    torch.cuda.synchronize()
    ex, sv = exact.cpu().numpy(), so.cpu().numpy()
    net.close()
    for t, (ys, xs) in enumerate(_tiles()):
        py, px = sites[t]
        assert ys.start <= py and px >= xs.start and py < ys.stop and px < xs.stop
        e = ex[py:py + PATCH, px:px + PATCH]
        s = sv[py:py + PATCH, px:px + PATCH]
        m = np.abs(e) >= 0.1
        r = np.sqrt(np.mean(np.angle(s[m] * np.conj(e[m])) ** 2)) if m.any() else 0.0
        assert abs(r - resid[t]) <= 1e-3 + 1e-3 * r, (t, r, resid[t])
    print("probe residuals (rad):", np.round(resid, 3))


@pytest.mark.parametrize("which", ["direct", "fft"])
def test_mixed_tiles_come_from_the_right_path(glsu, synth, which):
    method = glsu.METHOD_DIRECT if which == "direct" else glsu.METHOD_FFT
    p = _params(glsu)
    _, stats, _ = _run(glsu, synth, p, 1e9, nframes=2, method=method)
    resid = stats[0][2]
    tol = float(np.median(resid))
    plain, _, _ = _run(glsu, synth, None, 0, nframes=2, method=method)
    net_only, _, _ = _run(glsu, synth, p, 1e9, nframes=2, method=method)
    mixed, mstats, _ = _run(glsu, synth, p, tol, nframes=2, method=method)
    flagged = resid > tol
    assert 0 < flagged.sum() < len(resid)
    assert mstats[0][1] == flagged.sum()
    for t, (ys, xs) in enumerate(_tiles()):
        ref = plain[0][0] if flagged[t] else net_only[0][0]
        assert np.array_equal(mixed[0][0][ys, xs], ref[ys, xs]), t
    print("%s, tol %.3f: %d of %d tiles recomputed" % (which, tol, flagged.sum(), len(resid)))


def test_probe_overlap_gives_the_serial_result(glsu, synth):
    """The probe sweep on its own stream beside the network (the default), on
    one stream after it, and beside it with the handle on a caller's stream:
    the same phases bit for bit and the same tile decisions."""
    torch = _torch()
    p = _params(glsu)
    frames, phi0, _ = synth.sequence(H, W, 4, seed=21)
    res = []
    for mode in ("overlap", "serial", "user_stream"):
        d = glsu.DPRA(phi0.astype(np.float32), 1, 3, "f32", glsu.WffParams(*WP))
        d.set_surrogate(p, DIL, TILE, PATCH, 0.3)
        if mode == "serial":
            d.set_probe_overlap(False)
        if mode == "user_stream":
            st = torch.cuda.Stream()
            d.set_stream(st.cuda_stream)
        out = []
        for f in frames[1:]:
            dphi, _ = d.per_frame(f)
            out.append(dphi)
            d.update_ref_phi()
        out.append(np.asarray(d.surrogate_stats()))
        d.close()
        res.append(out)
    for other in res[1:]:
        for a, b in zip(res[0], other):
            assert np.array_equal(a, b)
    print("probed, recomputed:", res[0][-1])


def test_surrogate_form_rejects_fp64_and_bad_patches(glsu):
    d = glsu.DPRA(np.zeros((32, 32)), 1, 1, "f64", glsu.WffParams(*WP))
    with pytest.raises(glsu.GlsuError) as e:
        d.set_surrogate(_params(glsu), DIL, 16, 8, 0.05)
    assert e.value.code == glsu.ERR_UNSUPPORTED
    d.close()
    d = glsu.DPRA(np.zeros((32, 32), np.float32), 1, 1, "f32", glsu.WffParams(*WP))
    with pytest.raises(glsu.GlsuError):
        d.set_surrogate(_params(glsu), DIL, 16, 9, 0.05)
    with pytest.raises(glsu.GlsuError):
        d.set_surrogate(_params(glsu), [1, 2, 3, 0, 1, 1, 1, 1], 16, 8, 0.05)
    d.close()
