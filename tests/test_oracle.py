"""CPU tests of the FP64 oracle: pinned against the reference's golden data
(tests/golden, made by tests/golden/make_golden.py) and cross-checked against
independent numpy formulations."""
import json
import os

import numpy as np
import pytest
from scipy.signal import fftconvolve

from conftest import GOLDEN


def test_fft_lut_matches_reference_table(oracle):
    ref = json.load(open(os.path.join(GOLDEN, "fft_lut.json")))["sizes"]
    assert oracle.fft_lut() == ref


def test_first_greater(oracle):
    lut = oracle.fft_lut()
    for x in [-5, 0, 1, 2, 3, 315, 316, 320, 321, 1084, 2048, 4095, 4096]:
        i = oracle.first_greater(x)
        assert lut[i] >= x and (i == 0 or lut[i - 1] < x)
    assert oracle.first_greater(4097) == -1
    assert oracle.opt_fft_size(256 + 60) == 320
    assert oracle.opt_fft_size(1024 + 60) == 1120
    assert oracle.opt_fft_size(2048 + 90) == 2160


def test_frequency_grid_matches_reference_csv(oracle):
    g = np.load(os.path.join(GOLDEN, "xfyf.npz"))
    xf, yf = oracle.freq_grid(64, 50)
    assert np.array_equal(xf, g["xf"]) and np.array_equal(yf, g["yf"])


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 12, 28, 50, 98, 320, 448, 576, 1120, 2160])
def test_fft_vs_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(oracle.fft1d(x) - ref).max() / scale < 1e-14
    assert np.abs(oracle.fft1d(x, inverse=True) - np.fft.ifft(x) * n).max() / scale < 1e-14


def test_fft2_vs_numpy(oracle):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((50, 64)) + 1j * rng.standard_normal((50, 64))
    assert np.abs(oracle.fft2d(x) - np.fft.fft2(x)).max() < 1e-11


def _round_half_away(v):
    return int(np.floor(v + 0.5))


def wff_direct(f, sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, thr, count):
    """Independent restatement: direct 'same' convolutions with the truncated window."""
    sx, sy = _round_half_away(3 * sigx), _round_half_away(3 * sigy)
    y, x = np.meshgrid(np.arange(-sy, sy + 1), np.arange(-sx, sx + 1), indexing="ij")
    g = np.exp(-x * x / 2 / sigx / sigx - y * y / 2 / sigy / sigy)
    g = g / np.sqrt((g * g).sum())
    if thr < 0:
        thr = 6 * np.sqrt(np.mean(np.abs(f) ** 2) / 3)
    out = np.zeros(f.shape, complex)
    for iy in range(count(wyl, wyh, wyi)):
        for ix in range(count(wxl, wxh, wxi)):
            w = g * np.exp(1j * ((wxl + ix * wxi) * x + (wyl + iy * wyi) * y))
            sf = fftconvolve(f, w, mode="same")
            sf = sf * (np.abs(sf) >= thr)
            out += fftconvolve(sf, w, mode="same")
    return out * 0.25 / np.pi ** 2 * wxi * wyi


@pytest.mark.parametrize("shape,params", [
    ((37, 44), (3.0, -1.0, 1.0, 0.25, 4.0, -0.8, 0.8, 0.2, 0.5)),
    ((32, 32), (2.0, -0.5, 0.5, 0.5, 2.0, -0.5, 0.5, 0.5, 0.0)),
    ((21, 30), (3.0, 0.3, 0.3, 0.1, 3.0, -0.2, -0.2, 0.1, 0.3)),  # single frequency
    ((40, 28), (2.5, -1.0, 1.0, 0.4, 3.5, -1.2, 1.2, 0.6, -1.0)),  # automatic threshold
])
def test_wff_fft_formulation_equals_direct_convolution(oracle, shape, params):
    rng = np.random.default_rng(sum(shape))
    phi = np.cumsum(rng.standard_normal(shape) * 0.3, axis=1)
    f = np.exp(1j * phi) * (1 + 0.1 * rng.standard_normal(shape))
    a, thr = oracle.wff2(f, *params)
    b = wff_direct(f, *params, count=oracle.wff_count)
    assert np.abs(a - b).max() < 1e-12 * max(1, np.abs(b).max())
    if params[-1] < 0:
        assert abs(thr - 6 * np.sqrt(np.mean(np.abs(f) ** 2) / 3)) < 1e-12


def test_wff_padding_out_of_range(oracle):
    f = np.ones((8, 4090), complex)
    with pytest.raises(ValueError):
        oracle.wff2(f, 10, -1, 1, 0.5, 10, -1, 1, 0.5, 0.1)


def test_wff_frequency_count(oracle):
    assert oracle.wff_count(-1.0, 1.0, 0.1) == 21
    assert oracle.wff_count(-1.5, 1.5, 0.1) == 31
    assert oracle.wff_count(-0.15, 0.15, 0.05) == 7


def dpra_numpy(img, phiref, r):
    """Loop restatement of DPRA/dpra_cpu.cpp:162-230 with radius r."""
    H, W = img.shape
    z = np.zeros((H, W), complex)
    for i in range(H):
        for j in range(W):
            sl = (slice(max(i - r, 0), min(i + r, H - 1) + 1), slice(max(j - r, 0), min(j + r, W - 1) + 1))
            c, s, ft = np.cos(phiref[sl]).ravel(), np.sin(phiref[sl]).ravel(), img[sl].ravel()
            A = np.array([[(2 * r + 1) ** 2, c.sum(), s.sum()], [c.sum(), (c * c).sum(), (c * s).sum()],
                          [s.sum(), (c * s).sum(), (s * s).sum()]])
            b = np.array([ft.sum(), (ft * c).sum(), (ft * s).sum()])
            x = np.linalg.solve(A, b)
            z[i, j] = np.exp(1j * np.arctan2(-x[2], x[1]))
    return z


@pytest.mark.parametrize("r", [1, 2, 3])
def test_dpra_ls_vs_numpy(oracle, synth, r):
    frames, phi0, _ = synth.sequence(19, 23, 2, seed=r)
    z = oracle.dpra_ls(frames[1].astype(np.float64), phi0, r)
    zr = dpra_numpy(frames[1].astype(np.float64), phi0, r)
    assert np.abs(np.angle(z * np.conj(zr))).max() < 1e-9


def test_dpra_update(oracle):
    rng = np.random.default_rng(5)
    filt = rng.standard_normal((6, 7)) + 1j * rng.standard_normal((6, 7))
    pr, dpr = rng.uniform(-3, 3, (6, 7)), rng.uniform(-3, 3, (6, 7))
    pc, dp = oracle.dpra_update(filt, pr, dpr)
    t = np.angle(filt)
    assert np.allclose(dp, dpr + t, atol=1e-14)
    assert np.allclose(pc, np.angle(np.exp(1j * (t + pr))), atol=1e-12)


def test_aia_pixel_solve_matches_reference_phi_cpu_csv(oracle):
    """Test/Phi_CPU.csv: the first per-pixel AIA solve on Test/{1,2,3}.bmp with
    deltas {0.8622, 0.3188, -1.3077} (float), printed to 6 significant digits."""
    g = np.load(os.path.join(GOLDEN, "aia_bmp.npz"))
    frames = g["frames"].astype(np.float64)
    _, x = oracle.aia_phi_solve(frames, g["deltas0"].astype(np.float64))
    xs = x[g["pix"]]
    ref = g["x"]
    assert np.abs(xs - ref).max() < 2e-3
    assert (np.abs(xs - ref) <= 1e-5 * np.abs(ref) + 1e-3).all()


def test_aia_recovers_known_shifts(oracle, synth):
    frames, phi, shifts = synth.aia_frames(64, 64, 5, seed=1, noise=0.0, bump=False)
    d0 = np.concatenate([[0.0], np.random.default_rng(0).standard_normal(4)])
    est, d, it, err = oracle.aia(frames.astype(np.float64), d0, max_iter=200, max_err=1e-12)
    true_rel = synth.wrap(shifts - shifts[0])
    # AIA's solution is defined up to the sign convention (phi, d) -> (-phi, -d)
    e = min(np.abs(synth.phase_err(d, true_rel)).max(), np.abs(synth.phase_err(-d, true_rel)).max())
    assert e < 1e-6, (d, true_rel)


def test_sequence_reference_update_rate(oracle, synth):
    """DPRA_CPU::operator(): the reference is updated after frame i when i % rr == 0."""
    frames, phi0, _ = synth.sequence(24, 24, 4, seed=2)
    wp = oracle.WffParams(2.0, -0.5, 0.5, 0.5, 2.0, -0.5, 0.5, 0.5, 0.1)
    pcs, dps = oracle.glsu_sequence(frames.astype(np.float64), phi0, 1, wp, rr=2)
    # frame 1 uses the reference set after frame 0; frame 2 the same one
    pc1, dp1, _, _ = oracle.glsu_frame(frames[1].astype(np.float64), pcs[0], dps[0], 1, wp)
    pc2, dp2, _, _ = oracle.glsu_frame(frames[2].astype(np.float64), pcs[0], dps[0], 1, wp)
    assert np.allclose(pcs[1], pc1) and np.allclose(dps[2], dp2)


def test_dpra_stable_and_literal_forms_agree_where_well_posed(oracle, synth):
    """or_dpra_ls (centre-shifted Schur complement) and or_dpra_ls_raw (the
    literal raw-sum 3x3 of DPRA/dpra_cpu.cpp) solve the same normal
    equations; they agree to 1e-9 rad wherever the 3x3 system is
    well-conditioned, and the literal form drifts where it is not."""
    frames, phi0, _ = synth.sequence(96, 96, 2, seed=4)
    img = frames[1].astype(np.float64)
    for r in (1, 3):
        zs = oracle.dpra_ls(img, phi0, r)
        zr = oracle.dpra_ls(img, phi0, r, raw=True)
        kap = oracle.dpra_kappa(phi0, r)
        e = np.abs(np.angle(zs * np.conj(zr)))
        good = kap > 1e-3
        assert good.mean() > 0.2
        assert e[good].max() < 1e-9, (r, e[good].max())


def unwrap_matlab(p, sx, sy):
    """Loop restatement of MatLab/fp_unwrapping.m:41-71 (0-based starts)."""
    p = np.array(p, np.float64)
    m, n = p.shape

    def u1(v, s):
        v = v.copy()
        for i in range(s + 1, len(v)):
            v[i] += np.trunc((v[i - 1] - v[i]) / 2 / np.pi + np.copysign(0.5, (v[i - 1] - v[i]))) * 2 * np.pi
        for i in range(s - 1, -1, -1):
            v[i] += np.trunc((v[i + 1] - v[i]) / 2 / np.pi + np.copysign(0.5, (v[i + 1] - v[i]))) * 2 * np.pi
        return v
    p[:, sy] = u1(p[:, sy], sx)
    for i in range(m):
        p[i, :] = u1(p[i, :], sy)
    return p


@pytest.mark.parametrize("shape,start", [((40, 50), (10, 20)), ((33, 17), (0, 0)), ((1, 30), (0, 29)),
                                         ((25, 1), (12, 0))])
def test_unwrap_matches_matlab_loops(oracle, shape, start):
    rng = np.random.default_rng(sum(shape))
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    true = 0.4 * x - 0.3 * y + 2 * np.sin(x / 7.0) + 0.2 * rng.standard_normal(shape)
    w = np.angle(np.exp(1j * true))
    a = oracle.unwrap2(w, *start)
    b = unwrap_matlab(w, *start)
    assert np.array_equal(a, b)
    # a smooth field is recovered up to one 2pi offset
    smooth = np.angle(np.exp(1j * (0.4 * x - 0.3 * y)))
    u = oracle.unwrap2(smooth, *start)
    d = u - (0.4 * x - 0.3 * y)
    assert np.allclose(d, d[start], atol=1e-12)


def test_aia_iterates_drift_along_the_common_rotation(oracle):
    """AIA's phase and frame steps leave a common rotation of all shifts
    free.  On the synthetic 5-frame data the iterates drift along it by a
    constant step per iteration, so the reference's measure max|delta - old|
    (aia_cpu.cpp:249-263) stays constant and the run stops at the cap, while
    the normalised shifts have settled; the measure of AIA_CUDAF_YC2
    (aia_cudaf_v2.cu:665-677), relative to the first shift, converges, to the
    same normalised shifts and phase."""
    import glsu
    from glsu import synth
    fr, _, _ = synth.aia_frames(96, 80, 5, seed=1000)
    f = fr.astype(np.float64)
    d0 = glsu.random_deltas(5, 1000).astype(np.float64)
    _, da, it_a, err_a = oracle.aia(f, d0, 40, 1e-4)
    _, db, it_b, err_b = oracle.aia(f, d0, 41, 1e-4)
    assert it_a == 40 and it_b == 41 and abs(err_a - err_b) < 1e-6 * err_a
    assert err_a > 1e-4
    assert np.abs(da - db).max() < 1e-9                      # settled, although the measure is not small
    pr, dr, it_r, err_r = oracle.aia(f, d0, 40, 1e-4, relative=True)
    print("abs measure: %d iterations, err %.3g; relative measure: %d iterations, err %.3g" % (it_a, err_a, it_r,
                                                                                            err_r))
    assert it_r < 40 and err_r <= 1e-4
    assert np.abs(np.angle(np.exp(1j * (dr - da)))).max() < 1e-3  # within a few stopping tolerances
