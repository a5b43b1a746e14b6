"""The FP32 CPU variant (oracle/glsu_oracle_f32.c: the reference's float CPU
classes DPRA_CPUF and WFT2_cpuF restated) against the FP64 oracle.  It is the
timed FP32 CPU baseline, so it is pinned here: its float FFT and WFF2 agree
with the FP64 oracle to FP32 rounding, and its least squares (raw float
window sums and a float 3x3 solve, as DPRA/dpra_cpuf.cpp:130-230) where the
3x3 system is well conditioned."""
import numpy as np

from oracle import oracle as O


def test_f32_wff2_matches_fp64_oracle():
    rng = np.random.default_rng(2)
    H, W = 70, 90
    y, x = np.mgrid[0:H, 0:W]
    f = np.exp(1j * (0.3 * x - 0.2 * y + np.sin(x / 11.0))) + 0.1 * (rng.standard_normal((H, W)) +
                                                                       1j * rng.standard_normal((H, W)))
    for p in ((4.0, -1.0, 1.0, 0.25, 4.0, -1.0, 1.0, 0.25, 0.5), (5.0, -1.0, 1.0, 0.4, 6.0, -0.8, 0.8, 0.4, -1.0)):
        ref, _ = O.wff2(f.astype(np.complex64).astype(np.complex128), *p)
        got = O.wff2_f32(f.astype(np.complex64), *p)
        m = np.abs(ref) >= 0.05 * np.abs(ref).max()
        assert np.abs(np.angle(got[m] * np.conj(ref[m]))).max() < 1e-4
        assert np.abs(got - ref).max() < 1e-5 * np.abs(ref).max()


def test_f32_least_squares_where_well_conditioned():
    """Steep fringes (phi_ref changing by about 1 rad per pixel) make the
    3x3 normal equations well conditioned; there the float form follows the
    FP64 solution.  On smooth phases the float raw sums lose it (measured:
    0.1 to 0.4 rad RMS on the benchmark generator), which is the reference
    float class's own precision."""
    rng = np.random.default_rng(5)
    H, W = 48, 64
    y, x = np.mgrid[0:H, 0:W]
    phiref = 1.1 * x + 0.7 * y + 0.3 * np.sin(y / 5.0)
    dphi = 0.4 + 0.2 * np.cos(x / 9.0)
    img = 0.5 + 0.4 * np.cos(phiref + dphi) + 0.01 * rng.standard_normal((H, W))
    for r in (1, 3):
        ref = O.dpra_ls(img.astype(np.float32).astype(np.float64), phiref.astype(np.float32).astype(np.float64), r)
        got = O.dpra_ls_f32(img, phiref, r)
        e = np.abs(np.angle(got * np.conj(ref)))
        assert e.max() < 1e-3, (r, e.max())


def test_f32_frame_update():
    rng = np.random.default_rng(6)
    filt = (rng.standard_normal((20, 30)) + 1j * rng.standard_normal((20, 30))).astype(np.complex64)
    pref = rng.uniform(-np.pi, np.pi, (20, 30)).astype(np.float32)
    dref = rng.standard_normal((20, 30)).astype(np.float32)
    pc, dp = O.dpra_update_f32(filt, pref, dref)
    pc64, dp64 = O.dpra_update(filt.astype(np.complex128), pref.astype(np.float64), dref.astype(np.float64))
    assert np.abs(np.angle(np.exp(1j * (pc - pc64)))).max() < 1e-5
    assert np.abs(dp - dp64).max() < 1e-5
