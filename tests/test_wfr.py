"""WFR2 (windowed Fourier ridges, WFT/WFT2_CPU.cpp:391-694): the FP64 oracle
pinned by analytic cases and an independent direct-sum restatement (CPU),
and the CUDA path (FP32 / FP64) against the oracle (GPU).

Arg-max parity: the ridge frequency is an arg-max over the frequency grid,
so where two frequencies give |sf| within the arithmetic's rounding of each
other FP32 may pick the other one.  The GPU tests compare r everywhere, and
wx, wy, phase where both sides pick the same frequency (at least 99% of the
pixels in FP32, all of them in FP64); cxx, cyy, phase_comp and b depend on a
window of the wx / wy maps and are compared where the whole window agrees.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _direct_wfr(f, sig, lo, hi, step):
    """Literal restatement: sf by direct 2-D sums, the arg-max loop in
    wy-major, wx-minor order with `>=`, the curvature convolutions with the
    border replicated."""
    H, W = f.shape
    s = int(np.floor(3 * sig + 0.5))
    m = np.arange(-s, s + 1)
    g = np.exp(-(m[:, None] ** 2) / (2 * sig * sig) - (m[None, :] ** 2) / (2 * sig * sig))
    g /= np.sqrt((g * g).sum())
    n = int((hi - lo) * (1 / step)) + 1
    fp = np.zeros((H + 2 * s, W + 2 * s), complex)
    fp[s:s + H, s:s + W] = f
    r = np.zeros((H, W))
    wx = np.zeros((H, W))
    wy = np.zeros((H, W))
    ph = np.zeros((H, W))
    for iy in range(n):
        for ix in range(n):
            wyt, wxt = lo + iy * step, lo + ix * step
            k = g * np.exp(1j * (wxt * m[None, :] + wyt * m[:, None]))
            sf = np.zeros((H, W), complex)
            for a in range(2 * s + 1):
                for b in range(2 * s + 1):
                    # f(y - (a - s), x - (b - s)) k(a, b)
                    sf += fp[2 * s - a:2 * s - a + H, 2 * s - b:2 * s - b + W] * k[a, b]
            mag = np.abs(sf)
            t = mag >= r
            r = np.where(t, mag, r)
            wx = np.where(t, wxt, wx)
            wy = np.where(t, wyt, wy)
            ph = np.where(t, np.angle(sf), ph)
    yy = np.clip(np.arange(H)[:, None, None, None] - m[None, None, :, None], 0, H - 1)
    xx = np.clip(np.arange(W)[None, :, None, None] - m[None, None, None, :], 0, W - 1)
    cxx = -(g[None, None] * m[None, None, None, :] * wx[yy, xx]).sum((2, 3)) / (g * m[None, :] ** 2).sum()
    cyy = -(g[None, None] * m[None, None, :, None] * wy[yy, xx]).sum((2, 3)) / (g * m[:, None] ** 2).sum()
    pc = ph - 0.5 * np.arctan(sig * sig * cxx) - 0.5 * np.arctan(sig * sig * cyy)
    pc = np.arctan2(np.sin(pc), np.cos(pc))
    q = 0.25 / np.pi / (sig * sig)
    b = r * ((1 + sig ** 4 * cxx ** 2) * q) ** 0.25 * ((1 + sig ** 4 * cyy ** 2) * q) ** 0.25
    return dict(wx=wx, wy=wy, phase=ph, phase_comp=pc, b=b, r=r, cxx=cxx, cyy=cyy)


def test_oracle_wfr_plane_wave_is_exact():
    H, W = 48, 56
    y, x = np.mgrid[0:H, 0:W]
    f = np.exp(1j * (0.3 * x - 0.2 * y + 0.7))
    res = O.wfr2(f, 5.0, -1, 1, 0.1, 5.0, -1, 1, 0.1)
    c = (slice(15, 33), slice(15, 41))  # beyond one window from the border
    assert np.all(np.abs(res["wx"][c] - 0.3) < 1e-12) and np.all(np.abs(res["wy"][c] + 0.2) < 1e-12)
    assert np.abs(np.angle(np.exp(1j * (res["phase"][c] - np.angle(f[c]))))).max() < 1e-12
    assert np.abs(res["cxx"][c]).max() < 1e-12 and np.abs(res["cyy"][c]).max() < 1e-12
    # amplitude: b = r (4 pi s^2)^(-1/2) -> 1 for a unit fringe (up to the 3-sigma truncation)
    assert np.abs(res["b"][c] - 1).max() < 5e-3


def test_oracle_wfr_matches_direct_sums():
    rng = np.random.default_rng(4)
    H, W = 13, 17
    y, x = np.mgrid[0:H, 0:W]
    f = np.exp(1j * (0.4 * x + 0.02 * x * y - 0.3 * y)) + 0.1 * (rng.standard_normal((H, W)) +
                                                                 1j * rng.standard_normal((H, W)))
    ref = _direct_wfr(f, 1.4, -1.0, 1.0, 0.5)
    res = O.wfr2(f, 1.4, -1.0, 1.0, 0.5, 1.4, -1.0, 1.0, 0.5)
    for k in ("r", "b"):
        assert np.abs(res[k] - ref[k]).max() < 1e-12 * np.abs(ref[k]).max(), k
    for k in ("wx", "wy", "cxx", "cyy"):
        assert np.abs(res[k] - ref[k]).max() < 1e-12, k
    for k in ("phase", "phase_comp"):
        assert np.abs(np.angle(np.exp(1j * (res[k] - ref[k])))).max() < 1e-11, k


def test_oracle_wfr_curvature_of_a_chirp():
    """phi = a x^2: the local frequency 2 a x, so cxx ~ 2 a inside."""
    H, W, a = 40, 96, 0.004
    x = np.arange(W)[None, :].repeat(H, 0)
    f = np.exp(1j * a * (x - W / 2) ** 2)
    res = O.wfr2(f, 4.0, -0.5, 0.5, 0.02, 4.0, -0.2, 0.2, 0.02)
    c = (slice(14, 26), slice(30, 66))
    assert abs(np.median(res["cxx"][c]) - 2 * a) < 0.1 * 2 * a
    assert np.abs(res["cyy"][c]).max() < 1e-12


# ---------------------------------------------------------------------------
def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def _run_gpu(glsu, f, prec, sigx, lo, hi, step, sigy=None, ylo=None, yhi=None, ystep=None):
    torch = _torch()
    H, W = f.shape
    sigy = sigx if sigy is None else sigy
    ylo, yhi, ystep = (lo, hi, step) if ylo is None else (ylo, yhi, ystep)
    cdt, rdt = (torch.complex64, torch.float32) if prec == "f32" else (torch.complex128, torch.float64)
    df = torch.from_numpy(f).to(cdt).cuda()
    maps = {k: torch.zeros((H, W), dtype=rdt, device="cuda") for k in glsu.WFR_FIELDS}
    p = glsu.WffParams(sigma_x=sigx, wxl=lo, wxh=hi, wxi=step, sigma_y=sigy, wyl=ylo, wyh=yhi, wyi=ystep, thr=0)
    w = glsu.WFR2(W, H, prec, p)
    w.run(df.data_ptr(), {k: v.data_ptr() for k, v in maps.items()})
    w.close()
    return {k: v.cpu().numpy().astype(np.float64) for k, v in maps.items()}


def _window_agrees(same, s):
    """Pixels whose (2s+1)^2 window (border replicated) agrees entirely."""
    H, W = same.shape
    yy = np.clip(np.arange(H)[:, None] + np.arange(-s, s + 1)[None, :], 0, H - 1)
    xx = np.clip(np.arange(W)[:, None] + np.arange(-s, s + 1)[None, :], 0, W - 1)
    return same[yy[:, :, None, None], xx[None, None, :, :]].transpose(0, 2, 1, 3).all((2, 3))


def _field(H, W, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W]
    phi = 0.25 * x - 0.15 * y + 2.0 * np.sin(x / 17.0) * np.cos(y / 23.0)
    return np.exp(1j * phi) + 0.05 * (rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W)))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f32", "f64"])
# grid steps are binary fractions so that the FP32 handle (which counts the
# frequencies in float, as WFT2_CUDAF does) and the oracle sweep the same grid
@pytest.mark.parametrize("H,W,sig,grid,sigy,ygrid", [
    (70, 90, 4.0, (-1.0, 1.0, 0.125), None, None),
    (45, 133, 3.0, (-0.75, 0.75, 0.25), 5.0, (-0.5, 0.5, 0.125)),  # ragged, sigma_x != sigma_y
    (150, 40, 6.0, (0.25, 0.25, 0.125), None, None),              # one frequency
])
def test_wfr_gpu_matches_oracle(glsu, prec, H, W, sig, grid, sigy, ygrid):
    f = _field(H, W, H + W)
    ys = sig if sigy is None else sigy
    yg = grid if ygrid is None else ygrid
    got = _run_gpu(glsu, f, prec, sig, *grid, sigy=ys, ylo=yg[0], yhi=yg[1], ystep=yg[2])
    ref = O.wfr2(f, sig, *grid, ys, *yg)
    rtol = 1e-5 if prec == "f32" else 1e-12
    atol_ph = 1e-3 if prec == "f32" else 1e-10
    assert np.abs(got["r"] - ref["r"]).max() <= rtol * ref["r"].max()
    same = (np.abs(got["wx"] - ref["wx"]) < 1e-6) & (np.abs(got["wy"] - ref["wy"]) < 1e-6)
    print("%s %dx%d: frequency agreement %.5f" % (prec, H, W, same.mean()))
    assert same.mean() >= (0.99 if prec == "f32" else 1.0)
    dph = np.abs(np.angle(np.exp(1j * (got["phase"] - ref["phase"]))))
    assert dph[same].max() < atol_ph
    s = max(int(np.floor(3 * sig + 0.5)), int(np.floor(3 * ys + 0.5)))
    ok = _window_agrees(same, s)
    assert ok.mean() > 0.9
    for k in ("cxx", "cyy"):
        assert np.abs(got[k] - ref[k])[ok].max() < (1e-6 if prec == "f32" else 1e-12), k
    dpc = np.abs(np.angle(np.exp(1j * (got["phase_comp"] - ref["phase_comp"]))))
    assert dpc[ok].max() < atol_ph
    assert np.abs(got["b"] - ref["b"])[ok].max() <= rtol * 10 * ref["b"].max()


@pytest.mark.gpu
def test_wfr_gpu_default_grid_plane_wave(glsu):
    """The reference's WFR defaults (sigma 10, 161 x 161 frequencies on [-2, 2]):
    a plane wave on the grid is found exactly inside the image."""
    H, W = 96, 128
    y, x = np.mgrid[0:H, 0:W]
    f = np.exp(1j * (0.475 * x - 1.2 * y))
    got = _run_gpu(glsu, f, "f32", 10.0, -2.0, 2.0, 0.025)
    c = (slice(30, 66), slice(30, 98))
    assert np.all(np.abs(got["wx"][c] - 0.475) < 1e-6) and np.all(np.abs(got["wy"][c] + 1.2) < 1e-6)
    assert np.abs(np.angle(np.exp(1j * (got["phase"][c] - np.angle(f[c]))))).max() < 1e-3
