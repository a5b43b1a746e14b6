"""FP64 CPU oracle for the G-LS3U hot path -- TEST INFRASTRUCTURE ONLY.

This module wraps ``glsu_oracle.c`` (a restatement of the reference's own CPU
code: ``DPRA/dpra_cpu.cpp``, ``WFT/WFT2_CPU.cpp``, ``AIA/aia_cpu.cpp``) with
ctypes.  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may import it, and only as the checker or the timed CPU
baseline.  The product library never calls it.

``build()`` compiles the C file with gcc into ``oracle/_build/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "glsu_oracle.c")
_SRCS = [_SRC, os.path.join(_HERE, "glsu_oracle_f32.c"), os.path.join(_HERE, "or_fft_gen.h")]
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "libglsu_oracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc -O3 -fopenmp) and return its path."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(f) for f in _SRCS)):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11"] + [f for f in _SRCS if f.endswith(".c")] + [
        "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            L = ctypes.CDLL(path)
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int)
            c_int, c_double = ctypes.c_int, ctypes.c_double
            L.or_fft_lut.argtypes = [ip, c_int]
            L.or_first_greater.argtypes = [c_int]
            L.or_opt_fft_size.argtypes = [c_int]
            L.or_freq_grid.argtypes = [c_int, c_int, dp, dp]
            L.or_fft1d.argtypes = [c_int, dp, c_int]
            L.or_fft2d.argtypes = [c_int, c_int, dp, c_int]
            L.or_wff_count.argtypes = [c_double, c_double, c_double]
            L.or_wff2.argtypes = [c_int, c_int, dp, c_double, c_double, c_double, c_double,
                                  c_double, c_double, c_double, c_double, c_double, dp, dp,
                                  c_int, c_int, c_int]
            L.or_dpra_ls.argtypes = [c_int, c_int, c_int, dp, dp, dp, c_int]
            L.or_dpra_ls_raw.argtypes = [c_int, c_int, c_int, dp, dp, dp, c_int]
            L.or_dpra_update.argtypes = [c_int, dp, dp, dp, dp, dp]
            L.or_aia_phi_solve.argtypes = [c_int, c_int, dp, dp, dp, dp]
            L.or_aia.argtypes = [c_int, c_int, dp, dp, c_int, c_double, dp, ip, dp]
            L.or_aia_mode.argtypes = [c_int, c_int, dp, dp, c_int, c_double, c_int, dp, ip, dp]
            L.or_unwrap2.argtypes = [c_int, c_int, dp, c_int, c_int]
            L.or_wfr2.argtypes = [c_int, c_int, dp] + [c_double] * 8 + [dp] * 8 + [c_int]
            fp = ctypes.POINTER(ctypes.c_float)
            L.orf_dpra_ls.argtypes = [c_int, c_int, c_int, fp, fp, fp, c_int]
            L.orf_dpra_update.argtypes = [c_int, fp, fp, fp, fp, fp]
            L.orf_wff2.argtypes = [c_int, c_int, fp] + [c_double] * 9 + [fp, c_int, c_int, c_int]
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# --------------------------------------------------------------------------
def fft_lut() -> list[int]:
    buf = (ctypes.c_int * 512)()
    n = lib().or_fft_lut(buf, 512)
    return list(buf[:n])


def first_greater(x: int) -> int:
    return lib().or_first_greater(int(x))


def opt_fft_size(x: int) -> int:
    return lib().or_opt_fft_size(int(x))


def freq_grid(W: int, H: int):
    xf = np.zeros((H, W)); yf = np.zeros((H, W))
    lib().or_freq_grid(W, H, _dp(xf), _dp(yf))
    return xf, yf


def fft1d(x, inverse=False):
    a = _c128(x).copy()
    if lib().or_fft1d(a.size, _dp(a.view(np.float64)), int(inverse)):
        raise ValueError("unsupported FFT length")
    return a


def fft2d(x, inverse=False):
    a = _c128(x).copy()
    H, W = a.shape
    if lib().or_fft2d(W, H, _dp(a.view(np.float64)), int(inverse)):
        raise ValueError("unsupported FFT size")
    return a


def wff_count(lo, hi, step) -> int:
    return lib().or_wff_count(float(lo), float(hi), float(step))


def wff2(f, sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, thr, nthreads=0, ky=None):
    """WFF2 of complex H x W ``f`` (reference argument order: sigma, low, high, step).

    Returns (filtered, threshold_used).  ``ky=(k0, k1)`` sweeps only frequency
    rows k0..k1-1 (bounded CPU samples)."""
    a = _c128(f)
    H, W = a.shape
    out = np.zeros((H, W), np.complex128)
    thr_used = ctypes.c_double(0)
    k0, k1 = (ky if ky is not None else (0, -1))
    rc = lib().or_wff2(W, H, _dp(a.view(np.float64)), sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi,
                       float(thr), _dp(out.view(np.float64)), ctypes.byref(thr_used),
                       int(nthreads), int(k0), int(k1))
    if rc == -1:
        raise ValueError("FFT padding is out of range [4096]")
    if rc:
        raise MemoryError("oracle allocation failed")
    return out, thr_used.value


WFR_FIELDS = ("wx", "wy", "phase", "phase_comp", "b", "r", "cxx", "cyy")


def wfr2(f, sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, nthreads=0):
    """WFR2 (windowed Fourier ridges) of complex H x W ``f``
    (WFT/WFT2_CPU.cpp:391-694).  Returns a dict of the eight H x W result
    maps of WFT2_HostResults: wx, wy, phase, phase_comp, b, r, cxx, cyy."""
    a = _c128(f)
    H, W = a.shape
    out = {k: np.zeros((H, W), np.float64) for k in WFR_FIELDS}
    rc = lib().or_wfr2(W, H, _dp(a.view(np.float64)), sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi,
                       *[_dp(out[k]) for k in WFR_FIELDS], int(nthreads))
    if rc == -1:
        raise ValueError("FFT padding is out of range [4096]")
    if rc:
        raise MemoryError("oracle allocation failed")
    return out


def dpra_ls(img, phiref, r=1, nthreads=0, raw=False):
    """exp(j dphi) of DPRA's windowed least squares.  raw=True: the literal
    raw-sum 3x3 form of DPRA/dpra_cpu.cpp; default: the same normal
    equations solved through the centre-shifted Schur complement."""
    img = _f64(img); phiref = _f64(phiref)
    H, W = img.shape
    z = np.zeros((H, W), np.complex128)
    fn = lib().or_dpra_ls_raw if raw else lib().or_dpra_ls
    fn(W, H, int(r), _dp(img), _dp(phiref), _dp(z.view(np.float64)), int(nthreads))
    return z


def dpra_kappa(phiref, r=1):
    """Conditioning of DPRA's reduced 2x2 normal matrix per pixel:
    det / trace^2 of [[a, b], [b, d]] (<= 1/4; small = ill-conditioned)."""
    phi = np.asarray(phiref, np.float64)
    H, W = phi.shape
    c, s = np.cos(phi), np.sin(phi)
    n0 = (2 * r + 1) ** 2
    ones = np.ones((H, W))
    sums = {}
    for name, v in (("c", c), ("s", s), ("cc", c * c), ("ss", s * s), ("cs", c * s), ("n", ones)):
        p = np.pad(v, r)
        acc = np.zeros((H, W))
        for dy in range(2 * r + 1):
            for dx in range(2 * r + 1):
                acc += p[dy:dy + H, dx:dx + W]
        sums[name] = acc
    a = sums["cc"] - sums["c"] ** 2 / n0
    d = sums["ss"] - sums["s"] ** 2 / n0
    b = sums["cs"] - sums["c"] * sums["s"] / n0
    return (a * d - b * b) / np.maximum((a + d) ** 2, 1e-300)


def dpra_update(filtered, phiref, dphiref):
    filtered = _c128(filtered); phiref = _f64(phiref); dphiref = _f64(dphiref)
    pc = np.zeros_like(phiref); dp_ = np.zeros_like(phiref)
    lib().or_dpra_update(phiref.size, _dp(filtered.view(np.float64)), _dp(phiref), _dp(dphiref),
                         _dp(pc), _dp(dp_))
    return pc, dp_


def aia_phi_solve(frames, deltas):
    f = _f64(frames)
    M = f.shape[0]
    N = f[0].size
    d = _f64(deltas)
    phi = np.zeros(N); x = np.zeros(3 * N)
    info = lib().or_aia_phi_solve(M, N, _dp(f), _dp(d), _dp(phi), _dp(x))
    if info:
        raise ValueError("matrix not positive definite")
    return phi.reshape(f.shape[1:]), x.reshape(-1, 3)


def aia(frames, deltas, max_iter=20, max_err=1e-4, relative=False):
    """AIA (aia_cpu.cpp:16-100); relative=True measures convergence as
    AIA_CUDAF_YC2 does (aia_cudaf_v2.cu:665-677)."""
    f = _f64(frames)
    M = f.shape[0]
    N = f[0].size
    d = _f64(deltas).copy()
    phi = np.zeros(N)
    it = ctypes.c_int(0); err = ctypes.c_double(0)
    info = lib().or_aia_mode(M, N, _dp(f), _dp(d), int(max_iter), float(max_err), int(relative), _dp(phi),
                             ctypes.byref(it), ctypes.byref(err))
    if info:
        raise ValueError("matrix not positive definite")
    return phi.reshape(f.shape[1:]), d, it.value, err.value


def unwrap2(p, start_row=None, start_col=None):
    """Line-scanning unwrapping of MatLab/fp_unwrapping.m (0-based starts;
    default: MATLAB's round(m/2), round(n/2) converted to 0-based)."""
    a = _f64(p).copy()
    H, W = a.shape
    if start_row is None:
        start_row = int(np.floor(H / 2 + 0.5)) - 1
    if start_col is None:
        start_col = int(np.floor(W / 2 + 0.5)) - 1
    lib().or_unwrap2(W, H, _dp(a), int(start_row), int(start_col))
    return a


class WffParams:
    """WFF2 parameters in the reference's C++ order (sigma, low, high, step)."""

    def __init__(self, sigx=10.0, wxl=-1.0, wxh=1.0, wxi=0.1, sigy=10.0, wyl=-1.0, wyh=1.0,
                 wyi=0.1, thr=0.2):
        self.sigx, self.wxl, self.wxh, self.wxi = sigx, wxl, wxh, wxi
        self.sigy, self.wyl, self.wyh, self.wyi = sigy, wyl, wyh, wyi
        self.thr = thr

    def tuple(self):
        return (self.sigx, self.wxl, self.wxh, self.wxi, self.sigy, self.wyl, self.wyh,
                self.wyi, self.thr)


def glsu_frame(img, phiref, dphiref, r, wp: WffParams, nthreads=0, ky=None):
    """One G-LS3U frame: DPRA LS -> WFF2 -> update.  Returns (phicurr, dphi, z, filtered)."""
    z = dpra_ls(img, phiref, r, nthreads)
    filt, _ = wff2(z, *wp.tuple(), nthreads=nthreads, ky=ky)
    pc, dphi = dpra_update(filt, phiref, dphiref)
    return pc, dphi, z, filt


def glsu_sequence(frames, phi0, r, wp: WffParams, rr=1, nthreads=0):
    """Frame loop of DPRA_CPU::operator() (DPRA/dpra_cpu.cpp:58-89):
    the reference is updated after frame i when i % rr == 0."""
    phiref = _f64(phi0).copy()
    dphiref = np.zeros_like(phiref)
    pcs, dps = [], []
    for i, img in enumerate(frames):
        pc, dphi, _, _ = glsu_frame(img, phiref, dphiref, r, wp, nthreads)
        pcs.append(pc); dps.append(dphi)
        if i % rr == 0:
            phiref, dphiref = pc, dphi
    return np.stack(pcs), np.stack(dps)


# ---------------------------------------------------------------------------
# FP32 variant (glsu_oracle_f32.c): the reference's float CPU classes
# (DPRA/dpra_cpuf.cpp, WFT/WFT2_CPUf.cpp), for the timed CPU baseline.
# ---------------------------------------------------------------------------
def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def dpra_ls_f32(img, phiref, r=1, nthreads=0):
    img, phiref = _f32(img), _f32(phiref)
    H, W = img.shape
    z = np.empty((H, W), np.complex64)
    lib().orf_dpra_ls(W, H, r, _fptr(img), _fptr(phiref), _fptr(z.view(np.float32)), nthreads)
    return z


def wff2_f32(f, sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, thr, nthreads=0, ky=None):
    f = np.ascontiguousarray(f, dtype=np.complex64)
    H, W = f.shape
    out = np.empty((H, W), np.complex64)
    ky0, ky1 = ky if ky is not None else (0, -1)
    rc = lib().orf_wff2(W, H, _fptr(f.view(np.float32)), sigx, wxl, wxh, wxi, sigy, wyl, wyh, wyi, thr,
                        _fptr(out.view(np.float32)), nthreads, ky0, ky1)
    if rc:
        raise RuntimeError("orf_wff2 failed (%d)" % rc)
    return out


def dpra_update_f32(filtered, phiref, dphiref):
    filtered = np.ascontiguousarray(filtered, dtype=np.complex64)
    phiref, dphiref = _f32(phiref), _f32(dphiref)
    pc, dp = np.empty_like(phiref), np.empty_like(phiref)
    lib().orf_dpra_update(phiref.size, _fptr(filtered.view(np.float32)), _fptr(phiref), _fptr(dphiref), _fptr(pc),
                          _fptr(dp))
    return pc, dp


def glsu_frame_f32(img, phiref, dphiref, r, wp: WffParams, nthreads=0, ky=None):
    """One frame of the FP32 CPU variant.  Returns (phicurr, dphi, z, filtered)."""
    z = dpra_ls_f32(img, phiref, r, nthreads)
    filt = wff2_f32(z, *wp.tuple(), nthreads=nthreads, ky=ky)
    pc, dphi = dpra_update_f32(filt, phiref, dphiref)
    return pc, dphi, z, filt

