"""Python host interface of the GB300 G-LS3U hot path (ctypes over ``libglsu.so``).

The classes mirror the reference's C++ interfaces (paths inside the
reference project):

- :class:`WFF2` -- ``WFT_FPA::WFT::WFT2_CUDAF`` / ``WFT2_CUDA`` with
  ``WFT_TYPE::WFF`` (``WFT/WFT2_CUDAf.h:11-40``); arguments in the C++ order
  sigma, low, high, step.
- :class:`DPRA` -- ``DPRA::DPRA_CUDAF`` (``DPRA/dpra_cudaf.h:21-46``) and the FP64
  ``DPRA::DPRA_CUDA``, with ``DPRA_CPU::operator()`` semantics for sequences
  (``DPRA/dpra_cpu.cpp:58-89``).
- :class:`AIA` -- ``AIA::AIA_CUDAF`` (``AIA/aia_cudaf.h:15-38``).

There is no CPU fallback: importing works anywhere, but every compute call
goes through the CUDA library and raises if it is not built or no GPU is
present.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libglsu.so")
HEADER = os.path.join(os.path.dirname(PKG_ROOT), "include", "glsu.h")

OK = 0
ERR_INVALID, ERR_PADDING, ERR_CUDA, ERR_ALLOC = -1, -2, -3, -4
ERR_UNSUPPORTED, ERR_NOT_POSDEF, ERR_TIMEOUT, ERR_NO_DEVICE = -5, -6, -7, -8
F32, F64, U8 = 0, 1, 2
PHI_REF, PHI_CURR, DPHI_REF, DPHI = 0, 1, 2, 3
WFT_WFF, WFT_WFR = 0, 1
METHOD_AUTO, METHOD_DIRECT, METHOD_FFT, METHOD_TIMED = 0, 1, 2, 3
AIA_ERR_ABS, AIA_ERR_RELATIVE = 0, 1
LS_FLOAT_FLOAT, LS_FP64_SUMS = 0, 1

_lock = threading.Lock()
_lib = None


class GlsuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("glsu error %d: %s" % (code, msg))
        self.code = code


WFR_FIELDS = ("wx", "wy", "phase", "phase_comp", "b", "r", "cxx", "cyy")


class WfrResultsC(ctypes.Structure):
    """glsu_wfr_results: device addresses of the eight H*W WFR2 result maps."""
    _fields_ = [(n, ctypes.c_void_p) for n in WFR_FIELDS]


class WffTuningC(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("fft_length", ctypes.c_int), ("fft_columns", ctypes.c_int),
                ("fft_radix_order", ctypes.c_int), ("tuned", ctypes.c_int), ("ms_direct", ctypes.c_float),
                ("ms_fft", ctypes.c_float)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class WffParamsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("sigma_x", "wxl", "wxh", "wxi", "sigma_y", "wyl", "wyh", "wyi", "thr")]


@dataclass
class WffParams:
    """WFF2 parameters in the reference's C++ order (sigma, low, high, step)."""
    sigma_x: float = 10.0
    wxl: float = -1.0
    wxh: float = 1.0
    wxi: float = 0.1
    sigma_y: float = 10.0
    wyl: float = -1.0
    wyh: float = 1.0
    wyi: float = 0.1
    thr: float = 0.2

    def c(self) -> WffParamsC:
        return WffParamsC(*[float(getattr(self, f[0])) for f in WffParamsC._fields_])

    def tuple(self):
        return tuple(float(getattr(self, f[0])) for f in WffParamsC._fields_)


def exported_symbols() -> list[str]:
    """Function names declared in include/glsu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(glsu_\w+)\s*\(", txt, re.M)))


def lib() -> ctypes.CDLL:
    """Load libglsu.so; raises if the CUDA library has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libglsu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        c_int, c_double, c_void_p, c_float = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_float
        pp = ctypes.POINTER(c_void_p)
        dblp = ctypes.POINTER(c_double)
        intp = ctypes.POINTER(c_int)
        fltp = ctypes.POINTER(c_float)
        prm = ctypes.POINTER(WffParamsC)
        sig = {
            "glsu_last_error": ([], ctypes.c_char_p),
            "glsu_version": ([], c_int),
            "glsu_opt_fft_size": ([c_int], c_int),
            "glsu_wft_default_params": ([c_int, prm], c_int),
            "glsu_dpra_default_wff_params": ([prm], c_int),
            "glsu_wff_count": ([c_double, c_double, c_double, c_int], c_int),
            "glsu_aia_random_deltas": ([c_int, ctypes.c_uint64, fltp], c_int),
            "glsu_wff_create": ([pp, c_int, c_int, c_int, prm], c_int),
            "glsu_wfr_create": ([pp, c_int, c_int, c_int, prm], c_int),
            "glsu_wfr_destroy": ([c_void_p], c_int),
            "glsu_wfr_set_stream": ([c_void_p, c_void_p], c_int),
            "glsu_wfr_run": ([c_void_p, c_void_p, ctypes.POINTER(WfrResultsC), dblp], c_int),
            "glsu_wfr_run_async": ([c_void_p, c_void_p, ctypes.POINTER(WfrResultsC)], c_int),
            "glsu_wff_destroy": ([c_void_p], c_int),
            "glsu_wff_set_stream": ([c_void_p, c_void_p], c_int),
            "glsu_wff_run": ([c_void_p, c_void_p, c_void_p, dblp], c_int),
            "glsu_wff_run_async": ([c_void_p, c_void_p, c_void_p], c_int),
            "glsu_wff_threshold": ([c_void_p, dblp], c_int),
            "glsu_wff_set_method": ([c_void_p, c_int], c_int),
            "glsu_dpra_set_method": ([c_void_p, c_int], c_int),
            "glsu_wff_get_tuning": ([c_void_p, ctypes.POINTER(WffTuningC)], c_int),
            "glsu_dpra_batch_step": ([ctypes.POINTER(c_void_p), c_int, ctypes.POINTER(c_void_p), c_int], c_int),
            "glsu_dpra_batch_wait": ([ctypes.POINTER(c_void_p), c_int], c_int),
            "glsu_dpra_get_tuning": ([c_void_p, ctypes.POINTER(WffTuningC)], c_int),
            "glsu_wff_set_fft_plan": ([c_void_p, c_int, c_int], c_int),
            "glsu_wff_set_fft_length": ([c_void_p, c_int], c_int),
            "glsu_wff_fft_lengths": ([c_void_p, intp, c_int], c_int),
            "glsu_dpra_set_unwrap": ([c_void_p, c_int, c_int, c_int], c_int),
            "glsu_unwrap2_device": ([c_int, c_void_p, c_int, c_int, c_int, c_int, c_void_p], c_int),
            "glsu_wff_padded_size": ([c_void_p, intp, intp], c_int),
            "glsu_wff_run_noalloc": ([c_int, c_int, prm, c_void_p, c_void_p, c_void_p], c_int),
            "glsu_dpra_create": ([pp, c_int, c_void_p, c_int, c_int, c_int, c_int, prm], c_int),
            "glsu_dpra_destroy": ([c_void_p], c_int),
            "glsu_dpra_set_stream": ([c_void_p, c_void_p], c_int),
            "glsu_dpra_per_frame": ([c_void_p, c_void_p, c_int, c_void_p, dblp], c_int),
            "glsu_dpra_per_frame_device": ([c_void_p, c_void_p, c_int, c_void_p], c_int),
            "glsu_dpra_update_ref_phi": ([c_void_p], c_int),
            "glsu_dpra_sequence": ([c_void_p, c_int, c_void_p, c_int, c_void_p, dblp], c_int),
            "glsu_dpra_get": ([c_void_p, c_int, c_void_p], c_int),
            "glsu_dpra_device_ptr": ([c_void_p, c_int, pp], c_int),
            "glsu_dpra_get_lsq": ([c_void_p, c_void_p], c_int),
            "glsu_dpra_stage_timing": ([c_void_p, c_int], c_int),
            "glsu_dpra_stage_times": ([c_void_p, fltp, c_int], c_int),
            "glsu_aia_create": ([pp, c_int, c_int, c_int], c_int),
            "glsu_aia_destroy": ([c_void_p], c_int),
            "glsu_aia_set_convergence": ([c_void_p, c_int], c_int),
            "glsu_aia_set_stream": ([c_void_p, c_void_p], c_int),
            "glsu_aia_run": ([c_void_p, pp, c_int, fltp, fltp, c_int, dblp, intp, fltp, c_int, c_float,
                              ctypes.c_uint64], c_int),
            "glsu_aia_run_device": ([c_void_p, c_void_p, c_int, fltp, fltp, c_int, intp, fltp, c_int, c_float,
                                     ctypes.c_uint64], c_int),
            "glsu_sur_param_count": ([], c_int),
            "glsu_sur_create": ([pp, c_int, c_int, c_int, intp, c_int], c_int),
            "glsu_sur_destroy": ([c_void_p], c_int),
            "glsu_sur_set_stream": ([c_void_p, c_void_p], c_int),
            "glsu_sur_set_params": ([c_void_p, fltp], c_int),
            "glsu_sur_get_params": ([c_void_p, fltp], c_int),
            "glsu_sur_forward": ([c_void_p, c_void_p, c_void_p], c_int),
            "glsu_sur_backward": ([c_void_p, c_void_p, c_void_p, dblp, fltp], c_int),
            "glsu_sur_adam": ([c_void_p, c_float, c_float, c_float, c_float], c_int),
            "glsu_sur_set_loss_scale": ([c_void_p, c_float], c_int),
            "glsu_sur_output": ([c_void_p, c_void_p], c_int),
            "glsu_sur_gather": ([c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, intp, c_void_p, c_void_p],
                                c_int),
            "glsu_sur_conv32": ([c_void_p, c_void_p, c_int, c_int, c_int, c_int, fltp, fltp, c_int, c_void_p,
                                 c_void_p], c_int),
            "glsu_sur_wgrad32": ([c_void_p, c_void_p, c_int, c_int, c_int, c_int, fltp, c_void_p], c_int),
            "glsu_dpra_set_surrogate": ([c_void_p, fltp, intp, c_int, c_int, c_double], c_int),
            "glsu_dpra_set_probe_overlap": ([c_void_p, c_int, c_int], c_int),
            "glsu_dpra_set_graph": ([c_void_p, c_int], c_int),
            "glsu_dpra_surrogate_stats": ([c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                           ctypes.POINTER(ctypes.c_longlong), fltp, intp], c_int),
            "glsu_dpra_lsq_device": ([c_void_p, c_void_p], c_int),
            "glsu_dpra_set_ls_method": ([c_void_p, c_int], c_int),
            "glsu_dpra_set_ls_tile": ([c_void_p, c_int, c_int], c_int),
            "glsu_dpra_batch_create": ([pp, c_void_p, c_int], c_int),
            "glsu_dpra_batch_destroy": ([c_void_p], c_int),
            "glsu_dpra_batch_set_graph": ([c_void_p, c_int], c_int),
            "glsu_dpra_batch_run": ([c_void_p, c_void_p, c_int], c_int),
            "glsu_dpra_batch_sync": ([c_void_p], c_int),
            "glsu_dpra_get_ls_tile": ([c_void_p, intp, intp], c_int),
            "glsu_dpra_tune_ls_tile": ([c_void_p, fltp], c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def check(rc: int) -> int:
    if rc < 0:
        raise GlsuError(rc, lib().glsu_last_error().decode(errors="replace"))
    return rc


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def opt_fft_size(x: int) -> int:
    return lib().glsu_opt_fft_size(int(x))


def wff_count(lo: float, hi: float, step: float, precision: int = F64) -> int:
    return check(lib().glsu_wff_count(lo, hi, step, precision))


def default_params(wft_type: int = WFT_WFF) -> WffParams:
    c = WffParamsC()
    check(lib().glsu_wft_default_params(wft_type, ctypes.byref(c)))
    return WffParams(*[getattr(c, f[0]) for f in WffParamsC._fields_])


def dpra_default_params() -> WffParams:
    c = WffParamsC()
    check(lib().glsu_dpra_default_wff_params(ctypes.byref(c)))
    return WffParams(*[getattr(c, f[0]) for f in WffParamsC._fields_])


def random_deltas(M: int, seed: int) -> np.ndarray:
    d = np.zeros(M, np.float32)
    check(lib().glsu_aia_random_deltas(M, ctypes.c_uint64(seed), d.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
    return d


def unwrap2_device(precision, d_p: int, width: int, height: int, start_row: int = -1, start_col: int = -1,
                   stream: int = 0):
    """Line-scanning unwrapping (MatLab/fp_unwrapping.m) of a device phase map, in place."""
    check(lib().glsu_unwrap2_device(_prec(precision), ctypes.c_void_p(d_p), width, height, start_row, start_col,
                                    ctypes.c_void_p(stream) if stream else None))


def _prec(p) -> int:
    if p in (F32, "f32", "float32", np.float32):
        return F32
    if p in (F64, "f64", "float64", np.float64):
        return F64
    raise ValueError("precision must be f32 or f64")


def _img_type(a: np.ndarray) -> int:
    if a.dtype == np.uint8:
        return U8
    if a.dtype == np.float32:
        return F32
    if a.dtype == np.float64:
        return F64
    raise TypeError("frames must be uint8, float32 or float64")


class WFR2:
    """Windowed Fourier ridges (WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFR).

    ``run(d_f, maps)`` takes the device address of the H*W complex input
    (complex64 for f32, complex128 for f64) and a dict of the device
    addresses of the eight H*W real result maps (float32 / float64) named as
    in ``WFR_FIELDS``: wx, wy, phase, phase_comp, b, r, cxx, cyy."""

    def __init__(self, width: int, height: int, precision="f32", params: WffParams | None = None):
        self.width, self.height, self.precision = width, height, _prec(precision)
        h = ctypes.c_void_p()
        pc = ctypes.byref(params.c()) if params is not None else None
        check(lib().glsu_wfr_create(ctypes.byref(h), self.precision, width, height, pc))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().glsu_wfr_destroy(self._h)
            self._h = None

    __del__ = close

    def set_stream(self, stream_ptr: int):
        check(lib().glsu_wfr_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    @staticmethod
    def _maps(maps) -> WfrResultsC:
        return WfrResultsC(*[ctypes.c_void_p(int(maps[k])) for k in WFR_FIELDS])

    def run(self, d_f: int, maps) -> float:
        t = ctypes.c_double(0)
        z = self._maps(maps)
        check(lib().glsu_wfr_run(self._h, ctypes.c_void_p(d_f), ctypes.byref(z), ctypes.byref(t)))
        return t.value

    def run_async(self, d_f: int, maps):
        z = self._maps(maps)
        check(lib().glsu_wfr_run_async(self._h, ctypes.c_void_p(d_f), ctypes.byref(z)))


class WFF2:
    """Windowed Fourier filtering (WFT2_CUDAF / WFT2_CUDA with WFT_TYPE::WFF).

    Operates on device buffers: ``run(d_f, d_out)`` takes device addresses of
    H*W complex arrays (complex64 for f32, complex128 for f64)."""

    def __init__(self, width: int, height: int, precision="f32", params: WffParams | None = None,
                 wft_type: int = WFT_WFF):
        if wft_type != WFT_WFF:
            raise GlsuError(ERR_UNSUPPORTED, "WFT_TYPE::WFR is the WFR2 class")
        self.width, self.height, self.precision = width, height, _prec(precision)
        h = ctypes.c_void_p()
        pc = ctypes.byref(params.c()) if params is not None else None
        check(lib().glsu_wff_create(ctypes.byref(h), self.precision, width, height, pc))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().glsu_wff_destroy(self._h)
            self._h = None

    __del__ = close

    def set_stream(self, stream_ptr: int):
        check(lib().glsu_wff_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def run(self, d_f: int, d_out: int) -> float:
        t = ctypes.c_double(0)
        check(lib().glsu_wff_run(self._h, ctypes.c_void_p(d_f), ctypes.c_void_p(d_out), ctypes.byref(t)))
        return t.value

    def run_async(self, d_f: int, d_out: int):
        check(lib().glsu_wff_run_async(self._h, ctypes.c_void_p(d_f), ctypes.c_void_p(d_out)))

    def set_method(self, method: int):
        """Column-sweep method: METHOD_AUTO, METHOD_DIRECT, METHOD_FFT or METHOD_TIMED."""
        check(lib().glsu_wff_set_method(self._h, method))

    def tuning(self) -> dict:
        """The autotuner's choice for this shape (method, FFT plan, timings)."""
        t = WffTuningC()
        check(lib().glsu_wff_get_tuning(self._h, ctypes.byref(t)))
        return t.asdict()

    def set_fft_plan(self, columns_per_cta: int, radix_order: int):
        """Force an FFT plan variant (4 or 2 columns per CTA; radix order 0, 1 or 2)."""
        check(lib().glsu_wff_set_fft_plan(self._h, columns_per_cta, radix_order))

    def set_fft_length(self, length: int):
        """Rebuild the FFT sweep for another transform length (default plan variant)."""
        check(lib().glsu_wff_set_fft_length(self._h, length))

    def fft_lengths(self, n: int = 3) -> list:
        """The transform lengths the autotuner times, cheapest first."""
        out = (ctypes.c_int * max(n, 1))()
        k = check(lib().glsu_wff_fft_lengths(self._h, out, n))
        return list(out[:k])

    @property
    def threshold(self) -> float:
        t = ctypes.c_double(0)
        check(lib().glsu_wff_threshold(self._h, ctypes.byref(t)))
        return t.value

    @property
    def padded_size(self):
        w, h = ctypes.c_int(0), ctypes.c_int(0)
        check(lib().glsu_wff_padded_size(self._h, ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value


class DPRA:
    """DPRA_CUDAF (precision f32) / DPRA_CUDA (precision f64)."""

    def __init__(self, phi0: np.ndarray, ref_update_rate: int = 1, window_radius: int = 1, precision="f32",
                 wff: WffParams | None = None):
        self.precision = _prec(precision)
        dt = np.float32 if self.precision == F32 else np.float64
        phi0 = np.ascontiguousarray(phi0, dtype=dt)
        self.height, self.width = phi0.shape
        self.dtype = dt
        self.rr = ref_update_rate
        h = ctypes.c_void_p()
        pc = ctypes.byref(wff.c()) if wff is not None else None
        check(lib().glsu_dpra_create(ctypes.byref(h), self.precision, _ptr(phi0), self.width, self.height,
                                     ref_update_rate, window_radius, pc))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().glsu_dpra_destroy(self._h)
            self._h = None

    __del__ = close

    def set_stream(self, stream_ptr: int):
        check(lib().glsu_dpra_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def per_frame(self, img: np.ndarray, out: np.ndarray | None = None):
        img = np.ascontiguousarray(img)
        if out is None:
            out = np.empty((self.height, self.width), self.dtype)
        t = ctypes.c_double(0)
        check(lib().glsu_dpra_per_frame(self._h, _ptr(img), _img_type(img), _ptr(out), ctypes.byref(t)))
        return out, t.value

    def per_frame_ptr(self, h_img_ptr: int, img_type: int, h_out_ptr: int) -> float:
        t = ctypes.c_double(0)
        check(lib().glsu_dpra_per_frame(self._h, ctypes.c_void_p(h_img_ptr), img_type, ctypes.c_void_p(h_out_ptr),
                                        ctypes.byref(t)))
        return t.value

    def per_frame_device(self, d_img: int, img_type: int, d_dphi: int = 0):
        check(lib().glsu_dpra_per_frame_device(self._h, ctypes.c_void_p(d_img), img_type,
                                               ctypes.c_void_p(d_dphi) if d_dphi else None))

    def update_ref_phi(self):
        check(lib().glsu_dpra_update_ref_phi(self._h))

    def sequence(self, frames: np.ndarray):
        frames = np.ascontiguousarray(frames)
        out = np.empty((frames.shape[0], self.height, self.width), self.dtype)
        t = ctypes.c_double(0)
        check(lib().glsu_dpra_sequence(self._h, frames.shape[0], _ptr(frames), _img_type(frames), _ptr(out),
                                       ctypes.byref(t)))
        return out, t.value

    def sequence_ptr(self, nframes: int, h_frames_ptr: int, img_type: int, h_out_ptr: int) -> float:
        """Sequence over raw host pointers.  When both buffers are page-locked
        (e.g. ``torch.empty(..., pin_memory=True)``) the uploads and downloads
        overlap the compute of neighbouring frames; the returned time is then
        the device time from the first upload to the last download."""
        t = ctypes.c_double(0)
        check(lib().glsu_dpra_sequence(self._h, nframes, ctypes.c_void_p(h_frames_ptr), img_type,
                                       ctypes.c_void_p(h_out_ptr), ctypes.byref(t)))
        return t.value

    def get(self, which: int) -> np.ndarray:
        out = np.empty((self.height, self.width), self.dtype)
        check(lib().glsu_dpra_get(self._h, which, _ptr(out)))
        return out

    def get_lsq(self) -> np.ndarray:
        """exp(j dphi) of the last frame's least-squares stage (the WFF2 input)."""
        out = np.empty((self.height, self.width), np.complex64 if self.precision == F32 else np.complex128)
        check(lib().glsu_dpra_get_lsq(self._h, _ptr(out)))
        return out

    def device_ptr(self, which: int) -> int:
        p = ctypes.c_void_p()
        check(lib().glsu_dpra_device_ptr(self._h, which, ctypes.byref(p)))
        return p.value

    def set_method(self, method: int):
        """Column-sweep method of the WFF2: METHOD_AUTO, METHOD_DIRECT, METHOD_FFT or METHOD_TIMED."""
        check(lib().glsu_dpra_set_method(self._h, method))

    def tuning(self) -> dict:
        """The autotuner's choice for this handle's WFF2 shape."""
        t = WffTuningC()
        check(lib().glsu_dpra_get_tuning(self._h, ctypes.byref(t)))
        return t.asdict()

    def set_ls_tile(self, width: int, height: int):
        """Output tile of the FP32 float-float least squares: 32x16 (default), 32x8 or 32x32."""
        check(lib().glsu_dpra_set_ls_tile(self._h, width, height))

    def ls_tile(self):
        w, h = ctypes.c_int(0), ctypes.c_int(0)
        check(lib().glsu_dpra_get_ls_tile(self._h, ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value

    def tune_ls_tile(self):
        """Time the three least-squares tiles and select the fastest; returns their times (ms),
        -1 for a tile whose shared memory does not fit at the handle's radius."""
        ms = (ctypes.c_float * 3)()
        check(lib().glsu_dpra_tune_ls_tile(self._h, ms))
        return list(ms)

    def set_ls_method(self, method: int):
        """FP32 least-squares arithmetic: LS_FLOAT_FLOAT (default) or LS_FP64_SUMS."""
        check(lib().glsu_dpra_set_ls_method(self._h, method))

    def set_unwrap(self, enable: bool = True, start_row: int = -1, start_col: int = -1):
        """dphi = dphi_ref + unwrap(t) (MatLab/fp_ls3u.m:104) instead of dphi_ref + t."""
        check(lib().glsu_dpra_set_unwrap(self._h, int(enable), start_row, start_col))

    def set_surrogate(self, params, dilations, tile: int = 256, patch: int = 8, tol: float = 0.05):
        """Surrogate form (FP32): the learned network replaces WFF2, one exact
        WFF2 patch per tile judges it, tiles above ``tol`` rad fall back to the
        plain WFF2.  ``params=None`` restores the plain form."""
        if params is None:
            check(lib().glsu_dpra_set_surrogate(self._h, None, None, 0, 0, 0.0))
            self._surrogate = False
            return
        p = np.ascontiguousarray(params, np.float32)
        d = np.ascontiguousarray(dilations, np.int32)
        check(lib().glsu_dpra_set_surrogate(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                            d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), tile, patch,
                                            float(tol)))
        self._surrogate = tol > 0

    def surrogate_stats(self, ntiles: int = 0):
        """(tiles probed, tiles recomputed by the plain WFF2[, last residuals,
        last probe sites (row, col)]) -- the last two when ntiles > 0."""
        a, b = ctypes.c_longlong(0), ctypes.c_longlong(0)
        r = np.zeros(max(ntiles, 1), np.float32)
        st = np.zeros((max(ntiles, 1), 2), np.int32)
        check(lib().glsu_dpra_surrogate_stats(
            self._h, ctypes.byref(a), ctypes.byref(b),
            r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if ntiles else None,
            st.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if ntiles else None))
        return (a.value, b.value, r, st) if ntiles else (a.value, b.value)

    def lsq_device(self, d_out: int):
        """Device copy of the last least-squares output (enqueued on the handle's stream)."""
        check(lib().glsu_dpra_lsq_device(self._h, ctypes.c_void_p(d_out)))

    def stage_timing(self, enable: bool = True):
        check(lib().glsu_dpra_stage_timing(self._h, int(enable)))

    def stage_times(self):
        """Stage times (ms) of the last frame: 4 stages, plus in the surrogate
        form the network's layer 0 / tensor-core layers / layer 7 split and
        the probe sweep on its own stream."""
        ms = (ctypes.c_float * 8)()
        n = check(lib().glsu_dpra_stage_times(self._h, ms, 8))
        return list(ms[:n])

    def set_graph(self, enable: bool = True):
        """Replay each frame's device work as a captured CUDA graph."""
        check(lib().glsu_dpra_set_graph(self._h, int(enable)))

    def set_probe_overlap(self, enable: bool = True, conv_ctas_per_sm: int = 0):
        """Surrogate form: probe sweep beside the network on a second stream."""
        check(lib().glsu_dpra_set_probe_overlap(self._h, int(enable), int(conv_ctas_per_sm)))


def _handle_array(handles):
    return (ctypes.c_void_p * len(handles))(*[h._h.value for h in handles])


def dpra_batch_step(handles, d_frames, img_type: int):
    """One frame of each of several DPRA sequences (handles of any sizes), each
    on its handle's stream, in flight together; d_frames[i] is a device
    pointer, or 0 / None for a sequence that has ended.  Returns without
    waiting: call dpra_batch_wait."""
    fs = (ctypes.c_void_p * len(handles))(*[f or None for f in d_frames])
    check(lib().glsu_dpra_batch_step(_handle_array(handles), len(handles), fs, img_type))


class DpraBatch:
    """Staged batch of FP32 plain-form DPRA handles (glsu_dpra_batch_*): one
    frame of each active sequence per step, the FFT column sweeps of all
    sequences of a transform length in one persistent launch."""

    def __init__(self, handles, graph: bool = False):
        self._handles = list(handles)
        arr = _handle_array(self._handles)
        h = ctypes.c_void_p()
        check(lib().glsu_dpra_batch_create(ctypes.byref(h), arr, len(self._handles)))
        self._h = h
        if graph:
            check(lib().glsu_dpra_batch_set_graph(self._h, 1))

    def close(self):
        if self._h:
            lib().glsu_dpra_batch_destroy(self._h)
            self._h = None

    def run(self, d_frames, img_type: int):
        """d_frames: one device pointer (or 0 / None for an ended sequence) per handle."""
        arr = (ctypes.c_void_p * len(d_frames))(*[p or None for p in d_frames])
        check(lib().glsu_dpra_batch_run(self._h, arr, img_type))

    def sync(self):
        check(lib().glsu_dpra_batch_sync(self._h))


def dpra_batch_wait(handles):
    check(lib().glsu_dpra_batch_wait(_handle_array(handles), len(handles)))


class AIA:
    """AIA_CUDAF: initial phase from M frames with unknown phase shifts."""

    def __init__(self, M: int, cols: int, rows: int):
        self.M, self.cols, self.rows = M, cols, rows
        h = ctypes.c_void_p()
        check(lib().glsu_aia_create(ctypes.byref(h), M, cols, rows))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().glsu_aia_destroy(self._h)
            self._h = None

    __del__ = close

    def set_convergence(self, relative: bool):
        """Convergence measure: relative=False is AIA_CUDAF's max |delta - old|,
        True the change of the shifts relative to the first (AIA_CUDAF_YC2)."""
        check(lib().glsu_aia_set_convergence(self._h, AIA_ERR_RELATIVE if relative else AIA_ERR_ABS))

    def run(self, frames, deltas=None, max_iter: int = 20, max_err: float = 1e-4, seed: int = 0):
        frames = [np.ascontiguousarray(f) for f in frames]
        it = _img_type(frames[0])
        ptrs = (ctypes.c_void_p * len(frames))(*[f.ctypes.data for f in frames])
        d = np.zeros(self.M, np.float32)
        n_in = 0
        if deltas is not None:
            d[:len(deltas)] = np.asarray(deltas, np.float32)[:self.M]
            n_in = len(deltas)
        phi = np.empty((self.rows, self.cols), np.float32)
        t, iters, err = ctypes.c_double(0), ctypes.c_int(0), ctypes.c_float(0)
        fp = ctypes.POINTER(ctypes.c_float)
        check(lib().glsu_aia_run(self._h, ptrs, it, phi.ctypes.data_as(fp), d.ctypes.data_as(fp), n_in,
                                 ctypes.byref(t), ctypes.byref(iters), ctypes.byref(err), max_iter,
                                 ctypes.c_float(max_err), ctypes.c_uint64(seed)))
        return phi, d, t.value, iters.value, err.value


# ---------------------------------------------------------------------------
# learned WFF2 surrogate
# ---------------------------------------------------------------------------
def sur_param_count() -> int:
    return lib().glsu_sur_param_count()


def conv32(d_in: int, d_out: int, batch: int, width: int, height: int, dilation: int, w: np.ndarray, b=None,
           relu: bool = True, d_mask: int = 0, stream: int = 0):
    """One 32 -> 32 tensor-core layer on BF16 NHWC device buffers (synchronous)."""
    fp = ctypes.POINTER(ctypes.c_float)
    w = np.ascontiguousarray(w, np.float32)
    bb = None if b is None else np.ascontiguousarray(b, np.float32)
    check(lib().glsu_sur_conv32(ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), batch, width, height, dilation,
                                w.ctypes.data_as(fp), None if bb is None else bb.ctypes.data_as(fp), int(relu),
                                ctypes.c_void_p(d_mask) if d_mask else None,
                                ctypes.c_void_p(stream) if stream else None))


def wgrad32(d_g: int, d_in: int, batch: int, width: int, height: int, dilation: int, stream: int = 0):
    """Weight and bias gradient of one 32 -> 32 layer (BF16 NHWC device
    buffers; synchronous): (dW [32][32][3][3], db [32])."""
    out = np.empty(9216 + 32, np.float32)
    check(lib().glsu_sur_wgrad32(ctypes.c_void_p(d_g), ctypes.c_void_p(d_in), batch, width, height, dilation,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                 ctypes.c_void_p(stream) if stream else None))
    return out[:9216].reshape(32, 32, 3, 3), out[9216:]


class Surrogate:
    """The residual CNN that stands in for WFF2 (see ``include/glsu.h``)."""

    def __init__(self, batch: int, width: int, height: int, dilations, training: bool = False):
        self.batch, self.width, self.height = batch, width, height
        self.dilations = list(dilations)
        d = np.ascontiguousarray(dilations, np.int32)
        h = ctypes.c_void_p()
        check(lib().glsu_sur_create(ctypes.byref(h), batch, width, height,
                                    d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(training)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().glsu_sur_destroy(self._h)
            self._h = None

    __del__ = close

    def set_stream(self, stream: int):
        check(lib().glsu_sur_set_stream(self._h, ctypes.c_void_p(stream)))

    @property
    def params(self) -> np.ndarray:
        p = np.empty(sur_param_count(), np.float32)
        check(lib().glsu_sur_get_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != sur_param_count():
            raise ValueError("expected %d parameters" % sur_param_count())
        check(lib().glsu_sur_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def forward(self, d_z: int, d_out: int):
        check(lib().glsu_sur_forward(self._h, ctypes.c_void_p(d_z), ctypes.c_void_p(d_out)))

    def backward(self, d_z: int, d_target: int, want_grad: bool = False, want_loss: bool = True):
        loss = ctypes.c_double(0)
        g = np.empty(sur_param_count(), np.float32) if want_grad else None
        check(lib().glsu_sur_backward(self._h, ctypes.c_void_p(d_z), ctypes.c_void_p(d_target),
                                      ctypes.byref(loss) if want_loss else None,
                                      g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if want_grad else None))
        return (loss.value if want_loss else None), g

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        check(lib().glsu_sur_adam(self._h, lr, beta1, beta2, eps))

    def set_loss_scale(self, scale: float):
        """Training loss weight of a pixel: min(scale |target|, 1)."""
        check(lib().glsu_sur_set_loss_scale(self._h, float(scale)))

    def output(self) -> np.ndarray:
        o = np.empty((self.batch, self.height, self.width), np.complex64)
        check(lib().glsu_sur_output(self._h, _ptr(o)))
        return o

    def gather(self, d_pool_x: int, d_pool_t: int, pool_n: int, pool_h: int, pool_w: int, crops, d_x: int,
               d_t: int):
        """crops: rows (pool index, row, col) of the batch's windows."""
        c = np.ascontiguousarray(crops, np.int32).reshape(-1)
        check(lib().glsu_sur_gather(self._h, ctypes.c_void_p(d_pool_x), ctypes.c_void_p(d_pool_t), pool_n,
                                    pool_h, pool_w,
                                    c.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.c_void_p(d_x),
                                    ctypes.c_void_p(d_t)))
