"""CPU tests of the C ABI: the library loads, exports every declared symbol,
and its host-only logic (padding table, frequency counts, defaults, argument
validation, seeded AIA start) matches the reference behaviour.  No compute
call is made here."""
import ctypes

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(glsu):
    L = glsu.lib()
    names = glsu.exported_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_opt_fft_size_matches_reference_lut(glsu, oracle):
    for x in range(-3, 4200):
        assert glsu.opt_fft_size(x) == oracle.opt_fft_size(x), x


def test_frequency_count_in_each_precision(glsu):
    # WFT/WFT2_CPU.cpp:222-223 (double) and WFT/WFT2_CUDAf.cu:1062-1063 (float)
    assert glsu.wff_count(-1.0, 1.0, 0.1, glsu.F64) == 21
    assert glsu.wff_count(-1.0, 1.0, 0.1, glsu.F32) == 21
    assert glsu.wff_count(-1.5, 1.5, 0.1, glsu.F64) == 31
    assert glsu.wff_count(-0.15, 0.15, 0.05, glsu.F32) == 7
    for lo, hi, st in [(-2.3, 2.3, 0.1), (-0.7, 0.9, 0.05), (0.0, 0.0, 0.3)]:
        assert glsu.wff_count(lo, hi, st, glsu.F64) == int((hi - lo) * (1.0 / st)) + 1
        f = np.float32
        assert glsu.wff_count(lo, hi, st, glsu.F32) == int((f(hi) - f(lo)) * (f(1.0) / f(st))) + 1
    with pytest.raises(glsu.GlsuError):
        glsu.wff_count(0, 1, 0, glsu.F64)


def test_default_parameters(glsu):
    p = glsu.default_params(glsu.WFT_WFF)
    f = np.float32
    assert p.sigma_x == 10 and p.thr == -1
    assert p.wxl == float(f(-2) - f(3) / f(10)) and p.wxi == float(f(1) / f(10))
    d = glsu.dpra_default_params()
    assert (d.sigma_x, d.sigma_y, d.thr) == (20, 20, 15)
    assert d.wxl == float(f(-0.15)) and d.wxi == float(f(0.05))


def test_random_deltas_are_seeded(glsu):
    a, b, c = glsu.random_deltas(6, 1), glsu.random_deltas(6, 1), glsu.random_deltas(6, 2)
    assert a[0] == 0 and np.array_equal(a, b) and not np.array_equal(a, c)
    big = glsu.random_deltas(20001, 7)[1:]
    assert abs(big.mean()) < 0.05 and abs(big.std() - 1) < 0.05


def _wff_create(glsu, prec, W, H, p):
    h = ctypes.c_void_p()
    rc = glsu.lib().glsu_wff_create(ctypes.byref(h), prec, W, H, ctypes.byref(p.c()) if p else None)
    if rc == 0:
        glsu.lib().glsu_wff_destroy(h)
    return rc


def test_wff_create_rejects_bad_arguments_before_touching_the_device(glsu):
    P = glsu.WffParams
    assert _wff_create(glsu, 7, 64, 64, P()) == glsu.ERR_INVALID
    assert _wff_create(glsu, glsu.F32, 0, 64, P()) == glsu.ERR_INVALID
    assert _wff_create(glsu, glsu.F32, 64, 64, P(sigma_x=-1)) == glsu.ERR_INVALID
    assert _wff_create(glsu, glsu.F32, 64, 64, P(wxi=0)) == glsu.ERR_INVALID
    assert _wff_create(glsu, glsu.F32, 64, 64, P(wxl=1, wxh=0)) == glsu.ERR_INVALID
    # padded width 4090 + 60 leaves the FFT size table (the reference throws -1)
    assert _wff_create(glsu, glsu.F32, 4090, 8, P()) == glsu.ERR_PADDING
    assert "4096" in glsu.lib().glsu_last_error().decode()
    # window half-size round(3*sigma) = 63 is beyond the supported 60
    assert _wff_create(glsu, glsu.F32, 64, 64, P(sigma_x=21)) == glsu.ERR_UNSUPPORTED


def test_dpra_create_rejects_bad_arguments(glsu):
    L = glsu.lib()
    h = ctypes.c_void_p()
    phi = np.zeros((8, 8), np.float32)
    assert L.glsu_dpra_create(ctypes.byref(h), glsu.F32, None, 8, 8, 1, 1, None) == glsu.ERR_INVALID
    assert L.glsu_dpra_create(ctypes.byref(h), glsu.F32, phi.ctypes.data, 8, 8, 0, 1, None) == glsu.ERR_INVALID
    assert L.glsu_dpra_create(ctypes.byref(h), glsu.F32, phi.ctypes.data, 8, 8, 1, 9, None) == glsu.ERR_UNSUPPORTED
    assert L.glsu_aia_create(ctypes.byref(h), 2, 8, 8) == glsu.ERR_INVALID


def test_no_silent_cpu_path_without_a_device(glsu):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(glsu.GlsuError) as e:
        glsu.WFF2(64, 64, "f32", glsu.WffParams())
    assert e.value.code == glsu.ERR_NO_DEVICE


def test_frequency_count_float_and_double_can_differ(glsu):
    """The reference counts frequencies in the class's precision, so the same
    grid can hold a different number of frequencies in WFT2_CUDAF (float)
    and WFT2_cpu / WFT2_CUDA (double): int(1.8 * (1/0.3)) + 1."""
    assert glsu.wff_count(-0.9, 0.9, 0.3, glsu.F64) == 7
    assert glsu.wff_count(-0.9, 0.9, 0.3, glsu.F32) == 6


def test_kernel_attribute_record_is_per_device(tmp_path):
    """The record of raised shared-memory limits (csrc/func_attr.hpp) is kept
    per kernel and device and is consistent across threads (g++, no GPU)."""
    import os
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "test_func_attr")
    r = subprocess.run([gxx, "-O1", "-std=c++17", "-pthread", "-I", os.path.join(root, "g-ls3u_gb300", "csrc"),
                        os.path.join(root, "tests", "cpp", "test_func_attr.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
