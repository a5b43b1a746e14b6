"""The no-allocation WFF2 entry point (glsu_wff_run_noalloc).

Callers that may not call cudaMalloc -- a plugin whose host application owns
all device memory, a real-time loop that must not stall in the allocator, a
deployment with a fixed memory budget -- get WFF2 with scratch taken from a
fixed array inside the library.  These checks call it through the C ABI and
compare it with the allocating entry point (glsu_wff_create / glsu_wff_run)
on the same inputs, two calls in a row each, so that a call reading what the
previous call left in the shared scratch would show.  This file is named to
be collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    H, W = shape
    y, x = np.mgrid[0:H, 0:W]
    phi = 0.04 * x + 0.05 * y + 1.5 * np.sin(x / 13.0) * np.cos(y / 19.0) + 0.3 * seed
    return (np.exp(1j * phi) * (1 + 0.1 * rng.standard_normal(shape))).astype(np.complex64)


def _noalloc(glsu, torch, f, params, stream=None):
    """One call of the entry point.  With a torch stream, the input is written
    and the output read on that stream and the call is given its handle."""
    if stream is None:
        a = torch.from_numpy(f).cuda()
        out = torch.full_like(a, complex(np.nan, np.nan))
        torch.cuda.synchronize()
        sp = None
    else:
        host = torch.from_numpy(f).pin_memory()
        with torch.cuda.stream(stream):
            a = host.to("cuda", non_blocking=True)
            out = torch.full_like(a, complex(np.nan, np.nan))
        sp = ctypes.c_void_p(stream.cuda_stream)
    rc = glsu.lib().glsu_wff_run_noalloc(f.shape[1], f.shape[0], ctypes.byref(params.c()),
                                         ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(out.data_ptr()), sp)
    glsu.check(rc)
    if stream is None:
        return out.cpu().numpy()
    with torch.cuda.stream(stream):
        res = out.cpu().numpy()
    return res


def _allocating(glsu, torch, f, params, method=None):
    a = torch.from_numpy(f).cuda()
    out = torch.empty_like(a)
    w = glsu.WFF2(f.shape[1], f.shape[0], "f32", params)
    if method is not None:
        w.set_method(method)
    w.run(a.data_ptr(), out.data_ptr())
    w.close()
    return out.cpu().numpy()


CASES = [
    ((256, 256), (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)),   # the 21x21 sweep
    ((96, 130), (6.5, -0.8, 0.8, 0.4, 6.5, -0.8, 0.8, 0.4, -1.0)),      # automatic threshold
]


@pytest.mark.parametrize("case,on_stream", [(0, False), (1, False), (0, True)])
def test_no_alloc_matches_allocating_entry_point(glsu, case, on_stream):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "needs a CUDA device"
    shape, p = CASES[case]
    params = glsu.WffParams(*p)
    stream = torch.cuda.Stream() if on_stream else None
    for seed in (case * 10 + 1, case * 10 + 2):  # two calls in a row on different inputs
        f = _field(shape, seed)
        got = _noalloc(glsu, torch, f, params, stream)
        ref = _allocating(glsu, torch, f, params)
        mag = np.abs(ref)
        m = mag > 0.05 * mag.max()
        perr = np.abs(np.angle(got[m] * np.conj(ref[m]))).max()
        rel = np.abs(got - ref).max() / mag.max()
        print("no-alloc case %d seed %d: phase diff %.3g rad, rel diff %.3g" % (case, seed, perr, rel))
        assert np.isfinite(got).all()
        assert perr < 1e-3 and rel < 1e-4  # the FP32 tolerance of the WFF2 parity tests


def test_no_alloc_rejects_problems_beyond_its_scratch(glsu):
    torch = pytest.importorskip("torch")
    a = torch.zeros((8, 8), dtype=torch.complex64, device="cuda")
    p = glsu.WffParams(10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
    rc = glsu.lib().glsu_wff_run_noalloc(2048, 2048, ctypes.byref(p.c()), ctypes.c_void_p(a.data_ptr()),
                                         ctypes.c_void_p(a.data_ptr()), None)
    assert rc == glsu.ERR_INVALID
    msg = glsu.lib().glsu_last_error().decode()
    assert "64 MiB" in msg and "needs" in msg


def test_no_alloc_equals_direct_sweep_bit_for_bit(glsu):
    """The entry point runs the direct column sweep, so against an allocating
    handle forced onto that sweep the two outputs are identical."""
    torch = pytest.importorskip("torch")
    shape, p = CASES[0]
    params = glsu.WffParams(*p)
    for seed in (5, 6):
        f = _field(shape, seed)
        got = _noalloc(glsu, torch, f, params)
        ref = _allocating(glsu, torch, f, params, method=glsu.METHOD_DIRECT)
        assert np.array_equal(got, ref)
