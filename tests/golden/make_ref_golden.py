"""Golden vectors from the reference's own CPU classes (WFT2_cpu, DPRA_CPU).

Builds oracle/_ref from the reference checkout (oracle/ref_build.py: the
reference's WFT/WFT2_CPU.cpp, DPRA/dpra_cpu.cpp, WFT/WFT.cpp and
Utils/Utils.cpp, unchanged, on stand-ins for FFTW3, LAPACKE_dsysv and
cv::Mat) and writes ``ref_golden.npz`` here:

- ``wff{k}_*``: WFT2_cpu (WFF) on three complex fields: the synthetic
  config-0 parameters (sigma 10, 21 x 21 frequencies on [-1, 1], thr 0.2),
  the parameters DPRA hard-wires (sigma 20, 7 x 7 frequencies, thr 15), and
  an automatic threshold with sigma_x != sigma_y on a ragged size.  Inputs
  are stored as complex64 values (so an FP32 path reads the same numbers);
  outputs and the threshold used are FP64.
- ``dpra_*``: DPRA_CPU (3 x 3 window and the WFF parameters it hard-wires)
  over 5 8-bit frames of the seeded synthetic sequence at 96 x 80, reference
  rate 1, from phi0: per frame the returned dphi, phi_curr, and the
  least-squares output exp(j dphi_ls) of its LAPACKE_dsysv solves.

    python tests/golden/make_ref_golden.py <path of the reference checkout>

Tests read only the .npz; nothing at test time touches the reference.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "g-ls3u_gb300"))

WFF_CASES = [
    ((96, 128), (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)),
    ((96, 128), (20.0, -0.15, 0.15, 0.05, 20.0, -0.15, 0.15, 0.05, 15.0)),
    ((75, 90), (5.0, -0.9, 0.9, 0.3, 6.0, -0.6, 0.6, 0.3, -1.0)),
]
DPRA_SHAPE, DPRA_FRAMES = (96, 80), 5


def field(shape, seed):
    H, W = shape
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W]
    phi = 0.3 * x + 0.2 * y + 2.0 * np.sin(x / 11.0) * np.cos(y / 17.0)
    f = np.exp(1j * phi) + 0.1 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    return f.astype(np.complex64)


def main(ref: str) -> None:
    from oracle import ref_build
    from glsu import synth
    lib = ctypes.CDLL(ref_build.build(ref, force=True))
    dp = ctypes.POINTER(ctypes.c_double)

    def P(a):
        return a.ctypes.data_as(dp)

    out = {}
    for k, (shape, p) in enumerate(WFF_CASES):
        H, W = shape
        f = field(shape, 100 + k)
        f64 = np.ascontiguousarray(f.astype(np.complex128))
        res = np.zeros_like(f64)
        thr = ctypes.c_double()
        rc = lib.ref_wff2(W, H, P(np.array(p, np.float64)), P(f64.view(np.float64)), P(res.view(np.float64)),
                          ctypes.byref(thr), os.cpu_count() or 1)
        assert rc == 0
        out["wff%d_in" % k] = f
        out["wff%d_out" % k] = res
        out["wff%d_params" % k] = np.array(p, np.float64)
        out["wff%d_thr" % k] = np.float64(thr.value)

    H, W = DPRA_SHAPE
    frames, phi0, _ = synth.sequence(H, W, DPRA_FRAMES + 1, seed=31)
    u8 = np.clip(np.round(frames * 255.0), 0, 255).astype(np.uint8)[1:]
    phi0 = np.ascontiguousarray(phi0, np.float64)
    dphi = np.zeros((DPRA_FRAMES, H, W))
    pc = np.zeros((DPRA_FRAMES, H, W))
    lsq = np.zeros((DPRA_FRAMES, H, W), np.complex128)
    rc = lib.ref_dpra_sequence(W, H, DPRA_FRAMES, np.ascontiguousarray(u8).ctypes.data_as(ctypes.c_void_p), P(phi0),
                               1, os.cpu_count() or 1, P(dphi), P(pc), P(lsq.view(np.float64)))
    assert rc == 0
    out.update(dpra_frames=u8, dpra_phi0=phi0, dpra_dphi=dphi, dpra_phi_curr=pc, dpra_lsq=lsq)
    np.savez_compressed(os.path.join(HERE, "ref_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_golden.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_golden.py <path of the reference checkout>")
    main(sys.argv[1])
