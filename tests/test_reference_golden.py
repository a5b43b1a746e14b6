"""Parity pinned to the reference's own CPU classes.

tests/golden/ref_golden.npz holds outputs of the reference's WFT2_cpu (WFF)
and DPRA_CPU, compiled here from the reference's sources
(oracle/ref_build.py; script tests/golden/make_ref_golden.py).  These tests
check the FP64 oracle against them on the CPU; tests/test_gpu_parity.py
checks the CUDA paths against the same vectors.

DPRA's 3x3 normal equations are stated per conditioning bucket of the
reduced 2x2 matrix, kappa = det / trace^2 (at most 1/4): where kappa <= 1e-4
the window's reference phase is nearly constant, the system is numerically
singular, and the reference's literal arithmetic (raw sums, LAPACKE_dsysv)
and any other evaluation of it give unrelated answers (up to pi apart), so
no bound is asserted there.  The reference also rounds the WFF2 angle to
float before the update (DPRA/dpra_cpu.cpp:246); its phases carry that
rounding (at most 2^-24 pi, 1.9e-7 rad).
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_golden.npz")
DPRA_WFF = (20.0, -0.15, 0.15, 0.05, 20.0, -0.15, 0.15, 0.05, 15.0)  # DPRA/dpra_cpu.cpp:22-25
FLOAT_ANGLE = 2.0 ** -24 * np.pi * 1.01  # the reference's float rounding of the angle
# (kappa range, largest phase difference allowed against the reference's literal arithmetic)
LS_BUCKETS = [((1e-3, 1.0), 1e-9), ((1e-4, 1e-3), 1e-6), ((-1.0, 1e-4), None)]


def gold():
    return np.load(GOLD)


def ls_bucket_errors(z, zref, kappa):
    e = np.abs(np.angle(z * np.conj(zref)))
    out = []
    for (lo, hi), bar in LS_BUCKETS:
        m = (kappa > lo) & (kappa <= hi)
        out.append(((lo, hi), bar, int(m.sum()), float(e[m].max()) if m.any() else 0.0))
    return out


def test_oracle_wff2_matches_reference_wft2_cpu(oracle):
    g = gold()
    for k in range(3):
        f = g["wff%d_in" % k].astype(np.complex128)
        p = tuple(g["wff%d_params" % k])
        out, thr = oracle.wff2(f, *p)
        ref = g["wff%d_out" % k]
        rel = np.abs(out - ref).max() / np.abs(ref).max()
        m = np.abs(ref) > 1e-3 * np.abs(ref).max()
        ph = np.abs(np.angle(out[m] * np.conj(ref[m]))).max()
        print("WFF2 case %d %s: rel %.3g, phase %.3g rad, thr %.15g / %.15g" % (k, p, rel, ph, thr, g["wff%d_thr" % k]))
        assert rel < 1e-12 and ph < 1e-10
        assert abs(thr - g["wff%d_thr" % k]) <= 1e-12 * abs(thr)


def test_oracle_dpra_ls_matches_reference_by_conditioning(oracle):
    g = gold()
    u8, pc = g["dpra_frames"], g["dpra_phi_curr"]
    pref = g["dpra_phi0"]
    for k in range(u8.shape[0]):
        kap = oracle.dpra_kappa(pref, 1)
        z = oracle.dpra_ls(u8[k].astype(np.float64), pref, 1)
        for (lo, hi), bar, n, emax in ls_bucket_errors(z, g["dpra_lsq"][k], kap):
            print("frame %d kappa (%g, %g]: %d pixels, max %.3g rad" % (k, lo, hi, n, emax))
            if bar is not None:
                assert emax <= bar
        pref = pc[k]


def test_oracle_wff2_and_update_match_reference_frames(oracle):
    """WFF2 of the reference's own least-squares output, then the phase
    update, give the reference's phi_curr and dphi to its float rounding."""
    g = gold()
    pref, dref = g["dpra_phi0"], np.zeros_like(g["dpra_phi0"])
    for k in range(g["dpra_frames"].shape[0]):
        filt, _ = oracle.wff2(g["dpra_lsq"][k], *DPRA_WFF)
        pc, dp = oracle.dpra_update(filt, pref, dref)
        e = np.abs(np.angle(np.exp(1j * (pc - g["dpra_phi_curr"][k]))))
        ed = np.abs(dp - g["dpra_dphi"][k])
        print("frame %d: phi_curr max %.3g, dphi max %.3g" % (k, e.max(), ed.max()))
        assert e.max() <= FLOAT_ANGLE and ed.max() <= FLOAT_ANGLE
        pref, dref = g["dpra_phi_curr"][k], g["dpra_dphi"][k]


def test_reference_rate_semantics_in_the_fixture():
    """With rate 1 the reference updates after every frame: each frame's
    dphi is the previous frame's dphi plus the new increment."""
    g = gold()
    d = g["dpra_dphi"]
    assert d.shape[0] == 5 and np.isfinite(d).all()
    inc = np.diff(d, axis=0)
    assert np.abs(inc).max() < np.pi + 1e-6
