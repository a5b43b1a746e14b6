"""Accuracy of the surrogate form in deployment (the learned WFF2 stand-in
with its sparse exact probes and per-tile plain fallback).

For each held-out seed a sequence of the synthetic generator (glsu.synth,
frames made on the GPU: DeviceSequence) runs free through a surrogate-form
DPRA handle.  At every `every`-th frame k the handle's own reference phase
phi_ref is taken and, from that same phi_ref and frame:

* the FP64 G-LS3U frame (FP64 DPRA least squares and FP64 WFF2, which
  match the FP64 oracle and the reference's CPU classes to 1e-10 rad) gives
  phi_curr64, the target;
* the surrogate form's own frame gives phi_curr (what a user gets);
* the same network without fallback (probes on, nothing recomputed) gives
  the network's phases and each tile's probe residual;
* the raw least-squares phase (no filtering) shows what the network gains.

Reported per sampled frame: RMSE and max |error| (wrapped, all pixels) of
each against phi_curr64, the tiles recomputed, and the probe's recall: of
the tiles whose network-only RMSE against phi_curr64 exceeds the tolerance
(over the tile's pixels where the FP64 WFF2 magnitude is at least 0.1, the
probe's own mask: elsewhere the phase is not defined), the fraction the
probe flagged; and the tiles flagged although within the tolerance.

The recall needs tiles that the network gets wrong, which the generator's
sequences do not produce (nor do noise far outside the training range, steps
and high-frequency ripples in the phase change: the network stays within
0.015 rad on them).  Two cases make them:
* ``carrier_region``: a linear phase ramp of 0.9 rad/px in the per-frame
  phase change over a centred square, near the edge of the WFF2 frequency
  range; the network's error there is tile-local and partial;
* ``reversed_residual``: the network with its last layer negated (its
  correction applied backwards), wrong on every tile: the mechanism check of
  probe, flag and fallback.

    python -m glsu.surrogate_eval [--seeds 10] [--frames 200] [--every 20]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import synth

DPRA_RADIUS = 3
WFF_SIGMA10 = (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)


def _wrap(d):
    return np.angle(np.exp(1j * d))


def _stats(e):
    return float(np.sqrt(np.mean(e * e))), float(np.abs(e).max())


def deployment(glsu, params, dil, seeds, nframes=200, every=20, size=1024, noise=0.02, wff=WFF_SIGMA10,
               radius=DPRA_RADIUS, tile=256, patch=4, tol=0.05, graph=True, delta_extra=None, n_gauss=4):
    """Run the deployment evaluation; returns a dict of per-frame records and
    summaries.  noise: the generator's noise level, or an H x W map of it;
    delta_extra: an H x W addition to the per-frame phase change."""
    import torch
    wp = glsu.WffParams(*wff)
    ntx, nty = -(-size // tile), -(-size // tile)
    recs = []
    w64 = glsu.WFF2(size, size, "f64", wp)
    zd = torch.empty((size, size), dtype=torch.complex128, device="cuda")
    fd = torch.empty_like(zd)
    for seed in seeds:
        seq = synth.DeviceSequence(size, size, seed=seed, noise=noise, delta_extra=delta_extra, n_gauss=n_gauss)
        ds = glsu.DPRA(seq.phi0.astype(np.float32), 1, radius, "f32", wp)
        ds.set_surrogate(params, dil, tile, patch, tol)
        if graph:
            ds.set_graph(True)
        buf = torch.empty((size, size), dtype=torch.float32, device="cuda")
        for k in range(1, nframes + 1):
            buf.copy_(seq.frame(k))
            torch.cuda.synchronize()
            if k % every:
                ds.per_frame_device(buf.data_ptr(), glsu.F32)
                ds.update_ref_phi()
                continue
            pref = ds.get(glsu.PHI_REF)
            # FP64 frame from the same reference phase
            d64 = glsu.DPRA(pref.astype(np.float64), 1, radius, "f64", wp)
            d64.per_frame_device(buf.data_ptr(), glsu.F32)
            pc64 = d64.get(glsu.PHI_CURR)
            d64.lsq_device(zd.data_ptr())
            torch.cuda.synchronize()
            d64.close()
            w64.run(zd.data_ptr(), fd.data_ptr())
            defined = np.abs(fd.cpu().numpy()) >= 0.1  # where the WFF2 phase is defined (the probe's mask)
            # the network alone: probes on, no tile recomputed
            dn = glsu.DPRA(pref, 1, radius, "f32", wp)
            dn.set_surrogate(params, dil, tile, patch, 1e9)
            dn.per_frame_device(buf.data_ptr(), glsu.F32)
            pc_net = dn.get(glsu.PHI_CURR)
            z = dn.get_lsq()
            _, _, resid, _ = dn.surrogate_stats(ntx * nty)
            dn.close()
            # the surrogate form's own frame
            p0, f0 = ds.surrogate_stats()
            ds.per_frame_device(buf.data_ptr(), glsu.F32)
            pc = ds.get(glsu.PHI_CURR)
            p1, f1 = ds.surrogate_stats()
            ds.update_ref_phi()
            e = _wrap(pc.astype(np.float64) - pc64)
            en = _wrap(pc_net.astype(np.float64) - pc64)
            els = _wrap(pref.astype(np.float64) + np.angle(z) - pc64)
            bad = flagged_bad = good_flagged = 0
            tiles_bad_rmse = []
            for ty in range(nty):
                for tx in range(ntx):
                    sl = (slice(ty * tile, (ty + 1) * tile), slice(tx * tile, (tx + 1) * tile))
                    t = en[sl][defined[sl]]
                    r = float(np.sqrt(np.mean(t * t))) if t.size else 0.0
                    flagged = int(resid[ty * ntx + tx] > tol)
                    if r > tol:
                        bad += 1
                        tiles_bad_rmse.append(r)
                        flagged_bad += flagged
                    else:
                        good_flagged += flagged
            rm, mx = _stats(e)
            rn, mn = _stats(en)
            rl, ml = _stats(els)
            recs.append({"seed": int(seed), "frame": k, "rmse": rm, "max": mx, "rmse_network_only": rn,
                         "max_network_only": mn, "rmse_without_network": rl, "max_without_network": ml,
                         "tiles_flagged": int(f1 - f0), "tiles": int(p1 - p0), "tiles_bad": bad,
                         "tiles_bad_flagged": flagged_bad, "tiles_good_flagged": good_flagged,
                         "bad_tile_rmse": tiles_bad_rmse})
        ds.close()
    w64.close()
    return summarise(recs, tol)


def noisy_region(size, level=0.2, base=0.02, frac=0.25):
    """A noise map for the probe's recall check: `base` everywhere, `level`
    in a centred square covering `frac` of the frame, far outside the
    training range U(0.01, 0.08), where the network's output degrades."""
    m = np.full((size, size), base)
    h = int(round(size * np.sqrt(frac) / 2))
    c = size // 2
    m[c - h:c + h, c - h:c + h] = level
    return m


def carrier_region(size, slope=0.9, frac=0.25):
    """A per-frame phase-change addition for the probe's recall check: a
    linear ramp of `slope` rad/px along x in a centred square covering `frac`
    of the frame, zero elsewhere."""
    m = np.zeros((size, size))
    h = int(round(size * np.sqrt(frac) / 2))
    c = size // 2
    x = np.arange(size, dtype=np.float64)[None, :]
    m[c - h:c + h, c - h:c + h] = (slope * x)[:, c - h:c + h]
    return m


def reversed_residual(params):
    """The network's parameters with the last layer (weights and bias)
    negated: y = z - conv7(a6) instead of z + conv7(a6)."""
    from .train_surrogate import LAYER_SIZES
    p = np.array(params, np.float32, copy=True)
    n_last = LAYER_SIZES[-1][0] * LAYER_SIZES[-1][1] * 9 + LAYER_SIZES[-1][0]
    p[-n_last:] = -p[-n_last:]
    return p


def summarise(recs, tol=0.05):
    r = np.array([x["rmse"] for x in recs])
    rn = np.array([x["rmse_network_only"] for x in recs])
    rl = np.array([x["rmse_without_network"] for x in recs])
    bad = sum(x["tiles_bad"] for x in recs)
    caught = sum(x["tiles_bad_flagged"] for x in recs)
    return {
        "frames_sampled": len(recs), "seeds": sorted({x["seed"] for x in recs}),
        "rmse_median": float(np.median(r)), "rmse_p90": float(np.percentile(r, 90)), "rmse_max": float(r.max()),
        "rmse_mean": float(r.mean()),
        "max_abs_max": float(max(x["max"] for x in recs)),
        "rmse_network_only_median": float(np.median(rn)), "rmse_network_only_p90": float(np.percentile(rn, 90)),
        "rmse_without_network_median": float(np.median(rl)),
        "tiles_recomputed_fraction": float(sum(x["tiles_flagged"] for x in recs) /
                                           max(1, sum(x["tiles"] for x in recs))),
        "tiles_over_tol": bad, "probe_recall": (caught / bad) if bad else None,
        "tiles_flagged_within_tol": sum(x["tiles_good_flagged"] for x in recs), "tol_rad": tol,
        "per_frame": recs,
    }


def main():
    import glsu
    from . import train_surrogate as T
    ap = argparse.ArgumentParser()
    ap.add_argument("--weights", default=None)
    ap.add_argument("--seeds", type=int, default=10)
    ap.add_argument("--seed0", type=int, default=50000)
    ap.add_argument("--frames", type=int, default=200)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    params, dil = T.load(a.weights) if a.weights else T.load()
    res = deployment(glsu, params, dil, range(a.seed0, a.seed0 + a.seeds), a.frames, a.every, a.size)
    short = {k: v for k, v in res.items() if k != "per_frame"}
    print(json.dumps(short, indent=1))
    if a.out:
        json.dump(res, open(a.out, "w"))


if __name__ == "__main__":
    main()
