"""Train the learned WFF2 surrogate with this library's own CUDA kernels.

Training pairs come from the plain G-LS3U pipeline on the GPU: for every
frame of a synthetic fringe sequence, the input is the DPRA least-squares
output z = exp(j dphi) and the target is WFF2(z), the plain frequency sweep
the surrogate stands in for.  Two pools are generated:

- 256 x 256 frames of the sequence generator with 4 Gaussian phase bumps and
  intensity noise sigma ~ U(0.01, 0.08), one noise level per sequence;
- 1024 x 1024 frames of the same generator scaled to that size (the
  deployment frames), from which 256 x 256 windows are cut.

Each step draws a batch of 256 x 256 windows (alternating pools), runs the
network forward and backward (tensor-core convolutions, FP32 weight
gradients) and one Adam step with a one-cycle learning rate.  The result is
saved as an ``.npz`` holding ``params`` (FP32), ``dilations`` and the WFF2
parameters it was trained for.

    python -m glsu.train_surrogate --out glsu/surrogate_sigma10.npz

For a large deployment shape, pairs come from sequences of that size only
(frames made on the GPU), e.g. the 2048^2 workload with sigma 15:

    python -m glsu.train_surrogate --size 2048 --wff 15,-1.5,1.5,0.1,15,-1.5,1.5,0.1,0.2 --radius 4 \
        --n-gauss 8 --noise 0.02,0.08 --dilations 1,3,9,27,27,9,3,1 --out glsu/surrogate_sigma15.npz
"""
from __future__ import annotations

import argparse
import math
import os
import time

import numpy as np

DILATIONS = (1, 2, 4, 8, 16, 8, 4, 1)
WFF = (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)  # sigma, low, high, step (x, y), threshold
RADIUS = 3
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "surrogate_sigma10.npz")


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("training the surrogate needs a CUDA device")
    return torch


def make_pool(size: int, nseq: int, nframes: int, seed: int, noise=(0.01, 0.08), wff=WFF, radius=RADIUS):
    """(x, t): complex64 device tensors [n][size][size] of (DPRA LS output, WFF2 output)."""
    torch = _torch()
    import glsu
    from glsu import synth
    wp = glsu.WffParams(*wff)
    rng = np.random.default_rng(seed)
    n = nseq * (nframes - 1)
    x = torch.empty((n, size, size), dtype=torch.complex64, device="cuda")
    t = torch.empty_like(x)
    w = glsu.WFF2(size, size, "f32", wp)
    k = 0
    for s in range(nseq):
        frames, phi0, _ = synth.sequence(size, size, nframes, seed=seed + s, noise=float(rng.uniform(*noise)))
        d = glsu.DPRA(phi0.astype(np.float32), 1, radius, "f32", wp)
        fr = torch.from_numpy(frames).cuda()
        torch.cuda.synchronize()
        for f in range(1, nframes):
            d.per_frame_device(fr[f].data_ptr(), glsu.F32)
            d.lsq_device(x[k].data_ptr())
            d.update_ref_phi()
            torch.cuda.synchronize()
            w.run(x[k].data_ptr(), t[k].data_ptr())
            k += 1
        d.close()
    w.close()
    torch.cuda.synchronize()
    return x, t


def make_pool_device(size: int, nseq: int, nframes: int, seed: int, noise=(0.01, 0.08), wff=WFF, radius=RADIUS,
                     n_gauss: int = 4, stride: int = 1):
    """Like make_pool, with the frames made on the GPU (synth.DeviceSequence),
    for large deployment sizes: every `stride`-th frame of each sequence
    gives a pair (the sequence itself runs through every frame)."""
    torch = _torch()
    import glsu
    from glsu import synth
    wp = glsu.WffParams(*wff)
    rng = np.random.default_rng(seed)
    per = (nframes - 1) // stride
    x = torch.empty((nseq * per, size, size), dtype=torch.complex64, device="cuda")
    t = torch.empty_like(x)
    w = glsu.WFF2(size, size, "f32", wp)
    buf = torch.empty((size, size), dtype=torch.float32, device="cuda")
    k = 0
    for s in range(nseq):
        seq = synth.DeviceSequence(size, size, seed=seed + s, noise=float(rng.uniform(*noise)), n_gauss=n_gauss)
        d = glsu.DPRA(seq.phi0.astype(np.float32), 1, radius, "f32", wp)
        for f in range(1, nframes):
            buf.copy_(seq.frame(f))
            torch.cuda.synchronize()
            d.per_frame_device(buf.data_ptr(), glsu.F32)
            if f % stride == 0 and k < x.shape[0]:
                d.lsq_device(x[k].data_ptr())
                torch.cuda.synchronize()
                w.run(x[k].data_ptr(), t[k].data_ptr())
                k += 1
            d.update_ref_phi()
        d.close()
    w.close()
    torch.cuda.synchronize()
    return x[:k], t[:k]


def phase_rmse(out, t, mask_mag: float = 0.0) -> float:
    """RMS of the wrapped phase difference (all pixels, or |t| >= mask_mag)."""
    e = np.angle(out * np.conj(t))
    if mask_mag > 0:
        e = e[np.abs(t) >= mask_mag]
    return float(np.sqrt(np.mean(e ** 2)))


def evaluate(params, x, t, dilations=DILATIONS, limit: int = 16):
    """Phase RMSE of the surrogate and of the identity (no filtering) on pool frames."""
    torch = _torch()
    import glsu
    n, H, W = x.shape
    net = glsu.Surrogate(1, W, H, dilations)
    net.params = params
    out = torch.empty_like(x[0])
    se = si = cnt = 0.0
    for k in range(min(n, limit)):
        net.forward(x[k].data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        o, tt, xx = out.cpu().numpy(), t[k].cpu().numpy(), x[k].cpu().numpy()
        se += float(np.sum(np.angle(o * np.conj(tt)) ** 2))
        si += float(np.sum(np.angle(xx * np.conj(tt)) ** 2))
        cnt += o.size
    net.close()
    return math.sqrt(se / cnt), math.sqrt(si / cnt)


LAYER_SIZES = [(32, 2)] + [(32, 32)] * 6 + [(2, 32)]  # (out, in) channels of the 8 layers


def init_params(seed: int = 0, scale_last: float = 0.1) -> np.ndarray:
    """He-normal 3x3 kernels, zero biases, a small last layer (starts near the
    identity y = z).  Layout: per layer W[co][ci][3][3] then b[co]."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (co, ci) in enumerate(LAYER_SIZES):
        std = math.sqrt(2.0 / (ci * 9)) * (scale_last if l == len(LAYER_SIZES) - 1 else 1.0)
        parts += [rng.normal(0.0, std, co * ci * 9), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


def one_cycle(step: int, steps: int, peak: float, warm: float = 0.25) -> float:
    """Linear warm-up to peak over warm*steps, then cosine decay to peak/1000."""
    w = max(1, int(warm * steps))
    if step < w:
        return peak * (0.04 + 0.96 * step / w)
    q = (step - w) / max(1, steps - w)
    return peak * (1e-3 + (1 - 1e-3) * 0.5 * (1 + math.cos(math.pi * q)))


def train(pools, steps: int, batch: int = 16, crop: int = 256, lr: float = 1.5e-3, dilations=DILATIONS,
          seed: int = 0, init=None, log_every: int = 500, log=print, time_budget: float = 0.0,
          loss_scale: float = 1.0):
    """Train on a list of (x, t) pools, alternating between them; returns the
    FP32 parameters and a list of (step, loss).  With time_budget > 0 the
    learning-rate schedule runs over elapsed seconds instead of steps and
    training stops when the budget is spent (at most `steps` steps).  A
    pixel's loss weight is min(loss_scale |target|, 1)."""
    torch = _torch()
    import glsu
    rng = np.random.default_rng(seed)
    net = glsu.Surrogate(batch, crop, crop, dilations, training=True)
    net.params = init_params(seed) if init is None else np.asarray(init, np.float32)
    if loss_scale != 1.0:
        net.set_loss_scale(loss_scale)
    xb = torch.empty((batch, crop, crop), dtype=torch.complex64, device="cuda")
    tb = torch.empty_like(xb)
    hist = []
    t0 = time.time()
    it = 0
    while it < steps:
        if time_budget > 0:
            el = time.time() - t0
            if el >= time_budget:
                break
            cur_lr = one_cycle(int(1e6 * el / time_budget), 1_000_000, lr)
        else:
            cur_lr = one_cycle(it, steps, lr)
        x, t = pools[it % len(pools)]
        n, H, W = x.shape
        crops = np.stack([rng.integers(0, n, batch), rng.integers(0, H - crop + 1, batch),
                          rng.integers(0, W - crop + 1, batch)], 1)
        net.gather(x.data_ptr(), t.data_ptr(), n, H, W, crops, xb.data_ptr(), tb.data_ptr())
        want = (it + 1) % log_every == 0 or it == 0
        loss, _ = net.backward(xb.data_ptr(), tb.data_ptr(), want_loss=want)
        net.adam(cur_lr)
        if want:
            hist.append((it + 1, loss))
            log("step %6d  loss %.5f  lr %.2e  %.1f s" % (it + 1, loss, cur_lr, time.time() - t0))
        it += 1
    hist.append((it, float("nan")))  # steps taken
    params = net.params
    net.close()
    return params, hist


def load(path: str = DEFAULT_WEIGHTS):
    """(params, dilations) of a saved surrogate."""
    z = np.load(path)
    return z["params"].astype(np.float32), [int(d) for d in z["dilations"]]


def main_large(a):
    """Train for a large deployment shape (e.g. 2048^2 with sigma 15): pairs
    from sequences of the generator at that size, made on the GPU."""
    wff = tuple(float(v) for v in a.wff.split(","))
    dil = tuple(int(v) for v in a.dilations.split(","))
    noise = tuple(float(v) for v in a.noise.split(","))
    t0 = time.time()
    pool = make_pool_device(a.size, a.seqs, a.frames, seed=30_000 + a.seed, noise=noise, wff=wff, radius=a.radius,
                            n_gauss=a.n_gauss, stride=a.stride)
    held = make_pool_device(a.size, 2, 6, seed=97_000 + a.seed, noise=noise, wff=wff, radius=a.radius,
                            n_gauss=a.n_gauss)
    print("pool: %d training frames of %d^2, generated in %.1f s" % (pool[0].shape[0], a.size, time.time() - t0),
          flush=True)
    params, hist = train([pool], a.steps, a.batch, lr=a.lr, dilations=dil, seed=a.seed, time_budget=a.time_budget,
                         log=lambda m: print(m, flush=True), loss_scale=a.loss_scale)
    r = evaluate(params, *held, dilations=dil, limit=8)
    print("held-out phase RMSE vs WFF2 at %d^2: %.4f (identity %.4f)" % (a.size, r[0], r[1]), flush=True)
    np.savez(a.out, params=params, dilations=np.array(dil, np.int32), wff=np.array(wff), radius=a.radius,
             steps=int(hist[-1][0]) if hist else 0, batch=a.batch, lr=a.lr, seed=a.seed, size=a.size,
             pairs=pool[0].shape[0], rmse_heldout=r[0], rmse_identity=r[1], loss_history=np.array(hist),
             loss_scale=a.loss_scale)
    print("saved", a.out)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--steps", type=int, default=30000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1.5e-3)
    ap.add_argument("--seqs256", type=int, default=1000, help="256^2 sequences (19 pairs each)")
    ap.add_argument("--seqs1024", type=int, default=20, help="1024^2 sequences (20 frames each)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--time-budget", type=float, default=0.0, help="seconds of training (schedule over time)")
    ap.add_argument("--loss-scale", type=float, default=1.0, help="pixel loss weight min(scale |WFF2|, 1)")
    ap.add_argument("--size", type=int, default=0,
                    help="large deployment size: train on pairs from sequences of that size only (GPU-made frames)")
    ap.add_argument("--wff", default=",".join(str(v) for v in WFF), help="WFF2 parameters (with --size)")
    ap.add_argument("--radius", type=int, default=RADIUS, help="DPRA window radius (with --size)")
    ap.add_argument("--dilations", default=",".join(str(v) for v in DILATIONS), help="(with --size)")
    ap.add_argument("--noise", default="0.01,0.08", help="noise range per sequence (with --size)")
    ap.add_argument("--n-gauss", type=int, default=4, help="Gaussians of the phase (with --size)")
    ap.add_argument("--seqs", type=int, default=16, help="sequences (with --size)")
    ap.add_argument("--frames", type=int, default=41, help="frames per sequence (with --size)")
    ap.add_argument("--stride", type=int, default=2, help="every stride-th frame gives a pair (with --size)")
    a = ap.parse_args(argv)
    if a.size:
        return main_large(a)
    t0 = time.time()
    small = make_pool(256, a.seqs256, 20, seed=10_000 + a.seed)
    big = make_pool(1024, a.seqs1024, 21, seed=20_000 + a.seed)
    held_small = make_pool(256, 8, 5, seed=90_000 + a.seed)
    held_big = make_pool(1024, 2, 5, seed=95_000 + a.seed)
    print("pools: %d + %d training frames, generated in %.1f s" % (small[0].shape[0], big[0].shape[0],
                                                                   time.time() - t0), flush=True)
    params, hist = train([big, small], a.steps, a.batch, lr=a.lr, seed=a.seed, time_budget=a.time_budget,
                         log=lambda m: print(m, flush=True), loss_scale=a.loss_scale)
    r_small = evaluate(params, *held_small)
    r_big = evaluate(params, *held_big)
    print("held-out phase RMSE vs WFF2: 256^2 %.4f (identity %.4f), 1024^2 %.4f (identity %.4f)"
          % (r_small[0], r_small[1], r_big[0], r_big[1]), flush=True)
    np.savez(a.out, params=params, dilations=np.array(DILATIONS, np.int32), wff=np.array(WFF),
             radius=RADIUS, steps=int(hist[-1][0]) if hist else 0, batch=a.batch, lr=a.lr, seed=a.seed,
             pairs=small[0].shape[0] + 16 * big[0].shape[0],
             rmse_heldout_256=r_small[0], rmse_heldout_1024=r_big[0],
             rmse_identity_256=r_small[1], rmse_identity_1024=r_big[1], loss_history=np.array(hist),
             loss_scale=a.loss_scale)
    print("saved", a.out)


if __name__ == "__main__":
    main()
