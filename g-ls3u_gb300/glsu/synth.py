"""Seeded synthetic fringe sequences of the benchmark workloads.

    I_k = a + b cos(phi_k) + N(0, noise),  phi_k = phi_0 + k * Delta
    a   = 0.5 + 0.1 * (one unit-peak Gaussian bump, sigma 80 px at 256 px)
    b   = 0.4
    phi_0 = sum of n_gauss Gaussians: centres U(0, size), amplitudes
            U(5, 15) rad, widths U(20, 60) px (lengths scale with size/256)
    Delta = 2 Gaussians rescaled to a 0.3 rad/frame peak

Seeds feed numpy's PCG64.  This replaces recorded fringe data (none is
public with the reference); the shapes, value ranges and noise levels are
those of the workloads the hot path is measured on.
"""
from __future__ import annotations

import numpy as np


def _gauss(rng, H, W, n, amp_lo, amp_hi, s_lo, s_hi, scale):
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    out = np.zeros((H, W))
    for _ in range(n):
        cy, cx = rng.uniform(0, H), rng.uniform(0, W)
        a = rng.uniform(amp_lo, amp_hi)
        s = rng.uniform(s_lo, s_hi) * scale
        out += a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
    return out


def sequence(H: int, W: int, nframes: int, seed: int = 0, noise: float = 0.02, n_gauss: int = 4,
             dtype=np.float32):
    """Return (frames [n,H,W], phi0 [H,W] float64, delta [H,W] float64)."""
    rng = np.random.default_rng(seed)
    scale = max(H, W) / 256.0
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    cy, cx = rng.uniform(0, H), rng.uniform(0, W)
    sa = 80.0 * scale
    a = 0.5 + 0.1 * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sa * sa))
    b = 0.4
    phi0 = _gauss(rng, H, W, n_gauss, 5.0, 15.0, 20.0, 60.0, scale)
    delta = _gauss(rng, H, W, 2, 0.5, 1.0, 20.0, 60.0, scale)
    delta *= 0.3 / max(np.abs(delta).max(), 1e-12)
    frames = np.empty((nframes, H, W), dtype)
    for k in range(nframes):
        frames[k] = a + b * np.cos(phi0 + k * delta) + rng.normal(0.0, noise, (H, W))
    return frames, phi0, delta


def sequence_params(H: int, W: int, seed: int = 0, n_gauss: int = 4):
    """The deterministic part of ``sequence``'s generator for a seed:
    (a, b, phi0, delta), drawn in the same order, so that
    a + b cos(phi0 + k delta) is its noise-free frame k."""
    rng = np.random.default_rng(seed)
    scale = max(H, W) / 256.0
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    cy, cx = rng.uniform(0, H), rng.uniform(0, W)
    sa = 80.0 * scale
    a = 0.5 + 0.1 * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sa * sa))
    phi0 = _gauss(rng, H, W, n_gauss, 5.0, 15.0, 20.0, 60.0, scale)
    delta = _gauss(rng, H, W, 2, 0.5, 1.0, 20.0, 60.0, scale)
    delta *= 0.3 / max(np.abs(delta).max(), 1e-12)
    return a, 0.4, phi0, delta


class DeviceSequence:
    """Frames of ``sequence``'s generator made on the GPU with torch, for
    long sequences at large sizes: I_k = a + b cos(phi0 + k delta) + N(0,
    noise), with the noise drawn by a torch generator seeded from `seed`
    (the same distribution as ``sequence``, not the same numbers).  noise
    may also be an H x W array of per-pixel standard deviations;
    delta_extra (H x W, rad/frame) is added to the per-frame phase change."""

    def __init__(self, H: int, W: int, seed: int = 0, noise=0.02, n_gauss: int = 4, device="cuda",
                 delta_extra=None):
        import torch
        a, b, phi0, delta = sequence_params(H, W, seed, n_gauss)
        if delta_extra is not None:
            delta = delta + np.asarray(delta_extra, np.float64)
        self.phi0, self.delta = phi0, delta
        self._t = torch
        self._a = torch.from_numpy(a).to(device)
        self._b = b
        self._phi0 = torch.from_numpy(phi0).to(device)
        self._delta = torch.from_numpy(delta).to(device)
        self._noise = noise if np.isscalar(noise) else torch.from_numpy(np.asarray(noise, np.float64)).to(device)
        self._gen = torch.Generator(device=device)
        self._gen.manual_seed(int(seed) * 7919 + 17)
        self._dev = device

    def frame(self, k: int):
        """Frame k as a float32 device tensor (the noise of successive calls is fresh)."""
        t = self._t
        clean = self._a + self._b * t.cos(self._phi0 + k * self._delta)
        n = t.randn(clean.shape, generator=self._gen, device=self._dev, dtype=t.float64) * self._noise
        return (clean + n).to(t.float32).contiguous()


def aia_frames(H: int, W: int, M: int, seed: int = 0, noise: float = 0.02, n_gauss: int = 4,
               bump: bool = True):
    """M frames with unknown phase shifts U(0, 2 pi): returns (frames, phi, shifts).

    ``bump=False`` keeps the background uniform, the case in which AIA's
    frame step is an exact model and recovers the shifts exactly."""
    rng = np.random.default_rng(seed + 7919)
    _, phi0, _ = sequence(H, W, 0, seed, noise, n_gauss)
    scale = max(H, W) / 256.0
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    cy, cx = rng.uniform(0, H), rng.uniform(0, W)
    sa = 80.0 * scale
    a = 0.5 + (0.1 if bump else 0.0) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sa * sa))
    shifts = rng.uniform(0, 2 * np.pi, M)
    frames = np.empty((M, H, W), np.float32)
    for k in range(M):
        frames[k] = a + 0.4 * np.cos(phi0 + shifts[k]) + rng.normal(0.0, noise, (H, W))
    return frames, phi0, shifts


def wrap(p):
    return np.angle(np.exp(1j * p))


def phase_err(a, b):
    """Wrapped phase difference a - b in (-pi, pi]."""
    return np.angle(np.exp(1j * (np.asarray(a, np.float64) - np.asarray(b, np.float64))))
