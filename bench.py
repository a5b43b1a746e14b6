#!/usr/bin/env python
"""G-LS3U benchmark: frames/s of the per-frame hot path at 1024x1024 FP32,
surrogate form against plain form.

A step is one frame of a seeded synthetic sequence (glsu/synth.py) with the
frame already in HBM:

* plain form -- DPRA least squares (7x7 window) -> WFF2 (sigma 10, 21x21
  frequencies on [-1, 1], threshold 0.2) -> phase update -> reference update
  (rate 1);
* surrogate form (the headline "value") -- DPRA least squares -> the learned
  8-layer dilated residual network (BF16 tcgen05 convolutions) in place of
  WFF2 -> exact FP32 WFF2 on one 4x4 probe patch per 256x256 tile -> plain
  WFF2 recomputation of every tile whose RMS phase residual exceeds 0.05 rad
  -> phase update -> reference update.

Both forms are timed with CUDA events over K consecutive frames after W
warm-up frames, L2 flushed (256 MiB write) before each frame outside the
events.  "e2e" runs K further frames of the same sequence through
glsu_dpra_sequence (pinned host frames in, dphi out).  The surrogate form's
accuracy is measured teacher-forced against the plain FP32 WFF2 of the same
least-squares output over 6 frames.  The sequence's initial phase comes from
AIA on 5 phase-shifted frames (timed separately, reported under "aia").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs its own sequence (weak scaling, no collective
on the data path); the reported time is the max over ranks.
``--impl reference`` times the reference's CPU algorithm (the FP64 oracle
restatement of DPRA_CPU + WFT2_cpu; the reference's own MKL/FFTW/OpenCV/MSVC
build cannot be compiled here) on the host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "g-ls3u_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "G-LS3U frames/s at 1024\u00b2 FP32, surrogate vs plain, at \u22640.02 rad RMSE vs FP64"
# surrogate form: one exact WFF2 probe patch per 256x256 tile (4x4 for
# sigma = 10), plain fallback for tiles whose RMS phase residual exceeds 0.05 rad
SUR_TILE, SUR_PATCH, SUR_TOL = 256, 4, 0.05
# algorithmic bytes and flops per pixel of the network: layer 0 reads z (8 B)
# and writes 32 BF16 channels (64 B); each of the six 32->32 layers reads and
# writes 64 B; layer 7 reads 64 B + z and writes the complex output (8 B)
SUR_BYTES_PER_PX = 72 + 6 * 128 + 80
SUR_FLOPS_PER_PX = 2 * 18 * 32 + 6 * 2 * 288 * 32 + 2 * 288 * 2
# kernels per frame: plain = LS, rows, column sweep, final (with the update);
# surrogate = LS, the probe's row and column passes, layer 0, six tensor-core
# layers, layer 7, the residuals, the tile list, three masked WFF2 passes and
# the update
PLAIN_LAUNCHES, SUR_LAUNCHES = 4, 17
# one 32->32 tensor-core layer per pixel: read 64 B, write 64 B; 2*288*32 flops
SUR_CONV_BYTES_PER_PX, SUR_CONV_FLOPS_PER_PX = 128, 2 * 288 * 32
# DRAM bytes (read + write) of one sur_conv_tc_kernel launch at 1024x1024,
# from the ncu capture summarised in profiles/sur_conv_tc_kernel_1024.md
SUR_CONV_TRAFFIC_1024 = 67.170304e6 + 21.358592e6
SIZE = 1024
# the surrogate form's deployment check: held-out seeds (training used
# 10000.., 20000.., 90000.., 95000..), free-running frames, sampling period
DEPLOY_SEED0, DEPLOY_SEEDS, DEPLOY_FRAMES, DEPLOY_EVERY = 50000, 10, 200, 20
RADIUS = 3
WFF = (10.0, -1.0, 1.0, 0.1, 10.0, -1.0, 1.0, 0.1, 0.2)
NFX = NFY = 21
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=SIZE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--frames-only", action="store_true",
                    help="only the timed plain and surrogate frames (no AIA, WFR, e2e or accuracy runs): "
                         "for profiler captures")
    return ap.parse_args()


def fft_padded(n):
    """Smallest even 7-smooth size >= n: the reference's FFT size table
    (WFT/WFT.h:18-32) is exactly the even 7-smooth numbers up to 4096."""
    while True:
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        if m == 1 and n % 2 == 0:
            return n
        n += 1


def fft_model_bytes(size):
    """Algorithmic bytes of one frame of the FFT formulation of WFF2 (the
    reference's WFT2_CUDAF::cuWFF2, WFT/WFT2_CUDAf.cu:1016-1173): four passes
    over the padded complex64 plane per frequency (16 B each way per element)
    plus the forward transform of the input: (64 * n_freq + 32) * P bytes."""
    s = int(np.floor(3 * WFF[0] + 0.5))
    P = fft_padded(size + 2 * s) ** 2
    return (64 * NFX * NFY + 32) * P, P


def workload_config(size):
    return {
        "workload": "G-LS3U per-frame path, %dx%d FP32, DPRA %dx%d window, WFF2 sigma=%g, "
                    "xi in [%g,%g] step %g (%dx%d frequencies), thr=%g, reference rate 1; surrogate form "
                    "(8-layer dilated residual CNN, BF16 tcgen05, one %dx%d exact-WFF2 probe per %dx%d tile, "
                    "plain fallback above %g rad) vs plain form; 200-frame sequence generator with AIA "
                    "(5 frames) initial phase"
                    % (size, size, 2 * RADIUS + 1, 2 * RADIUS + 1, WFF[0], WFF[1], WFF[2], WFF[3], NFX, NFY,
                       WFF[8], SUR_PATCH, SUR_PATCH, SUR_TILE, SUR_TILE, SUR_TOL),
        "frame": [size, size],
        "dpra_window": 2 * RADIUS + 1,
        "wff": {"sigma": WFF[0], "wl": WFF[1], "wh": WFF[2], "wi": WFF[3], "thr": WFF[8], "n_freq": NFX * NFY},
        "surrogate": {"tile": SUR_TILE, "probe_patch": SUR_PATCH, "tol_rad": SUR_TOL},
        "frame_launch": "each handle in graph mode: a frame's kernels (both streams of the surrogate form) "
                        "captured once as a CUDA graph and replayed; the stage-split frames run eagerly",
        "l2": "flushed before every timed step (256 MiB device write outside the timed events)",
        "e2e_path": "glsu_dpra_sequence over K consecutive pinned host frames after W warm-up frames on a "
                    "fresh handle (H2D, D2H on their own streams, overlapped with neighbouring frames); L2 "
                    "flushed once before; each plain frame streams 352 MB of WFF2 planes (more than the "
                    "129 MB L2)",
    }


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_init():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        from datetime import timedelta
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend, timeout=timedelta(minutes=30))
    return rank, world, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
def cpu_sample(size, rows=None, seed=1000, prec="f32"):
    """One frame of the CPU path with the oracle restatements of the
    reference's CPU classes: DPRA LS, WFF2 over `rows` of the 21 frequency
    rows (all of them by default: the whole frame), phase update.  The WFF2
    sweep runs one frequency row per OpenMP thread at a time, as the
    reference's does (WFT/WFT2_CPU.cpp:227-237).  prec "f64": DPRA_CPU /
    WFT2_cpu (glsu_oracle.c); "f32": the float classes DPRA_CPUF / WFT2_cpuF
    (glsu_oracle_f32.c).  Returns (frames_per_s, seconds, threads, rows);
    with rows < 21 the rate is that of the partial frame (warm-up only)."""
    from oracle import oracle as O
    from glsu import synth
    O.build()
    frames, phi0, _ = synth.sequence(size, size, 2, seed=seed)
    threads = os.cpu_count() or 1
    rows = NFY if rows is None else max(1, min(NFY, rows))
    wp = O.WffParams(*WFF)
    if prec == "f64":
        ls, wff, upd, img, pref = O.dpra_ls, O.wff2, O.dpra_update, frames[1].astype(np.float64), phi0
    else:
        ls, wff, upd, img, pref = O.dpra_ls_f32, O.wff2_f32, O.dpra_update_f32, frames[1], phi0.astype(np.float32)
    t0 = time.perf_counter()
    z = ls(img, pref, RADIUS, threads)
    filt = wff(z, *wp.tuple(), nthreads=threads, ky=(0, rows))
    if isinstance(filt, tuple):
        filt = filt[0]
    upd(filt, pref, np.zeros_like(pref))
    el = time.perf_counter() - t0
    return 1.0 / el, el, threads, rows


def run_reference(args, rank, world):
    """The reference's CPU algorithm (the oracle restatements of its CPU
    classes) on the host cores, rank 0 only: every timed step is one whole
    1024^2 frame (all 441 frequencies).  The first warm-up step times one
    round of frequency rows in each precision to pick the faster variant;
    the other warm-up steps run one frequency row."""
    if rank != 0:
        return None
    steps, warm = args.steps, args.warmup
    threads = os.cpu_count() or 1
    vw = {}
    for prec in ("f32", "f64"):
        vw[prec] = cpu_sample(args.size, rows=min(NFY, threads), prec=prec)[1]
    best = min(vw, key=vw.get)
    for _ in range(max(0, warm - 1)):
        cpu_sample(args.size, rows=1, prec=best)
    times = []
    for _ in range(steps):
        _, el, threads, rows = cpu_sample(args.size, prec=best)
        times.append(el)
    tot = float(sum(times))
    value = steps / tot
    sample = ("per step: one whole %dx%d frame on the host cores (%d threads): DPRA LS (7x7), WFF2 over all "
              "21 x 21 frequencies (one frequency row per OpenMP thread at a time, as the reference schedules "
              "it), phase update; the restatement of the reference's %s CPU classes (%s), the faster variant "
              "in the warm-up (one round of rows: FP32 %.1f s, FP64 %.1f s)"
              % (args.size, args.size, threads, "float" if best == "f32" else "double",
                 "DPRA_CPUF/WFT2_cpuF" if best == "f32" else "DPRA_CPU/WFT2_cpu", vw["f32"], vw["f64"]))
    return {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": args.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": 1e3 * tot / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": best, "data": "synthetic",
        "config": workload_config(args.size), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port", "sample": sample,
                         "step_seconds": times},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


STAGE_FRAMES = 5  # frames after the timed ones that are run with stage events


def timed_frames(glsu, torch, d, dfr, nfr, args, stream, flush, world, local):
    """Device time of K frames through handle d (per-frame device call + reference
    update), L2 flushed before each frame outside the events; max over ranks.
    The timed frames run without the handle's stage events (they cost about
    17 us a frame); STAGE_FRAMES further frames of the sequence, run with the
    events and with the stages one after another, give the per-stage split."""
    d.stage_timing(False)
    for k in range(args.warmup):
        d.per_frame_device(dfr[k % nfr].data_ptr(), glsu.F32)
        d.update_ref_phi()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        evs[k][0].record(stream)
        d.per_frame_device(dfr[(args.warmup + k) % nfr].data_ptr(), glsu.F32)
        d.update_ref_phi()
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    max_ms = reduce_max(sum(a.elapsed_time(b) for a, b in evs), world)
    # the stage split with the stages one after another (surrogate form: the
    # probe sweep not overlapped), so that each kernel is timed on its own
    overlap = hasattr(d, "set_probe_overlap") and getattr(d, "_surrogate", False)
    if overlap:
        d.set_probe_overlap(False)
    d.stage_timing(True)
    stage = None
    for k in range(STAGE_FRAMES):
        with torch.cuda.stream(stream):
            flush.zero_()
        d.per_frame_device(dfr[(args.warmup + args.steps + k) % nfr].data_ptr(), glsu.F32)
        d.update_ref_phi()
        st = np.array(d.stage_times())
        stage = st if stage is None else stage + st
    d.stage_timing(False)
    if overlap:
        d.set_probe_overlap(True)
    return world * args.steps / (max_ms / 1e3), max_ms, stage / STAGE_FRAMES, clk


E2E_FRAMES, E2E_RUNS = 200, 3


def host_sequence(torch, size, nframes, seed):
    """nframes consecutive frames of the seeded generator in pinned host
    memory (made on the GPU: synth.DeviceSequence), and its phi0."""
    from glsu import synth
    seq = synth.DeviceSequence(size, size, seed=seed)
    h = torch.empty((nframes, size, size), dtype=torch.float32).pin_memory()
    for k in range(nframes):
        h[k].copy_(seq.frame(k + 1), non_blocking=False)
    return h, seq.phi0


def copy_times(torch, size, reps=20):
    """Device time (ms) of one frame's H2D copy (4 B/px from pinned memory)
    and one dphi D2H copy, each alone on a stream."""
    st = torch.cuda.Stream()
    hin = torch.empty((size, size), dtype=torch.float32).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    dev = torch.empty((size, size), dtype=torch.float32, device="cuda")
    res = []
    for direction in ("h2d", "d2h"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            for k in range(reps + 2):
                if k == 2:
                    e0.record(st)
                if direction == "h2d":
                    dev.copy_(hin, non_blocking=True)
                else:
                    hout.copy_(dev, non_blocking=True)
            e1.record(st)
        st.synchronize()
        res.append(e0.elapsed_time(e1) / reps)
    return res


def e2e_sequence(glsu, torch, make_handle, hframes, args, stream, flush, world):
    """Frames/s end to end through glsu_dpra_sequence, the public sequence
    call: after one untimed pass over the pinned buffers, and W warm-up
    frames on a fresh handle (reference phase phi0), one call runs
    E2E_FRAMES pinned host frames, uploads, compute and dphi downloads
    overlapped on the handle's copy streams, and returns when every output is
    on the host; wall clock around that call, max over ranks, the median of
    E2E_RUNS runs."""
    W = args.warmup
    K = hframes.shape[0] - W
    hout = torch.empty(hframes.shape[1:], dtype=torch.float32).unsqueeze(0).expand(K, -1, -1).contiguous()
    hout = hout.pin_memory()
    # one untimed pass over the whole pinned input and output first: the
    # first DMA through freshly pinned pages is slower (about 1300 against
    # 1700 frames/s for the surrogate form), a one-time cost of the buffers
    d = make_handle()
    d.sequence_ptr(K, hframes[W].data_ptr(), glsu.F32, hout.data_ptr())
    d.close()
    vals = []
    for _ in range(E2E_RUNS):
        d = make_handle()
        d.sequence_ptr(W, hframes.data_ptr(), glsu.F32, hout.data_ptr())  # warms the copy streams
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        d.sequence_ptr(K, hframes[W].data_ptr(), glsu.F32, hout.data_ptr())
        el = reduce_max(time.perf_counter() - t0, world)
        d.close()
        vals.append(world * K / el)
    return float(np.median(vals)), vals


def surrogate_accuracy(glsu, torch, dfr, phi0, wp, params, dil, nframes):
    """Teacher-forced phase error of the surrogate form (per frame, all pixels)
    against the FP64 G-LS3U frame from the same reference phase (FP64 DPRA
    least squares and FP64 WFF2: the oracle's arithmetic, which the FP64
    kernels match to 1e-11 rad), against the plain FP32 WFF2 of the same
    least-squares output, and of the raw least-squares phase (no filtering)."""
    size = dfr.shape[-1]
    d = glsu.DPRA(phi0.astype(np.float32), 1, RADIUS, "f32", wp)
    d.set_surrogate(params, dil, SUR_TILE, SUR_PATCH, SUR_TOL)
    w = glsu.WFF2(size, size, "f32", wp)
    z = torch.empty((size, size), dtype=torch.complex64, device="cuda")
    ref = torch.empty_like(z)
    rm, mx, rid, rm64, mx64 = [], [], [], [], []
    for k in range(1, nframes + 1):
        pref = d.get(glsu.PHI_REF).astype(np.float64)
        d64 = glsu.DPRA(pref, 1, RADIUS, "f64", wp)
        d64.per_frame_device(dfr[k].data_ptr(), glsu.F32)
        pc64 = d64.get(glsu.PHI_CURR)
        d64.close()
        d.per_frame_device(dfr[k].data_ptr(), glsu.F32)
        d.lsq_device(z.data_ptr())
        torch.cuda.synchronize()
        w.run(z.data_ptr(), ref.data_ptr())
        pc = d.get(glsu.PHI_CURR).astype(np.float64)
        tp = np.angle(ref.cpu().numpy())
        e = np.angle(np.exp(1j * (pc - pref - tp)))
        eid = np.angle(z.cpu().numpy() * np.exp(-1j * tp))
        rm.append(float(np.sqrt(np.mean(e ** 2))))
        mx.append(float(np.abs(e).max()))
        rid.append(float(np.sqrt(np.mean(eid ** 2))))
        e64 = np.angle(np.exp(1j * (pc - pc64)))
        rm64.append(float(np.sqrt(np.mean(e64 ** 2))))
        mx64.append(float(np.abs(e64).max()))
        d.update_ref_phi()
    probed, flagged = d.surrogate_stats()
    d.close()
    w.close()
    return {"rmse_vs_fp64": float(np.sqrt(np.mean(np.square(rm64)))), "max_abs_vs_fp64": max(mx64),
            "rmse_vs_fp64_per_frame": rm64,
            "rmse_per_frame": rm, "rmse": float(np.sqrt(np.mean(np.square(rm)))), "max_abs": max(mx),
            "rmse_without_network": float(np.sqrt(np.mean(np.square(rid)))), "frames": nframes,
            "tiles_probed": probed, "tiles_recomputed": flagged}


def aligned_phase_error(est, truth):
    """Phase error of est against truth up to the global constant (and sign)
    that AIA cannot determine: (rmse, max, sign, offset)."""
    best = None
    for sgn in (1.0, -1.0):
        d = np.angle(np.exp(1j * (sgn * np.asarray(est, np.float64) - truth)))
        c = float(np.angle(np.mean(np.exp(1j * d))))
        e = np.angle(np.exp(1j * (d - c)))
        r = (float(np.sqrt(np.mean(e * e))), float(np.abs(e).max()), sgn, c)
        if best is None or r[0] < best[0]:
            best = r
    return best


def fp64_frame_error(glsu, pref, dev_frame, radius, wp, pc):
    """Phase error (wrapped, all pixels) of a frame's phi_curr against the
    FP64 G-LS3U frame from the same reference phase: (rmse, max)."""
    d64 = glsu.DPRA(np.asarray(pref, np.float64), 1, radius, "f64", wp)
    d64.per_frame_device(dev_frame.data_ptr(), glsu.F32)
    pc64 = d64.get(glsu.PHI_CURR)
    d64.close()
    e = np.angle(np.exp(1j * (np.asarray(pc, np.float64) - pc64)))
    return float(np.sqrt(np.mean(e * e))), float(np.abs(e).max())


def precision_form(glsu, torch, seed, size=SIZE, nframes=200, every=20):
    """The precision form (AIA initial phase, then the FP32 G-LS3U sequence):
    AIA on 5 frames with shifts U(0, 2 pi) (at most 30 iterations or a shift
    change below 1e-4) against the generator's phase and shifts, with the
    reference's convergence measure and with the relative one of its second
    AIA variant; then `nframes` frames of the generator from AIA's phase,
    DPRA 7x7 + WFF2 in FP32, graph mode, with every `every`-th frame compared
    with the FP64 frame from the same reference phase."""
    from glsu import synth
    out = {"shifts": None}
    fr, phi_true, shifts = synth.aia_frames(size, size, 5, seed=seed)
    out["shifts"] = [float(v) for v in shifts]
    for rel in (False, True):
        a = glsu.AIA(5, size, size)
        a.set_convergence(rel)
        a.run(list(fr), None, max_iter=30, max_err=1e-4, seed=seed)  # warm
        phi, deltas, ms, iters, err = a.run(list(fr), None, max_iter=30, max_err=1e-4, seed=seed)
        a.close()
        rm, mx, sgn, c = aligned_phase_error(phi, phi_true)
        ds = np.angle(np.exp(1j * (sgn * np.asarray(deltas, np.float64) - (shifts - shifts[0]))))
        ds = np.angle(np.exp(1j * (ds - ds[0])))
        out["aia_relative_measure" if rel else "aia"] = {
            "ms": ms, "iterations": int(iters), "last_change": float(err), "phase_rmse_vs_truth": rm,
            "phase_max_vs_truth": mx, "shift_max_err_vs_truth": float(np.abs(ds).max()),
            "measure": ("change of the shifts relative to the first (AIA_CUDAF_YC2, AIA/aia_cudaf_v2.cu:665-677)"
                        if rel else "max |delta - delta_old| (AIA_CUDAF, AIA/aia_cpu.cpp:249-263)")}
        if not rel:
            phi_aia = np.asarray(phi, np.float64)
    out["note"] = ("the phase and frame steps leave a common rotation of the shifts free; the iterates drift along "
                   "it by a constant step per iteration, so the first measure stays at that step and the run "
                   "stops at the cap while the normalised shifts have settled; the phase error against the "
                   "generator's phase (up to the global constant AIA cannot fix) is set by the 5 shifts' spread "
                   "and the noise")
    wp = glsu.WffParams(*WFF)
    seq = synth.DeviceSequence(size, size, seed=seed)
    d = glsu.DPRA(phi_aia.astype(np.float32), 1, RADIUS, "f32", wp)
    st = torch.cuda.Stream()
    d.set_stream(st.cuda_stream)
    d.set_graph(True)
    buf = torch.empty((size, size), dtype=torch.float32, device="cuda")
    dev_ms, errs = 0.0, []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for k in range(1, nframes + 1):
        buf.copy_(seq.frame(k))
        sample = k % every == 0
        pref = d.get(glsu.PHI_REF) if sample else None
        torch.cuda.synchronize()
        e0.record(st)
        d.per_frame_device(buf.data_ptr(), glsu.F32)
        d.update_ref_phi()
        e1.record(st)
        torch.cuda.synchronize()
        dev_ms += e0.elapsed_time(e1)
        if sample:
            errs.append((k,) + fp64_frame_error(glsu, pref, buf, RADIUS, wp, d.get(glsu.PHI_REF)))
    d.close()
    out["sequence"] = {
        "frames": nframes, "device_ms_per_frame": dev_ms / nframes, "frames_per_s": nframes / (dev_ms * 1e-3),
        "initial_phase": "AIA output", "fp64_samples": [{"frame": k, "rmse": r, "max": m} for k, r, m in errs],
        "rmse_vs_fp64": float(np.sqrt(np.mean([r * r for _, r, _ in errs]))),
        "max_abs_vs_fp64": max(m for _, _, m in errs), "bar_rad": 1e-3,
        "note": "each sampled frame is compared with the FP64 frame (FP64 DPRA LS + FP64 WFF2) run from the same "
                "reference phase; frames are made on the GPU from the seeded generator"}
    return out


CONFIG4 = dict(size=2048, radius=4, wff=(15.0, -1.5, 1.5, 0.1, 15.0, -1.5, 1.5, 0.1, 0.2), noise=0.05, n_gauss=8)
# Surrogate tiles of the large workload: 512^2.  An exact probe patch at
# sigma 15 with 31 x 31 frequencies costs about 7x one at sigma 10 with
# 21 x 21 (window area x frequency count), so 512^2 tiles keep the probe's
# share of the frame near the 1024^2 benchmark's (16 probes a frame).
SUR4_TILE = 512


SIGMA15_WEIGHTS = os.path.join(PKG, "glsu", "surrogate_sigma15.npz")


def _large_run(glsu, torch, seed, form, nframes, warm, fp64_frames):
    """One form of the large workload (plain, or the surrogate with the
    sigma-15 network): device time per frame over `nframes` frames after
    `warm`, graph mode, stage split of one further eager frame, and the
    FP64 check of the sampled frames."""
    from glsu import synth
    from glsu import train_surrogate as TS
    c = CONFIG4
    size, wp = c["size"], glsu.WffParams(*c["wff"])
    seq = synth.DeviceSequence(size, size, seed=seed, noise=c["noise"], n_gauss=c["n_gauss"])
    d = glsu.DPRA(seq.phi0.astype(np.float32), 1, c["radius"], "f32", wp)
    tu = d.tuning()
    if form == "surrogate":
        params, dil = TS.load(SIGMA15_WEIGHTS)
        d.set_surrogate(params, dil, SUR4_TILE, 0, SUR_TOL)
    st = torch.cuda.Stream()
    d.set_stream(st.cuda_stream)
    d.set_graph(True)
    buf = torch.empty((size, size), dtype=torch.float32, device="cuda")
    ms, errs, fp64_s = [], [], 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for k in range(1, warm + nframes + 1):
        buf.copy_(seq.frame(k))
        sample = k - warm in fp64_frames
        pref = d.get(glsu.PHI_REF) if sample else None
        torch.cuda.synchronize()
        e0.record(st)
        d.per_frame_device(buf.data_ptr(), glsu.F32)
        d.update_ref_phi()
        e1.record(st)
        torch.cuda.synchronize()
        if k > warm:
            ms.append(e0.elapsed_time(e1))
        if sample:
            t0 = time.perf_counter()
            errs.append((k,) + fp64_frame_error(glsu, pref, buf, c["radius"], wp, d.get(glsu.PHI_REF)))
            fp64_s += time.perf_counter() - t0
    d.set_graph(False)
    if form == "surrogate":
        d.set_probe_overlap(False)  # stage split with the stages one after another
    d.stage_timing(True)
    buf.copy_(seq.frame(warm + nframes + 1))
    d.per_frame_device(buf.data_ptr(), glsu.F32)
    stg = d.stage_times()
    stats = d.surrogate_stats() if form == "surrogate" else None
    d.close()
    mean_ms = float(np.mean(ms))
    out = {"frames_per_s": 1e3 / mean_ms, "ms_per_frame": mean_ms, "frames_timed": nframes,
           "fp64_samples": [{"frame": k, "rmse": r, "max": m} for k, r, m in errs],
           "rmse_vs_fp64": float(np.sqrt(np.mean([r * r for _, r, _ in errs]))) if errs else None,
           "max_abs_vs_fp64": max(m for _, _, m in errs) if errs else None, "fp64_check_s": fp64_s}
    if form == "plain":
        out["stages_ms"] = {"dpra_ls": stg[0], "wff_rows": stg[1], "wff_column_sweep": stg[2],
                            "wff_final_update": stg[3]}
        out["column_sweep"] = tu
    else:
        out["stages_ms"] = {"dpra_ls": stg[0], "network": stg[1], "wff2_probe_and_residuals": stg[2],
                            "fallback_and_update": stg[3], "wff2_probe_sweep": stg[7]}
        out["tiles_probed_recomputed"] = list(stats)
        out["probe"] = {"tile": SUR4_TILE, "patch": 4, "tol_rad": SUR_TOL}
    return out


def large_workload(glsu, torch, seed, nframes=20, warm=2, fp64_frames=tuple(range(2, 21, 2))):
    """The large streaming workload (2048^2, 8 Gaussians, noise 0.05, DPRA
    9x9, WFF2 sigma 15 with 31 x 31 frequencies on [-1.5, 1.5]): the plain
    FP32 form and, with the sigma-15 network (glsu/surrogate_sigma15.npz),
    the surrogate form, on the same sequence in graph mode; frames/s, stage
    split, HBM figures and the FP64 check on sampled frames."""
    c = CONFIG4
    size = c["size"]
    plain = _large_run(glsu, torch, seed, "plain", nframes, warm, fp64_frames)
    s = int(np.floor(3 * c["wff"][0] + 0.5))
    nfx = glsu.wff_count(c["wff"][1], c["wff"][2], c["wff"][3], glsu.F32)
    P = fft_padded(size + 2 * s) ** 2
    fft_bytes = (64 * nfx * nfx + 32) * P
    pitch = (size + 127) // 128 * 128
    col_bytes = 2 * nfx * size * pitch * 8
    plain["hbm"] = {"compulsory_gb_per_s": col_bytes / (plain["stages_ms"]["wff_column_sweep"] * 1e-3) / 1e9,
                    "fft_model_bytes_per_frame": fft_bytes,
                    "fft_model_gb_per_s": fft_bytes / (plain["ms_per_frame"] * 1e-3) / 1e9,
                    "what": "compulsory: the column sweep's R-plane read and C-plane write over its time; "
                            "fft_model: frame throughput x the FFT formulation's algorithmic bytes per frame "
                            "((64 n_freq + 32) P, P = %d^2)" % int(P ** 0.5)}
    out = {"workload": "2048x2048 FP32, 8 Gaussians, noise 0.05, DPRA 9x9, WFF2 sigma 15, xi in [-1.5, 1.5] step "
                       "0.1 (%dx%d frequencies), thr 0.2, graph mode" % (nfx, nfx),
           "plain": plain}
    if os.path.exists(SIGMA15_WEIGHTS):
        sur = _large_run(glsu, torch, seed, "surrogate", nframes, warm, fp64_frames)
        out["surrogate"] = sur
        out["speedup_surrogate_vs_plain"] = sur["frames_per_s"] / plain["frames_per_s"]
    else:
        out["surrogate"] = {"unavailable": "no sigma-15 weights (glsu/surrogate_sigma15.npz)"}
    return out


BATCH_SIZES = ((256, 256), (384, 512), (1024, 1024), (1536, 2048))  # (H, W) of the batched form's mix


def batched_measure(glsu, torch, seed, sizes=BATCH_SIZES, per_size=2, nframes=4):
    """The batched form on a small mix of uneven sequences (per_size sequences
    of each of four sizes, DPRA 7x7, the plain WFF2 with 21x21 frequencies,
    every handle in graph mode): nframes frames of each through
    glsu_dpra_batch_step (each sequence's frame on its own stream), against
    the same sequences run one after another on one stream.  Device time
    from CUDA events around the frames, after one warm-up frame each."""
    from glsu import synth
    wp = glsu.WffParams(*WFF)
    seqs, handles, px = [], [], 0
    for k, (H, W) in enumerate(tuple(sizes) * per_size):
        frames, phi0, _ = synth.sequence(H, W, nframes + 1, seed=seed + 7 * k)
        seqs.append((torch.from_numpy(frames).cuda(), phi0.astype(np.float32)))
        px += H * W * nframes

    def make():
        hs = []
        for fr, phi0 in seqs:
            d = glsu.DPRA(phi0, 1, RADIUS, "f32", wp)
            d.set_graph(True)
            hs.append(d)
        return hs

    def run(hs, batched):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for step in range(nframes + 1):
            if step == 1:
                torch.cuda.synchronize()
                e0.record()
            if batched:
                glsu.dpra_batch_step(hs, [fr[step].data_ptr() for fr, _ in seqs], glsu.F32)
            else:
                for d, (fr, _) in zip(hs, seqs):
                    d.per_frame_device(fr[step].data_ptr(), glsu.F32)
                    d.update_ref_phi()
                    torch.cuda.synchronize()  # one sequence's frame at a time
        glsu.dpra_batch_wait(hs)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    hs = make()
    ms_b = run(hs, True)
    for d in hs:
        d.close()
    hs = make()
    ms_s = run(hs, False)
    for d in hs:
        d.close()
    nf = len(seqs) * nframes
    return {"workload": "%d sequences (%s, %d each), %d frames each after one warm-up frame, DPRA %dx%d, "
                        "WFF2 21x21 frequencies, FP32, graph mode" % (
                            len(seqs), ", ".join("%dx%d" % (w, h) for h, w in sizes), per_size, nframes,
                            2 * RADIUS + 1, 2 * RADIUS + 1),
            "batched_ms": ms_b, "sequential_ms": ms_s, "frames": nf, "megapixels": px / 1e6,
            "batched_frames_per_s": nf / (ms_b * 1e-3), "batched_mpixels_per_s": px / 1e6 / (ms_b * 1e-3),
            "speedup_vs_sequential": ms_s / ms_b}


MIX_SIZES = ((256, 256), (384, 512), (1024, 1024), (1536, 2048))  # (H, W), 16 sequences each


def batched_mix(glsu, torch, seed, per_size=16, fmin=10, fmax=100):
    """The batched form at its full mix: 16 sequences each of 256^2,
    512x384, 1024^2 and 1536x2048 (W x H), frame counts U[fmin, fmax],
    DPRA windows 5, 7 or 9, WFF2 with 21 x 21 frequencies, FP32, frames of
    each sequence's own seeded generator (made on the GPU before each step,
    outside the timing).  The staged batch (glsu_dpra_batch_*, graph mode:
    the FFT column sweeps of all sequences of a transform length in one
    persistent launch) against the same sequences run one after another
    (graph-mode handles, one frame at a time); device time per step bracketed
    by synchronisation, summed over the steps.  The two runs' final phases
    are compared bit for bit."""
    from glsu import synth
    rng = np.random.default_rng(seed + 77)
    wp = glsu.WffParams(*WFF)
    specs = []
    for (H, W) in MIX_SIZES:
        for k in range(per_size):
            specs.append((H, W, int(rng.integers(fmin, fmax + 1)), int(rng.choice([2, 3, 4])),
                          seed * 1000 + len(specs)))
    nsteps = max(sp[2] for sp in specs)
    frames_total = sum(sp[2] for sp in specs)
    px_total = sum(sp[0] * sp[1] * sp[2] for sp in specs)

    def make():
        seqs, hs = [], []
        for (H, W, nf, r, sd) in specs:
            q = synth.DeviceSequence(H, W, seed=sd)
            d = glsu.DPRA(q.phi0.astype(np.float32), 1, r, "f32", wp)
            d.set_graph(True)
            seqs.append(q)
            hs.append(d)
        return seqs, hs

    def run(batched):
        seqs, hs = make()
        bufs = [torch.empty((H, W), dtype=torch.float32, device="cuda") for (H, W, _, _, _) in specs]
        b = glsu.DpraBatch(hs, graph=True) if batched else None
        total = 0.0
        for step in range(nsteps):
            act = [step < sp[2] for sp in specs]
            for k, q in enumerate(seqs):
                if act[k]:
                    bufs[k].copy_(q.frame(step + 1))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if batched:
                b.run([bufs[k].data_ptr() if act[k] else None for k in range(len(specs))], glsu.F32)
                b.sync()
            else:  # the handles share the legacy stream: one frame after another, no host round trips
                for k, d in enumerate(hs):
                    if act[k]:
                        d.per_frame_device(bufs[k].data_ptr(), glsu.F32)
                        d.update_ref_phi()
                torch.cuda.synchronize()
            total += time.perf_counter() - t0
        phases = [d.get(glsu.PHI_REF) for d in hs]
        if b is not None:
            b.close()
        for d in hs:
            d.close()
        return total, phases

    t_b, ph_b = run(True)
    t_s, ph_s = run(False)
    same = all(np.array_equal(a, c) for a, c in zip(ph_b, ph_s))
    return {"workload": "64 sequences: 16 each of 256x256, 512x384, 1024x1024, 2048x1536 (W x H), frame counts "
                        "U[%d, %d] (%d frames, %.0f megapixels in all), DPRA windows 5/7/9, WFF2 21x21 "
                        "frequencies, FP32; staged batch in graph mode against the same sequences one after "
                        "another" % (fmin, fmax, frames_total, px_total / 1e6),
            "batched_s": t_b, "sequential_s": t_s, "steps": nsteps, "frames": frames_total,
            "batched_frames_per_s": frames_total / t_b, "sequential_frames_per_s": frames_total / t_s,
            "batched_mpixels_per_s": px_total / 1e6 / t_b, "speedup_vs_sequential": t_s / t_b,
            "outputs_identical": bool(same)}


def plain_accuracy(glsu, torch, dfr, phi0, wp, nframes):
    """Teacher-forced phase error of the plain FP32 form against the FP64
    G-LS3U frame from the same reference phase (per frame, all pixels and
    pixels with |WFF2| >= 0.1)."""
    d = glsu.DPRA(phi0.astype(np.float32), 1, RADIUS, "f32", wp)
    rm, mx, mxm = [], [], []
    for k in range(1, nframes + 1):
        pref = d.get(glsu.PHI_REF).astype(np.float64)
        d64 = glsu.DPRA(pref, 1, RADIUS, "f64", wp)
        d64.per_frame_device(dfr[k].data_ptr(), glsu.F32)
        pc64 = d64.get(glsu.PHI_CURR)
        d64.close()
        d.per_frame_device(dfr[k].data_ptr(), glsu.F32)
        pc = d.get(glsu.PHI_CURR).astype(np.float64)
        e = np.abs(np.angle(np.exp(1j * (pc - pc64))))
        rm.append(float(np.sqrt(np.mean(e ** 2))))
        mx.append(float(e.max()))
        d.update_ref_phi()
    d.close()
    return {"rmse_vs_fp64": float(np.sqrt(np.mean(np.square(rm)))), "max_abs_vs_fp64": max(mx),
            "frames": nframes, "bar_rad": 1e-3}


def wfr_measure(glsu, torch, phi0, size, seed):
    """WFR2 (windowed Fourier ridges) with the reference's WFR defaults
    (sigma 10, 161 x 161 frequencies on [-2, 2] step 0.025, counted in float as
    WFT2_CUDAF does) on the fringe field exp(j phi0) + noise at size^2, FP32:
    device time of one run (after one warm-up) and the FP32-pipe fraction of
    its algorithmic FMAs (per frequency and pixel, 2 (2s+1) for the column
    filter; per wx and pixel, 2 (2s+1) for the row filter)."""
    rng = np.random.default_rng(seed)
    f = np.exp(1j * phi0) + 0.05 * (rng.standard_normal(phi0.shape) + 1j * rng.standard_normal(phi0.shape))
    df = torch.from_numpy(f.astype(np.complex64)).cuda()
    maps = {k: torch.empty((size, size), dtype=torch.float32, device="cuda") for k in glsu.WFR_FIELDS}
    ptrs = {k: v.data_ptr() for k, v in maps.items()}
    p = glsu.default_params(glsu.WFT_WFR)
    w = glsu.WFR2(size, size, "f32", p)
    w.run(df.data_ptr(), ptrs)
    ms = min(w.run(df.data_ptr(), ptrs) for _ in range(3))
    w.close()
    n = glsu.wff_count(p.wxl, p.wxh, p.wxi, glsu.F32)
    s = int(np.floor(3 * p.sigma_x + 0.5))
    fma = float(n) * n * size * size * 2 * (2 * s + 1) + float(n) * size * size * 2 * (2 * s + 1)
    return {"workload": "WFR2 of exp(j phi0) + noise, %dx%d FP32, sigma %g, %dx%d frequencies on [%g, %g] step %g"
                        % (size, size, p.sigma_x, n, n, p.wxl, p.wxh, p.wxi),
            "ms": ms, "frames_per_s": 1e3 / ms, "algorithmic_fma": fma,
            "fp32_tflops": 2 * fma / (ms * 1e-3) / 1e12,
            "fp32_frac_of_peak_at_2070mhz": 2 * fma / (ms * 1e-3) / (152 * 128 * 2 * 2070e6)}


def fft_sweep_flops(size, nfx, nfy, L, pitch):
    """Algorithmic FP32 flops of one FFT column sweep: per column and
    x-frequency, 2 nfy + 2 transforms of length L at 5 L log2 L each, plus
    per wy the two window products (6 flops a point each), the threshold and
    the accumulation (4)."""
    return float(pitch) * nfx * ((2 * nfy + 2) * 5.0 * L * np.log2(L) + nfy * 16.0 * L)


def probe_recall(glsu, SE, params, dil, size):
    """The sparse probe's recall on tiles the network gets wrong (network-only
    RMSE above the tolerance over the pixels where the WFF2 phase is
    defined): with the network's last layer negated (wrong on every tile: the
    probe, flag and fallback mechanism), and with a 0.9 rad/px carrier in the
    phase change over the centre quarter of the frame (tile-local, partial
    errors), 12 frames with every 2nd checked."""
    keys = ("frames_sampled", "tiles_over_tol", "probe_recall", "tiles_flagged_within_tol", "rmse_median",
            "rmse_network_only_median", "tiles_recomputed_fraction")
    out = {}
    for name, prm, kw, nf, ev in (("reversed_residual", SE.reversed_residual(params), {}, 4, 4),
                                  ("carrier_0.9", params, {"delta_extra": SE.carrier_region(size)}, 12, 2)):
        r = SE.deployment(glsu, prm, dil, [60100], nf, ev, size, wff=WFF, radius=RADIUS, tile=SUR_TILE,
                          patch=SUR_PATCH, tol=SUR_TOL, **kw)
        out[name] = {k: r[k] for k in keys}
        out[name]["bad_tile_rmse"] = [round(v, 4) for x in r["per_frame"] for v in x["bad_tile_rmse"]]
    return out


def surrogate_training(glsu, torch, steps=20, warm=3, batch=16, crop=256):
    """Training throughput of the surrogate's own kernels: one step is the
    forward pass, the loss, the backward pass (data and weight gradients of
    the hidden layers on the tensor cores) and the Adam update, for a
    batch of `batch` crop x crop pairs already on the device; CUDA events on
    the handle's stream around `steps` steps after `warm`.  The forward pass
    alone is timed the same way, so the backward + update share follows."""
    from glsu import train_surrogate as TS
    net = glsu.Surrogate(batch, crop, crop, TS.DILATIONS, training=True)
    net.params = TS.init_params(0)
    st = torch.cuda.Stream()
    net.set_stream(st.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)
    ph = torch.rand((batch, crop, crop), generator=g, device="cuda") * (2 * np.pi)
    z = torch.polar(torch.ones_like(ph), ph).to(torch.complex64)
    t = torch.polar(torch.ones_like(ph), ph + 0.1 * torch.randn(ph.shape, generator=g, device="cuda"))
    t = t.to(torch.complex64)
    out = torch.empty_like(z)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(steps):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def step():
        net.backward(z.data_ptr(), t.data_ptr(), want_loss=False)
        net.adam(1e-4)

    ms_step = timed(step)
    ms_fwd = timed(lambda: net.forward(z.data_ptr(), out.data_ptr()))
    loss, _ = net.backward(z.data_ptr(), t.data_ptr(), want_loss=True)
    net.close()
    px = batch * crop * crop
    hidden = 2 * 288 * 32  # flops a pixel of one 32 -> 32 layer
    fwd = 2 * 9 * 2 * 32 + 6 * hidden + 2 * 288 * 2
    flops = 3 * fwd * px  # forward, data gradients, weight gradients
    return {"steps_per_s": 1e3 / ms_step, "ms_per_step": ms_step, "pairs_per_s": batch * 1e3 / ms_step,
            "batch": batch, "crop": crop, "ms_forward": ms_fwd, "ms_backward_and_update": ms_step - ms_fwd,
            "tflops": flops / (ms_step * 1e-3) / 1e12, "flops_per_step": flops,
            "tensor_core_share_of_flops": 3 * 6 * hidden / (3 * fwd),
            "loss_after": loss, "steps_timed": steps,
            "what": "forward + loss + backward + Adam on device-resident synthetic pairs; the hidden layers' "
                    "forward, data gradients and weight gradients on tcgen05 (FP32 accumulation), layers 0 and 7 "
                    "and the bias gradients on CUDA cores"}


def run_ours(args, rank, world, local):
    import torch
    import glsu
    from glsu import synth
    from glsu import train_surrogate as TS
    from glsu import surrogate_eval as SE
    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device: the GB300 path has no CPU fallback")
    torch.cuda.set_device(local)
    size = args.size
    N = size * size
    wp = glsu.WffParams(*WFF)
    seed = 1000 + rank
    # one consecutive frame of the sequence per warm-up and timed step (a
    # wrapped index would feed frame 0 after frame k, a k-frame phase jump)
    nfr = args.warmup + args.steps + STAGE_FRAMES + 1
    frames, phi0, _ = synth.sequence(size, size, nfr, seed=seed)
    # the legs beside the headline run in the single-GPU run only (rank 0 of
    # one): under torchrun the other ranks would wait for them at the first
    # collective
    extras = not args.frames_only and rank == 0 and world == 1

    wfr = batched = prec1 = large = training = None
    if extras:
        wfr = wfr_measure(glsu, torch, phi0, size, seed)
        batched = {"config_mix": batched_mix(glsu, torch, seed),
                   "streams_uneven_sizes": batched_measure(glsu, torch, seed),
                   "streams_small_frames": batched_measure(glsu, torch, seed, sizes=((256, 256),), per_size=16,
                                                           nframes=8)}
        prec1 = precision_form(glsu, torch, seed, size)
        large = large_workload(glsu, torch, seed)
        training = surrogate_training(glsu, torch)

    stream = torch.cuda.Stream()
    dfr = torch.from_numpy(frames).cuda()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # ---- plain form: DPRA LS -> WFF2 -> update
    dp = glsu.DPRA(phi0.astype(np.float32), 1, RADIUS, "f32", wp)
    dp.set_stream(stream.cuda_stream)
    dp.set_graph(True)
    p_val, p_ms, p_st, p_clk = timed_frames(glsu, torch, dp, dfr, nfr, args, stream, flush, world, local)
    p_tuning = dp.tuning()
    dp.close()

    hseq = hphi0 = None
    if not args.frames_only:
        hseq, hphi0 = host_sequence(torch, size, args.warmup + E2E_FRAMES, seed)

    def plain_handle():
        h = glsu.DPRA(hphi0.astype(np.float32), 1, RADIUS, "f32", wp)
        h.set_stream(stream.cuda_stream)
        h.set_graph(True)
        return h

    p_e2e = p_e2e_runs = p_acc = copies = None
    if not args.frames_only:
        p_e2e, p_e2e_runs = e2e_sequence(glsu, torch, plain_handle, hseq, args, stream, flush, world)
        p_acc = plain_accuracy(glsu, torch, dfr, phi0, wp, 3)
        copies = copy_times(torch, size)

    # ---- surrogate form: DPRA LS -> network -> probes -> per-tile fallback -> update
    sur = None
    try:
        params, dil = TS.load()
    except (OSError, KeyError) as e:
        params, dil = None, None
        sur = {"unavailable": "no trained weights (%s)" % e}
    if params is not None:
        ds = glsu.DPRA(phi0.astype(np.float32), 1, RADIUS, "f32", wp)
        ds.set_stream(stream.cuda_stream)
        ds.set_surrogate(params, dil, SUR_TILE, SUR_PATCH, SUR_TOL)
        ds.set_graph(True)
        s_val, s_ms, s_st, s_clk = timed_frames(glsu, torch, ds, dfr, nfr, args, stream, flush, world, local)
        probed, flagged = ds.surrogate_stats()
        ds.close()
        # the probe's cost scales with the number of tiles: the same frames
        # with 128^2 tiles (64 probes a frame) and 512^2 tiles (4 probes)
        tile_variants = None
        if extras:
            tile_variants = {}
            for tv in (128, 512):
                dv = glsu.DPRA(phi0.astype(np.float32), 1, RADIUS, "f32", wp)
                dv.set_stream(stream.cuda_stream)
                dv.set_surrogate(params, dil, tv, SUR_PATCH, SUR_TOL)
                dv.set_graph(True)
                v_val, v_ms, v_st, _ = timed_frames(glsu, torch, dv, dfr, nfr, args, stream, flush, world, local)
                dv.close()
                tile_variants["tile_%d" % tv] = {"frames_per_s": v_val, "ms_per_step": v_ms / args.steps,
                                                 "probes_per_frame": (-(-size // tv)) ** 2,
                                                 "probe_sweep_ms": v_st[7]}

        def sur_handle():
            h = plain_handle()
            h.set_surrogate(params, dil, SUR_TILE, SUR_PATCH, SUR_TOL)
            return h

        s_e2e = s_e2e_runs = deploy = None
        acc = {"rmse": None, "rmse_vs_fp64": None}
        if not args.frames_only:
            s_e2e, s_e2e_runs = e2e_sequence(glsu, torch, sur_handle, hseq, args, stream, flush, world)
            acc = surrogate_accuracy(glsu, torch, dfr, phi0, wp, params, dil, min(6, nfr - 1))
        if extras:
            dep = SE.deployment(glsu, params, dil, range(DEPLOY_SEED0, DEPLOY_SEED0 + DEPLOY_SEEDS),
                                DEPLOY_FRAMES, DEPLOY_EVERY, size, wff=WFF, radius=RADIUS, tile=SUR_TILE,
                                patch=SUR_PATCH, tol=SUR_TOL)
            deploy = {k: v for k, v in dep.items() if k != "per_frame"}
            deploy["rmse_per_sampled_frame"] = [round(x["rmse"], 5) for x in dep["per_frame"]]
            deploy["workload"] = ("%d held-out seeds (%d..) of the 1024^2 generator, %d free-running frames each in "
                                  "the surrogate form (graph mode); every %d-th frame against the FP64 frame from "
                                  "the same reference phase" % (DEPLOY_SEEDS, DEPLOY_SEED0, DEPLOY_FRAMES,
                                                                 DEPLOY_EVERY))
            deploy["probe_recall"] = probe_recall(glsu, SE, params, dil, size)
        sur = {"frames_per_s": s_val, "ms_per_step": s_ms / args.steps, "speedup_vs_plain": s_val / p_val,
               "tile_variants": tile_variants,
               "e2e_frames_per_s": s_e2e, "e2e_runs": s_e2e_runs,
               "stages_ms": {"dpra_ls": s_st[0], "network": s_st[1], "wff2_probe_and_residuals": s_st[2],
                             "fallback_and_update": s_st[3]},
               "network_ms": {"layer0": s_st[4], "tensor_core_layers_1_6": s_st[5], "layer7": s_st[6]},
               "wff2_probe_sweep_ms": s_st[7],
               "probe_overlap": "in the timed frames the probe sweep runs on a second stream beside the "
                                "network; the stage split is taken with the stages one after another",
               "fallback_fraction_timed": flagged / probed if probed else None,
               "probe": {"tile": SUR_TILE, "patch": SUR_PATCH, "tol_rad": SUR_TOL},
               "dilations": dil, "params": int(params.size),
               "accuracy": acc,
               "deployment": deploy,
               "rmse_target_rad": 0.02,
               "meets_rmse_target": (None if deploy is None else
                                     bool(deploy["rmse_median"] <= 0.02 and deploy["rmse_p90"] <= 0.02))}

    # ---- rooflines
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    peak_kind = "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback"
    pitch = (size + 127) // 128 * 128
    col_bytes = 2 * NFX * size * pitch * 8  # read R_i planes + write C_i planes (complex64)
    sm_mhz = p_clk.get("sm_mhz") or 1900.0
    fp32_peak_tflops = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    if p_tuning["method"] == glsu.METHOD_FFT:
        col_flops = fft_sweep_flops(size, NFX, NFY, p_tuning["fft_length"], pitch)
        col_kernel, flop_rule = "wff_colfft_kernel (WFF2 FFT column sweep, L = %d)" % p_tuning["fft_length"], \
            "5 L log2 L per transform, 2 nfy + 2 transforms per column and wx, + 16 L per wy"
    else:
        sx = int(np.floor(3 * WFF[0] + 0.5))
        col_flops = float(NFX * NFY * N * 2 * (2 * sx + 1) * 2)
        col_kernel, flop_rule = "wff_cols_kernel (WFF2 direct column sweep)", "2 column filters x (2s+1) taps x 2"
    col_s = p_st[2] * 1e-3
    fb, P = fft_model_bytes(size)
    plain_roof = {"kernel": col_kernel, "bound": "fp32",
                  "achieved": col_flops / col_s / 1e12, "peak": fp32_peak_tflops, "unit": "TFLOP/s",
                  "frac": col_flops / col_s / 1e12 / fp32_peak_tflops,
                  "peak_source": "152 SMs x 128 FP32 lanes x 2 x sampled SM clock (%.0f MHz)" % sm_mhz,
                  "algorithmic_flops_per_launch": col_flops, "flop_rule": flop_rule, "launch_ms": p_st[2],
                  "hbm_compulsory": {"bytes_per_launch": col_bytes, "achieved": col_bytes / col_s / 1e9,
                                     "peak": hbm_peak, "unit": "GB/s", "frac": col_bytes / col_s / 1e9 / hbm_peak},
                  "fft_model": {
                      "what": "side figure: frame throughput x the reference FFT formulation's algorithmic bytes "
                              "per frame ((64 n_freq + 32) P, P = padded plane %d^2)" % int(P ** 0.5),
                      "bytes_per_frame": fb, "achieved": fb * p_val / world / 1e9, "peak": hbm_peak, "unit": "GB/s",
                      "frac": fb * p_val / world / 1e9 / hbm_peak}}
    roof = plain_roof
    if sur and "stages_ms" in sur:
        net_ms = sur["stages_ms"]["network"]
        # the tensor-core layer: six launches per frame, timed together
        conv_ms = sur["network_ms"]["tensor_core_layers_1_6"] / 6
        conv_bytes, conv_flops = SUR_CONV_BYTES_PER_PX * N, SUR_CONV_FLOPS_PER_PX * N
        traffic = SUR_CONV_TRAFFIC_1024 if size == 1024 else None
        conv_roof = {"kernel": "sur_conv_tc_kernel (tcgen05 32->32 dilated 3x3 layer, per launch)", "bound": "tensor",
                     "achieved": conv_flops / (conv_ms * 1e-3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": conv_flops / (conv_ms * 1e-3) / 1e12 / bf16_peak,
                     "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at "
                                       "1024x1024 (profiles/sur_conv_tc_kernel_1024.md)",
                     "peak_source": peak_kind + ", dense bf16 burst",
                     "algorithmic_flops_per_launch": conv_flops, "launch_ms": conv_ms,
                     "hbm": {"algorithmic_bytes_per_launch": conv_bytes,
                             "achieved": conv_bytes / (conv_ms * 1e-3) / 1e9,
                             "dram_achieved": None if traffic is None else traffic / (conv_ms * 1e-3) / 1e9,
                             "peak": hbm_peak, "unit": "GB/s",
                             "dram_frac": None if traffic is None else traffic / (conv_ms * 1e-3) / 1e9 / hbm_peak}}
        net_flops = SUR_FLOPS_PER_PX * N
        sur["roofline_network"] = {"kernels": "sur_l0 + 6 x sur_conv_tc (tcgen05) + sur_l7", "bound": "tensor",
                                   "achieved": net_flops / (net_ms * 1e-3) / 1e12, "peak": bf16_peak,
                                   "unit": "TFLOP/s", "frac": net_flops / (net_ms * 1e-3) / 1e12 / bf16_peak}
        sur["roofline_tensor_core_layer"] = conv_roof
        sur["roofline_plain_column_sweep"] = plain_roof
        kern = {"sur_conv_tc_kernel x6": sur["network_ms"]["tensor_core_layers_1_6"],
                "wff_probe_kernels (beside the network)": sur["wff2_probe_sweep_ms"],
                "dpra_ls_ff_kernel": sur["stages_ms"]["dpra_ls"],
                "sur_l7_kernel": sur["network_ms"]["layer7"], "sur_l0_kernel": sur["network_ms"]["layer0"]}
        sur["dominant_kernel"] = max(kern, key=kern.get)
        roof = conv_roof

    headline = sur if (sur and "frames_per_s" in sur) else None
    e2e_val = headline["e2e_frames_per_s"] if headline else p_e2e
    out = {
        "metric": METRIC, "value": headline["frames_per_s"] if headline else p_val, "unit": "frames/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": headline["ms_per_step"] if headline else p_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "form": "surrogate" if headline else "plain",
        "config": workload_config(size),
        "clocks": s_clk if headline else p_clk,
        "e2e": {"value": e2e_val, "unit": "frames/s", "h2d_bytes_per_step": 4 * N, "d2h_bytes_per_step": 4 * N,
                "frames_per_run": E2E_FRAMES, "runs": headline["e2e_runs"] if headline else p_e2e_runs,
                "statistic": "median of the runs",
                "h2d_ms_per_frame": copies[0] if copies else None, "d2h_ms_per_frame": copies[1] if copies else None,
                "overhead_ms_per_frame": None if not e2e_val else 1e3 / e2e_val -
                (headline["ms_per_step"] if headline else p_ms / args.steps)},
        "gpu_launches": (SUR_LAUNCHES if headline else PLAIN_LAUNCHES) * args.steps,
        "roofline": roof,
        "plain": {"frames_per_s": p_val, "ms_per_step": p_ms / args.steps, "e2e_frames_per_s": p_e2e,
                  "e2e_runs": p_e2e_runs,
                  "stages_ms": {"dpra_ls": p_st[0], "wff_rows": p_st[1], "wff_column_sweep": p_st[2],
                                "wff_final_update": p_st[3]},
                  "roofline": plain_roof, "clocks": p_clk, "gpu_launches_per_step": PLAIN_LAUNCHES,
                  "column_sweep_autotune": p_tuning, "accuracy": p_acc},
        "surrogate": sur,
        "precision_form": prec1,
        "large_workload": large,
        "surrogate_training": training,
        "wfr": wfr,
        "batched_form": batched,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline: rank 0 at N = 1 only
        v32, secs, threads, rows = cpu_sample(size, prec="f32")
        v64, secs64, _, _ = cpu_sample(size, prec="f64")
        out["cpu_baseline"] = {
            "value": max(v32, v64), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": "one whole %dx%d frame in each precision (%d threads; FP32 %.1f s, FP64 %.1f s): DPRA LS, "
                      "WFF2 over all 441 frequencies (one frequency row per OpenMP thread at a time), update, "
                      "with the restatements of the reference's CPU classes in FP32 (DPRA_CPUF/WFT2_cpuF) and "
                      "FP64 (DPRA_CPU/WFT2_cpu); value is the faster of the two"
                      % (size, size, threads, secs, secs64),
            "fp32_value": v32, "fp64_value": v64}
    return out if rank == 0 else None


def main():
    args = parse()
    rank, world, local = dist_init()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
