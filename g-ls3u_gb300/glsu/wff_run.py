"""Run the WFF2 (or the column-sweep candidates) on a synthetic fringe field
and print the autotuner's choice and the device time of each run.

    python -m glsu.wff_run --size 1024 --sigma 15 --wl -1.5 --wh 1.5 --step 0.1 --method fft --runs 2

(from ``g-ls3u_gb300/``).  The field is exp(j phi) + 0.05 complex noise with
phi = 0.3 x + 0.1 y + 3 sin(x / 90), seeded; FP32 unless --f64.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import glsu  # noqa: E402


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--sigma", type=float, default=10.0)
    ap.add_argument("--wl", type=float, default=-1.0)
    ap.add_argument("--wh", type=float, default=1.0)
    ap.add_argument("--step", type=float, default=0.1)
    ap.add_argument("--thr", type=float, default=0.2)
    ap.add_argument("--method", choices=["auto", "direct", "fft", "timed"], default="auto")
    ap.add_argument("--runs", type=int, default=2)
    ap.add_argument("--f64", action="store_true")
    args = ap.parse_args(argv)
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("no CUDA device")
    n = args.size
    rng = np.random.default_rng(0)
    y, x = np.mgrid[0:n, 0:n]
    f = np.exp(1j * (0.3 * x + 0.1 * y + 3 * np.sin(x / 90.0))) + 0.05 * (rng.standard_normal((n, n)) +
                                                                        1j * rng.standard_normal((n, n)))
    prec, dt = ("f64", torch.complex128) if args.f64 else ("f32", torch.complex64)
    df = torch.from_numpy(f).to(dt).cuda()
    out = torch.empty_like(df)
    p = glsu.WffParams(args.sigma, args.wl, args.wh, args.step, args.sigma, args.wl, args.wh, args.step, args.thr)
    w = glsu.WFF2(n, n, prec, p)
    w.set_method({"auto": glsu.METHOD_AUTO, "direct": glsu.METHOD_DIRECT, "fft": glsu.METHOD_FFT,
                  "timed": glsu.METHOD_TIMED}[args.method])
    print("tuning:", w.tuning())
    for _ in range(args.runs):
        print("ms %.3f" % w.run(df.data_ptr(), out.data_ptr()))
    w.close()


if __name__ == "__main__":
    main()
