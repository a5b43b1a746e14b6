"""Host-side pieces of bench.py that need no GPU: the FFT-model byte count
used for the plain form's HBM roofline, and the CPU baseline's sample."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_padded_size_equals_the_reference_fft_table():
    import bench
    lut = json.load(open(os.path.join(ROOT, "tests", "golden", "fft_lut.json")))["sizes"]
    for x in range(1, max(lut) + 1):
        assert bench.fft_padded(x) == min(v for v in lut if v >= x), x


def test_fft_model_bytes_at_1024():
    import bench
    b, P = bench.fft_model_bytes(1024)
    assert P == 1120 * 1120                     # 1024 + 2 * round(3 * 10) -> 1120
    assert abs(b / 1e9 - 35.44) < 0.01          # (64 * 441 + 32) * P bytes


def test_cpu_sample_runs_whole_frames_in_both_variants(monkeypatch):
    """The CPU baseline's sample is a whole frame (all 21 frequency rows, at
    any host thread count) in the FP32 and the FP64 restatement; a partial
    sample (warm-up) sweeps fewer rows."""
    import bench
    for threads in (4, 16, 32):
        monkeypatch.setattr(os, "cpu_count", lambda t=threads: t)
        fps, secs, th, rows = bench.cpu_sample(64, prec="f32")
        assert th == threads and rows == bench.NFY
        assert fps > 0 and secs > 0 and abs(fps * secs - 1.0) < 1e-9
    monkeypatch.setattr(os, "cpu_count", lambda: 8)
    fps64, _, _, rows = bench.cpu_sample(64, 3, prec="f64")
    assert rows == 3 and fps64 > 0


def test_reference_arm_times_every_step_as_a_whole_frame(monkeypatch):
    """--impl reference: each timed step is one whole frame, and the line's
    time per step is the mean of the timed steps (no extrapolation)."""
    import argparse
    import bench
    calls = []

    def fake(size, rows=None, seed=1000, prec="f32"):
        calls.append((rows, prec))
        el = 0.5 if rows is None else 0.1
        return 1.0 / el, el, 4, bench.NFY if rows is None else rows

    monkeypatch.setattr(bench, "cpu_sample", fake)
    args = argparse.Namespace(steps=3, warmup=2, size=64, gpus=1)
    res = bench.run_reference(args, 0, 1)
    timed = [c for c in calls if c[0] is None]
    assert len(timed) == 3
    assert abs(res["ms_per_step"] - 500.0) < 1e-9 and abs(res["value"] - 2.0) < 1e-9
    assert res["impl"] == "reference" and res["e2e"]["value"] == res["value"]
    assert bench.run_reference(args, 1, 2) is None


def test_aligned_phase_error_removes_the_global_constant_and_sign():
    """AIA determines the phase up to a global constant and sign; the
    precision form's accuracy figure removes both before measuring."""
    import numpy as np
    import bench
    rng = np.random.default_rng(3)
    truth = rng.uniform(-np.pi, np.pi, (40, 50))
    noise = 1e-3 * rng.standard_normal(truth.shape)
    for sgn in (1.0, -1.0):
        est = np.angle(np.exp(1j * (sgn * (truth + 1.234) + noise)))
        rm, mx, s, c = bench.aligned_phase_error(est, truth)
        assert s == sgn and abs(np.angle(np.exp(1j * (c - 1.234)))) < 1e-3
        assert abs(rm - np.sqrt(np.mean(noise ** 2))) < 2e-4 and mx < 6e-3


def test_fft_sweep_flop_count():
    import bench
    f = bench.fft_sweep_flops(1024, 21, 21, 1280, 1024)
    assert abs(f - 1024 * 21 * (44 * 5 * 1280 * 10.321928094887362 + 21 * 16 * 1280)) < 1e3


def test_recall_cases_and_summary():
    """Host side of the probe-recall legs: the carrier ramp covers the centre
    quarter only, the reversed network negates exactly the last layer, and
    the summary counts bad and caught tiles."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "g-ls3u_gb300"))
    from glsu import surrogate_eval as SE
    from glsu import train_surrogate as T
    m = SE.carrier_region(64, slope=0.9)
    assert m[:16].max() == 0 and m[48:].max() == 0 and m[:, :16].max() == 0
    assert np.allclose(np.diff(m[32, 16:48]), 0.9)
    p = T.init_params(3)
    r = SE.reversed_residual(p)
    n_last = T.LAYER_SIZES[-1][0] * T.LAYER_SIZES[-1][1] * 9 + T.LAYER_SIZES[-1][0]
    assert np.array_equal(r[:-n_last], p[:-n_last]) and np.array_equal(r[-n_last:], -p[-n_last:])
    recs = [{"seed": 1, "frame": 2, "rmse": 0.01, "max": 1.0, "rmse_network_only": 0.02, "max_network_only": 1.0,
             "rmse_without_network": 0.6, "max_without_network": 3.0, "tiles_flagged": 1, "tiles": 16,
             "tiles_bad": 2, "tiles_bad_flagged": 1, "tiles_good_flagged": 0, "bad_tile_rmse": [0.06, 0.1]}]
    s = SE.summarise(recs, 0.05)
    assert s["tiles_over_tol"] == 2 and s["probe_recall"] == 0.5 and s["tiles_recomputed_fraction"] == 1 / 16
