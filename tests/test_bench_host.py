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


def test_cpu_sample_runs_both_variants_and_extrapolates_by_rounds(monkeypatch):
    """The CPU baseline's sample: one round of frequency rows (one per host
    thread, at most 21), extrapolated by ceil(21 / threads) rounds; both the
    FP64 and the FP32 restatements run."""
    import bench
    for threads in (4, 16, 32):
        monkeypatch.setattr(os, "cpu_count", lambda t=threads: t)
        fps, secs, th, rows = bench.cpu_sample(64, prec="f32")
        assert th == threads and rows == min(bench.NFY, threads)
        assert fps > 0 and secs > 0
    monkeypatch.setattr(os, "cpu_count", lambda: 8)
    fps64, _, _, rows = bench.cpu_sample(64, 3, prec="f64")
    assert rows == 3 and fps64 > 0
