"""File formats of the reference's data (glsu/io.py, include/glsu_io.hpp)."""
import os

import numpy as np

from conftest import GOLDEN


def test_reads_reference_phase_map(tmp_path):
    from glsu import io
    a = io.read_matrix_bin(os.path.join(GOLDEN, "phi_1.bin"))
    assert a.shape == (256, 256) and a.dtype == np.float32
    assert np.isfinite(a).all() and -np.pi - 1e-5 <= a.min() and a.max() <= np.pi + 1e-5
    p = str(tmp_path / "copy.bin")
    io.write_matrix_bin(p, a)
    assert open(p, "rb").read() == open(os.path.join(GOLDEN, "phi_1.bin"), "rb").read()


def test_complex_text_round_trip(tmp_path):
    from glsu import io
    rng = np.random.default_rng(0)
    a = (rng.standard_normal((7, 5)) + 1j * rng.standard_normal((7, 5))).astype(np.complex64)
    p = str(tmp_path / "f.fp")
    io.write_complex_text(p, a)
    assert open(p).readline().strip() == "7,5"
    assert np.array_equal(io.read_complex_text(p), a)


def test_bmp_reader_matches_fixture_frames(tmp_path):
    from glsu import io
    from test_cpp_classes import write_bmp8
    g = np.load(os.path.join(GOLDEN, "aia_bmp.npz"))
    p = str(tmp_path / "f.bmp")
    write_bmp8(p, g["frames"][1])
    assert np.array_equal(io.read_bmp(p), g["frames"][1])


def test_cpp_readers_match_python(tmp_path):
    """include/glsu_io.hpp (reference names) on the reference's own phase map."""
    import shutil
    import subprocess
    from glsu import io
    gxx = shutil.which("g++")
    if gxx is None:
        import pytest
        pytest.skip("g++ not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "test_io")
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", os.path.join(root, "include"), "-I", cuda_inc,
                    os.path.join(root, "tests", "cpp", "test_io.cpp"), "-o", exe], check=True)
    src = os.path.join(GOLDEN, "phi_1.bin")
    out = subprocess.run([exe, src, str(tmp_path / "o.bin"), str(tmp_path / "t.fp")], check=True,
                         capture_output=True, text=True).stdout.split()
    a = io.read_matrix_bin(src)
    assert (int(out[0]), int(out[1])) == a.shape
    assert abs(float(out[2]) - a.astype(np.float64).sum()) <= 1e-6 * np.abs(a).sum()
    assert open(str(tmp_path / "o.bin"), "rb").read() == open(src, "rb").read()
    assert io.read_complex_text(str(tmp_path / "t.fp")).shape == (2, 3)
