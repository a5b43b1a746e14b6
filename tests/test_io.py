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
