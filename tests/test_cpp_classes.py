"""The reference's C++ class interfaces (DPRA_CUDAF, DPRA_CUDA, DPRA_HYBRID[F], WFT2_CUDAF
with WFT_TYPE::WFF and WFR, AIA_CUDAF) driven from a compiled C++ program
(tests/cpp/test_classes.cpp) and checked against the FP64 oracle."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG

pytestmark = pytest.mark.gpu
BIN = os.path.join(PKG, "lib", "glsu_cpp_test")


def write_bmp8(path, img):
    """Minimal 8-bit grey-palette bottom-up BMP writer."""
    h, w = img.shape
    stride = (w + 3) & ~3
    pal = b"".join(struct.pack("<BBBB", i, i, i, 0) for i in range(256))
    off = 14 + 40 + len(pal)
    data = b"".join(img[h - 1 - y].tobytes() + b"\0" * (stride - w) for y in range(h))
    hdr = struct.pack("<2sIHHI", b"BM", off + len(data), 0, 0, off)
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 8, 0, len(data), 2835, 2835, 256, 0)
    open(path, "wb").write(hdr + info + pal + data)


def test_reference_class_interfaces(tmp_path, oracle, synth):
    assert os.path.exists(BIN), "C++ test driver not built"
    W, H, nf, r, rr = 48, 40, 3, 2, 1
    wpar = (3.0, -0.5, 0.5, 0.25, 0.1)
    frames, phi0, _ = synth.sequence(H, W, nf, seed=5)
    d = str(tmp_path)
    open(os.path.join(d, "params.txt"), "w").write("%d %d %d %d %d %r %r %r %r %r\n" % ((W, H, nf, r, rr) + wpar))
    phi0.astype(np.float64).tofile(os.path.join(d, "phi0.f64"))
    frames.astype(np.float32).tofile(os.path.join(d, "frames.f32"))
    rng = np.random.default_rng(0)
    field = np.exp(1j * rng.uniform(0, 0.3, (H, W)).cumsum(1)).astype(np.complex64)
    field.tofile(os.path.join(d, "field.c64"))
    g = np.load(os.path.join(GOLDEN, "aia_bmp.npz"))
    for k in range(3):
        write_bmp8(os.path.join(d, "aia%d.bmp" % (k + 1)), g["frames"][k])
    out = subprocess.run([BIN, d], capture_output=True, text=True, timeout=600)
    print(out.stdout, out.stderr)
    assert out.returncode == 0
    assert "errors_caught=2" in out.stdout
    assert "DPRA_HYBRID equal=1" in out.stdout

    wp = oracle.WffParams(wpar[0], wpar[1], wpar[2], wpar[3], wpar[0], wpar[1], wpar[2], wpar[3], wpar[4])
    # DPRA_CUDA (FP64): every frame against the oracle sequence
    dp64 = np.fromfile(os.path.join(d, "dpra_f64_dphi.f64")).reshape(nf, H, W)
    _, odp = oracle.glsu_sequence(frames.astype(np.float32).astype(np.float64), phi0, r, wp, rr=rr)
    assert np.abs(dp64 - odp).max() < 1e-9
    # DPRA_CUDAF (FP32)
    dp32 = np.fromfile(os.path.join(d, "dpra_f32_dphi.f32"), np.float32).reshape(nf, H, W)
    assert np.abs(dp32 - odp).max() < 1e-3
    # WFT2_CUDAF
    wf = np.fromfile(os.path.join(d, "wff_f32.c64"), np.complex64).reshape(H, W)
    ref, _ = oracle.wff2(field.astype(np.complex128), *wp.tuple())
    assert np.abs(wf - ref).max() < 1e-4 * np.abs(ref).max()
    # WFT2_CUDAF with WFT_TYPE::WFR: the ridge maps against the oracle's WFR2
    wr = np.fromfile(os.path.join(d, "wfr_f32.f32"), np.float32).reshape(8, H, W)
    ow = oracle.wfr2(field.astype(np.complex128), wpar[0], wpar[1], wpar[2], wpar[3], wpar[0], wpar[1], wpar[2],
                     wpar[3])
    got = dict(zip(oracle.WFR_FIELDS, wr))
    assert np.abs(got["r"] - ow["r"]).max() < 1e-4 * ow["r"].max()
    same = (got["wx"] == ow["wx"].astype(np.float32)) & (got["wy"] == ow["wy"].astype(np.float32))
    assert same.mean() > 0.99
    assert np.abs(np.angle(np.exp(1j * (got["phase"] - ow["phase"]))))[same].max() < 1e-3
    # AIA_CUDAF on BMPs read by the class layer's imread
    img1 = np.fromfile(os.path.join(d, "aia_img1.u8"), np.uint8).reshape(256, 256)
    assert np.array_equal(img1, g["frames"][0])
    phi = np.fromfile(os.path.join(d, "aia_phi.f32"), np.float32).reshape(256, 256)
    ophi, od, _, _ = oracle.aia(g["frames"].astype(np.float64), g["deltas0"].astype(np.float64), 20, 1e-4)
    delta = np.fromfile(os.path.join(d, "aia_delta.f32"), np.float32)
    assert np.abs(delta - od).max() < 1e-4
    assert np.abs(np.angle(np.exp(1j * (phi - ophi)))).max() < 1e-3
