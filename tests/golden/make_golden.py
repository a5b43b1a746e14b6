"""Regenerate the golden fixtures in this folder from the reference project.

Run with the path of a reference checkout (read only):

    python tests/golden/make_golden.py REF

Nothing at test time reads the reference; the tests read only the files this
script writes:

- ``fft_lut.json``: the FFT size table of ``WFT/WFT.h:18-32``.
- ``xfyf.npz``: the ifftshift-ed integer frequency grid printed by the
  reference's GPU test into ``Test/xfyf.csv`` (64 x 50 plane).
- ``phi_1.bin``: the reference's phase map ``Experiments/imgs/1/1_phi.bin``,
  byte for byte: the ``matrixIO`` binary format (int32 rows, int32 cols,
  row-major float32), which pins the readers in ``glsu/io.py`` and
  ``include/glsu_io.hpp``.
- ``aia_bmp.npz``: the three 256x256 fringe frames ``Test/{1,2,3}.bmp``
  (decoded top-down, as OpenCV's imread + BGR2GRAY does for these 8-bit
  grey-palette files), the initial deltas used by the reference's AIA tests
  (``Test/AIA_CUDA_YC_Test.cpp:33-36``), and a seeded sample of 4096 pixels of
  ``Test/Phi_CPU.csv``: the per-pixel 3-vector solutions of the first AIA
  pixel solve (written by ``AIA/aia_cpuf.cpp:157-166``).
"""
from __future__ import annotations

import json
import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_bmp_gray(path: str) -> np.ndarray:
    """Decode an uncompressed 8-bit paletted or 24-bit BMP to grey uint8 (top-down)."""
    data = open(path, "rb").read()
    if data[:2] != b"BM":
        raise ValueError("not a BMP: " + path)
    off = struct.unpack_from("<I", data, 10)[0]
    hdr = struct.unpack_from("<I", data, 14)[0]
    w, h = struct.unpack_from("<ii", data, 18)
    bpp = struct.unpack_from("<H", data, 28)[0]
    comp = struct.unpack_from("<I", data, 30)[0]
    if comp != 0:
        raise ValueError("compressed BMP not supported")
    top_down = h < 0
    h = abs(h)
    if bpp == 8:
        ncol = struct.unpack_from("<I", data, 46)[0] or 256
        pal = np.frombuffer(data, np.uint8, ncol * 4, 14 + hdr).reshape(ncol, 4)
        # OpenCV BGR2GRAY: 0.299 R + 0.587 G + 0.114 B in 14-bit fixed point
        b, g, r = (pal[:, 0].astype(np.int64), pal[:, 1].astype(np.int64), pal[:, 2].astype(np.int64))
        grey = ((r * 4899 + g * 9617 + b * 1868 + (1 << 13)) >> 14).astype(np.uint8)
        stride = (w + 3) & ~3
        idx = np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)[:, :w]
        img = grey[idx]
    elif bpp == 24:
        stride = (3 * w + 3) & ~3
        px = np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)[:, :3 * w]
        px = px.reshape(h, w, 3).astype(np.int64)
        img = ((px[..., 2] * 4899 + px[..., 1] * 9617 + px[..., 0] * 1868 + (1 << 13)) >> 14)
        img = img.astype(np.uint8)
    else:
        raise ValueError("unsupported bit depth %d" % bpp)
    return np.ascontiguousarray(img if top_down else img[::-1])


def main(ref: str) -> None:
    # 1. FFT size LUT
    src = open(os.path.join(ref, "WFT", "WFT.h"), encoding="latin-1").read()
    body = src[src.index("OPT_FFT_SIZE"):]
    body = body[body.index("{") + 1: body.index("}")]
    lut = [int(t) for t in re.findall(r"\d+", body)]
    with open(os.path.join(HERE, "fft_lut.json"), "w") as fh:
        json.dump({"source": "WFT/WFT.h:18-32", "sizes": lut}, fh)

    # 2. frequency grid
    rows = open(os.path.join(ref, "Test", "xfyf.csv")).read().strip().splitlines()
    xf, yf = [], []
    for line in rows:
        cells = [c for c in line.strip().split(",") if c]
        xr, yr = [], []
        for c in cells:
            m = re.fullmatch(r"\[(-?\d+)-(-?\d+)\]", c)
            xr.append(int(m.group(1))); yr.append(int(m.group(2)))
        xf.append(xr); yf.append(yr)
    np.savez_compressed(os.path.join(HERE, "xfyf.npz"), xf=np.array(xf, np.int16),
                        yf=np.array(yf, np.int16))

    # 3. AIA frames + Phi_CPU sample
    frames = np.stack([read_bmp_gray(os.path.join(ref, "Test", "%d.bmp" % k)) for k in (1, 2, 3)])
    vals = np.loadtxt(os.path.join(ref, "Test", "Phi_CPU.csv"), dtype=np.float64)
    x = vals.reshape(-1, 3)
    rng = np.random.default_rng(20240601)
    idx = np.sort(rng.choice(x.shape[0], 4096, replace=False))
    np.savez_compressed(os.path.join(HERE, "aia_bmp.npz"), frames=frames,
                        deltas0=np.array([0.8622, 0.3188, -1.3077], np.float32),
                        pix=idx.astype(np.int32), x=x[idx])
    # 4. matrixIO phase map, copied as is
    raw = open(os.path.join(ref, "Experiments", "imgs", "1", "1_phi.bin"), "rb").read()
    open(os.path.join(HERE, "phi_1.bin"), "wb").write(raw)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
