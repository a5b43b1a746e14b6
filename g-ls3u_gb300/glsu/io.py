"""File formats of the reference's frame and phase data.

- ``read_matrix_bin`` / ``write_matrix_bin``: the ``matrixIO`` binary format
  (``Utils/matrixIO.h:17-55``, ``Utils/matrixIO.inl``): int32 rows, int32
  cols, then rows*cols row-major elements (float32 phase maps in
  ``Experiments/imgs/*/*_phi.bin``; ``MatLab/Load2DMatrix.m``).
- ``read_complex_text`` / ``write_complex_text``: the ``.fp`` text format of
  ``fftwComplexMatRead2D`` / ``Write2D`` (``Utils/Utils.cpp:80-123``): a first
  line ``rows,cols`` then one ``re,im`` line per element, row-major.
- ``read_bmp``: 8-bit grey-palette or 24-bit BMP frames as uint8, top-down,
  grey as OpenCV's ``imread`` + ``BGR2GRAY``.
"""
from __future__ import annotations

import struct

import numpy as np


def read_matrix_bin(path: str, dtype=np.float32) -> np.ndarray:
    with open(path, "rb") as fh:
        hdr = fh.read(8)
        if len(hdr) < 8:
            raise ValueError("matrix header truncated: " + path)
        rows, cols = struct.unpack("<ii", hdr)
        if rows < 0 or cols < 0:
            raise ValueError("bad matrix size %d x %d" % (rows, cols))
        n = rows * cols
        data = np.fromfile(fh, dtype=dtype, count=n)
    if data.size < n:
        raise ValueError("matrix data truncated: read %d of %d elements" % (data.size, n))
    return data.reshape(rows, cols)


def write_matrix_bin(path: str, a: np.ndarray) -> None:
    a = np.ascontiguousarray(a)
    if a.ndim != 2:
        raise ValueError("a 2-D matrix is required")
    with open(path, "wb") as fh:
        fh.write(struct.pack("<ii", a.shape[0], a.shape[1]))
        a.tofile(fh)


def read_complex_text(path: str, dtype=np.complex64) -> np.ndarray:
    with open(path) as fh:
        first = fh.readline().strip().split(",")
        if len(first) != 2:
            raise ValueError("first line must be 'rows,cols'")
        rows, cols = int(first[0]), int(first[1])
        vals = []
        for line in fh:
            line = line.strip()
            if not line:
                continue
            re_, im_ = line.split(",")
            vals.append(complex(float(re_), float(im_)))
    if len(vals) != rows * cols:
        raise ValueError("expected %d elements, read %d" % (rows * cols, len(vals)))
    return np.array(vals, dtype=dtype).reshape(rows, cols)


def write_complex_text(path: str, a: np.ndarray) -> None:
    a = np.asarray(a)
    with open(path, "w") as fh:
        fh.write("%d,%d\n" % a.shape)
        for v in a.ravel():
            fh.write("%.9g,%.9g\n" % (v.real, v.imag))


def read_bmp(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    if data[:2] != b"BM":
        raise ValueError("not a BMP file: " + path)
    off, hdr = struct.unpack_from("<I", data, 10)[0], struct.unpack_from("<I", data, 14)[0]
    w, h = struct.unpack_from("<ii", data, 18)
    bpp, comp = struct.unpack_from("<H", data, 28)[0], struct.unpack_from("<I", data, 30)[0]
    if comp != 0:
        raise ValueError("compressed BMP files are not supported")
    top_down, h = h < 0, abs(h)
    if bpp == 8:
        ncol = struct.unpack_from("<I", data, 46)[0] or 256
        pal = np.frombuffer(data, np.uint8, ncol * 4, 14 + hdr).reshape(ncol, 4).astype(np.int64)
        grey = ((pal[:, 2] * 4899 + pal[:, 1] * 9617 + pal[:, 0] * 1868 + (1 << 13)) >> 14).astype(np.uint8)
        stride = (w + 3) & ~3
        img = grey[np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)[:, :w]]
    elif bpp == 24:
        stride = (3 * w + 3) & ~3
        px = np.frombuffer(data, np.uint8, stride * h, off).reshape(h, stride)[:, :3 * w].reshape(h, w, 3)
        px = px.astype(np.int64)
        img = ((px[..., 2] * 4899 + px[..., 1] * 9617 + px[..., 0] * 1868 + (1 << 13)) >> 14).astype(np.uint8)
    else:
        raise ValueError("unsupported BMP bit depth %d" % bpp)
    return np.ascontiguousarray(img if top_down else img[::-1])
