"""Build the reference's own CPU DPRA / WFF2 classes into oracle/_ref.

TEST INFRASTRUCTURE ONLY.  Compiles, unchanged and where they lie in the
reference checkout, DPRA/dpra_cpu.cpp (DPRA_CPU), WFT/WFT2_CPU.cpp
(WFT2_cpu), WFT/WFT.cpp and Utils/Utils.cpp, against stand-ins for the
libraries the reference links that are absent here (oracle/ref_shims/:
the FFTW3 API on the oracle's own FFT, LAPACKE_dsysv restated from LAPACK,
and an 8-bit cv::Mat), plus the C entry points of ref_shims/ref_driver.cpp,
into oracle/_ref/libglsu_ref.so.  The library generates the golden vectors
under tests/golden/ (tests/golden/make_ref_golden.py); no test, bench or
product code loads it.

    python oracle/ref_build.py --reference <path to the reference checkout>

The reference is Windows/MSVC code: its headers include
"opencv2\\opencv.hpp" with a backslash, which the stand-in satisfies with a
file of that literal name in the generated include folder.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIMS = os.path.join(HERE, "ref_shims")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
REF_SOURCES = ["DPRA/dpra_cpu.cpp", "WFT/WFT2_CPU.cpp", "WFT/WFT.cpp", "Utils/Utils.cpp"]
LIB = os.path.join(OUT, "libglsu_ref.so")


def build(reference: str, force: bool = False) -> str:
    for s in REF_SOURCES:
        if not os.path.exists(os.path.join(reference, s)):
            raise FileNotFoundError("reference source missing: %s" % os.path.join(reference, s))
    inc = os.path.join(OUT, "include")
    os.makedirs(os.path.join(inc, "opencv2"), exist_ok=True)
    shutil.copyfile(os.path.join(SHIMS, "opencv_shim.hpp"), os.path.join(inc, "opencv2", "opencv.hpp"))
    shutil.copyfile(os.path.join(SHIMS, "opencv_shim.hpp"), os.path.join(inc, "opencv2\\opencv.hpp"))
    if os.path.exists(LIB) and not force:
        return LIB
    objs = []
    common = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w"]
    incs = ["-I", inc, "-I", SHIMS, "-I", os.path.join(reference, "Utils"), "-I", os.path.join(reference, "WFT"),
            "-I", os.path.join(reference, "DPRA"), "-I", os.path.join(CUDA_HOME, "include")]
    units = [(os.path.join(reference, s), "g++") for s in REF_SOURCES]
    units += [(os.path.join(SHIMS, "ref_driver.cpp"), "g++"), (os.path.join(SHIMS, "fftw_shim.c"), "gcc"),
              (os.path.join(SHIMS, "lapacke_shim.c"), "gcc")]
    for src, cc in units:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        # the MSVC build reached <iostream> and the CUDA samples' helper
        # header transitively; here the first is included up front and the
        # second replaced by its one macro the CPU path uses
        std = (["-std=c++17", "-include", "iostream", "-DHELPER_CUDA_H", "-include",
                os.path.join(SHIMS, "helper_cuda_shim.h")] if cc == "g++" else ["-std=gnu11"])
        cmd = [cc] + common + std + incs + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        objs.append(obj)
    cmd = ["g++", "-shared", "-fopenmp", "-o", LIB] + objs + ["-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart",
                                                                "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="path of the reference checkout (read only)")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.reference, a.force))
    sys.exit(0)
