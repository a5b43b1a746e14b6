"""Build the G-LS3U CUDA library for sm_103a (in-tree, no cmake).

    python g-ls3u_gb300/build.py [--force]

Compiles every ``csrc/*.cu`` / ``csrc/*.cpp`` translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and links
``lib/libglsu.so`` (CUDA runtime linked statically), plus the C++ class test
driver ``lib/glsu_cpp_test`` used by the GPU tests.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libglsu.so")
CPP_TEST_SRC = os.path.join(ROOT, "tests", "cpp", "test_classes.cpp")
CPP_TEST_BIN = os.path.join(LIB_DIR, "glsu_cpp_test")
NVCC = os.environ.get("NVCC", "nvcc")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _compile(src: str, force: bool, hdr_time: float) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= hdr_time):
        return obj
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", obj + ".tmp"]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = _sources()
    hdr_time = _newest(_headers())
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, hdr_time), srcs))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if os.path.exists(CPP_TEST_SRC):
        if force or not os.path.exists(CPP_TEST_BIN) or os.path.getmtime(CPP_TEST_BIN) < max(
                os.path.getmtime(LIB), os.path.getmtime(CPP_TEST_SRC), hdr_time):
            tmp = CPP_TEST_BIN + ".tmp"
            cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                   "-I", os.path.join(CUDA_HOME, "include"), CPP_TEST_SRC, "-o", tmp,
                   "-L", LIB_DIR, "-lglsu", "-Wl,-rpath,$ORIGIN",
                   "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart",
                   "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("C++ test driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
            os.replace(tmp, CPP_TEST_BIN)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
