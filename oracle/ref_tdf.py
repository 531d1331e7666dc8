"""The reference's own ComputeTDF kernel as a GPU reference -- TEST INFRASTRUCTURE ONLY.

Only tests/ use this module: it is a checker for the ref-compat index-decode
modes of the TDF (core/demo.cu:32-34 decodes the linear voxel index through
float32), never part of the product.

core/demo.cu cannot be compiled whole here: core/utils.hpp needs OpenCV (absent)
and core/marvin.hpp needs cuDNN and does not compile under CUDA 13.  Its TDF
kernel (core/demo.cu:18-57, with the launch constants of :18-19) is
self-contained, so this recipe

  1. copies those lines out of the reference tree, where it is mounted, into
     oracle/_ref/compute_tdf_ref.cu, between a header and a launcher written
     here.  The launcher runs the kernel as core/demo.cu:151-158 does:
     <<<2880, 512>>> once per loop index until every voxel is covered;
  2. compiles that file the way core/compile.sh builds demo.cu -- nvcc -O3 with
     the default floating-point flags, so multiply-add contraction is on --
     for sm_103a, into oracle/_ref/libref_tdf.<machine>.so.

oracle/_ref/ is not committed (.gitignore).  The extracted source travels with
the working tree to a GPU machine without the reference tree, where step 2 runs
again.  The kernel's bounds test (voxel_idx > V) lets voxel_idx == V through,
so callers pass occupancy and TDF buffers of V + 1 floats.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(REF_DIR, "compute_tdf_ref.cu")
LIB_PATH = os.path.join(REF_DIR, "libref_tdf.%s.so" % platform.machine())
REFERENCE = os.environ.get("TDM_REFERENCE_ROOT", "/root/reference")

_HEADER = """// Generated by oracle/ref_tdf.py from core/demo.cu of the reference tree
// (lines of the launch constants and of ComputeTDF, unmodified).  Not
// committed; test infrastructure only.
#include <cuda_runtime.h>
#include <math.h>
"""

_LAUNCHER = """
// Launcher (oracle/ref_tdf.py): the loop of core/demo.cu:151-158.
extern "C" int ref_compute_tdf(float* occ, float* tdf, int dx, int dy, int dz, float ox, float oy, float oz,
                               float vs, float trunc) {
  const long long V = (long long)dx * dy * dz;
  const long long per = (long long)CUDA_NUM_THREADS * CUDA_MAX_NUM_BLOCKS;
  const int loops = (int)((V + per - 1) / per);
  for (int l = 0; l < loops; ++l)
    ComputeTDF<<<CUDA_MAX_NUM_BLOCKS, CUDA_NUM_THREADS>>>(l, occ, tdf, dx, dy, dz, ox, oy, oz, vs, trunc);
  if (cudaGetLastError() != cudaSuccess) return 1;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}
"""


def extract() -> bool:
    """Step 1: writes SRC from the reference tree; False when it is absent."""
    demo = os.path.join(REFERENCE, "core", "demo.cu")
    if not os.path.exists(demo):
        return False
    lines = open(demo).read().split("\n")
    consts = [l for l in lines if l.startswith("#define CUDA_NUM_THREADS") or
              l.startswith("#define CUDA_MAX_NUM_BLOCKS")]
    start = next(i for i, l in enumerate(lines) if l.startswith("void ComputeTDF("))
    if lines[start - 1].strip() == "__global__":
        start -= 1
    end = next(i for i in range(start, len(lines)) if lines[i] == "}")
    body = "\n".join(consts + [""] + lines[start:end + 1])
    os.makedirs(REF_DIR, exist_ok=True)
    text = _HEADER + body + "\n" + _LAUNCHER
    if not os.path.exists(SRC) or open(SRC).read() != text:
        with open(SRC, "w") as f:
            f.write(text)
    return True


def build() -> str | None:
    """Steps 1 and 2; returns the library path, or None when neither the
    reference tree nor a previously extracted source is present."""
    extract()
    if not os.path.exists(SRC):
        return None
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc, "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
                               "-shared", SRC, "-o", tmp])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        f32, i32, P = ctypes.c_float, ctypes.c_int, ctypes.c_void_p
        L.ref_compute_tdf.restype = i32
        L.ref_compute_tdf.argtypes = [P, P, i32, i32, i32, f32, f32, f32, f32, f32]
        _lib = L
    return _lib
