"""Build recipe for libtdm.so (sm_103a) and the drop-in command-line tools.

Compiles every translation unit in parallel with nvcc / g++ and links in-tree:
    lib/libtdm.so      the C ABI of include/tdm.h
    bin/demo           drop-in for core/demo.cu's `demo <cloud.ply> <out_prefix>`
    bin/fuse           drop-in for depth-fusion/demo.cu
    bin/descriptors    drop-in for evaluation/*/get3DMatchDescriptors.cu
Objects go to _build/.  Rebuilds only what changed (sources or headers).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
LIB_PATH = os.path.join(LIB, "libtdm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + INC, "-I" + CSRC] + ARCH
# Extra flags for diagnostic builds (e.g. -DTDM_WAIT_STATS); objects built
# with different flags are not mixed (the flags are part of the stamp).
EXTRA = os.environ.get("TDM_EXTRA_NVCC_FLAGS", "").split()
# Translation units whose float results are compared bit for bit with the
# CPU restatement: no multiply-add contraction on the device either.
NO_FMAD = {"ransac.cu", "tsdf.cu", "batch.cu", "overlap.cu", "icp.cu"}
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + INC, "-I" + CSRC,
             "-I/usr/local/cuda/include"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _compile(src: str, hdrs) -> str:
    name = os.path.basename(src)
    obj = os.path.join(OBJ, name + ".o")
    if not _stale(obj, [src] + hdrs):
        return obj
    tmp = obj + ".tmp%d" % os.getpid()
    if src.endswith(".cu"):
        flags = list(NVCC_FLAGS) + EXTRA
        if name in NO_FMAD:
            flags.append("-fmad=false")
        _run([_nvcc()] + flags + ["-c", src, "-o", tmp])
    else:
        _run(["g++"] + CXX_FLAGS + ["-c", src, "-o", tmp])
    os.replace(tmp, obj)
    return obj


def _arch_guard() -> None:
    """Objects built on another host architecture are discarded."""
    stamp = os.path.join(OBJ, "ARCH")
    mach = platform.machine() + " " + " ".join(EXTRA)
    old = open(stamp).read().strip() if os.path.exists(stamp) else None
    if old != mach:
        for d in (OBJ, LIB, BIN):
            shutil.rmtree(d, ignore_errors=True)
        os.makedirs(OBJ, exist_ok=True)
        with open(stamp, "w") as f:
            f.write(mach)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    _arch_guard()
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    hdrs = _headers()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdrs), srcs))
    if _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        _run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
        os.replace(tmp, LIB_PATH)
    # the command-line drop-ins; a tool that cannot be built (fuse needs zlib)
    # is reported and left out, the library stands on its own
    for tool, libs in (("demo", []), ("fuse", ["-lz"]), ("descriptors", [])):
        src = os.path.join(HOST, tool + ".cpp")
        out = os.path.join(BIN, tool)
        if os.path.exists(src) and _stale(out, [src, LIB_PATH] + hdrs):
            try:
                _run(["g++"] + CXX_FLAGS + [src, "-o", out, "-L" + LIB, "-ltdm", "-Wl,-rpath,$ORIGIN/../lib",
                                           "-L/usr/local/cuda/lib64", "-lcudart"] + libs)
            except RuntimeError as e:
                print("warning: bin/%s not built: %s" % (tool, str(e).splitlines()[-1][:300]))
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
