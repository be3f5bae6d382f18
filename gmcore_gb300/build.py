"""In-tree build of the GB300 library (nvcc, sm_103a only).

    python -m gmcore_gb300.build        # builds gmcore_gb300/lib/libgmcore_gpu.so

Translation units are compiled in parallel and linked into one shared
library with a plain C ABI (include/gmcore_gpu.h).
"""
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libgmcore_gpu.so")

CUDA_SOURCES = ["dyn.cu", "adv.cu", "tlad.cu", "gmcore_gpu.cu", "peak.cu", "out.cu"]
CXX_SOURCES = ["grid.cpp", "ncfile.cpp", "output.cpp"]
HEADERS = ["common.cuh", "stencil.cuh", "kernels.hpp", "grid.hpp", "ncfile.hpp", "output.hpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


# FP32 arithmetic of the mixed form: subnormals flushed, division and square
# root to the hardware approximations (within 2 ulp).  FP64 arithmetic, and so
# the FP64 form, is unaffected by these flags.
FP32_FLAGS = ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]


def build(verbose=False, force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "gmcore_gpu.h"),
                                                           os.path.abspath(__file__)]
    cmds, objs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmds.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", *FP32_FLAGS,
                         "-Xcompiler", "-fPIC", *inc, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-fno-fast-math", *inc, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(cmds), os.cpu_count() or 1))) as ex:
        list(ex.map(run, cmds))
    if force or cmds or _stale(LIB, objs):
        libs = (["-lquadmath"] if platform.machine() in ("x86_64", "AMD64") else []) + ["-lpthread"]
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, *libs])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
