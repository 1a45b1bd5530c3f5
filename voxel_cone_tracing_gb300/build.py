"""Build recipe of libvct.so (the CUDA kernels + the C ABI of include/vct.h).

nvcc compiles every translation unit of csrc/ for sm_103a in parallel, then
links one shared library next to this file.  Host code is built without
floating-point contraction so that its FP32 matrix products equal the
oracle's bit for bit on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvct.so")
DEMO_SRC = os.path.join(HERE, "demo", "vct_demo.cpp")
DEMO = os.path.join(HERE, "vct_demo")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC]
# Per-file flags: the cone tracer fuses products and sums only where its
# code says so, so that its frames do not change with the code's arrangement.
FILE_FLAGS = {"k_trace.cu": ["-fmad=false"]}
# Extra nvcc flags (e.g. -DVCT_TRACE_MIN_BLOCKS=3 for tuning sweeps); the
# library is rebuilt when they differ from the ones it was built with.
EXTRA = os.environ.get("VCT_NVCC_FLAGS", "").split()
STAMP = LIB + ".flags"


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libvct.so")
    return p


def sources() -> list:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps() -> list:
    return sources() + [os.path.abspath(__file__)] + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    try:
        with open(STAMP) as f:
            if f.read() != " ".join(EXTRA):
                return False
    except OSError:
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build_demo(force: bool = False) -> str:
    """The headless demo executable (C++ host over include/vct_renderer.hpp),
    linked against libvct.so next to it."""
    deps = [DEMO_SRC, LIB] + glob.glob(os.path.join(HERE, "..", "include", "*"))
    if not force and os.path.exists(DEMO) and os.path.getmtime(DEMO) >= max(map(os.path.getmtime, deps)):
        return DEMO
    tmp = DEMO + f".tmp{os.getpid()}"
    cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"), DEMO_SRC,
           "-L", HERE, "-lvct", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"demo build failed:\n{r.stderr}")
    os.replace(tmp, DEMO)
    return DEMO


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        build_demo()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *FLAGS, *FILE_FLAGS.get(os.path.basename(src), []), *EXTRA, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, sources()))
    if verbose:
        for _, err in results:
            print(err)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(" ".join(EXTRA))
    build_demo(force=True)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
