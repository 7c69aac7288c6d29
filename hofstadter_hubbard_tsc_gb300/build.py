"""Builds ``libhh_dmrg.so`` in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into one shared
library exporting the C ABI of ``include/hh_dmrg.h``.  No CMake and no torch
extension machinery: the library has no Python or torch dependency.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhh_dmrg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
          "--expt-relaxed-constexpr"]
SOURCES = ["su2.cpp", "plan.cpp", "gemm_fp64.cu", "hh_api.cu", "noalloc.cu", "tc_gemm.cu", "tc_plan.cpp", "step.cu", "eig.cu", "eig_tri.cu", "mlp.cu", "enlarge.cu"]
LIBS = ["-lcudart", "-lcusolver"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and all(os.path.getmtime(obj) >= os.path.getmtime(os.path.join(CSRC, h))
                    for h in os.listdir(CSRC) if h.endswith((".h", ".cuh")))
            and os.path.getmtime(obj) >= os.path.getmtime(os.path.join(HERE, "..", "include", "hh_dmrg.h"))):
        return obj, ""
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + ARCH + COMMON + extra + lang + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=None):
    """Compile every CUDA/C++ source and link libhh_dmrg.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = list(extra or [])
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log:
                print(log, file=sys.stderr)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + LIBS
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
