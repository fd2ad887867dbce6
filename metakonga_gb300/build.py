"""In-tree build of libxdem (sm_103a) and the reference-API shim libraries.

    python -m metakonga_gb300.build          # or __graft_entry__.build()

Outputs (git-ignored, rebuilt on every machine):
    metakonga_gb300/libxdem.so            the CUDA library + C ABI (include/xdem.h)
    metakonga_gb300/libxdem_mphysics.so   C++ shim with the exact functions of the
                                          reference's include/mphysics_cuda_dec.cuh
Objects go to metakonga_gb300/_build/.  Translation units are compiled in
parallel with one -gencode (compute_103a/sm_103a).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIBXDEM = os.path.join(PKG, "libxdem.so")
LIBSHIM = os.path.join(PKG, "libxdem_mphysics.so")
LIBLEGACY = os.path.join(PKG, "libxdem_legacy.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]

# FP64 translation units whose results must match the reference's arithmetic
# are compiled without multiply-add contraction.
NO_FMAD = {"xd_grid.cu", "xd_integrate.cu", "xd_contact64.cu", "xd_twin32.cu", "xd_legacy.cu"}
# The mixed form's FP32 contact arithmetic carries its own error bounds and
# corrects its pair-arithmetic quotients and roots: approximate FP32 division
# and square root there (about 2 ulp, a few instructions instead of an IEEE
# sequence with a slow path).
FAST_DIV = {"xd_mixed.cu"}

CUDA_SOURCES = ["xd_capi.cu", "xd_sort.cu", "xd_grid.cu", "xd_integrate.cu", "xd_contact64.cu",
                "xd_scene.cu", "xd_noalloc.cu", "xd_mixed.cu", "xd_twin32.cu", "xd_legacy.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libxdem")


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(INCLUDE, "xdem.h"))
    deps.append(os.path.abspath(__file__))   # the flags
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    flags = list(NVCC_COMMON)
    if src in NO_FMAD:
        flags.append("--fmad=false")
    if src in FAST_DIV:
        flags += ["-prec-div=false", "-prec-sqrt=false"]
    cmd = [nvcc(), "-c", srcp, "-o", obj] + flags
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _newer(out: str, inputs) -> bool:
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(i) for i in inputs)


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, CUDA_SOURCES))
    if not _newer(LIBXDEM, objs):
        cmd = [nvcc(), "-shared", "-o", LIBXDEM] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libxdem.so failed:\n{r.stdout}\n{r.stderr}")
    for out, src, heads in ((LIBSHIM, "shim_mphysics.cpp", ("mphysics_cuda_dec.cuh", "xdem_host.h", "xdem.h")),
                            (LIBLEGACY, "shim_legacy.cpp", ("cu_dem_dec.cuh", "xdem_legacy.h", "xdem.h"))):
        shim_src = os.path.join(CSRC, src)
        shim_deps = [shim_src, LIBXDEM] + [os.path.join(INCLUDE, h) for h in heads]
        if os.path.exists(shim_src) and not _newer(out, shim_deps):
            cuda_root = os.path.dirname(os.path.dirname(nvcc()))
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", out, shim_src,
                   "-I", INCLUDE, "-I", os.path.join(cuda_root, "include"), "-L", PKG, "-lxdem",
                   "-L", os.path.join(cuda_root, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
                   "-Wl,-rpath," + os.path.join(cuda_root, "lib64")]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"build of {os.path.basename(out)} failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIBXDEM, file=sys.stderr)
    return LIBXDEM


if __name__ == "__main__":
    build(verbose=True)
