"""Build libtopo_gb300.so in-tree: nvcc for sm_103a, one process per source.

Usage: python -m topoptspline3d_gb300.build [--force]

Extra nvcc flags for the CUDA sources (e.g. -DTOPO_FINE32_MIN_CTAS=3) can be
given in the TOPO_NVCC_FLAGS environment variable; rebuild with --force after
changing them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libtopo_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["capi.cu", "k_fine.cu", "k_coarse.cu", "k_vec.cu", "k_design.cu", "k_noalloc.cu", "k_mma.cu", "k_unet.cu", "k_conv_tc.cu", "unet.cu", "k_multi.cu", "worst.cu", "io.cu", "voxel.cu", "support.cu"]
CPP_SOURCES = ["host_setup.cpp", "bc_regions.cpp"]
# per-file nvcc flags: the voxeliser reproduces the reference's FP32 tests
# operation for operation, so no multiply-add contraction there
FILE_FLAGS = {"voxel.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtopo_gb300")


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "topo_gb300.h"))
    cpp = os.path.join(HERE, "cpp")
    hs += [os.path.join(cpp, f) for f in os.listdir(cpp) if f.endswith((".hpp", ".cpp"))]
    return hs


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > t for p in _sources() + _headers() + [__file__])


def _compile(src: str) -> str:
    nvcc = _nvcc()
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        cmd = [nvcc, ARCH, "-lineinfo", "--expt-relaxed-constexpr", "-c", src, "-o", obj] + common
        cmd += FILE_FLAGS.get(os.path.basename(src), [])
        cmd += os.environ.get("TOPO_NVCC_FLAGS", "").split()
    else:
        cmd = [nvcc, "-x", "c++", "-c", src, "-o", obj] + common
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [_nvcc(), ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    build_driver()
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


DRIVER_PATH = os.path.join(OUT_DIR, "topopt_driver")


def build_driver() -> str:
    """C++ driver (cpp/topopt_driver.cpp) linked against the in-tree library."""
    src = os.path.join(HERE, "cpp", "topopt_driver.cpp")
    tmp = DRIVER_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include"),
           "-I" + os.path.join(HERE, "cpp"), src, "-o", tmp, "-L" + OUT_DIR, "-ltopo_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER_PATH)
    return DRIVER_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
