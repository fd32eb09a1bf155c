"""In-tree build of libgbdx.so for sm_103a.

Each CUDA translation unit under ``csrc/`` is compiled by its own ``nvcc``
process (in parallel) and linked into ``diffrax_gb300/_lib/libgbdx.so``.  The
library is rebuilt whenever a source or header is newer than it.

``build(bounds=True)`` makes the bounds-checked variant
``libgbdx_bounds.so`` from the same sources with ``-DGBDX_BOUNDS`` (every
kernel index into a caller buffer checked; include/gbdx.h, GBDX_ERR_BOUNDS);
``GBDX_BOUNDS=1`` in the environment makes the package load it.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_lib", "obj")
LIB_PATH = os.path.join(OUT_DIR, "libgbdx.so")
BOUNDS_LIB_PATH = os.path.join(OUT_DIR, "libgbdx_bounds.so")
BOUNDS_OBJ_DIR = os.path.join(PKG, "_lib", "obj_bounds")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr"] + ARCH
# The FP64-state kernels are the parity mode: no FMA contraction, so their
# arithmetic rounds like the oracle's (built with -ffp-contract=off).
PER_FILE_FLAGS = {"gbdx_ode_f64.cu": ["-fmad=false"], "gbdx_ode_f64_xo.cu": ["-fmad=false"],
                  "gbdx_dense.cu": ["-fmad=false"], "gbdx_ode_adj_f64.cu": ["-fmad=false"]}


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgbdx.so")
    return cand


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps() -> list[str]:
    return (sources() + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)])


def is_stale(bounds: bool = False) -> bool:
    lib = BOUNDS_LIB_PATH if bounds else LIB_PATH
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False, bounds: bool = False) -> str:
    """Compile every translation unit and link libgbdx.so (libgbdx_bounds.so
    with bounds=True).  Returns its path."""
    lib_path = BOUNDS_LIB_PATH if bounds else LIB_PATH
    obj_dir = BOUNDS_OBJ_DIR if bounds else OBJ_DIR
    if not force and not is_stale(bounds):
        return lib_path
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()
    srcs = sources()
    extra = ["-DGBDX_BOUNDS"] if bounds else []

    def compile_one(src: str) -> str:
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [cc] + NVCC_FLAGS + extra + PER_FILE_FLAGS.get(os.path.basename(src), []) + [
            "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib_path + f".tmp{os.getpid()}"
    cmd = [cc, "-shared", "-cudart", "shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {os.path.basename(lib_path)} failed:\n{r.stdout}\n"
                           f"{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force=True, verbose=True))
