"""Build libnatgpu.so in-tree (nvcc, sm_103a only).

The CUDA translation units are compiled in parallel and linked with the
CUDA runtime into ``natrium_gb300/_lib/libnatgpu.so``.  Run as
``python -m natrium_gb300.build`` or through ``__graft_entry__.build()``.
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
LIB = os.path.join(OUT_DIR, "libnatgpu.so")

SOURCES = ["natgpu_api.cu", "k_d2q9.cu", "k_d3q19.cu", "k_d3q27.cu", "k_v2.cu", "k_v2_small.cu", "k_row_d2q9.cu",
           "k_row_d3q19.cu", "k_row_d3q27.cu", "serve.cu",
           "natgpu_noalloc.cu", "k_thermal.cu", "k_rowt_d3q19.cu", "k_rowt_d3q27_bgk.cu",
           "k_rowt_d3q27_kbc.cu", "k_row_ss_d3q19.cu", "k_row_ss_d3q27.cu",
           "k_rowg_d3q19.cu", "k_rowg_d3q27.cu", "k_mapped_d2q9.cu", "k_mapped_d3q19.cu",
           "k_mapped_d3q27.cu", "tracker.cu", "io.cu", "k_cell.cu", "k_cell_q27f.cu", "k_cell_q27fz.cu",
           "k_cell_q27d.cu", "k_cell_q19f.cu", "k_cell_q19d.cu", "k_thermal_p2.cu",
           "k_cell_q19feq.cu", "k_cell_wide.cu",
           "k_cell_wide128.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# the departure-path tracker runs on the host and on the device and must give
# the same rows bit for bit: no floating-point contraction on either side
FILE_FLAGS = {"tracker.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libnatgpu.so")
    return cand


def _deps_mtime() -> float:
    t = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    nv = nvcc()
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nv, *FLAGS, *FILE_FLAGS.get(src, []), *ARCH, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nv, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:  # every build recompiles all sources; the objects are not kept
        try:
            os.remove(o)
        except OSError:
            pass
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
