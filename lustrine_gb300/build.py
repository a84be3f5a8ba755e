"""Build the CUDA library liblustrine_gb300.so in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into
lustrine_gb300/_build/liblustrine_gb300.so.  pbf_compat.cu and sand.cu are
compiled with --fmad=false: the reference-semantics steps must not contract
a * b + c into fused multiply-adds (the reference's arithmetic has none).
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
LIB = os.path.join(BUILD, "liblustrine_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
# translation unit -> extra flags
UNITS = {
    "pbf_sort.cu": [],
    "pbf_compat.cu": ["--fmad=false"],
    "sand.cu": ["--fmad=false"],
    "pbf_solver.cu": [],
    "pbf_compact.cu": [],
    "pbf_scene_solve.cu": [],
    "pbf_context.cu": [],
    "pbf_dynamic.cu": [],
    "pbf_sort_api.cu": [],
    "pbf_sort_noalloc.cu": [],
    # host float math of scene construction and sources as the reference's
    # (no FMA contraction, which GCC applies by default on aarch64)
    "lustrine_wrapper.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "vox.cpp": [],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build lustrine_gb300")
    return p


def _sources_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "lustrine_gb300.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def up_to_date() -> bool:
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime()


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(unit: str) -> str:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.rsplit(".", 1)[0] + ".o")
        cmd = [cc, *ARCH, *COMMON, *UNITS[unit], "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
