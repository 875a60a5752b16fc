"""Build recipe for libmddem_gb300.so (sm_103a only).

Compiles each CUDA translation unit with nvcc in parallel and links the
shared library in-tree at ``mddem_gb300/_lib/libmddem_gb300.so``.  The FP64
kernels are compiled with ``-fmad=false`` so that multiply-adds fuse only
where the source calls ``fma()`` (the reference's ``mul_add`` sites); the
mixed-precision kernels keep nvcc's default contraction.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB = os.path.join(OUT_DIR, "libmddem_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
          "-I", os.path.join(ROOT, "include")]

UNITS = [
    ("mdg_kernels_fp64.cu", ["-fmad=false"]),
    ("mdg_kernels_mixed.cu", []),
    ("mdg_api.cu", ["-fmad=false"]),
    ("mdg_noalloc.cu", ["-fmad=false"]),
    ("mdg_measure.cu", ["-fmad=false"]),
    ("mdg_serve.cpp", []),
    ("mdg_insert.cpp", []),
    ("mdg_tune.cpp", []),
]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmddem_gb300.so")


def _compile(src: str, extra: list[str], verbose: bool, ptxas_v: bool) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if ptxas_v:
        cmd.insert(1, "-Xptxas=-v")
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if ptxas_v:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "mdg.h"),
                                                                 os.path.abspath(__file__)]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> str:
    """Compile (if stale) and return the path of libmddem_gb300.so."""
    if not force and not ptxas_v and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose, ptxas_v), UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="-v" in sys.argv))
