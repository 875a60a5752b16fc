"""Build recipe for libmddem_gb300.so (sm_103a only) and the mdg_run host.

Compiles each CUDA translation unit with nvcc in parallel and links the
shared library in-tree at ``mddem_gb300/_lib/libmddem_gb300.so``; the C++
host above the ABI (``csrc/host``) is compiled with g++ into
``mddem_gb300/_lib/mdg_run``, linked against the library.  The FP64
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
HOST_DIR = os.path.join(CSRC, "host")
RUNNER = os.path.join(OUT_DIR, "mdg_run")
# the C++ host above the ABI (App, plugins, TOML reader) and its CLI
HOST_SOURCES = ["toml.cpp", "app.cpp", "plugins.cpp", "restart.cpp", "mdg_run.cpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
          "-I", os.path.join(ROOT, "include")]

UNITS = [
    ("mdg_kernels_fp64.cu", ["-fmad=false"]),
    ("mdg_kernels_mixed.cu", []),
    ("mdg_api.cu", ["-fmad=false"]),
    ("mdg_noalloc.cu", ["-fmad=false"]),
    ("mdg_measure.cu", ["-fmad=false"]),
    ("mdg_generate.cu", ["-fmad=false"]),
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
    if not os.path.exists(LIB) or not os.path.exists(RUNNER):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(RUNNER))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HOST_DIR, f) for f in os.listdir(HOST_DIR)]
    deps += [os.path.join(ROOT, "include", "mdg.h"), os.path.abspath(__file__)]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def _host_compile(src: str, verbose: bool) -> str:
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("g++ not found: needed for the mdg_run host")
    obj = os.path.join(OBJ_DIR, "host_" + os.path.splitext(src)[0] + ".o")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include"), "-c",
           os.path.join(HOST_DIR, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _link_runner(objs: list[str], verbose: bool) -> None:
    cxx = shutil.which("g++") or shutil.which("c++")
    tmp = RUNNER + ".tmp"
    cmd = [cxx, "-o", tmp, *objs, "-L", OUT_DIR, "-lmddem_gb300", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of mdg_run failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, RUNNER)


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> str:
    """Compile (if stale) and return the path of libmddem_gb300.so."""
    if not force and not ptxas_v and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS) + len(HOST_SOURCES)) as ex:
        futs = [ex.submit(_compile, u[0], u[1], verbose, ptxas_v) for u in UNITS]
        hfuts = [ex.submit(_host_compile, h, verbose) for h in HOST_SOURCES]
        objs = [f.result() for f in futs]
        hobjs = [f.result() for f in hfuts]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    _link_runner(hobjs, verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="-v" in sys.argv))
