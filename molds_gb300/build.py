"""Builds the CUDA library molds_gb300/_build/libnddo_gb300.so for sm_103a.

Every translation unit is compiled by nvcc in parallel and linked with the
static CUDA runtime, so the library has no dependency besides the driver.
Run as ``python -m molds_gb300.build`` or through ``__graft_entry__.build()``.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnddo_gb300.so")
# host-only helper library: the alkane geometry generator of the workloads
HOST_LIB = os.path.join(BUILD, "libworkloads.so")
HOST_SOURCES = ["alkane_gen.c"]
SOURCES = ["nddo_tables.cpp", "pair_fock.cu", "jacobi.cu", "tridiag.cu", "tridiag_grid.cu", "scf_kernels.cu", "engine.cu", "capi.cu", "noalloc.cu", "server.cu", "block_jacobi.cu", "tc_gemm.cu", "grouped.cu", "tuning.cpp", "scf_text.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "nddo_gpu.h"))
    return files


def needs_build() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(HOST_LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps() + [os.path.abspath(__file__)])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + ARCH + COMMON + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    def compile_host():
        cc_host = shutil.which("gcc") or "cc"
        tmp = HOST_LIB + f".tmp{os.getpid()}"
        cmd = [cc_host, "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-shared", "-fPIC", "-o", tmp] + \
              [os.path.join(CSRC, f) for f in HOST_SOURCES] + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gcc failed for {HOST_SOURCES}:\n{r.stderr}")
        os.replace(tmp, HOST_LIB)

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        host = ex.submit(compile_host)
        objs = list(ex.map(compile_one, SOURCES))
        host.result()
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
