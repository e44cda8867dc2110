"""Builds the in-tree CUDA library libscirs_sparse_gpu.so for sm_103a.

Each translation unit is compiled by nvcc in parallel into _build/, then
linked into scirs_gb300/libscirs_sparse_gpu.so (CUDA runtime linked
statically).  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libscirs_sparse_gpu.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

SOURCES = [
    "sx_core.cu",
    "sx_precond.cu",
    "sx_krylov.cu",
    "sx_ic0.cu",
    "sx_mixed.cu",
    "sx_batched.cu",
    "sx_noalloc.cu",
    "sx_gnn.cu",
    "sx_sym.cu",
    "sx_krylov2.cu",
    "sx_ilu.cu",
    "sx_io.cu",
    "sx_eigen.cu",
    "sx_probe.cu",
    "sx_gen.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build scirs_gb300")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj: str, src: str, headers: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def build(verbose: bool = False, jobs: int | None = None, extra: list[str] | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    extra = list(extra or [])

    def compile_one(src: str) -> str:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if not _stale(obj, path, headers) and not extra:
            return obj
        cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", path, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, *COMMON, "-x", "c++", *extra, "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if not os.path.exists(LIB_PATH) or any(os.path.getmtime(o) > os.path.getmtime(LIB_PATH) for o in objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
