"""Builds libtqf.so (the sm_103a kernels and the C ABI) in-tree.

Each translation unit is compiled by nvcc in parallel for exactly one target,
``-gencode arch=compute_103a,code=sm_103a``, then linked into
``tqf/_lib/libtqf.so`` next to the Python package.  No cmake, no torch
extension machinery: the library exports a plain C ABI (include/tqf.h) that
the Python host side loads with ctypes.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)  # tf-quant-finance_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
INCLUDE = os.path.join(REPO_ROOT, "include")
OUT_DIR = os.path.join(PKG_ROOT, "tqf", "_lib")
OBJ_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libtqf.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "-Xcompiler",
    "-Wall",
    "--expt-relaxed-constexpr",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the tqf kernels need the CUDA toolkit to build")


def sources() -> list[str]:
    return sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".cu"))


def _needs_rebuild(lib: str, inputs: list[str]) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(p) > t for p in inputs)


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compiles every csrc/*.cu and links libtqf.so; returns its path."""
    srcs = sources()
    headers = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if not force and not _needs_rebuild(LIB_PATH, srcs + headers + [__file__]):
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + NVCC_FLAGS + ["-I", INCLUDE, "-I", HERE] + list(extra_flags or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr, file=sys.stderr)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as pool:
        objs = list(pool.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link of libtqf.so failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
