"""Build libpsdgb.so in-tree with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel into _build/, then
linked into psd_projection_gb300/libpsdgb.so (CUDA runtime linked statically,
cuBLAS / cuSOLVER dynamically for the EVD entry points and the cuBLAS-handle
stream lookup of the C++ shim).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libpsdgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    f"-I{ROOT / 'include'}", f"-I{CSRC}",
]
SOURCES = ["capi.cu", "composite.cu", "elem.cu", "lanczos.cu", "gemm_simt.cu", "gemm_tc.cu", "gemm_tc2.cu", "gemm_wide.cu", "gemm_pairwide.cu", "eigenpairs.cu", "lobpcg.cu", "refapi.cu",
           "static_scratch.cu", "serve.cu", "batch.cu", "batch_chain.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def cuda_lib_dir() -> str:
    base = Path(nvcc()).resolve().parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (base / sub / "libcublas.so").exists():
            return str(base / sub)
    return str(base / "lib64")


def _headers() -> list[Path]:
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").rglob("*.h"))


def _compile(src: str, force: bool) -> Path:
    s = CSRC / src
    o = BUILD / (s.stem + ".o")
    newest_dep = max([s.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if not force and o.exists() and o.stat().st_mtime >= newest_dep:
        return o
    cmd = [nvcc(), *ARCH, *CFLAGS, "-c", str(s), "-o", str(o)]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *CFLAGS, "-x", "c++", "-c", str(s), "-o", str(o)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return o


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), SOURCES))
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    libdir = cuda_lib_dir()
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), f"-L{libdir}", "-lcublas", "-lcusolver",
           "-Xlinker", f"-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
