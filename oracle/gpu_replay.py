"""The reference's GPU methods, replayed on cuBLAS / cuSOLVER (oracle/ref_replay.cu).

TEST / BENCHMARK INFRASTRUCTURE ONLY (bench.py --impl reference).  The
reference library's own build cannot travel to the GPU host, so
oracle/ref_replay.cu restates its call sequence — the same cuBLAS and
cuSOLVER calls with the same operand and compute types, per-call allocation
and blocking synchronisations — for approximate_two_norm and the three
composite methods with their auto-scaling (src/lanczos.cu:41-293,
src/composite_FP32.cu:15-191, src/composite_FP16.cu:16-274,
src/composite_FP32_emulated.cu:20-262).  build() compiles it into
oracle/_build/libref_replay.so; auto_scale() runs one projection.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from pathlib import Path

from oracle.reference_port import schedule_coefficients

HERE = Path(__file__).resolve().parent
SRC = HERE / "ref_replay.cu"
OUT = HERE / "_build" / "libref_replay.so"

METHODS = {"composite_FP32": 0, "composite_FP16": 1, "composite_FP32_emulated": 2}

_lib = None


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def build() -> Path:
    """Compile ref_replay.cu for sm_103a (skipped when the library is newer than the source)."""
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", str(SRC), "-o", str(OUT), "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_replay build failed: {r.stderr[-2000:]}")
    return OUT


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.ref_replay_auto_scale.restype = ctypes.c_int
        _lib.ref_replay_auto_scale.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_double)]
        _lib.ref_replay_ws_bytes.restype = ctypes.c_size_t
        _lib.ref_replay_ws_bytes.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int]
    return _lib


class Workspaces:
    """Caller workspaces of the documented sizes for one method and n (torch device buffers)."""

    def __init__(self, method: str, n: int):
        import torch

        m = METHODS[method]
        fb = lib().ref_replay_ws_bytes(m, n, 0)
        hb = lib().ref_replay_ws_bytes(m, n, 1)
        self.f = torch.empty(fb, dtype=torch.uint8, device="cuda")
        self.h = torch.empty(max(hb, 1), dtype=torch.uint8, device="cuda") if hb else None

    def ptrs(self):
        return ctypes.c_void_p(self.f.data_ptr()), (ctypes.c_void_p(self.h.data_ptr()) if self.h is not None
                                                   else None)


def auto_scale(method: str, mat, workspaces: Workspaces | None = None, seed: int = 1) -> float:
    """composite_*_auto_scale of `method` on the FP64 CUDA tensor mat (n x n,
    column-major storage), in place; returns the bound used as the scale."""
    import numpy as np

    sched = "fp16" if method == "composite_FP16" else "fp32"
    coef = np.array([float(v) for t in schedule_coefficients(sched) for v in t], dtype=np.float32)
    up = ctypes.c_double(0.0)
    f, h = workspaces.ptrs() if workspaces is not None else (None, None)
    rc = lib().ref_replay_auto_scale(METHODS[method], ctypes.c_void_p(mat.data_ptr()), mat.shape[0],
                                     coef.ctypes.data_as(ctypes.c_void_p), len(coef) // 3, seed, f, h,
                                     ctypes.byref(up))
    if rc != 0:
        raise RuntimeError(f"ref_replay {method}: {rc} library calls failed")
    return up.value
