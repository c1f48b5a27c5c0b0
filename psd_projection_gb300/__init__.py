"""psd_projection_gb300 — GB300-native PSD-cone projection (Python mirror of the C ABI).

The functions here mirror the reference library's C++ entry points
(ComputationalRobotics/psd_projection include/psd_projection/*.h) with the same
names and argument meaning, on torch CUDA tensors:

    composite_FP16(mat)                 composite_FP16_auto_scale(mat)
    composite_FP32(mat)                 composite_FP32_auto_scale(mat)
    composite_FP32_emulated(mat)        composite_FP32_emulated_auto_scale(mat)
    approximate_two_norm(A, max_iter=20, tol=1e-10) -> (lo, up)
    eig_FP64_psd(mat, return_eigenvalues=False)
    eig_FP32_psd(mat, return_eigenvalues=False)
    project(method, mat)                # the MATLAB wrapper's method strings
    project_host(method, array)         # the same on host (numpy) buffers

`mat` is an n x n float64 CUDA tensor projected in place.  Its memory is read
as the reference reads `double* mat`: column-major.  A C-contiguous torch
tensor M therefore stands for the column-major matrix M^T; for the symmetric
matrices these functions take, the two are the same.  Where a matrix is not
exactly symmetric, its upper triangle (row <= column in the column-major
sense) defines it, as in cuSOLVER syevd with CUBLAS_FILL_MODE_UPPER.

Error behaviour: the reference prints and continues; this mirror raises
PsdgbError with the library's message.  Every call runs the CUDA kernels of
libpsdgb.so — there is no CPU path.
"""
from __future__ import annotations

import ctypes

from . import _capi
from ._capi import (DEFAULT_SEED, PREC_BF16, PREC_BF16X3, PREC_BF16X6, PREC_BF16X9, PREC_FP8, PREC_FP16,
                    PREC_FP16X3, PREC_FP32_SIMT, PRECISIONS, RESIDUAL_EXACT, RESIDUAL_REFERENCE, SCHEDULE_FP8,
                    SCHEDULE_FP16, SCHEDULE_FP32, PsdgbError)

__all__ = [
    "composite", "composite_mixed", "composite_FP16", "composite_FP16_auto_scale", "composite_FP32", "composite_FP32_auto_scale",
    "composite_FP32_emulated", "composite_FP32_emulated_auto_scale", "approximate_two_norm", "lanczos_details",
    "eig_FP64_psd", "eig_FP32_psd", "project", "project_host", "workspace_size", "filter_coefficients",
    "kernel_launch_count", "rel_frobenius", "PsdgbError", "PRECISIONS", "METHODS",
]

# MATLAB method string -> (precision, schedule), MATLAB/psd_projection_MATLAB.cu:112-166.
METHODS = {
    "composite_FP16": (PREC_FP16, SCHEDULE_FP16),
    "composite_FP32": (PREC_FP16X3, SCHEDULE_FP32),
    "composite_FP32_emulated": (PREC_BF16X9, SCHEDULE_FP32),
    "eig_FP64": None,
    "eig_FP32": None,
}


def _torch():
    import torch  # deferred: the C ABI itself needs no torch
    return torch


def _stream_ptr(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _check_mat(mat, name="mat"):
    torch = _torch()
    if not isinstance(mat, torch.Tensor) or not mat.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if mat.dtype != torch.float64:
        raise TypeError(f"{name} must be float64 (the reference's double* mat)")
    if mat.dim() != 2 or mat.shape[0] != mat.shape[1]:
        raise ValueError(f"{name} must be square, got {tuple(mat.shape)}")
    if not mat.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return mat.shape[0]


def _ws_args(workspace):
    if workspace is None:
        return None, 0
    return ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()


def workspace_size(n: int, precision: int = PREC_FP16X3) -> int:
    """Device bytes of filter workspace for an n x n matrix at a precision."""
    return int(_capi.lib().psdgb_composite_workspace_size(n, precision))


def filter_coefficients(schedule: int = SCHEDULE_FP32) -> list[tuple[float, float, float]]:
    """The (a, b, c) of every filter step after the safety scaling, as FP32."""
    buf = (ctypes.c_float * 64)()
    k = _capi.lib().psdgb_filter_coefficients(schedule, buf, 21)
    if k < 0:
        raise ValueError("unknown schedule")
    return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(k)]


def composite(mat, precision: int = PREC_FP16X3, schedule: int = SCHEDULE_FP32, auto_scale: bool = True,
              max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED,
              residual: int = RESIDUAL_REFERENCE, workspace=None, stream=None) -> float:
    """Project mat in place with the composite filter; returns the scale used (up, or 1)."""
    n = _check_mat(mat)
    ws, wsb = _ws_args(workspace)
    lib = _capi.lib()
    if auto_scale:
        up = ctypes.c_double(1.0)
        st = lib.psdgb_composite_auto_scale(precision, schedule, ctypes.c_void_p(mat.data_ptr()), n, max_iter, tol,
                                            seed, residual, ws, wsb, _stream_ptr(stream), ctypes.byref(up))
        _capi.check(st, "psdgb_composite_auto_scale")
        return up.value
    st = lib.psdgb_composite(precision, schedule, ctypes.c_void_p(mat.data_ptr()), n, ws, wsb, _stream_ptr(stream))
    _capi.check(st, "psdgb_composite")
    return 1.0


def composite_mixed(mat, bulk: str = "bf16", refine: str = "bf16x9", refine_steps: int = 2,
                    bulk_schedule: int | None = None, stream=None) -> None:
    """Low-precision bulk (one-term products) followed by refine_steps
    FP32-class refinement steps and reconstruction, auto-scaled, in place.
    The bulk schedule defaults to the FP8 schedule for bulk="fp8", else FP16."""
    n = _check_mat(mat)
    if bulk_schedule is None:
        bulk_schedule = SCHEDULE_FP8 if bulk == "fp8" else SCHEDULE_FP16
    st = _capi.lib().psdgb_composite_mixed_auto_scale(PRECISIONS[bulk], bulk_schedule, PRECISIONS[refine],
                                                      refine_steps, ctypes.c_void_p(mat.data_ptr()), n,
                                                      _stream_ptr(stream))
    _capi.check(st, "psdgb_composite_mixed_auto_scale")


def composite_FP16(mat, workspace=None):
    """composite_FP16 (include/psd_projection/composite_FP16.h:12-18): spectrum must lie in [-1, 1]."""
    composite(mat, PREC_FP16, SCHEDULE_FP16, auto_scale=False, workspace=workspace)


def composite_FP16_auto_scale(mat, workspace=None):
    composite(mat, PREC_FP16, SCHEDULE_FP16, auto_scale=True, workspace=workspace)


def composite_FP32(mat, workspace=None):
    """composite_FP32 (include/psd_projection/composite_FP32.h:12-17): spectrum must lie in [-1, 1]."""
    composite(mat, PREC_FP16X3, SCHEDULE_FP32, auto_scale=False, workspace=workspace)


def composite_FP32_auto_scale(mat, workspace=None):
    composite(mat, PREC_FP16X3, SCHEDULE_FP32, auto_scale=True, workspace=workspace)


def composite_FP32_emulated(mat, workspace=None):
    composite(mat, PREC_BF16X9, SCHEDULE_FP32, auto_scale=False, workspace=workspace)


def composite_FP32_emulated_auto_scale(mat, workspace=None):
    composite(mat, PREC_BF16X9, SCHEDULE_FP32, auto_scale=True, workspace=workspace)


def lanczos_details(A, max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED,
                    residual: int = RESIDUAL_REFERENCE, stream=None) -> dict:
    """approximate_two_norm with its internals: lo, up, theta, nb_iter, alpha, beta."""
    n = _check_mat(A, "A")
    lo, up, theta = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    nb = ctypes.c_int64()
    m = max(int(max_iter), 1)
    alpha = (ctypes.c_double * m)()
    beta = (ctypes.c_double * m)()
    st = _capi.lib().psdgb_two_norm_ex(ctypes.c_void_p(A.data_ptr()), n, ctypes.byref(lo), ctypes.byref(up),
                                       max_iter, tol, seed, residual, None, 0, _stream_ptr(stream), alpha, beta,
                                       ctypes.byref(nb), ctypes.byref(theta))
    _capi.check(st, "psdgb_two_norm_ex")
    k = min(int(max_iter), n)
    return {"lo": lo.value, "up": up.value, "theta": theta.value, "nb_iter": nb.value,
            "alpha": list(alpha[:k]), "beta": list(beta[:k])}


def approximate_two_norm(A, max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED,
                         residual: int = RESIDUAL_REFERENCE, stream=None) -> tuple[float, float]:
    """approximate_two_norm (include/psd_projection/lanczos.h:11-17): returns (lo, up)."""
    d = lanczos_details(A, max_iter, tol, seed, residual, stream)
    return d["lo"], d["up"]


def _eig(fp64: int, mat, return_eigenvalues: bool, stream=None):
    torch = _torch()
    n = _check_mat(mat)
    eigs = torch.empty(n, dtype=torch.float64, device=mat.device) if return_eigenvalues else None
    st = _capi.lib().psdgb_eig_psd(fp64, ctypes.c_void_p(mat.data_ptr()), n,
                                   ctypes.c_void_p(eigs.data_ptr()) if eigs is not None else None,
                                   _stream_ptr(stream))
    _capi.check(st, "psdgb_eig_psd")
    return eigs


def eig_FP64_psd(mat, return_eigenvalues: bool = False):
    """eig_FP64_psd (include/psd_projection/eig_FP64_psd.h:14-20): in place; optional eigenvalues."""
    return _eig(1, mat, return_eigenvalues)


def eig_FP32_psd(mat, return_eigenvalues: bool = False):
    return _eig(0, mat, return_eigenvalues)


def project(method: str, mat, stream=None):
    """MATLAB psd_projection_MATLAB(A, method) on a device tensor, in place.

    Returns the eigenvalues for eig_* methods, else None."""
    torch = _torch()
    n = _check_mat(mat)
    eigs = None
    if method in ("eig_FP64", "eig_FP32"):
        eigs = torch.empty(n, dtype=torch.float64, device=mat.device)
    st = _capi.lib().psdgb_project(method.encode(), ctypes.c_void_p(mat.data_ptr()), n,
                                   ctypes.c_void_p(eigs.data_ptr()) if eigs is not None else None,
                                   _stream_ptr(stream))
    _capi.check(st, "psdgb_project")
    return eigs


def project_host(method: str, a, out=None, stream=None):
    """psd_projection_MATLAB(A, method) on host memory: a is an (n, n) float64
    numpy array (or pinned CPU tensor) read as column-major; the projection is
    written to out (a new array when None).  Returns (out, eigenvalues|None)."""
    import numpy as np

    torch = _torch()
    if isinstance(a, torch.Tensor):
        src_ptr, n = a.data_ptr(), a.shape[0]
        if out is None:
            out = torch.empty_like(a)
        dst_ptr = out.data_ptr()
    else:
        a = np.ascontiguousarray(a, dtype=np.float64)
        n = a.shape[0]
        if out is None:
            out = np.empty_like(a)
        src_ptr, dst_ptr = a.ctypes.data, out.ctypes.data
    eigs = np.empty(n, dtype=np.float64) if method in ("eig_FP64", "eig_FP32") else None
    st = _capi.lib().psdgb_project_host(method.encode(), ctypes.c_void_p(src_ptr), ctypes.c_void_p(dst_ptr), n,
                                        ctypes.c_void_p(eigs.ctypes.data) if eigs is not None else None,
                                        _stream_ptr(stream))
    _capi.check(st, "psdgb_project_host")
    return out, eigs


def project_host_many(method: str, inputs, outputs, stream=None):
    """Project a sequence of (n, n) float64 host matrices (numpy arrays or
    pinned CPU tensors, column-major) with one method: inputs[i] -> outputs[i],
    the copies of neighbouring matrices overlapping each projection
    (psdgb_project_host_many).  outputs[i] must not be inputs[i + 1] or
    inputs[i + 2] (refused with PsdgbError)."""
    import numpy as np

    torch = _torch()
    if len(inputs) != len(outputs):
        raise ValueError("inputs and outputs differ in length")
    count = len(inputs)
    if count == 0:
        return outputs

    def ptr(x):
        if isinstance(x, torch.Tensor):
            if x.dtype != torch.float64 or x.device.type != "cpu" or not x.is_contiguous():
                raise ValueError("host tensors must be contiguous float64 CPU tensors")
            return x.data_ptr(), x.shape
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
            raise ValueError("host arrays must be C-contiguous float64")
        return x.ctypes.data, x.shape

    src = [ptr(x) for x in inputs]
    dst = [ptr(x) for x in outputs]
    n = src[0][1][0]
    for p_, shape in src + dst:
        if tuple(shape) != (n, n):
            raise ValueError("all matrices must be n x n with the same n")
    arr_in = (ctypes.c_void_p * count)(*[p_ for p_, _ in src])
    arr_out = (ctypes.c_void_p * count)(*[p_ for p_, _ in dst])
    st = _capi.lib().psdgb_project_host_many(method.encode(), ctypes.cast(arr_in, ctypes.c_void_p),
                                             ctypes.cast(arr_out, ctypes.c_void_p), n, count, _stream_ptr(stream))
    _capi.check(st, "psdgb_project_host_many")
    return outputs


def kernel_launch_count() -> int:
    return int(_capi.lib().psdgb_kernel_launch_count())


def rel_frobenius(a, b, stream=None) -> float:
    """||a - b||_F / ||b||_F of two n x n float64 CUDA tensors (FP64 reduction on the device)."""
    n = _check_mat(a, "a")
    _check_mat(b, "b")
    out = ctypes.c_double()
    st = _capi.lib().psdgb_rel_frobenius(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()), n,
                                         ctypes.byref(out), _stream_ptr(stream))
    _capi.check(st, "psdgb_rel_frobenius")
    return out.value


TUNE_TILE_GROUP = 1
TUNE_TILE_SHAPE = 2
TUNE_WIDE_KBLOCK = 3
TUNE_GROUP_EPI_WARPS = 4
TUNE_LANCZOS_SYMV = 5
TILE_AUTO, TILE_128X128, TILE_PAIR_256X128, TILE_WIDE_128X256, TILE_PAIR_256X256 = -1, 0, 1, 2, 3


def set_product_config(acc_mode: int) -> int:
    """Accumulator configuration of single-matrix products (-1 automatic, 0, 1, 2); returns the previous one."""
    return int(_capi.lib().psdgb_set_product_config(int(acc_mode)))


def set_product_tuning(knob: int, value: int) -> int:
    """Process-wide product / bound settings; returns the previous value.  TUNE_TILE_GROUP (tile rows
    per group of the tile order, 0 = row by row), TUNE_TILE_SHAPE (TILE_AUTO, TILE_128X128,
    TILE_PAIR_256X128, TILE_WIDE_128X256, TILE_PAIR_256X256), TUNE_WIDE_KBLOCK (0, 32, 64),
    TUNE_GROUP_EPI_WARPS (4, 8), TUNE_LANCZOS_SYMV (-1 automatic, 0 whole-matrix matvec, 1 lower
    block triangle)."""
    return int(_capi.lib().psdgb_set_product_tuning(int(knob), int(value)))


def compute_eigenpairs(A, k: int, upper_bound_only: bool = False, max_iter: int = 0, tol: float = 1e-10,
                       ortho_tol: float = 1e-5, seed: int = DEFAULT_SEED, stream=None) -> dict:
    """compute_eigenpairs (include/psd_projection/lanczos.h:19-44) on a float64
    CUDA matrix: {"upper": bound, "r": pairs kept (None when upper_bound_only),
    "values": (r,) tensor, "vectors": (r, n) tensor, row i = eigenvector i}."""
    torch = _torch()
    n = _check_mat(A)
    kk = max(int(k), 0)
    vals = torch.empty(max(kk, 1), dtype=torch.float64, device=A.device)
    vecs = torch.empty((max(kk, 1), max(n, 1)), dtype=torch.float64, device=A.device)
    r = ctypes.c_int64(-1)
    up = ctypes.c_double(0.0)
    st = _capi.lib().psdgb_compute_eigenpairs(
        ctypes.c_void_p(A.data_ptr()), n, kk, ctypes.byref(r),
        None if upper_bound_only else ctypes.c_void_p(vals.data_ptr()),
        None if upper_bound_only else ctypes.c_void_p(vecs.data_ptr()), 1 if upper_bound_only else 0,
        int(max_iter), float(tol), float(ortho_tol), int(seed), ctypes.byref(up), _stream_ptr(stream))
    _capi.check(st, "psdgb_compute_eigenpairs")
    if upper_bound_only:
        return {"upper": up.value, "r": None, "values": None, "vectors": None}
    return {"upper": up.value, "r": r.value, "values": vals[: r.value], "vectors": vecs[: r.value]}


def composite_auto_scale_deflate(mat, precision: int = PREC_FP16X3, schedule: int = SCHEDULE_FP32, k: int = 40,
                                 tol: float = 1e-10, ortho_tol: float = 1e-3, seed: int = DEFAULT_SEED,
                                 stream=None) -> None:
    """composite_FP32_auto_scale_deflate (include/psd_projection/composite_FP32.h:32-45)
    with any precision, in place on a float64 CUDA matrix."""
    n = _check_mat(mat)
    st = _capi.lib().psdgb_composite_auto_scale_deflate(int(precision), int(schedule), ctypes.c_void_p(mat.data_ptr()),
                                                        n, int(k), float(tol), float(ortho_tol), int(seed),
                                                        _stream_ptr(stream))
    _capi.check(st, "psdgb_composite_auto_scale_deflate")


def composite_FP32_auto_scale_deflate(mat, k: int = 40, tol: float = 1e-10, ortho_tol: float = 1e-3) -> None:
    composite_auto_scale_deflate(mat, PREC_FP16X3, SCHEDULE_FP32, k, tol, ortho_tol)


def composite_FP32_emulated_auto_scale_deflate(mat, k: int = 40, tol: float = 1e-10, ortho_tol: float = 1e-3) -> None:
    composite_auto_scale_deflate(mat, PREC_BF16X9, SCHEDULE_FP32, k, tol, ortho_tol)


def lobpcg(A, m: int, V0=None, maxiter: int = 100, tol: float = 1e-8, seed: int = 0, stream=None) -> dict:
    """lobpcg (include/psd_projection/lobpcg.h) on a float64 CUDA matrix: the
    m largest eigenpairs.  V0 (m, n), rows orthonormal, warm-starts.  Returns
    {"V": (m, n) tensor, row i = eigenvector i, "D": (m,) decreasing, "iters"}."""
    torch = _torch()
    n = _check_mat(A)
    V = torch.empty((max(int(m), 1), n), dtype=torch.float64, device=A.device)
    D = torch.empty(max(int(m), 1), dtype=torch.float64, device=A.device)
    if V0 is not None:
        V.copy_(V0)
    iters = ctypes.c_int(0)
    st = _capi.lib().psdgb_lobpcg(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(V.data_ptr()),
                                  ctypes.c_void_p(D.data_ptr()), n, int(m), 1 if V0 is not None else 0, int(maxiter),
                                  float(tol), int(seed), ctypes.byref(iters), _stream_ptr(stream))
    _capi.check(st, "psdgb_lobpcg")
    return {"V": V[: int(m)], "D": D[: int(m)], "iters": iters.value}


def eig_FP64_deflate(mat, k: int = 40, maxiter: int = 100, tol: float = 1e-10, seed: int = 0, stream=None) -> None:
    """eig_FP64_deflate (include/psd_projection/eig_FP64_psd.h:22-31), in place."""
    n = _check_mat(mat)
    st = _capi.lib().psdgb_eig_FP64_deflate(ctypes.c_void_p(mat.data_ptr()), n, int(k), int(maxiter), float(tol),
                                            int(seed), _stream_ptr(stream))
    _capi.check(st, "psdgb_eig_FP64_deflate")


def composite_FP16_auto_scale_deflate(mat, k: int = 40, maxiter: int = 100, tol: float = 1e-10, seed: int = 0,
                                      precision: int = PREC_FP16, schedule: int = SCHEDULE_FP16, stream=None) -> None:
    """composite_FP16_auto_scale_deflate (include/psd_projection/composite_FP16.h:35-50), in place;
    precision / schedule select the filter (the reference's is FP16)."""
    n = _check_mat(mat)
    st = _capi.lib().psdgb_composite_auto_scale_deflate_two_ends(int(precision), int(schedule),
                                                                 ctypes.c_void_p(mat.data_ptr()), n, int(k),
                                                                 int(maxiter), float(tol), int(seed),
                                                                 _stream_ptr(stream))
    _capi.check(st, "psdgb_composite_auto_scale_deflate_two_ends")


def async_buffers(n: int, precision: int = PREC_FP16X3, max_iter: int = 20):
    """Device buffers for composite_async: (workspace, Lanczos state), uint8 CUDA tensors."""
    torch = _torch()
    ws = torch.empty(max(workspace_size(n, precision), 1), dtype=torch.uint8, device="cuda")
    lz = torch.empty(max(_capi.lib().psdgb_lanczos_state_size(n, max_iter), 1), dtype=torch.uint8, device="cuda")
    return ws, lz


def composite_async(mat, workspace, lanczos_state, precision: int = PREC_FP16X3, schedule: int = SCHEDULE_FP32,
                    max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED,
                    residual: int = RESIDUAL_REFERENCE, warm_start=None, ritz_out=None, stream=None) -> None:
    """The auto-scaled projection of mat, in place, enqueued on the stream with
    no host synchronisation and no allocation (psdgb_composite_auto_scale_async);
    workspace / lanczos_state from async_buffers.  Calls on one stream may
    share the buffers; calls in flight on different streams may not."""
    n = _check_mat(mat)
    st = _capi.lib().psdgb_composite_auto_scale_async(
        int(precision), int(schedule), ctypes.c_void_p(mat.data_ptr()), n, int(max_iter), float(tol), int(seed),
        int(residual), ctypes.c_void_p(warm_start.data_ptr()) if warm_start is not None else None,
        ctypes.c_void_p(ritz_out.data_ptr()) if ritz_out is not None else None,
        ctypes.c_void_p(workspace.data_ptr()), workspace.numel(), ctypes.c_void_p(lanczos_state.data_ptr()),
        lanczos_state.numel(), _stream_ptr(stream))
    _capi.check(st, "psdgb_composite_auto_scale_async")


def composite_f32(mat, precision: int = PREC_FP16X3, schedule: int = SCHEDULE_FP32, max_iter: int = 20,
                  tol: float = 1e-10, seed: int = DEFAULT_SEED, residual: int = RESIDUAL_REFERENCE, warm_start=None,
                  ritz_out=None, stream=None) -> None:
    """The auto-scaled projection of a float32 CUDA matrix, in place, asynchronous
    (psdgb_composite_auto_scale_f32); warm_start / ritz_out are float64 (n,) CUDA tensors."""
    torch = _torch()
    if not isinstance(mat, torch.Tensor) or not mat.is_cuda or mat.dtype != torch.float32 or mat.dim() != 2 or \
            mat.shape[0] != mat.shape[1] or not mat.is_contiguous():
        raise TypeError("mat must be a contiguous square float32 CUDA tensor")
    n = mat.shape[0]
    st = _capi.lib().psdgb_composite_auto_scale_f32(
        int(precision), int(schedule), ctypes.c_void_p(mat.data_ptr()), n, int(max_iter), float(tol), int(seed),
        int(residual), ctypes.c_void_p(warm_start.data_ptr()) if warm_start is not None else None,
        ctypes.c_void_p(ritz_out.data_ptr()) if ritz_out is not None else None, None, 0, None, 0,
        _stream_ptr(stream))
    _capi.check(st, "psdgb_composite_auto_scale_f32")
