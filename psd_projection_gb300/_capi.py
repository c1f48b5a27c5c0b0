"""ctypes binding of libpsdgb.so (the C ABI declared in include/psdgb.h).

The library is built in-tree by psd_projection_gb300/build.py (or
__graft_entry__.build()).  Loading fails loudly when it is missing: there is
no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import re
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().with_name("libpsdgb.so")
HEADER_PATH = Path(__file__).resolve().parent.parent / "include" / "psdgb.h"

# psdgb_status
OK = 0
STATUS_NAMES = {
    0: "PSDGB_OK",
    1: "PSDGB_ERR_INVALID_ARGUMENT",
    2: "PSDGB_ERR_CUDA",
    3: "PSDGB_ERR_OUT_OF_MEMORY",
    4: "PSDGB_ERR_UNSUPPORTED",
    5: "PSDGB_ERR_DEVICE_TIMEOUT",
    6: "PSDGB_ERR_SOLVER",
    7: "PSDGB_ERR_WORKSPACE_TOO_SMALL",
}
ERR_INVALID_ARGUMENT = 1
ERR_DEVICE_TIMEOUT = 5

# psdgb_precision
PREC_FP32_SIMT = 0
PREC_FP16 = 1
PREC_BF16 = 2
PREC_FP16X3 = 3
PREC_BF16X3 = 4
PREC_BF16X6 = 5
PREC_BF16X9 = 6
PREC_FP8 = 7
PRECISIONS = {
    "fp32_simt": PREC_FP32_SIMT, "fp16": PREC_FP16, "bf16": PREC_BF16, "fp16x3": PREC_FP16X3,
    "bf16x3": PREC_BF16X3, "bf16x6": PREC_BF16X6, "bf16x9": PREC_BF16X9, "fp8": PREC_FP8,
}
# psdgb_schedule
SCHEDULE_FP32 = 0
SCHEDULE_FP16 = 1
SCHEDULE_FP8 = 2
# psdgb_residual
RESIDUAL_REFERENCE = 0
RESIDUAL_EXACT = 1

DEFAULT_SEED = 0x5EED5EED


class PsdgbError(RuntimeError):
    """A libpsdgb call returned a status other than PSDGB_OK."""

    def __init__(self, status: int, fn: str, message: str):
        self.status = status
        super().__init__(f"{fn}: {STATUS_NAMES.get(status, status)}: {message}")


_lib = None
_lock = threading.Lock()

c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_u64 = ctypes.c_uint64
c_size = ctypes.c_size_t
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
c_str = ctypes.c_char_p
P_dbl = ctypes.POINTER(ctypes.c_double)
P_i64 = ctypes.POINTER(ctypes.c_int64)

SIGNATURES = {
    "psdgb_version": (c_int, []),
    "psdgb_last_error": (c_str, []),
    "psdgb_precision_name": (c_str, [c_int]),
    "psdgb_composite_workspace_size": (c_size, [c_i64, c_int]),
    "psdgb_release_workspace": (c_int, []),
    "psdgb_composite": (c_int, [c_int, c_int, c_vp, c_i64, c_vp, c_size, c_vp]),
    "psdgb_composite_static": (c_int, [c_int, c_int, c_vp, c_i64, c_vp]),
    "psdgb_lanczos_state_size": (c_size, [c_i64, c_i64]),
    "psdgb_composite_auto_scale_async": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_dbl, c_u64, c_int, c_vp, c_vp,
                                                 c_vp, c_size, c_vp, c_size, c_vp]),
    "psdgb_check_device_error": (c_int, []),
    "psdgb_set_product_config": (c_int, [c_int]),
    "psdgb_set_product_tuning": (c_int, [c_int, c_int]),
    "psdgb_composite_mixed_auto_scale": (c_int, [c_int, c_int, c_int, c_int, c_vp, c_i64, c_vp]),
    "psdgb_composite_auto_scale": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_dbl, c_u64, c_int, c_vp, c_size,
                                           c_vp, P_dbl]),
    "psdgb_two_norm": (c_int, [c_vp, c_i64, P_dbl, P_dbl, c_i64, c_dbl, c_u64, c_int, c_vp, c_size, c_vp]),
    "psdgb_two_norm_ex": (c_int, [c_vp, c_i64, P_dbl, P_dbl, c_i64, c_dbl, c_u64, c_int, c_vp, c_size, c_vp,
                                  P_dbl, P_dbl, P_i64, P_dbl]),
    "psdgb_eig_psd": (c_int, [c_int, c_vp, c_i64, c_vp, c_vp]),
    "psdgb_project": (c_int, [c_str, c_vp, c_i64, c_vp, c_vp]),
    "psdgb_project_host": (c_int, [c_str, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "psdgb_project_host_many": (c_int, [c_str, c_vp, c_vp, c_i64, c_i64, c_vp]),
    "psdgb_compute_eigenpairs": (c_int, [c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_int, c_i64, c_dbl, c_dbl, c_u64,
                                         c_vp, c_vp]),
    "psdgb_composite_auto_scale_deflate": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_dbl, c_dbl, c_u64, c_vp]),
    "psdgb_selftest_wait_timeout": (c_int, [c_dbl, c_vp]),
    "psdgb_composite_auto_scale_f32": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_dbl, c_u64, c_int, c_vp, c_vp,
                                               c_vp, c_size, c_vp, c_size, c_vp]),
    "psdgb_lobpcg": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_int, c_int, c_dbl, c_u64, c_vp, c_vp]),
    "psdgb_eig_FP64_deflate": (c_int, [c_vp, c_i64, c_i64, c_int, c_dbl, c_u64, c_vp]),
    "psdgb_composite_auto_scale_deflate_two_ends": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_int, c_dbl, c_u64,
                                                            c_vp]),
    "psdgb_kernel_launch_count": (c_u64, []),
    "psdgb_rel_frobenius": (c_int, [c_vp, c_vp, c_i64, P_dbl, c_vp]),
    "psdgb_filter_coefficients": (c_int, [c_int, ctypes.POINTER(ctypes.c_float), c_int]),
    "psdgb_product_timing_enable": (c_int, [c_int]),
    "psdgb_product_timing_read": (c_int, [P_dbl, ctypes.POINTER(ctypes.c_uint64), P_dbl, c_int]),
}


def header_functions() -> list[str]:
    """Names of every function include/psdgb.h declares."""
    text = HEADER_PATH.read_text()
    decl = r"(?:psdgb_status|int|size_t|double|uint64_t|const char\s*\*|void)\s+(psdgb_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, text)))


def lib() -> ctypes.CDLL:
    """Load libpsdgb.so once; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def last_error() -> str:
    return lib().psdgb_last_error().decode()


def check(status: int, fn: str) -> None:
    if status != OK:
        raise PsdgbError(status, fn, last_error())
