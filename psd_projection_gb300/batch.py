"""Python handle on the block-diagonal batch (psdgb_batch_* in include/psdgb.h).

    plan = BatchPlan(sizes)                 # block sizes n_b
    plan.project(d_blocks)                  # packed column-major blocks, in place (async)
    plan.autotune(scratch)                  # pick the fastest accumulator mode / tile order / route
    plan.configure(acc_mode=2, small_on_chip=0, pair_tiles=1)   # or set them by hand

`pack` / `unpack` convert between a list of square matrices and the packed layout.
"""
from __future__ import annotations

import ctypes

from . import _capi

c_int, c_i64, c_size, c_dbl = ctypes.c_int, ctypes.c_int64, ctypes.c_size_t, ctypes.c_double
_bound = False


def _bind():
    global _bound
    lib = _capi.lib()
    if _bound:
        return lib
    vp = ctypes.c_void_p
    lib.psdgb_batch_create.restype = c_int
    lib.psdgb_batch_create.argtypes = [ctypes.POINTER(c_i64), c_i64, c_int, c_int, ctypes.POINTER(vp)]
    lib.psdgb_batch_destroy.restype = c_int
    lib.psdgb_batch_destroy.argtypes = [vp]
    lib.psdgb_batch_info.restype = c_int
    lib.psdgb_batch_info.argtypes = [vp, ctypes.POINTER(c_i64), ctypes.POINTER(c_size), ctypes.POINTER(c_i64),
                                     ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    lib.psdgb_batch_project.restype = c_int
    lib.psdgb_batch_project.argtypes = [vp, vp, vp]
    lib.psdgb_batch_project_graph.restype = c_int
    lib.psdgb_batch_project_graph.argtypes = [vp, vp, vp]
    lib.psdgb_batch_autotune.restype = c_int
    lib.psdgb_batch_autotune.argtypes = [vp, vp, vp, ctypes.POINTER(c_dbl)]
    lib.psdgb_batch_configure.restype = c_int
    lib.psdgb_batch_configure.argtypes = [vp, c_int, c_int, c_int, c_int, c_int]
    lib.psdgb_batch_tuning.restype = c_int
    lib.psdgb_batch_tuning.argtypes = [vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                       ctypes.POINTER(c_i64), ctypes.POINTER(c_int), ctypes.POINTER(c_i64),
                                       ctypes.POINTER(c_int)]
    _bound = True
    return lib


def pack(mats, device="cuda"):
    """Packed column-major storage of a list of square float64 matrices (numpy)."""
    import numpy as np
    import torch

    flat = np.concatenate([np.ascontiguousarray(np.asarray(m, dtype=np.float64).T).reshape(-1) for m in mats])
    return torch.from_numpy(flat).to(device)


def unpack(packed, sizes):
    """List of matrices (numpy) from packed column-major storage."""
    host = packed.detach().cpu().numpy()
    out, off = [], 0
    for n in sizes:
        out.append(host[off:off + n * n].reshape(n, n).T.copy())
        off += n * n
    return out


class BatchPlan:
    def __init__(self, sizes, precision: int = _capi.PREC_FP16X3, schedule: int = _capi.SCHEDULE_FP32):
        lib = _bind()
        self.sizes = [int(n) for n in sizes]
        arr = (c_i64 * max(len(self.sizes), 1))(*self.sizes)
        h = ctypes.c_void_p()
        _capi.check(lib.psdgb_batch_create(arr, len(self.sizes), precision, schedule, ctypes.byref(h)),
                    "psdgb_batch_create")
        self._h = h

    def info(self) -> dict:
        te, db, nt, am, to = c_i64(), c_size(), c_i64(), c_int(), c_int()
        _capi.check(_bind().psdgb_batch_info(self._h, ctypes.byref(te), ctypes.byref(db), ctypes.byref(nt),
                                             ctypes.byref(am), ctypes.byref(to)), "psdgb_batch_info")
        return {"total_elements": te.value, "device_bytes": db.value, "num_tiles": nt.value, "acc_mode": am.value,
                "tile_order": to.value}

    def configure(self, acc_mode: int = -1, tile_order: int = -1, small_on_chip: int = -1,
                  pair_tiles: int = -1, serpentine: int = -1) -> None:
        """Set the accumulator mode (0..2), tile order (0 largest first, 1 block
        order), the on-chip route for blocks of n <= 128 (0 / 1), the 256 x 256
        pair tiles for blocks of n > 128 (0 / 1) and the serpentine product
        order (0 / 1); -1 keeps."""
        _capi.check(_bind().psdgb_batch_configure(self._h, acc_mode, tile_order, small_on_chip, pair_tiles,
                                                  serpentine), "psdgb_batch_configure")

    def tuning(self) -> dict:
        am, to, oc, sb, pt, npt, sp = c_int(), c_int(), c_int(), c_i64(), c_int(), c_i64(), c_int()
        _capi.check(_bind().psdgb_batch_tuning(self._h, ctypes.byref(am), ctypes.byref(to), ctypes.byref(oc),
                                               ctypes.byref(sb), ctypes.byref(pt), ctypes.byref(npt),
                                               ctypes.byref(sp)), "psdgb_batch_tuning")
        return {"acc_mode": am.value, "tile_order": to.value, "small_on_chip": oc.value, "small_blocks": sb.value,
                "pair_tiles": pt.value, "num_pair_tiles": npt.value, "serpentine": sp.value}

    def project(self, d_blocks, stream=None) -> None:
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        _capi.check(_bind().psdgb_batch_project(self._h, ctypes.c_void_p(d_blocks.data_ptr()),
                                                ctypes.c_void_p(s.cuda_stream)), "psdgb_batch_project")

    def project_graph(self, d_blocks, stream=None) -> None:
        """project() as one launch of a graph the plan captures once (per
        d_blocks pointer and configuration) with the kernels' stream
        priorities kept."""
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        _capi.check(_bind().psdgb_batch_project_graph(self._h, ctypes.c_void_p(d_blocks.data_ptr()),
                                                      ctypes.c_void_p(s.cuda_stream)), "psdgb_batch_project_graph")

    def autotune(self, d_scratch, stream=None) -> float:
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        ms = c_dbl()
        _capi.check(_bind().psdgb_batch_autotune(self._h, ctypes.c_void_p(d_scratch.data_ptr()),
                                                 ctypes.c_void_p(s.cuda_stream), ctypes.byref(ms)),
                    "psdgb_batch_autotune")
        return ms.value

    def close(self) -> None:
        if self._h:
            _bind().psdgb_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
