"""Python handle on the library's request loop (psdgb_server_* in include/psdgb.h).

    srv = Server(hbm_budget_bytes=8 << 30, max_slots=8)
    t = srv.submit(key, d_in, d_out)          # torch CUDA float64 n x n tensors
    done = srv.poll(wait=True)                # list of Completion records
    srv.close()

The scheduling, slots, streams, admission and warm starts are native (csrc/serve.cu);
this module only marshals arguments.
"""
from __future__ import annotations

import ctypes

from . import _capi

c_int, c_i64, c_u64, c_dbl, c_size = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_size_t


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_size), ("max_slots", c_int), ("precision", c_int), ("schedule", c_int),
                ("max_iter", c_i64), ("warm_max_iter", c_i64), ("use_graphs", c_int), ("admission", c_int),
                ("priority_n", c_i64), ("reserve_sms", c_int), ("reserve_slots", c_int)]


class Completion(ctypes.Structure):
    _fields_ = [("ticket", c_u64), ("key", c_i64), ("n", c_i64), ("status", c_int), ("submit_s", c_dbl),
                ("start_s", c_dbl), ("end_s", c_dbl), ("gpu_ms", c_dbl)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_bound = False


def _bind():
    global _bound
    if _bound:
        return _capi.lib()
    lib = _capi.lib()
    vp = ctypes.c_void_p
    lib.psdgb_clock_seconds.restype = c_dbl
    lib.psdgb_clock_seconds.argtypes = []
    lib.psdgb_server_create.restype = c_int
    lib.psdgb_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]
    lib.psdgb_server_destroy.restype = c_int
    lib.psdgb_server_destroy.argtypes = [vp]
    lib.psdgb_server_submit.restype = c_int
    lib.psdgb_server_submit.argtypes = [vp, c_i64, vp, vp, c_i64, ctypes.POINTER(c_u64)]
    lib.psdgb_server_poll.restype = c_int
    lib.psdgb_server_poll.argtypes = [vp, c_int, ctypes.POINTER(Completion), c_int, ctypes.POINTER(c_int)]
    lib.psdgb_server_stats.restype = c_int
    lib.psdgb_server_stats.argtypes = [vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_size),
                                       ctypes.POINTER(c_u64)]
    _bound = True
    return lib


def clock() -> float:
    """The host clock the server stamps completions with (seconds)."""
    return _bind().psdgb_clock_seconds()


class Server:
    def __init__(self, hbm_budget_bytes: int = 16 << 30, max_slots: int = 8, precision: int = _capi.PREC_FP16X3,
                 schedule: int = _capi.SCHEDULE_FP32, max_iter: int = 20, warm_max_iter: int = 20,
                 use_graphs: bool = True, admission: str = "fifo", priority_n: int = 0, reserve_sms: int = 0,
                 reserve_slots: int = 0):
        lib = _bind()
        if admission not in ("fifo", "shortest_first"):
            raise ValueError("admission is 'fifo' or 'shortest_first'")
        self.cfg = ServerConfig(hbm_budget_bytes, max_slots, precision, schedule, max_iter, warm_max_iter,
                                1 if use_graphs else 0, 0 if admission == "fifo" else 1, priority_n, reserve_sms,
                                reserve_slots)
        h = ctypes.c_void_p()
        _capi.check(lib.psdgb_server_create(ctypes.byref(self.cfg), ctypes.byref(h)), "psdgb_server_create")
        self._h = h
        self._buf = (Completion * 256)()

    def submit(self, key: int, d_in, d_out=None) -> int:
        d_out = d_in if d_out is None else d_out
        t = c_u64()
        st = _bind().psdgb_server_submit(self._h, key, ctypes.c_void_p(d_in.data_ptr()),
                                         ctypes.c_void_p(d_out.data_ptr()), d_in.shape[0], ctypes.byref(t))
        _capi.check(st, "psdgb_server_submit")
        return t.value

    def poll(self, wait: bool = False) -> list[Completion]:
        k = c_int()
        _capi.check(_bind().psdgb_server_poll(self._h, 1 if wait else 0, self._buf, 256, ctypes.byref(k)),
                    "psdgb_server_poll")
        return [Completion.from_buffer_copy(self._buf[i]) for i in range(k.value)]

    def drain(self) -> list[Completion]:
        out = []
        while True:
            st = self.stats()
            if st["in_flight"] == 0 and st["queued"] == 0:
                return out
            out += self.poll(wait=True)

    def stats(self) -> dict:
        f, q, b, c = c_int(), c_int(), c_size(), c_u64()
        _capi.check(_bind().psdgb_server_stats(self._h, ctypes.byref(f), ctypes.byref(q), ctypes.byref(b),
                                               ctypes.byref(c)), "psdgb_server_stats")
        return {"in_flight": f.value, "queued": q.value, "bytes_used": b.value, "completed": c.value}

    def close(self) -> None:
        if self._h:
            _bind().psdgb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
