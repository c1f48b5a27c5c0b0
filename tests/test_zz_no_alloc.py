"""psdgb_composite_static: the composite filter without any device allocation.

Callers that cannot allocate device memory — a solver that has reserved the
GPU's memory and hands out only its own buffers, or a real-time loop that may
not wait on or fail in the allocator — use psdgb_composite_static, whose
scratch is a file-scope device array in the library's CUDA module.  This file
checks, through the C ABI, that two calls in a row match psdgb_composite
(which takes its scratch from a workspace) within the FP32-class tolerance of
the other GPU tests (3e-5 relative Frobenius), that a call leaves the device's
free memory unchanged (with the library's cached workspace released first, so
a hidden use of it would show), and that sizes beyond its 512 limit are
refused with a clear error.

It is named to be collected last, so a run that stops at the first failure
has already run every other test; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 3e-5  # relative Frobenius, the FP32-class bound used across tests/


def _spectrum_matrix(n, seed):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.linspace(-1.0, 1.0, n)
    x = (q * lam) @ q.T
    return 0.5 * (x + x.T)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision_name,n", [("fp16x3", 300), ("fp16x3", 512), ("fp16", 200)])
def test_static_matches_workspace_entry_point_twice(precision_name, n):
    import torch

    from psd_projection_gb300 import _capi

    lib = _capi.lib()
    prec = _capi.PRECISIONS[precision_name]
    sched = _capi.SCHEDULE_FP16 if precision_name == "fp16" else _capi.SCHEDULE_FP32
    x = _spectrum_matrix(n, seed=n)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    ref = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    _capi.check(lib.psdgb_composite(prec, sched, ctypes.c_void_p(ref.data_ptr()), n, None, 0, stream),
                "psdgb_composite")
    want = ref.cpu().numpy()
    # Drop the cached workspace psdgb_composite just filled: the static calls
    # must not use (or re-create) it.
    _capi.check(lib.psdgb_release_workspace(), "psdgb_release_workspace")

    bufs = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for _ in range(2)]
    torch.cuda.synchronize()
    for i, t in enumerate(bufs):  # two calls in a row share (and reuse) the static scratch
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.psdgb_composite_static(prec, sched, ctypes.c_void_p(t.data_ptr()), n, stream)
        free_after = torch.cuda.mem_get_info()[0]
        _capi.check(st, "psdgb_composite_static")
        if i == 1:  # the first call on a device may load the module that holds the array
            assert free_after == free_before, (free_before, free_after)
        got = t.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _rel(got, want) <= TOL


def test_static_refuses_sizes_beyond_its_scratch():
    import torch

    from psd_projection_gb300 import _capi

    lib = _capi.lib()
    t = torch.zeros((513, 513), dtype=torch.float64, device="cuda")
    st = lib.psdgb_composite_static(_capi.PREC_FP16X3, _capi.SCHEDULE_FP32, ctypes.c_void_p(t.data_ptr()), 513,
                                    None)
    assert st == 1  # PSDGB_ERR_INVALID_ARGUMENT
    assert "512" in _capi.last_error()
    st = lib.psdgb_composite_static(_capi.PREC_BF16X9, _capi.SCHEDULE_FP32, ctypes.c_void_p(t.data_ptr()), 8, None)
    assert st == 1
