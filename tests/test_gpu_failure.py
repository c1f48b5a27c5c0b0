"""Failure detection on the GPU without a fault: a bounded device-side wait
gives up, the host reads the error word, and the context stays usable.

psdgb_selftest_wait_timeout runs one thread that waits on an mbarrier nothing
arrives at, through the same bounded-wait helper as the product kernels'
pipeline waits, with a short limit.  The expected outcome is
PSDGB_ERR_DEVICE_TIMEOUT after at least the limit, then normal operation.
"""
import time

import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import from_dev, to_dev, uniform_spectrum

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives():
    import psd_projection_gb300 as psd

    lib = psd._capi.lib()
    t0 = time.perf_counter()
    st = lib.psdgb_selftest_wait_timeout(0.25, None)
    dt = time.perf_counter() - t0
    assert st == psd._capi.ERR_DEVICE_TIMEOUT
    assert "device error 5" in psd._capi.last_error()
    assert 0.25 <= dt < 5.0
    assert lib.psdgb_check_device_error() == 0  # the error word was cleared
    x = uniform_spectrum(200, 1.0, seed=3)
    t = to_dev(x)
    psd.composite(t)
    proj, _ = rp.eig_psd(x)
    assert rp.rel_frobenius(from_dev(t), proj) <= 1e-4


def test_selftest_limit_validation():
    import psd_projection_gb300 as psd

    assert psd._capi.lib().psdgb_selftest_wait_timeout(10.0, None) == psd._capi.ERR_INVALID_ARGUMENT
