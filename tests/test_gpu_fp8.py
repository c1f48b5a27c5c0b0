"""FP8 (E4M3) products: tcgen05.mma kind::f8f6f4 with FP32 accumulation.

The reference has no FP8 method.  These tests hold the FP8 mode to the
arithmetic model of this library's kernels (oracle/reference_port.py,
composite_split_model with "fp8": E4M3 operand copies scaled by 2^7, the FP16
pair as the stored iterate, the FP8 schedule), and check the mixed path
(an FP8 bulk followed by FP16x3 refinement steps).

Tolerances: E4M3 keeps 4 significant bits, so the GPU's FP32 accumulation
and the model's FP64 accumulation round a few operands differently and the
two errors (relative Frobenius against FP64 EVD) differ by tens of percent;
the GPU error must lie within a factor 2 of the model's.  The absolute level
(about 5e-2 for the FP8 bulk, 2e-2 after two refinement steps on the model)
is what an E4M3 chain reaches: refinement that iterates on the sign
approximation cannot undo the eigenvector error of the bulk.
"""
import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import from_dev, to_dev, uniform_spectrum

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def psd():
    import psd_projection_gb300 as psd

    return psd


@pytest.mark.parametrize("n", [100, 129, 300])
def test_fp8_matches_kernel_model(psd, n):
    x = uniform_spectrum(n, 1.0, seed=40 + n)
    proj, _ = rp.eig_psd(x)
    t = to_dev(x)
    psd.composite(t, psd.PREC_FP8, psd.SCHEDULE_FP8, auto_scale=False)
    out = from_dev(t)
    assert np.all(np.isfinite(out))
    err = rp.rel_frobenius(out, proj)
    model = rp.rel_frobenius(rp.composite_split_model(x, "fp8", "fp8"), proj)
    assert 0.5 * model <= err <= 2.0 * model, (err, model)
    assert err <= 0.15


def test_fp8_auto_scaled(psd):
    x = uniform_spectrum(256, 7.0, seed=3)
    proj, _ = rp.eig_psd(x)
    t = to_dev(x)
    psd.composite(t, psd.PREC_FP8, psd.SCHEDULE_FP8, auto_scale=True)
    out = from_dev(t)
    assert np.all(np.isfinite(out))
    assert rp.rel_frobenius(out, proj) <= 0.15


def test_fp8_bulk_with_fp16x3_refinement(psd):
    x = uniform_spectrum(384, 1.0, seed=5)
    proj, _ = rp.eig_psd(x)
    errs = []
    for steps in (0, 1, 2):
        t = to_dev(x)
        psd.composite_mixed(t, "fp8", "fp16x3", steps)
        out = from_dev(t)
        assert np.all(np.isfinite(out))
        errs.append(rp.rel_frobenius(out, proj))
    # the refinement steps never make it worse, and the result stays at the FP8 level
    assert errs[1] <= errs[0] * 1.05 and errs[2] <= errs[0] * 1.05, errs
    assert errs[2] <= 0.1, errs


def test_fp8_needs_fp8_schedule(psd):
    t = to_dev(np.eye(8) * 0.5)
    with pytest.raises(psd.PsdgbError, match="FP8 schedule"):
        psd.composite(t, psd.PREC_FP8, psd.SCHEDULE_FP16, auto_scale=False)
