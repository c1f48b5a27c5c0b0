"""EVD entry points, the MATLAB method dispatch and the host-buffer path (GPU)."""
import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import from_dev, gaussian_sym, to_dev, uniform_spectrum

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def psd():
    import psd_projection_gb300 as psd

    return psd


def test_eig_fp64(psd):
    x = gaussian_sym(200, seed=1)
    proj, w = rp.eig_psd(x)
    t = to_dev(x)
    eigs = psd.eig_FP64_psd(t, return_eigenvalues=True)
    assert rp.rel_frobenius(from_dev(t), proj) <= 1e-12
    np.testing.assert_allclose(eigs.cpu().numpy(), w, rtol=0, atol=1e-10)
    t = to_dev(x)
    assert psd.eig_FP64_psd(t) is None


def test_eig_fp32(psd):
    x = gaussian_sym(150, seed=2)
    proj, w = rp.eig_psd(x)
    t = to_dev(x)
    eigs = psd.eig_FP32_psd(t, return_eigenvalues=True)
    assert rp.rel_frobenius(from_dev(t), proj) <= 1e-5
    np.testing.assert_allclose(eigs.cpu().numpy(), w, rtol=0, atol=1e-4 * np.abs(w).max())


@pytest.mark.parametrize("method,tol", [("composite_FP32", 1e-4), ("composite_FP32_emulated", 1e-4),
                                        ("composite_FP16", 3e-3), ("eig_FP64", 1e-12), ("eig_FP32", 1e-5)])
def test_project_methods(psd, method, tol):
    x = uniform_spectrum(160, 5.0, seed=3)
    proj, w = rp.eig_psd(x)
    t = to_dev(x)
    eigs = psd.project(method, t)
    assert rp.rel_frobenius(from_dev(t), proj) <= tol
    if method.startswith("eig"):
        np.testing.assert_allclose(eigs.cpu().numpy(), w, rtol=0, atol=1e-4 * np.abs(w).max())
    else:
        assert eigs is None


def test_project_host_matches_device(psd):
    x = uniform_spectrum(130, 2.0, seed=4)
    t = to_dev(x)
    psd.project("composite_FP32", t)
    out, eigs = psd.project_host("composite_FP32", np.ascontiguousarray(x.T))  # column-major storage
    assert eigs is None
    assert np.array_equal(out.T, from_dev(t))
    out2, eigs2 = psd.project_host("eig_FP64", np.ascontiguousarray(x.T))
    assert eigs2 is not None and eigs2.shape == (130,)


def test_unknown_method_raises(psd):
    import torch

    t = torch.eye(4, dtype=torch.float64, device="cuda")
    with pytest.raises(psd.PsdgbError, match="Unknown method"):
        psd.project("composite_FP8", t)


def test_rel_frobenius_helper(psd):
    a = gaussian_sym(60, seed=5)
    b = gaussian_sym(60, seed=6)
    assert psd.rel_frobenius(to_dev(a), to_dev(b)) == pytest.approx(rp.rel_frobenius(a, b), rel=1e-12)


def test_kernel_launches_are_counted(psd):
    before = psd.kernel_launch_count()
    t = to_dev(uniform_spectrum(64, 1.0, seed=7))
    psd.composite_FP32_auto_scale(t)
    # prologue + 20 Lanczos steps x 3 + Ritz + 10 filter steps x 3 + final >= 90
    assert psd.kernel_launch_count() - before >= 90


def test_project_host_many_matches_one_call_per_matrix():
    """The pipelined host sequence (copies of neighbouring matrices
    overlapping each projection, three staging buffers) returns, for every
    matrix, exactly what one synchronous call returns: the same device path
    runs on the same input.  Buffers rotate (a buffer reused three steps
    later) and one result overwrites its own input."""
    import torch

    import psd_projection_gb300 as psd

    n = 300
    rng = np.random.default_rng(5)
    mats = []
    for _ in range(5):
        g = rng.standard_normal((n, n))
        mats.append(0.5 * (g + g.T))
    ins = [torch.from_numpy(m).pin_memory() for m in mats]
    outs = [torch.empty_like(ins[0]).pin_memory() for _ in range(3)]
    plan_out = [outs[0], outs[1], outs[2], outs[0], ins[4]]
    expect = [psd.project_host("composite_FP32", m)[0] for m in mats]
    psd.project_host_many("composite_FP32", ins, plan_out)
    got = [None] * 5
    got[4] = ins[4].numpy().copy()
    got[3] = outs[0].numpy().copy()
    got[2] = outs[2].numpy().copy()
    got[1] = outs[1].numpy().copy()
    for i in (1, 2, 3, 4):
        assert np.array_equal(got[i], expect[i]), i
    proj, _ = rp.eig_psd(mats[3])
    assert rp.rel_frobenius(got[3], proj) <= 1e-4


def test_project_host_many_validates():
    import psd_projection_gb300 as psd

    a = np.zeros((4, 4))
    with pytest.raises(ValueError):
        psd.project_host_many("composite_FP32", [a], [])
    with pytest.raises(psd.PsdgbError, match="Unknown method"):
        psd.project_host_many("nope", [a], [np.zeros((4, 4))])
    # A result may not land in the input of either of the next two matrices.
    bufs = [np.eye(4) for _ in range(3)]
    with pytest.raises(psd.PsdgbError, match="must not be"):
        psd.project_host_many("composite_FP32", bufs, [bufs[2], np.zeros((4, 4)), np.zeros((4, 4))])
