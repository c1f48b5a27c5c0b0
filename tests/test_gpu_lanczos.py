"""Lanczos bound on the GPU against the oracle and the reference's KAT."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_port as rp
from tests.gpu_util import gaussian_sym, to_dev, uniform_spectrum

pytestmark = pytest.mark.gpu
KAT = json.loads((Path(__file__).resolve().parent / "golden" / "kat.json").read_text())


@pytest.fixture(scope="module")
def psd():
    import psd_projection_gb300 as psd

    return psd


@pytest.mark.parametrize("residual", [0, 1])
def test_kat_two_norm(psd, residual):
    k = KAT["lanczos_two_norm"]
    a = np.array(k["matrix"])
    lo, up = psd.approximate_two_norm(to_dev(a), k["max_iter"], k["tol"], residual=residual)
    assert lo <= k["two_norm"] + k["two_norm_rounding"]
    assert k["two_norm"] <= up
    assert lo <= np.linalg.norm(a, 2) <= up


@pytest.mark.parametrize("n,residual", [(257, 0), (257, 1), (1000, 0), (64, 1)])
def test_parity_with_oracle(psd, n, residual):
    """Same seed, same recurrence: alpha/beta, nb_iter and the bounds agree with
    the FP64 oracle run on the FP32-rounded matrix (the GPU streams FP32)."""
    x = gaussian_sym(n, seed=n)
    x32 = x.astype(np.float32).astype(np.float64)
    want = rp.approximate_two_norm(x32, 20, 1e-10, residual=("reference", "exact")[residual])
    got = psd.lanczos_details(to_dev(x), 20, 1e-10, residual=residual)
    assert got["nb_iter"] == want["nb_iter"]
    nb = want["nb_iter"]
    # Without reorthogonalisation (as in the reference) the FP32 matvec
    # rounding is amplified in late steps: the first 12 coefficients agree to
    # 2e-5 / 2e-4, all of them to 1e-2; the bounds to 1e-6 / 1e-4.
    k = min(nb, 12)
    np.testing.assert_allclose(got["alpha"][:k], want["alpha"][:k], rtol=2e-5)
    np.testing.assert_allclose(got["beta"][:k], want["beta"][:k], rtol=2e-4)
    np.testing.assert_allclose(got["alpha"][:nb], want["alpha"][:nb], rtol=1e-2)
    assert got["lo"] == pytest.approx(want["lo"], rel=1e-6)
    assert got["up"] == pytest.approx(want["up"], rel=1e-4)
    sigma = np.linalg.norm(x, 2)
    assert got["lo"] <= sigma * (1 + 1e-6) and got["up"] >= sigma * (1 - 1e-6)


def test_zero_matrix_and_tiny_sizes(psd):
    lo, up = psd.approximate_two_norm(to_dev(np.zeros((7, 7))))
    assert (lo, up) == (0.0, 1.0)
    # n = 1: the first residual is exactly zero, so the reference's loop stops
    # before counting an iteration and returns its all-zero answer (0, 1)
    # (src/lanczos.cu:145-184); the GPU path reproduces that.
    lo, up = psd.approximate_two_norm(to_dev(np.array([[-3.0]])))
    want = rp.approximate_two_norm(np.array([[-3.0]]))
    assert (lo, up) == (want["lo"], want["up"]) == (0.0, 1.0)
    lo, up = psd.approximate_two_norm(to_dev(np.array([[1.0, 2.0], [2.0, -1.0]])), 5)
    assert lo <= np.sqrt(5.0) * (1 + 1e-7) <= up * (1 + 1e-7)


def test_early_stop_rank_one(psd):
    """The beta <= tol * alpha stop (src/lanczos.cu:145).  The GPU streams the
    matrix in FP32, so a residual that is zero in exact arithmetic sits near
    1e-7 * alpha: tolerances at or above ~1e-6 trigger the same stop as the
    FP64 reference; tighter ones run all max_iter steps (the bound is the same)."""
    v = np.random.default_rng(3).standard_normal(50)
    a = np.outer(v, v)
    got = psd.lanczos_details(to_dev(a), 20, 1e-5)
    want = rp.approximate_two_norm(a.astype(np.float32).astype(np.float64), 20, 1e-5)
    assert got["nb_iter"] == want["nb_iter"] < 20
    assert got["lo"] == pytest.approx(np.linalg.norm(a, 2), rel=1e-5)


def test_nonsymmetric_input_uses_upper_triangle(psd):
    x = np.random.default_rng(4).standard_normal((90, 90))
    got = psd.lanczos_details(to_dev(x), 20, 1e-10)
    ref = psd.lanczos_details(to_dev(rp.sym_upper(x)), 20, 1e-10)
    assert got == ref


def test_seed_changes_start_but_not_the_bound(psd):
    x = uniform_spectrum(300, 4.0, seed=9)
    a = psd.lanczos_details(to_dev(x), 20, 1e-10, seed=1, residual=1)
    b = psd.lanczos_details(to_dev(x), 20, 1e-10, seed=2, residual=1)
    assert a["alpha"] != b["alpha"]
    assert a["lo"] == pytest.approx(4.0, rel=1e-3) and b["lo"] == pytest.approx(4.0, rel=1e-3)


@pytest.fixture
def matvec_mode(psd):
    prev = psd.set_product_tuning(psd.TUNE_LANCZOS_SYMV, -1)
    yield lambda v: psd.set_product_tuning(psd.TUNE_LANCZOS_SYMV, v)
    psd.set_product_tuning(psd.TUNE_LANCZOS_SYMV, prev)


@pytest.mark.parametrize("n,residual", [(257, 0), (1000, 1), (2048, 0), (2100, 1)])
def test_triangle_matvec_parity_with_oracle(psd, matvec_mode, n, residual):
    """The matvec over the lower block triangle (128 x 128 tiles, each giving
    row and column sums) against the FP64 oracle, with the bars of the
    whole-matrix matvec."""
    matvec_mode(1)
    x = gaussian_sym(n, seed=n + 1)
    x32 = x.astype(np.float32).astype(np.float64)
    want = rp.approximate_two_norm(x32, 20, 1e-10, residual=("reference", "exact")[residual])
    got = psd.lanczos_details(to_dev(x), 20, 1e-10, residual=residual)
    assert got["nb_iter"] == want["nb_iter"]
    k = min(want["nb_iter"], 12)
    np.testing.assert_allclose(got["alpha"][:k], want["alpha"][:k], rtol=2e-5)
    np.testing.assert_allclose(got["beta"][:k], want["beta"][:k], rtol=2e-4)
    assert got["lo"] == pytest.approx(want["lo"], rel=1e-6)
    assert got["up"] == pytest.approx(want["up"], rel=1e-4)


@pytest.mark.parametrize("n", [2048, 4100])
def test_triangle_matvec_matches_column_matvec_and_repeats(psd, matvec_mode, n):
    """Both matvecs give the same bound; the triangle one is bit-for-bit
    repeatable (its cross-tile sums run in a fixed order whatever the CTA
    schedule)."""
    d = to_dev(gaussian_sym(n, seed=11))
    matvec_mode(0)
    col = psd.lanczos_details(d, 20, 1e-10)
    matvec_mode(1)
    tri = psd.lanczos_details(d, 20, 1e-10)
    again = psd.lanczos_details(d, 20, 1e-10)
    assert tri == again
    np.testing.assert_allclose(tri["alpha"][:12], col["alpha"][:12], rtol=2e-5)
    assert tri["lo"] == pytest.approx(col["lo"], rel=1e-6)
    assert tri["up"] == pytest.approx(col["up"], rel=1e-4)


def test_triangle_matvec_large(psd, matvec_mode):
    """n = 8192 (64 x 64 row blocks): both matvecs agree; with the automatic
    choice the triangle one runs."""
    d = to_dev(gaussian_sym(8192, seed=5))
    out = {}
    for mode in (0, 1, -1):
        matvec_mode(mode)
        out[mode] = psd.lanczos_details(d, 20, 1e-10)
    assert out[1] == out[-1]
    np.testing.assert_allclose(out[1]["alpha"][:12], out[0]["alpha"][:12], rtol=2e-5)
    assert out[1]["lo"] == pytest.approx(out[0]["lo"], rel=1e-6)
    assert out[1]["up"] == pytest.approx(out[0]["up"], rel=1e-4)
    assert out[1]["lo"] <= out[1]["up"]


@pytest.mark.parametrize("kind", ["gaussian", "clustered_top", "rank_two"])
@pytest.mark.parametrize("n", [300, 2100])
def test_tridiagonal_top_eigenvalue(psd, kind, n):
    """theta (the largest eigenvalue of the Lanczos tridiagonal, found by the
    four-warp Sturm multisection) against LAPACK on the same tridiagonal built
    from the returned alpha / beta: agreement to 32 ulps of ||T|| (both
    carry rounding errors of a few ulps of ||T||), also
    when the top of the spectrum is clustered (a near-double eigenvalue of
    A^T A) or when the recurrence stops early."""
    rng = np.random.default_rng(n + len(kind))
    if kind == "gaussian":
        a = gaussian_sym(n, seed=n + 3)
    elif kind == "clustered_top":
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = rng.uniform(-1.0, 1.0, n)
        lam[:3] = [2.0, -2.0 + 1e-9, 2.0 - 1e-9]
        a = (q * lam) @ q.T
        a = 0.5 * (a + a.T)
    else:
        u, v = rng.standard_normal(n), rng.standard_normal(n)
        a = np.outer(u, u) - 0.5 * np.outer(v, v)
    got = psd.lanczos_details(to_dev(a), 20, 1e-10)
    m = got["nb_iter"]
    assert m >= 1
    al = np.array(got["alpha"][:m])
    be = np.array(got["beta"][:m])
    t = np.diag(al) + np.diag(be[: m - 1], 1) + np.diag(be[: m - 1], -1)
    want = np.linalg.eigvalsh(t)[-1]
    tnorm = np.abs(t).sum(axis=1).max()
    assert abs(got["theta"] - want) <= 32 * np.finfo(float).eps * tnorm


def test_long_recurrence_tridiagonal_in_global_scratch(psd):
    """max_iter = 800: the tridiagonal solver's staged T and LU no longer fit
    its shared-memory allotment and live in the Lanczos state instead; theta
    still matches LAPACK on the returned coefficients and the bound brackets
    the two-norm."""
    n = 1000
    a = gaussian_sym(n, seed=17)
    got = psd.lanczos_details(to_dev(a), 800, 1e-10)
    m = got["nb_iter"]
    assert m > 760
    al = np.array(got["alpha"][:m])
    be = np.array(got["beta"][:m])
    t = np.diag(al) + np.diag(be[: m - 1], 1) + np.diag(be[: m - 1], -1)
    want = np.linalg.eigvalsh(t)[-1]
    tnorm = np.abs(t).sum(axis=1).max()
    assert abs(got["theta"] - want) <= 64 * np.finfo(float).eps * tnorm
    sigma = np.linalg.norm(a, 2)
    assert got["lo"] <= sigma * (1 + 1e-5) and got["up"] >= sigma * (1 - 1e-6)
