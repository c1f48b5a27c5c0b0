"""The oracle pinned against the reference's own known-answer tests and bars (CPU)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import reference_port as rp

GOLDEN = Path(__file__).resolve().parent / "golden"
KAT = json.loads((GOLDEN / "kat.json").read_text())


def uniform_spectrum(n, radius=1.0, seed=0):
    """Q diag(lambda) Q^T with lambda linearly spaced in [-radius, radius]
    (test/test_utils.hpp:20-97 uses srand(1) uniform entries, a QR, and this spectrum)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.uniform(-0.5, 0.5, (n, n)))
    lam = np.linspace(-radius, radius, n)
    x = (q * lam) @ q.T
    return 0.5 * (x + x.T)


def test_kat_composite_fp32_deterministic():
    k = KAT["composite_fp32_deterministic"]
    x = np.array(k["input_over_15"]) / 15.0
    out = rp.composite_fp32(x)
    assert np.abs(out - np.array(k["expected"])).max() <= k["tolerance"]


def test_kat_simple5():
    k = KAT["composite_simple5"]
    out, _ = rp.composite_auto_scale(np.diag(k["diagonal"]))
    assert np.abs(out - np.diag(k["expected_diagonal"])).max() <= k["tolerance"]


@pytest.mark.parametrize("residual", ["reference", "exact"])
def test_kat_lanczos_two_norm(residual):
    k = KAT["lanczos_two_norm"]
    a = np.array(k["matrix"])
    r = rp.approximate_two_norm(a, k["max_iter"], k["tol"], residual=residual)
    assert r["lo"] <= k["two_norm"] + k["two_norm_rounding"]
    assert k["two_norm"] <= r["up"]
    assert abs(np.linalg.norm(a, 2) - k["two_norm"]) <= k["two_norm_rounding"]
    assert r["lo"] <= np.linalg.norm(a, 2) <= r["up"]


def test_lanczos_reference_residual_is_loose_exact_is_tight():
    a = uniform_spectrum(200, 3.0, seed=5)
    ref = rp.approximate_two_norm(a, 20, 1e-10, residual="reference")
    ex = rp.approximate_two_norm(a, 20, 1e-10, residual="exact")
    sigma = np.linalg.norm(a, 2)
    assert ref["lo"] <= sigma * (1 + 1e-12) and ex["lo"] <= sigma * (1 + 1e-12)
    assert ref["up"] >= sigma and ex["up"] >= sigma * (1 - 1e-6)
    assert ex["up"] < ref["up"]


def test_lanczos_zero_and_empty():
    z = rp.approximate_two_norm(np.zeros((6, 6)))
    assert (z["lo"], z["up"], z["nb_iter"]) == (0.0, 1.0, 0)
    e = rp.approximate_two_norm(np.zeros((0, 0)))
    assert (e["lo"], e["up"]) == (0.0, 1.0)


def test_golden_rng_and_coefficients():
    g = json.loads((GOLDEN / "rng.json").read_text())
    assert np.array_equal(rp.start_vector(8, g["seed"]), np.array(g["first8"]))
    c = json.loads((GOLDEN / "coefficients.json").read_text())
    for s in ("fp32", "fp16"):
        got = [[float(v) for v in t] for t in rp.schedule_coefficients(s)]
        assert got == c[s]
    assert len(c["fp32"]) == 10 and len(c["fp16"]) == 7


def test_golden_cases_reproduce():
    g = np.load(GOLDEN / "cases.npz")
    for n in (16, 64, 100):
        x = g[f"x_{n}"]
        proj, _ = rp.eig_psd(x)
        assert np.allclose(proj, g[f"evd_{n}"], rtol=0, atol=1e-12)
        assert np.array_equal(rp.composite_fp32(x), g[f"fp32_{n}"])


def test_bar_uniform_scaled_rel():
    """CompositeFP32.UniformScaled bar (rel <= 1e-3, test/composite_FP32_test.hpp:121), n = 1000."""
    bar = KAT["oracle_bars"]["uniform_scaled_rel"]
    x = uniform_spectrum(bar["n"], bar["radius"], seed=1)
    proj, _ = rp.eig_psd(x)
    err = rp.rel_frobenius(rp.composite_fp32(x), proj)
    assert err <= bar["rel_frobenius_max"]
    assert err <= 1e-4


def test_bar_autoscaled_abs():
    """CompositeFP32.UniformAutoScaled1024 bar (abs <= 0.1, test/composite_FP32_test.hpp:239)."""
    bar = KAT["oracle_bars"]["uniform_autoscaled_abs"]
    x = uniform_spectrum(bar["n"], bar["radius"], seed=2)
    proj, _ = rp.eig_psd(x)
    out, up = rp.composite_auto_scale(x)
    assert np.linalg.norm(out - proj) <= bar["abs_frobenius_max"]
    assert up >= np.linalg.norm(x, 2)


def test_fp16_restatement_error_level():
    x = uniform_spectrum(300, 1.0, seed=3)
    proj, _ = rp.eig_psd(x)
    assert rp.rel_frobenius(rp.composite_fp16(x), proj) <= 2e-3


@pytest.mark.parametrize("precision,schedule,bound", [
    ("fp32_simt", "fp32", 1e-5), ("fp16x3", "fp32", 2e-5), ("bf16x3", "fp32", 5e-5), ("bf16x6", "fp32", 1e-5),
    ("bf16x9", "fp32", 1e-5), ("fp16", "fp16", 3e-3),
])
def test_split_model_error_levels(precision, schedule, bound):
    """The arithmetic model of the GPU kernels reaches the stated error levels."""
    x = uniform_spectrum(160, 1.0, seed=4)
    proj, _ = rp.eig_psd(x)
    assert rp.rel_frobenius(rp.composite_split_model(x, precision, schedule), proj) <= bound


def test_split_terms_reconstruct():
    rng = np.random.default_rng(0)
    x = rng.standard_normal(1000).astype(np.float32) * 0.05
    f16 = rp.split_terms(x, "f16")
    assert np.abs((f16[0].astype(np.float64) + f16[1]) - x).max() <= 2e-7 * 0.05 * 8
    b = rp.split_terms(x, "bf16")
    assert np.abs(sum(t.astype(np.float64) for t in b) - x).max() <= np.abs(x).max() * 2.0 ** -23


def test_f16_split_keeps_22_bits_over_the_operand_range():
    """hi + lo of the FP16 operand format is within 2.5e-7 relative of the
    FP32 value for every magnitude a filter operand takes (1e-4 to 1, and up
    to 15.99), because the split works on v * 2^12: unscaled, the low term of an
    entry near 1/sqrt(8192) is an FP16 subnormal and the pair keeps about 17
    bits (relative error near 1e-5)."""
    rng = np.random.default_rng(1)
    for lo_mag, hi_mag in ((1e-4, 1e-3), (1e-3, 1e-2), (1e-2, 1e-1), (1e-1, 1.0), (1.0, 15.99)):
        v = (np.exp(rng.uniform(np.log(lo_mag), np.log(hi_mag), 100_000)) *
             rng.choice([-1.0, 1.0], 100_000)).astype(np.float32)
        t = rp.split_terms(v, "f16")
        rel = np.abs((t[0].astype(np.float64) + t[1]) - v) / np.abs(v)
        assert rel.max() <= 2.5e-7, (lo_mag, rel.max())
    # Unscaled, the same pair loses the low bits at |v| ~ 0.006 (the reason for the factor).
    v = np.full(1000, 0.006, dtype=np.float32) * rng.uniform(0.9, 1.1, 1000).astype(np.float32)
    hi = v.astype(np.float16).astype(np.float32)
    lo = (v - hi).astype(np.float16).astype(np.float32)
    assert (np.abs((hi.astype(np.float64) + lo) - v) / v).max() > 1e-6


def test_sym_upper_convention():
    x = np.arange(9.0).reshape(3, 3)
    s = rp.sym_upper(x)
    assert np.array_equal(s, s.T) and s[2, 0] == x[0, 2] and s[0, 2] == x[0, 2]


# ---- eigenpairs and deflation (oracle/deflation_port.py) ----------------------

KAT5 = np.array([[4, 1, 2, 0, 0], [1, 3, 0, 1, 0], [2, 0, 5, 1, 1], [0, 1, 1, 2, 1], [0, 0, 1, 1, 3]], dtype=float)


def test_eigenpairs_port_kat():
    """Lanczos.Eigenpairs (test/lanczos_test.hpp:44-84): the bound is at least
    the quoted two-norm 7.0890; the three pairs kept are the top eigenpairs."""
    from oracle import deflation_port as dp

    ep = dp.compute_eigenpairs(KAT5, 3)
    assert ep["upper"] >= 7.0890
    w, V = np.linalg.eigh(KAT5)
    order = np.argsort(-np.abs(w))[:3]
    assert ep["r"] == 3
    assert np.allclose(ep["values"], w[order], atol=1e-12)
    assert np.allclose(np.abs(np.sum(ep["vectors"] * V[:, order], axis=0)), 1.0, atol=1e-10)
    assert dp.compute_eigenpairs(KAT5, 0)["r"] == 0


def test_deflate_port_kats():
    """CompositeFP32.Simple5Deflate (test/composite_FP32_test.hpp:248-290; its
    positional arguments give k = 0) within 1e-3 of diag(max(d, 0)), also
    with k = 2; UniformAutoScaleDeflate1024's bar (Frobenius <= 0.1, k = 0) on
    a smaller case of the same construction."""
    from oracle import deflation_port as dp

    d = np.diag([1.0, -2.0, 3.0, -4.0, 5.0])
    for k in (0, 2):
        out = dp.composite_auto_scale_deflate(d, "fp32", k=k, tol=2.0 if k == 0 else 1e-10)
        assert np.abs(out - np.maximum(d, 0)).max() <= 1e-3
    x = uniform_spectrum(256, 10.0, seed=4)
    proj, _ = rp.eig_psd(x)
    out = dp.composite_auto_scale_deflate(x, "fp32", k=0, tol=40, ortho_tol=1e-10)
    assert np.linalg.norm(out - proj) <= 0.1
    assert rp.rel_frobenius(out, proj) <= 1e-4


A6 = np.array([[4, 1, 2, 0, 0, 0], [1, 3, 0, 1, 0, 0], [2, 0, 5, 1, 1, 0], [0, 1, 1, 2, 1, 1], [0, 0, 1, 1, 3, 2],
               [0, 0, 0, 1, 2, 4]], dtype=float)


def test_lobpcg_port_kats():
    """LOBPCG.Simple (test/lobpcg_test.hpp:10-57: 7.3191, 5.6639 within 1e-4)
    and LOBPCG.Random (:59-130: the m = n / 10 largest eigenvalues of R + R^T,
    R ~ U[0, 1], within 1e-8 of EVD), at n = 100."""
    from oracle import deflation_port as dp

    r = dp.lobpcg(A6, 2)
    assert np.allclose(r["D"], [7.3191, 5.6639], atol=1e-4)
    rng = np.random.default_rng(0)
    R = rng.random((100, 100))
    A = R + R.T
    r = dp.lobpcg(A, 10)
    assert np.abs(r["D"] - np.linalg.eigvalsh(A)[::-1][:10]).max() <= 1e-8


def test_two_ended_deflations_port():
    """CompositeFP16.Random's bar (rel <= 1e-3 against EVD, n = 100, k = n / 10)
    and the EVD deflation (exact up to LOBPCG's tolerance)."""
    from oracle import deflation_port as dp

    rng = np.random.default_rng(1)
    R = rng.random((100, 100))
    A = R + R.T
    proj, _ = rp.eig_psd(A)
    assert rp.rel_frobenius(dp.composite_fp16_auto_scale_deflate(A, k=10), proj) <= 1e-3
    x = uniform_spectrum(120, 1.0, seed=2)
    proj, _ = rp.eig_psd(x)
    assert rp.rel_frobenius(dp.eig_deflate(x, k=10), proj) <= 1e-7
