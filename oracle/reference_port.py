"""CPU restatement of the reference's factorization-free PSD projection path.

TEST INFRASTRUCTURE ONLY: this module is the checker the CUDA path is
compared against (and the timed CPU baseline of bench.py).  It is never part
of the product path.

Parity pin: the restatement reproduces every known-answer test the reference
ships for this path — CompositeFP32.Deterministic
(test/composite_FP32_test.hpp:18-78), CompositeFP32.Simple5 (:249-290, the
expectation diag(max(d, 0)) holds for any correct projection),
Lanczos.TwoNorm (test/lanczos_test.hpp:8-42) — and the reference's
oracle-comparison bars (rel. Frobenius <= 1e-3 against FP64 EVD,
test/composite_FP32_test.hpp:121; absolute <= 0.1 at lambda in [-10, 10],
:191,239), see tests/test_oracle.py.  The reference itself is a CUDA library
built on cuBLAS/cuSOLVER and cannot run on this CPU-only host, so no output
of the reference binary pins it beyond those tests.

Matrices here are mathematical (numpy) matrices; the column-major storage of
the reference and of the C ABI is handled by the callers.

Functions and the reference lines they follow:
  start_vector            src/lanczos.cu:69 (fill_random) with the seeded
                          SplitMix64 stream the CUDA path uses instead of curand
  approximate_two_norm    src/lanczos.cu:41-293
  schedule_coefficients   src/composite_FP32.cu:73-99, src/composite_FP16.cu:93-113
  composite_fp32          src/composite_FP32.cu:15-164
  composite_fp16          src/composite_FP16.cu:16-246
  composite_auto_scale    src/composite_FP32.cu:166-191 (and the FP16 twin :248-274)
  eig_psd                 src/eig_FP64_psd.cu:24-85 (LAPACK dsyevd via scipy)
  composite_split_model   the arithmetic of this library's split-precision kernels
                          (operand terms, term products, fused epilogues)
"""
from __future__ import annotations

import numpy as np

DEFAULT_SEED = 0x5EED5EED

# Quintic coefficient tables of the reference (data, kept identical).
COEFF_FP32 = [  # src/composite_FP32.cu:73-84 (also src/composite_FP32_emulated.cu:78-89)
    (8.3119043343, -23.0739115930, 16.4664144722),
    (4.1439360087, -2.9176674704, 0.5246212487),
    (4.0257813209, -2.9025002398, 0.5334261214),
    (3.5118574347, -2.5740236523, 0.5050097282),
    (2.4398158400, -1.7586675341, 0.4191290613),
    (1.9779835097, -1.3337358510, 0.3772169049),
    (1.9559726949, -1.3091355170, 0.3746734515),
    (1.9282822454, -1.2823649693, 0.3704626545),
    (1.9220135179, -1.2812524618, 0.3707011753),
    (1.8942192942, -1.2613293407, 0.3676616051),
]
COEFF_FP16 = [  # src/composite_FP16.cu:93-101
    (8.2885332412, -22.5927099246, 15.8201383114),
    (4.1666196466, -2.9679004036, 0.5307623217),
    (4.0611848147, -2.9698947955, 0.5492133813),
    (3.6678301399, -2.7561018955, 0.5421513305),
    (2.7632556383, -2.0607754898, 0.4695405857),
    (2.0527445797, -1.4345145882, 0.4070669182),
    (1.8804816691, -1.2583997294, 0.3779501813),
]


# ---------------------------------------------------------------------------
# Symmetric matrix conventions
# ---------------------------------------------------------------------------

def sym_upper(x: np.ndarray) -> np.ndarray:
    """The symmetric matrix defined by the upper triangle of x (what cuSOLVER
    syevd with CUBLAS_FILL_MODE_UPPER reads, src/eig_FP64_psd.cu:38-43)."""
    u = np.triu(x)
    return u + np.triu(x, 1).T


def colmajor_to_matrix(buf: np.ndarray, n: int) -> np.ndarray:
    """Matrix whose column-major storage is buf (length n*n)."""
    return np.asarray(buf).reshape(n, n).T


def matrix_to_colmajor(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m).T).reshape(-1)


# ---------------------------------------------------------------------------
# Lanczos bound
# ---------------------------------------------------------------------------

_MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def start_vector(n: int, seed: int = DEFAULT_SEED) -> np.ndarray:
    """Uniform (0, 1] start vector: u_i = ((h >> 11) + 1) 2^-53 with
    h = SplitMix64(seed ^ SplitMix64(i)).  The reference draws
    curand_uniform_double from a nondeterministic seed (src/utils.cu:188-214)."""
    i = np.arange(n, dtype=np.uint64)
    h = _splitmix64(np.uint64(seed) ^ _splitmix64(i))
    return ((h >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53


def _tridiag_top(alpha: np.ndarray, beta: np.ndarray):
    import scipy.linalg

    m = len(alpha)
    if m == 1:
        return float(alpha[0]), np.ones(1)
    w, v = scipy.linalg.eigh_tridiagonal(alpha, beta[: m - 1])
    return float(w[-1]), v[:, -1]


def approximate_two_norm(A: np.ndarray, max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED,
                         residual: str = "reference") -> dict:
    """src/lanczos.cu:41-293 in FP64.  A is the matrix (not its storage).

    residual="reference" reproduces r = A y - theta y (the reference copies
    ry -> w1 at :255, so ry stays A y); residual="exact" uses A^T A y - theta y."""
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    m = min(int(max_iter), n)
    out = {"lo": 0.0, "up": 1.0, "theta": 0.0, "nb_iter": 0, "alpha": np.zeros(max(m, 0)),
           "beta": np.zeros(max(m, 0))}
    if m <= 0:
        return out
    q = start_vector(n, seed)
    nq = np.linalg.norm(q)
    if nq != 0.0:
        q = q / nq
    V = np.zeros((n, m))
    V[:, 0] = q
    vold = np.zeros(n)
    alpha, beta = out["alpha"], out["beta"]
    beta_old = 0.0
    nb = 0
    for k in range(m):
        w = A.T @ (A @ q)                                     # :118-128
        alpha[k] = q @ w                                      # :131
        w = w - alpha[k] * q - beta_old * vold                # :137-138
        beta[k] = np.linalg.norm(w)                           # :141
        if beta[k] <= tol * alpha[k] and k > 1:               # :145
            break
        vold = q.copy()                                       # :149
        if beta[k] == 0.0:                                    # :152-159
            break
        q = w / beta[k]
        if k < m - 1:
            V[:, k + 1] = q                                   # :161-164
        beta_old = beta[k]
        nb += 1
    out["nb_iter"] = nb
    if nb == 0:                                               # :171-184
        return out
    theta, u = _tridiag_top(alpha[:nb], beta[:nb])            # :186-231
    y = V[:, :nb] @ u                                         # :236-242
    ry = A @ y if residual == "reference" else A.T @ (A @ y)  # :244-256
    r = ry - theta * y                                        # :258-260
    out.update(theta=theta, lo=float(np.sqrt(theta)), up=float(np.sqrt(theta + np.linalg.norm(r))))  # :262-270
    return out


# ---------------------------------------------------------------------------
# Composite filter
# ---------------------------------------------------------------------------

def schedule_coefficients(schedule: str = "fp32") -> list[tuple[np.float32, np.float32, np.float32]]:
    """Per-step (a, b, c) after the safety scaling, in FP32 arithmetic like the
    reference: s = 1.001 on steps 0-7 of the FP32 table
    (src/composite_FP32.cu:86-99), s = 1.01 on every FP16 step (src/composite_FP16.cu:103-113).
    "fp8" (this library's FP8 schedule, no reference counterpart): the FP16
    table with s = 1.5 on every step."""
    f = np.float32
    out = []
    if schedule in ("fp16", "fp8"):
        s = f(1.5) if schedule == "fp8" else f(1.01)
        for a, b, c in COEFF_FP16:
            a, b, c = f(a), f(b), f(c)
            out.append((f(a / s), f(b / (s * s * s)), f(c / (s * s * s * s * s))))
    else:
        s = f(1.001)
        for i, (a, b, c) in enumerate(COEFF_FP32):
            a, b, c = f(a), f(b), f(c)
            if i < 8:
                a, b, c = f(a / s), f(b / (s * s * s)), f(c / (s * s * s * s * s))
            out.append((a, b, c))
    return out


def _sym32(m: np.ndarray) -> np.ndarray:
    """symmetrizeFloat, src/utils.cu:7-32: (M + M^T) * 0.5 in FP32."""
    return ((m + m.T) * np.float32(0.5)).astype(np.float32)


def composite_fp32(X: np.ndarray) -> np.ndarray:
    """composite_FP32 (src/composite_FP32.cu:15-164) in FP32; X spectrum in [-1, 1]."""
    f = np.float32
    A = np.asarray(X, dtype=np.float64).astype(np.float32)
    for a, b, c in schedule_coefficients("fp32"):
        A2 = A @ A                                            # :103
        A3 = A2 @ A                                           # :106
        A = (f(a) * A).astype(np.float32)                     # :109
        A = (f(b) * A3 + A).astype(np.float32)                # :111
        A = (f(c) * (A3 @ A2) + A).astype(np.float32)         # :115
        A = _sym32(A)                                         # :118
    n = A.shape[0]
    A = (A + np.eye(n, dtype=np.float32)).astype(np.float32)  # :143
    A = (f(0.5) * A).astype(np.float32)                       # :145
    W = np.asarray(X, dtype=np.float64).astype(np.float32) @ A  # :149-150
    return _sym32(W).astype(np.float64)                       # :153-156


def composite_fp16(X: np.ndarray) -> np.ndarray:
    """composite_FP16 (src/composite_FP16.cu:16-246): FP16 operands, FP32 accumulate."""
    f = np.float32

    def h(m):
        return m.astype(np.float16).astype(np.float32)

    A = np.asarray(X, dtype=np.float64).astype(np.float32)
    for a, b, c in schedule_coefficients("fp16"):
        hA = h(A)
        A2 = hA @ hA                                          # :117-127
        hA2 = h(A2)
        A3 = hA @ hA2                                         # :130-140
        A = (f(a) * A).astype(np.float32)                     # :143
        A = (f(b) * A3 + A).astype(np.float32)                # :145
        A = (f(c) * (hA2 @ h(A3)) + A).astype(np.float32)     # :153-163
        A = _sym32(A)                                         # :166
    n = A.shape[0]
    A = (f(0.5) * (A + np.eye(n, dtype=np.float32))).astype(np.float32)  # :210-212
    W = h(np.asarray(X, dtype=np.float64).astype(np.float32)) @ h(A)      # :215-227
    return _sym32(W).astype(np.float64)                       # :230-233


def composite_auto_scale(X: np.ndarray, method: str = "fp32", max_iter: int = 20, tol: float = 1e-10,
                         seed: int = DEFAULT_SEED, residual: str = "reference") -> tuple[np.ndarray, float]:
    """composite_*_auto_scale (src/composite_FP32.cu:166-191): Lanczos bound,
    X / up, filter, times up.  Returns (projection, up)."""
    X = np.asarray(X, dtype=np.float64)
    up = approximate_two_norm(X, max_iter, tol, seed, residual)["up"]
    scale = up if up > 0.0 else 1.0                           # :182
    Xs = X * (1.0 / scale)                                    # :183-184
    fn = composite_fp16 if method == "fp16" else composite_fp32
    return fn(Xs) * scale, scale                              # :187-190


# ---------------------------------------------------------------------------
# FP64 EVD projection (the ground truth)
# ---------------------------------------------------------------------------

def eig_psd(X: np.ndarray, upper: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """V max(L, 0) V^T by LAPACK dsyevd (scipy 'evd' driver): the math of
    eig_FP64_psd (src/eig_FP64_psd.cu:24-85).  Returns (projection, eigenvalues ascending)."""
    import scipy.linalg

    S = sym_upper(np.asarray(X, dtype=np.float64)) if upper else np.asarray(X, dtype=np.float64)
    w, V = scipy.linalg.eigh(S, driver="evd")
    return (V * np.maximum(w, 0.0)) @ V.T, w


def rel_frobenius(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    return float(d / nb) if nb > 0 else float(d)


# ---------------------------------------------------------------------------
# Model of this library's split-precision arithmetic
# ---------------------------------------------------------------------------

PRECISION_MODEL = {
    # name: (format, number of terms stored, term products)
    "fp32_simt": ("f32", 1, [(0, 0)]),
    "fp16": ("f16", 2, [(0, 0)]),
    "bf16": ("bf16", 3, [(0, 0)]),
    "fp16x3": ("f16", 2, [(0, 0), (0, 1), (1, 0)]),
    "bf16x3": ("bf16", 3, [(0, 0), (0, 1), (1, 0)]),
    "bf16x6": ("bf16", 3, [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (1, 1)]),
    "bf16x9": ("bf16", 3, [(i, j) for i in range(3) for j in range(3)]),
    # FP8: the products read an E4M3 copy (term index 2 of the "f16q8" format),
    # the stored value is the FP16 pair.
    "fp8": ("f16q8", 3, [(2, 2)]),
}


# Factor of the FP16 operand terms (psd_projection_gb300/csrc/common.cuh, kF16Scale).
F16_SCALE = np.float32(4096.0)
# Factor of the E4M3 plane (common.cuh, kE4M3Scale).
E4M3_SCALE = np.float32(128.0)


def to_e4m3(x: np.ndarray) -> np.ndarray:
    """Round FP32 to FP8 E4M3 (OCP: 4 exponent bits, bias 7, 3 mantissa bits,
    subnormals below 2^-6, largest finite 448; round to nearest even,
    saturating at +-448), returned as FP32."""
    x = np.asarray(x, dtype=np.float64)
    a = np.abs(x)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    e = np.maximum(e, -6.0)                      # subnormal spacing 2^-9 below 2^-6
    q = 2.0 ** (e - 3.0)                         # spacing of the 3-bit significand at exponent e
    r = np.round(a / q) * q                      # numpy rounds halves to even
    r = np.minimum(r, 448.0)
    return (np.sign(x) * r).astype(np.float32)


def _to_bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to BF16 (round to nearest even), returned as FP32."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + np.uint64(0x7FFF) + ((u >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)) << np.uint64(16)
    return (r & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32)


def split_terms(x32: np.ndarray, fmt: str) -> list[np.ndarray]:
    """Operand terms (FP32 arrays) of an FP32 matrix in a storage format."""
    x32 = np.asarray(x32, dtype=np.float32)
    if fmt == "f32":
        return [x32]
    if fmt == "f16q8":
        hi, lo = split_terms(x32, "f16")
        q = (to_e4m3((x32 * E4M3_SCALE).astype(np.float32)) / E4M3_SCALE).astype(np.float32)
        return [hi, lo, q]
    if fmt == "f16":
        # The kernels split v * 2^12 (F16_SCALE) so that the low term stays a
        # normal FP16 number, and take the factor out of every product and
        # load; both scalings are exact, so the terms are returned unscaled.
        xs = (x32 * F16_SCALE).astype(np.float32)
        hi = xs.astype(np.float16).astype(np.float32)
        lo = (xs - hi).astype(np.float16).astype(np.float32)
        return [(hi / F16_SCALE).astype(np.float32), (lo / F16_SCALE).astype(np.float32)]
    b0 = _to_bf16(x32)
    r1 = (x32 - b0).astype(np.float32)
    b1 = _to_bf16(r1)
    b2 = _to_bf16((r1 - b1).astype(np.float32))
    return [b0, b1, b2]


def _stored(terms: list[np.ndarray], fmt: str = "") -> np.ndarray:
    if fmt == "f16q8":
        terms = terms[:2]  # the stored value is the FP16 pair
    s = np.zeros_like(terms[0], dtype=np.float32)
    for t in reversed(terms):
        s = (s + t).astype(np.float32)
    return s


def _product(P: list[np.ndarray], Q: list[np.ndarray], prods, dual: bool = False) -> np.ndarray:
    """Symmetric product as the kernels form it: the lower triangle of
    sum_ab P_a Q_b mirrored (one triangle computed, stored twice), or for a
    dual product the symmetric part (PQ + QP)/2."""
    acc = np.zeros(P[0].shape, dtype=np.float64)
    for a, b in prods:
        acc += P[a].astype(np.float64) @ Q[b].astype(np.float64)
    acc = acc.astype(np.float32)
    if dual:
        return ((acc.astype(np.float64) + acc.T) * 0.5).astype(np.float32)
    return np.tril(acc) + np.tril(acc, -1).T


def composite_split_model(X: np.ndarray, precision: str = "fp16x3", schedule: str = "fp32",
                          up: float = 1.0) -> np.ndarray:
    """What this library's kernels compute for composite on X with scale up:
    operands split into terms, products summed over the precision's term
    pairs (accumulated here in FP64, on the GPU in FP32; one-term modes take
    the symmetric parts of the second and third products of each step), the step combination
    a*A + b*A3 + c*A3*A2 in FP32 on the stored values, and the final
    0.5 * (X + up * (Xs*A + A*Xs)/2) in FP64."""
    fmt, _, prods = PRECISION_MODEL[precision]
    one_term = len(prods) == 1 and fmt != "f32"
    X = sym_upper(np.asarray(X, dtype=np.float64))
    Xs32 = (X * (1.0 / up)).astype(np.float32)
    A_t = split_terms(Xs32, fmt)
    for a, b, c in schedule_coefficients(schedule):
        A2_t = split_terms(_product(A_t, A_t, prods), fmt)
        A3_t = split_terms(_product(A2_t, A_t, prods, dual=one_term), fmt)  # one-term modes: symmetric parts
        acc = _product(A3_t, A2_t, prods, dual=one_term)
        A_new = np.float32(c) * acc + (np.float32(b) * _stored(A3_t, fmt) + np.float32(a) * _stored(A_t, fmt))
        A_t = split_terms(A_new.astype(np.float32), fmt)
    PA = _product(split_terms(Xs32, fmt), A_t, prods, dual=True).astype(np.float64)
    out = 0.5 * (X + up * PA)   # symmetric part of Xs*A, one dual product on the GPU
    return sym_upper(out)
