"""CPU restatement of the reference's eigenpair and deflation routines.

TEST INFRASTRUCTURE ONLY: this module is the checker the CUDA path is
compared against; it is never part of the product path.

Parity pin: the reference's own tests for these routines are
Lanczos.Eigenpairs (test/lanczos_test.hpp:44-84: the returned bound is at
least the two-norm 7.0890 of its 5 x 5 matrix), CompositeFP32.Simple5Deflate
and UniformAutoScaleDeflate1024 (test/composite_FP32_test.hpp:248-333, which
by their positional arguments run with k = 0), LOBPCG.Simple / Random
(test/lobpcg_test.hpp: the two largest eigenvalues 7.3191, 5.6639 of a 6 x 6
matrix; the m = n / 10 largest of (R + R^T), R ~ U[0, 1], within 1e-8 of
EVD) and CompositeFP16.UniformAutoScaleDeflate1024 / Random
(test/composite_FP16_test.hpp: rel. Frobenius <= 5e-3 / 1e-3 against EVD).
tests/test_oracle.py checks this module against each of them.  The
reference is a CUDA library and cannot run on this CPU-only host.

Functions and the reference lines they follow:
  compute_eigenpairs        src/lanczos.cu:319-547 (plain Lanczos on A with the
                            basis kept, cuSOLVER syevd of T, residual filter
                            |beta_m Z[0, j]| < ortho_tol, ghost-orthogonality
                            filter, bound |theta_max| + res + 1e-3)
  rank_update               the cublasDger loops of the deflation routines
  composite_auto_scale_deflate
                            src/composite_FP32.cu:193-254 and
                            src/composite_FP32_emulated.cu:264-325
  lobpcg                    src/lobpcg.cu:12-255
  eig_deflate               src/eig_FP64_psd.cu:87-177
  composite_fp16_auto_scale_deflate
                            src/composite_FP16.cu:276-380
"""
from __future__ import annotations

import numpy as np

from oracle import reference_port as rp

EPS = np.finfo(np.float64).eps


def _lanczos_plain(A: np.ndarray, max_iter: int, seed: int):
    """src/lanczos.cu:340-394: Lanczos on A, basis Q kept, no
    reorthogonalisation, stop when beta <= machine epsilon (after storing it)."""
    n = A.shape[0]
    q = rp.start_vector(n, seed)
    nq = np.linalg.norm(q)
    if nq != 0.0:
        q = q / nq
    Q = np.zeros((n, max_iter + 1))
    Q[:, 0] = q
    alpha, beta = [], []
    b_prev = 0.0
    for m in range(max_iter):
        w = A @ Q[:, m]                                       # :361-364
        if m > 0:
            w = w - b_prev * Q[:, m - 1]                      # :367
        a = Q[:, m] @ w                                       # :370
        alpha.append(a)
        w = w - a * Q[:, m]                                   # :375
        b = np.linalg.norm(w)                                 # :378
        beta.append(b)
        b_prev = b
        if b <= EPS:                                          # :382-383
            break
        Q[:, m + 1] = w * (1.0 / b)                           # :386-388
    return Q, np.array(alpha), np.array(beta)


def compute_eigenpairs(A: np.ndarray, k: int, upper_bound_only: bool = False, max_iter: int = 0,
                       tol: float = 1e-10, ortho_tol: float = 1e-5, seed: int = rp.DEFAULT_SEED) -> dict:
    """src/lanczos.cu:319-547.  Returns {upper, r, values, vectors (n x r),
    alpha, beta, nb_iter}.  As in the reference, `tol` is not used (the
    residual filter compares with ortho_tol, :454) and the residual of Ritz
    pair j is |beta_m Z[0, j]| with Z's first row (:295-300).  k = 0 selects
    no pair (the reference's count test after the increment, :490-495, never
    stops at 0 and writes past its k-sized outputs)."""
    import scipy.linalg

    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    if max_iter == 0:
        max_iter = n                                          # :330-331
    Q, alpha, beta = _lanczos_plain(A, int(max_iter), seed)
    nb = len(alpha)
    T = np.diag(alpha) + np.diag(beta[: nb - 1], 1) + np.diag(beta[: nb - 1], -1)
    theta, Z = scipy.linalg.eigh(T, driver="evd")             # :418-422, ascending
    beta_m = beta[-1]
    res = np.abs(beta_m * Z[0, :])                            # :295-300, :427
    idx = sorted(range(nb), key=lambda i: -abs(theta[i]))     # :436-438
    out = {"alpha": alpha, "beta": beta, "nb_iter": nb, "r": None, "values": None, "vectors": None}
    if not upper_bound_only:
        sel_vals, basis = [], []
        for j in (idx if k > 0 else []):
            if not res[j] < ortho_tol:                        # :454
                continue
            x = Q[:, :nb] @ Z[:, j]                           # :457-459
            accept = all(abs(b @ x) <= ortho_tol for b in basis)  # :460-482
            if accept:
                basis.append(x)
                sel_vals.append(theta[j])
                if len(basis) == k:
                    break
        out["r"] = len(basis)
        out["values"] = np.array(sel_vals)
        out["vectors"] = np.array(basis).T.reshape(n, len(basis))
    i0 = idx[0]
    out["upper"] = float(abs(theta[i0]) + res[i0] + 1e-3)     # :509-517, :546
    return out


def rank_update(X: np.ndarray, coef, V: np.ndarray) -> np.ndarray:
    """X + sum_i coef_i v_i v_i^T (the cublasDger loops)."""
    return X + (V * np.asarray(coef, dtype=np.float64)) @ V.T


def composite_auto_scale_deflate(X: np.ndarray, method: str = "fp32", k: int = 40, tol: float = 1e-10,
                                 ortho_tol: float = 1e-3, seed: int = rp.DEFAULT_SEED) -> np.ndarray:
    """src/composite_FP32.cu:193-254: deflate the k largest-|lambda| Ritz pairs,
    bound the rest (100 Lanczos steps), scale by 1.1 up + 1e-5, filter, scale
    back, add the positive deflated pairs back."""
    X = rp.sym_upper(np.asarray(X, dtype=np.float64))
    ep = compute_eigenpairs(X, k, False, 0, tol, ortho_tol, seed)
    vals, V = ep["values"], ep["vectors"]
    Xd = rank_update(X, -vals, V)                             # :221-226
    up = compute_eigenpairs(Xd, 0, True, 100, 1e-10, 1e-5, seed + 1)["upper"]  # :229-231
    scale = 1.1 * up + 1e-5 if up > 0.0 else 1.0              # :234
    fn = rp.composite_fp16 if method == "fp16" else rp.composite_fp32
    P = fn(Xd * (1.0 / scale)) * scale                        # :236-243
    return rank_update(P, np.maximum(vals, 0.0), V)           # :245-252


def random_block(n: int, m: int, seed: int) -> np.ndarray:
    """n x m block, column-major fill of the seeded uniform stream (the
    reference fills with curand from seed 0, src/lobpcg.cu:93)."""
    return rp.start_vector(n * m, seed).reshape(m, n).T.copy()


def lobpcg(A: np.ndarray, m: int, warmstart_V=None, warmstart_D=None, maxiter: int = 100, tol: float = 1e-8,
           seed: int = 0) -> dict:
    """src/lobpcg.cu:12-255: block Rayleigh-Ritz on span[X, R, Delta] (QR of
    the n x 3m block), the m largest Ritz pairs kept.  The first Rayleigh-Ritz
    keeps its eigenvectors in ascending order while the values are reversed
    (:121-127), as the reference does; the product X = Q T is formed out of
    place (the reference's cublasDgemm writes over its own input, :125-127).
    Returns {V (n x m), D (m,), iters}."""
    import scipy.linalg

    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    assert 0 < m and 3 * m <= n
    if warmstart_V is not None:
        X, lam = np.array(warmstart_V, dtype=np.float64), np.array(warmstart_D, dtype=np.float64)
    else:
        X, _ = np.linalg.qr(random_block(n, m, seed))                 # :89-100
    T = X.T @ A @ X                                                   # :104-111
    T = 0.5 * (T + T.T)                                               # :115-119
    lt, Z = scipy.linalg.eigh(T, driver="evd")                        # :123-124
    lam = lt[::-1].copy()                                             # :126
    X = X @ Z                                                         # :129-131 (ascending order)
    D = X.copy()                                                      # :134
    iters = 0
    for it in range(1, maxiter + 1):
        R = A @ X - X * lam                                           # :138-152
        iters = it
        if np.linalg.norm(R) < tol:                                   # :154-163
            break
        Q, _ = np.linalg.qr(np.hstack([X, R, D]))                     # :166-172
        T = Q.T @ A @ Q                                               # :174-182
        T = 0.5 * (T + T.T)                                           # :186-190
        la, Z = scipy.linalg.eigh(T, driver="evd")                    # :194-195
        Z = Z[:, ::-1]                                                # :197
        Xn = Q @ Z[:, :m]                                             # :200-202, :209-211
        D = Xn - X                                                    # :205-214
        X = Xn
        lam = la[::-1][:m].copy()                                     # :217-218
    return {"V": X, "D": lam, "iters": iters}


def _deflate_both_ends(X: np.ndarray, k: int, maxiter: int, tol: float, seed: int):
    """The two LOBPCG runs and subtractions of src/eig_FP64_psd.cu:104-150."""
    top = lobpcg(X, k, maxiter=maxiter, tol=tol, seed=seed)
    X = rank_update(X, -top["D"], top["V"])                            # :113-122
    bot = lobpcg(-X, k, maxiter=maxiter, tol=tol, seed=seed)          # :125-131
    X = rank_update(X, bot["D"], bot["V"])                            # :135-145 (values of -X)
    return X, top, bot


def _add_back(X: np.ndarray, top: dict, bot: dict) -> np.ndarray:
    """src/eig_FP64_psd.cu:154-170: the positive parts of both deflated ends."""
    X = rank_update(X, np.maximum(top["D"], 0.0), top["V"])
    return rank_update(X, np.maximum(-bot["D"], 0.0), bot["V"])


def eig_deflate(X: np.ndarray, k: int = 40, maxiter: int = 100, tol: float = 1e-10, seed: int = 0) -> np.ndarray:
    """src/eig_FP64_psd.cu:87-177: deflate the k largest and k smallest
    eigenpairs (LOBPCG), EVD-project the rest, add back the positive pairs."""
    X = rp.sym_upper(np.asarray(X, dtype=np.float64))
    Xd, top, bot = _deflate_both_ends(X, k, maxiter, tol, seed)
    P, _ = rp.eig_psd(Xd)                                             # :150
    return _add_back(P, top, bot)


def composite_fp16_auto_scale_deflate(X: np.ndarray, k: int = 40, maxiter: int = 100, tol: float = 1e-10,
                                      seed: int = 0, method: str = "fp16") -> np.ndarray:
    """src/composite_FP16.cu:276-380: the same two-ended deflation, then the
    Lanczos bound (20 steps), scaling by 1.1 up + 1e-5, the FP16 composite
    filter, scaling back, and the positive pairs added back."""
    X = rp.sym_upper(np.asarray(X, dtype=np.float64))
    Xd, top, bot = _deflate_both_ends(X, k, maxiter, tol, seed)
    up = rp.approximate_two_norm(Xd)["up"]                           # :343-346
    scale = 1.1 * up + 1e-5 if up > 0.0 else 1.0                      # :349
    fn = rp.composite_fp16 if method == "fp16" else rp.composite_fp32
    P = fn(Xd * (1.0 / scale)) * scale                                # :351-358
    return _add_back(P, top, bot)
