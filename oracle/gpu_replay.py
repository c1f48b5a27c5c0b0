"""Replay of the reference's GPU call sequence on cuBLAS through torch.

TEST / BENCHMARK INFRASTRUCTURE ONLY (bench.py --impl reference).  The
reference library is a CUDA/cuBLAS library whose build needs its own x86
objects; this port issues the same sequence of library calls so its speed
can be measured on the GPU host:

  approximate_two_norm   src/lanczos.cu:41-293: two FP64 matvecs per step
                         (Dgemv N and T), dot, two axpys, nrm2 with a host
                         round trip per scalar, Dsyevd of the tridiagonal
  composite_FP32         src/composite_FP32.cu:15-164: per step three FP32
                         Sgemm (TF32 off), Sscal, Saxpy, Sgeam symmetrisation;
                         add identity, halve, final Sgemm, symmetrise, to FP64
"""
from __future__ import annotations

import numpy as np

from oracle.reference_port import DEFAULT_SEED, schedule_coefficients, start_vector


def approximate_two_norm(A, max_iter: int = 20, tol: float = 1e-10, seed: int = DEFAULT_SEED):
    import torch

    n = A.shape[0]
    m = min(max_iter, n)
    if m == 0:
        return 0.0, 1.0
    q = torch.from_numpy(start_vector(n, seed)).to(A.device)
    q = q / torch.linalg.vector_norm(q)
    V = torch.zeros((m, n), dtype=torch.float64, device=A.device)
    V[0] = q
    vold = torch.zeros_like(q)
    alpha, beta = [], []
    beta_old = 0.0
    nb = 0
    for k in range(m):
        w = A.T @ (A @ q)
        a = float(q @ w)                              # host round trip, like cublasDdot
        w = w - a * q - beta_old * vold
        b = float(torch.linalg.vector_norm(w))        # cublasDnrm2
        alpha.append(a)
        beta.append(b)
        if b <= tol * a and k > 1:
            break
        vold = q.clone()
        if b == 0.0:
            break
        q = w / b
        if k < m - 1:
            V[k + 1] = q
        beta_old = b
        nb += 1
    if nb == 0:
        return 0.0, 1.0
    T = torch.diag(torch.tensor(alpha[:nb], dtype=torch.float64, device=A.device))
    if nb > 1:
        off = torch.tensor(beta[: nb - 1], dtype=torch.float64, device=A.device)
        T += torch.diag(off, 1) + torch.diag(off, -1)
    ev, evec = torch.linalg.eigh(T)                   # cusolverDnDsyevd
    theta = float(ev[-1])
    y = V[:nb].T @ evec[:, -1]
    r = A @ y - theta * y                             # src/lanczos.cu:246-260
    return float(np.sqrt(theta)), float(np.sqrt(theta + float(torch.linalg.vector_norm(r))))


def composite_fp32_(mat) -> None:
    """In place on an FP64 CUDA matrix whose spectrum lies in [-1, 1]."""
    import torch

    A = mat.float()
    for a, b, c in schedule_coefficients("fp32"):
        A2 = A @ A
        A3 = A2 @ A
        A.mul_(float(a))
        A.add_(A3, alpha=float(b))
        A.addmm_(A3, A2, alpha=float(c))
        A = (A + A.T) * 0.5
    A.diagonal().add_(1.0)
    A.mul_(0.5)
    W = mat.float() @ A
    W = (W + W.T) * 0.5
    mat.copy_(W.double())


def composite_fp32_auto_scale_(mat) -> float:
    _, up = approximate_two_norm(mat)
    scale = up if up > 0.0 else 1.0
    mat.mul_(1.0 / scale)
    composite_fp32_(mat)
    mat.mul_(scale)
    return scale
