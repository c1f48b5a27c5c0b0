"""Helpers of the GPU tests: seeded inputs and column-major device transfers."""
import numpy as np


def to_dev(x):
    """Device float64 tensor holding the column-major storage of matrix x."""
    import torch

    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64).T)).cuda()


def from_dev(t):
    """Matrix whose column-major storage is the device tensor t."""
    return t.detach().cpu().numpy().T.copy()


def uniform_spectrum(n, radius=1.0, seed=0):
    """Q diag(lambda) Q^T, lambda linearly spaced in [-radius, radius]
    (the fixture of test/test_utils.hpp:20-97)."""
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.uniform(-0.5, 0.5, (n, n)))
    lam = np.linspace(-radius, radius, n)
    x = (q * lam) @ q.T
    return 0.5 * (x + x.T)


def gaussian_sym(n, seed=0):
    """(G + G^T) / 2 with G ~ N(0, 1)."""
    g = np.random.default_rng(seed).standard_normal((n, n))
    return 0.5 * (g + g.T)


def spectrum_workload_dev(n, seed=0, spectrum="uniform"):
    """X = Q diag(lambda) Q^T on the device (FP64 holding FP32 values, the
    column-major storage of a symmetric matrix is the matrix itself) and its
    exact projection P = Q diag(max(lambda, 0)) Q^T, Q from the QR of a seeded
    Gaussian.  spectrum "uniform": lambda ~ U[-1, 1]; "stress": 10 % of
    lambda in |lambda| < 1e-3, 60 % uniform in [-1, -1e-3], 30 % uniform in
    [1e-3, 10]."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    G = torch.randn((n, n), generator=g, dtype=torch.float64, device="cuda")
    Q, _ = torch.linalg.qr(G)
    del G
    g.manual_seed(seed + 1)
    u = torch.rand(n, generator=g, dtype=torch.float64, device="cuda")
    if spectrum == "uniform":
        lam = u * 2.0 - 1.0
    else:
        k1, k2 = n // 10, n // 10 + (6 * n) // 10
        lam = torch.empty_like(u)
        lam[:k1] = (u[:k1] * 2.0 - 1.0) * 1e-3
        lam[k1:k2] = -1e-3 - u[k1:k2] * (1.0 - 1e-3)
        lam[k2:] = 1e-3 + u[k2:] * (10.0 - 1e-3)
    A = (Q * lam) @ Q.T
    X = (0.5 * (A + A.T)).float().double().contiguous()
    del A
    P = (Q * lam.clamp(min=0.0)) @ Q.T
    P = (0.5 * (P + P.T)).contiguous()
    del Q
    torch.cuda.synchronize()
    return X, P
