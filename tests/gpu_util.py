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
