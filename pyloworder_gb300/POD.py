"""pyLOM.POD hot path on GB300: run / truncate / reconstruct.

Signatures, defaults and return tuples follow pyLOM/POD/wrapper.py:17-103
(pyLOM 3.2.8); ``precision`` is the one keyword-only addition (see
pyloworder_gb300.vmmath).
"""
from __future__ import annotations

import time

import numpy as np

from . import _lib as L
from . import vmmath as M

__all__ = ["run", "truncate", "reconstruct"]


def run_device(x, ld, remove_mean=True, divide_variance=False, randomized=False, r=1, q=3, seed=-1,
               precision=None):
    """POD of a CUDA tensor; returns device tensors (U, S, V)."""
    if remove_mean:
        Y, _, _ = M.remove_mean_device(x, ld, divide_variance)
        ldy = Y.shape[1]
    else:
        Y, ldy = x, ld  # read-only: the SVD never writes its input
    if randomized:
        seed = int(time.time()) if seed < 0 else int(seed)
        return M.randomized_svd_device(Y, ldy, int(r), int(q), seed, precision)
    return M.tsqr_svd_device(Y, ldy, precision)


def run(X, remove_mean: bool = True, divide_variance: bool = False, randomized: bool = False,
        r: int = 1, q: int = 3, seed: int = -1, *, precision=None):
    """POD of the snapshot matrix X (points x snapshots).  Returns the spatial
    modes U, singular values S and V (rows = temporal coefficients), as
    pyLOM/POD/wrapper.py:17-51."""
    cv = L.to_device(X)
    x, ld = L.as_rows(cv.t)
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("POD.run takes float32 or float64 data")
    U, S, V = run_device(x, ld, remove_mean, divide_variance, randomized, r, q, seed, precision)
    return cv.back(U), cv.back(S), cv.back(V)


def truncate(U, S, V, r: float = 1e-8):
    """Keep N modes: r >= 1 is the count, 0 < r < 1 a residual target, r < 0
    an energy fraction (pyLOM/POD/wrapper.py:56-82)."""
    N = int(r) if r >= 1 else M.compute_truncation_residual(S, r)
    return U[:, :N], S[:N], V[:N, :]


def reconstruct(U, S, V, *, precision=None):
    """X ~= U diag(S) V (pyLOM/POD/wrapper.py:87-103), one GEMM on the GPU."""
    return M.matmul(U, M.vecmat(S, V), precision=precision)
