"""pyLOM.PCA on the GB300 path.

PCA.run follows pyLOM/PCA/wrapper.py:17-38: the POD of the mean-removed (by
default also variance-normalised) snapshot matrix, returned as the
components U and the scores (diag(S) V)^T.  ``precision`` is the one
keyword-only addition (see pyloworder_gb300.vmmath).
"""
from __future__ import annotations

from . import POD
from . import vmmath as M

__all__ = ["run"]


def run(X, divide_variance: bool = True, randomized: bool = False, r: int = 1, q: int = 3,
        seed: int = -1, *, precision=None):
    """Components (points x modes) and scores (snapshots x modes) of X."""
    U, S, V = POD.run(X, remove_mean=True, divide_variance=divide_variance, randomized=randomized,
                      r=r, q=q, seed=seed, precision=precision)
    return U, M.vecmat(S, V).T
