"""ctypes access to pyLOM's own compiled SVD path (oracle/_ref/libpylom_ref.so,
built by oracle/build_ref.py) -- TEST INFRASTRUCTURE.

Only tests/ and bench.py's CPU-baseline / reference legs use it: it times and
checks the reference's C functions themselves (pyLOM/vmmath/src/svd.h:12-39:
stsqr_svd, dtsqr_svd, srandomized_svd, drandomized_svd) on numpy arrays, with
the OpenBLAS thread count set explicitly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libpylom_ref.so")
_lib = None


def available():
    return os.path.exists(LIB)


def load():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError(f"{LIB} is not built (python oracle/build_ref.py <pyLowOrder>)")
        lib = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
        vp, ci = ctypes.c_void_p, ctypes.c_int
        for nm in ("stsqr_svd", "dtsqr_svd"):
            getattr(lib, nm).argtypes = [vp, vp, vp, vp, ci, ci]
            getattr(lib, nm).restype = ci
        for nm in ("srandomized_svd", "drandomized_svd"):
            getattr(lib, nm).argtypes = [vp, vp, vp, vp, ci, ci, ci, ci, ctypes.c_uint]
            getattr(lib, nm).restype = ci
        _lib = lib
    return _lib


def _blas():
    """The bundled OpenBLAS the reference build links (its thread controls)."""
    from oracle import build_ref
    ob = ctypes.CDLL(build_ref.openblas())
    ob.scipy_openblas_set_num_threads.argtypes = [ctypes.c_int]
    ob.scipy_openblas_get_num_threads.restype = ctypes.c_int
    return ob


def set_threads(n):
    _blas().scipy_openblas_set_num_threads(int(n))


def get_threads():
    return int(_blas().scipy_openblas_get_num_threads())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def tsqr_svd(A):
    """pyLOM's compiled tsqr_svd (svd.c:529 stsqr_svd / :678 dtsqr_svd) on a
    C-contiguous float32/float64 matrix: (U m x n, S n, VT n x n).  The
    reference's C works on a private copy of A (svd.pyx passes a copy)."""
    A = np.ascontiguousarray(A)
    m, n = A.shape
    if A.dtype == np.float32:
        fn = load().stsqr_svd
    elif A.dtype == np.float64:
        fn = load().dtsqr_svd
    else:
        raise TypeError("tsqr_svd: float32 or float64")
    if m * n >= 2 ** 31:
        raise ValueError("the reference's C indexes with int: m * n must stay below 2^31")
    Ai = A.copy()
    U = np.empty((m, n), A.dtype)
    S = np.empty(n, A.dtype)
    VT = np.empty((n, n), A.dtype)
    info = fn(_ptr(U), _ptr(S), _ptr(VT), _ptr(Ai), m, n)
    if info != 0:
        raise RuntimeError(f"reference tsqr_svd returned info {info}")
    return U, S, VT


def randomized_svd(A, r, q, seed):
    """pyLOM's compiled randomized_svd (svd.c:1198 / :1453): (U m x r, S r, VT r x n);
    its test matrix comes from glibc rand() after srand(seed)."""
    A = np.ascontiguousarray(A)
    m, n = A.shape
    fn = load().srandomized_svd if A.dtype == np.float32 else load().drandomized_svd
    Ai = A.copy()
    U = np.empty((m, r), A.dtype)
    S = np.empty(r, A.dtype)
    VT = np.empty((r, n), A.dtype)
    info = fn(_ptr(U), _ptr(S), _ptr(VT), _ptr(Ai), m, n, int(r), int(q), int(seed))
    if info != 0:
        raise RuntimeError(f"reference randomized_svd returned info {info}")
    return U, S, VT
