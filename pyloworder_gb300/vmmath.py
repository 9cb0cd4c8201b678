"""pyLOM.math (pyLOM/vmmath) hot-path functions on GB300.

Same names, argument meanings, defaults and return tuples as pyLOM 3.2.8's
``pyLOM.math``; inputs may be numpy arrays or torch tensors and results come
back as the same kind (numpy in -> numpy out, CUDA tensor in -> CUDA tensor
out).  One extra keyword-only argument, ``precision``:

* ``'fp64'``  -- every product and reduction in FP64 on the GPU (default for
  float64 / complex128 input);
* ``'mixed'`` -- tall-skinny products on the tensor cores (each FP32 operand
  packed as an fp16 hi/lo pair with a power-of-two column scale, three f16
  products per tile, FP32 accumulation drained to FP64 or double-float
  partials), n x n factorizations in FP64 (default for float32 / complex64
  input, whose reference path runs in single precision).
"""
from __future__ import annotations

import time

import numpy as np

from . import _lib as L

__all__ = [
    "temporal_mean", "subtract_mean", "temporal_variance", "norm_variance",
    "matmul", "matmulp", "vecmat", "transpose", "tsqr", "tsqr_svd", "randomized_svd",
    "randomized_qr", "randomized_qr2", "qr", "svd", "init_qr_streaming", "update_qr_streaming", "compute_truncation_residual",
    "energy", "hammwin", "RMSE",
]


# --------------------------------------------------------------------------
# averaging: pyLOM/vmmath/averaging.py:18-75, src/averaging.c:10-157
# --------------------------------------------------------------------------

def _rows_in(X):
    cv = L.to_device(X)
    x, ld = L.as_rows(cv.t)
    if x.dim() != 2:
        raise ValueError("expected a 2-D snapshot matrix (points x snapshots)")
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("averaging takes float32 or float64 data")
    return cv, x, ld


def temporal_mean(X):
    """Mean over snapshots of each point (pyLOM/vmmath/averaging.py:18)."""
    cv, x, ld = _rows_in(X)
    t = L.torch()
    m, n = x.shape
    out = t.empty(m, dtype=x.dtype, device="cuda")
    L.call("plom_temporal_mean", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(out), L.stream_ptr())
    return cv.back(out)


def subtract_mean(X, X_mean):
    """X - mean over columns (pyLOM/vmmath/averaging.py:32)."""
    cv, x, ld = _rows_in(X)
    t = L.torch()
    m, n = x.shape
    mean = L.to_device(X_mean, x.dtype).t.contiguous().reshape(-1)
    Y = t.empty((m, n), dtype=x.dtype, device="cuda")
    L.call("plom_subtract_mean", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(mean), L.ptr(Y), n,
           L.stream_ptr())
    return cv.back(Y)


def temporal_variance(X, X_mean):
    """Population variance over snapshots, shape (m, 1) (averaging.py:47)."""
    cv, x, ld = _rows_in(X)
    t = L.torch()
    m, n = x.shape
    mean = L.to_device(X_mean, x.dtype).t.contiguous().reshape(-1)
    var = t.empty((m, 1), dtype=x.dtype, device="cuda")
    L.call("plom_temporal_variance", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(mean), L.ptr(var),
           L.stream_ptr())
    return cv.back(var)


def norm_variance(X, X_mean, X_var):
    """(X - mean) / variance (pyLOM/vmmath/averaging.py:62)."""
    cv, x, ld = _rows_in(X)
    t = L.torch()
    m, n = x.shape
    mean = L.to_device(X_mean, x.dtype).t.contiguous().reshape(-1)
    var = L.to_device(X_var, x.dtype).t.contiguous().reshape(-1)
    Y = t.empty((m, n), dtype=x.dtype, device="cuda")
    L.call("plom_norm_variance", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(mean), L.ptr(var),
           L.ptr(Y), n, L.stream_ptr())
    return cv.back(Y)


def temporal_mean_device(x, ld):
    """Mean over snapshots of each point of a CUDA tensor (rows ld apart)."""
    t = L.torch()
    m, n = x.shape
    out = t.empty(m, dtype=x.dtype, device="cuda")
    L.call("plom_temporal_mean", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(out), L.stream_ptr())
    return out


def remove_mean_device(x, ld, divide_variance=False):
    """Fused mean (+variance) and subtraction on a CUDA tensor: returns
    (Y, mean, var-or-None), all on the device."""
    t = L.torch()
    m, n = x.shape
    Y = t.empty((m, n), dtype=x.dtype, device="cuda")
    mean = t.empty(m, dtype=x.dtype, device="cuda")
    var = t.empty(m, dtype=x.dtype, device="cuda") if divide_variance else None
    L.call("plom_remove_mean", L.dtype_code(x), L.ptr(x), m, n, ld, L.ptr(mean), L.ptr(var),
           1 if divide_variance else 0, L.ptr(Y), n, L.stream_ptr())
    return Y, mean, var


# --------------------------------------------------------------------------
# products: pyLOM/vmmath/maths.py:77-130, src/vector_matrix.c:158-356
# --------------------------------------------------------------------------

def _operand(A):
    """-> (Converted, base tensor, ld, transposed?) for a 2-D operand that is
    row-major or the transpose of a row-major matrix."""
    t = L.torch()
    if isinstance(A, t.Tensor):
        x = A if A.device.type == "cuda" else A.to("cuda")
        cv = L.Converted(x, "torch", A.device)
        if x.dim() == 2 and x.shape[0] > 1 and x.shape[1] > 1 and x.stride(0) == 1 \
                and x.stride(1) >= x.shape[0]:
            return cv, x.t(), x.stride(1), True
        xx, ld = L.as_rows(x)
        return cv, xx, ld, False
    arr = np.asarray(A)
    if arr.ndim == 2 and not arr.flags.c_contiguous and arr.flags.f_contiguous and arr.shape[0] > 1:
        base = L.torch().from_numpy(np.ascontiguousarray(arr.T)).to("cuda")
        return L.Converted(base, "numpy", None), base, base.shape[1], True
    cv = L.to_device(arr)
    xx, ld = L.as_rows(cv.t)
    return cv, xx, ld, False


def _matmul_dev(a, lda, transA, b, ldb, m, n, k, precision=None, out=None, ldc=None):
    t = L.torch()
    prec = L.precision_code(precision, a)
    dt = L.dtype_code(a)
    C = out if out is not None else t.empty((m, n), dtype=a.dtype, device="cuda")
    ldc = ldc if ldc is not None else n
    nbytes = L.load().plom_matmul_workspace(dt, prec, transA, m, n, k)
    ws = L.workspace(nbytes)
    L.call("plom_matmul", dt, prec, transA, L.ptr(a), lda, L.ptr(b), ldb, L.ptr(C), ldc, m, n, k,
           L.ptr(ws), ws.numel(), L.stream_ptr())
    return C


def matmul(A, B, *, precision=None):
    """C = A @ B (pyLOM/vmmath/maths.py:77).  A may be the transpose of a
    row-major matrix (the ``A.T`` operands of pyLOM's matmulp calls); that
    form runs as a split-K reduction over A's long axis."""
    cva, a, lda, ta = _operand(A)
    cvb, b, ldb, tb = _operand(B)
    if tb:
        b = b.t().contiguous()
        ldb = b.shape[1]
    if b.dtype != a.dtype:
        b = b.to(a.dtype)
    m = a.shape[1] if ta else a.shape[0]
    k = a.shape[0] if ta else a.shape[1]
    if b.shape[0] != k:
        raise ValueError(f"matmul: shapes {tuple(A.shape)} and {tuple(B.shape)} do not align")
    n = b.shape[1]
    C = _matmul_dev(a, lda, 1 if ta else 0, b, ldb, m, n, k, precision)
    return cva.back(C)


def matmulp(A, B, *, precision=None):
    """Sum over ranks of A_i @ B_i; on one GPU the local product
    (pyLOM/vmmath/maths.py:93)."""
    return matmul(A, B, precision=precision)


def vecmat(v, A):
    """C[i,:] = v[i] * A[i,:] (pyLOM/vmmath/maths.py:113)."""
    t = L.torch()
    if isinstance(A, t.Tensor):
        vv = v if isinstance(v, t.Tensor) else t.as_tensor(np.asarray(v), device=A.device)
        return vv.to(A.dtype).reshape(-1, 1) * A
    return np.asarray(v).reshape(-1, 1) * np.asarray(A)


def transpose(A):
    """pyLOM/vmmath/maths.py:18."""
    return A.T


# --------------------------------------------------------------------------
# SVD family: pyLOM/vmmath/svd.py, src/svd.c
# --------------------------------------------------------------------------

def tsqr_svd_device(x, ld, precision=None, info_out=None):
    """TSQR-SVD of a CUDA tensor -> (U, S, V) CUDA tensors (V = V^T, n x n).
    With `info_out` (a list) the status words are appended to it unchecked
    instead of being read back at once, so that calls on several streams can
    overlap; the caller checks them with L.check_info afterwards."""
    t = L.torch()
    m, n = x.shape
    if m < n:
        # wide input: svd of the (tall) transpose, as LAPACK's gesdd would see it
        # x^T = Ut St Vt  ->  x = Vt^T St Ut^T (plain transposes, also for complex)
        Ut, St, Vt = tsqr_svd_device(x.transpose(0, 1).contiguous(), m, precision, info_out)
        return Vt.transpose(0, 1).contiguous(), St, Ut.transpose(0, 1).contiguous()
    dt = L.dtype_code(x)
    prec = L.precision_code(precision, x)
    U = t.empty((m, n), dtype=x.dtype, device="cuda")
    S = t.empty(n, dtype=L.real_dtype(x), device="cuda")
    V = t.empty((n, n), dtype=x.dtype, device="cuda")
    ws = L.workspace(L.load().plom_tsqr_svd_workspace(dt, prec, m, n))
    info = L.new_info()
    L.call("plom_tsqr_svd", dt, prec, L.ptr(x), m, n, ld, L.ptr(U), n, L.ptr(S), L.ptr(V),
           L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
    if info_out is None:
        L.check_info(info, "tsqr_svd")
    else:
        info_out.append(info)
    return U, S, V


def tsqr_svd_batched_device(x3, precision=None, info_out=None):
    """TSQR-SVD of each matrix of a (batch, m, n) CUDA tensor (m >= n, unit
    inner stride, equal strides between matrices) -> U (batch, m, n), S
    (batch, n), V (batch, n, n) holding V^T.  The mixed form on float32 /
    complex64 data runs every stage as one launch over the batch."""
    t = L.torch()
    b, m, n = x3.shape
    if x3.stride(2) != 1 or (b > 1 and x3.stride(0) < m * x3.stride(1)):
        x3 = x3.contiguous()
    dt = L.dtype_code(x3)
    prec = L.precision_code(precision, x3)
    U = t.empty((b, m, n), dtype=x3.dtype, device="cuda")
    S = t.empty((b, n), dtype=L.real_dtype(x3), device="cuda")
    V = t.empty((b, n, n), dtype=x3.dtype, device="cuda")
    ws = L.workspace(L.load().plom_tsqr_svd_batched_workspace(dt, prec, b, m, n))
    info = L.new_info()
    L.call("plom_tsqr_svd_batched", dt, prec, L.ptr(x3), b, m, n, x3.stride(1),
           x3.stride(0) if b > 1 else m * x3.stride(1), L.ptr(U), n, m * n, L.ptr(S), L.ptr(V),
           L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
    if info_out is None:
        L.check_info(info, "tsqr_svd_batched")
    else:
        info_out.append(info)
    return U, S, V


def _host_rows(Ai):
    """A host matrix (numpy array or CPU torch tensor) as a row-major CPU
    tensor with unit inner stride, or None when Ai lives on the device or is
    not a 2-D m >= n matrix of a supported type."""
    t = L.torch()
    if isinstance(Ai, t.Tensor):
        if Ai.device.type != "cpu":
            return None
        x = Ai
    else:
        arr = np.asarray(Ai)
        if arr.dtype not in (np.float32, np.float64, np.complex64, np.complex128):
            return None
        x = t.from_numpy(np.ascontiguousarray(arr))
    if x.dim() != 2 or x.shape[0] < x.shape[1] or x.shape[1] < 1:
        return None
    if x.dtype not in (t.float32, t.float64, t.complex64, t.complex128):
        return None
    if L.rows_ld(x) is None:
        x = x.contiguous()
    return x


def tsqr_svd_host(x, precision=None):
    """TSQR-SVD of a host matrix in one library call (plom_tsqr_svd_host):
    X streams to the device in row chunks while the first pass runs, and U,
    S, V come back to host memory -- page-locked when X is."""
    t = L.torch()
    m, n = x.shape
    ld = L.rows_ld(x)
    dt = L.dtype_code(x)
    prec = L.precision_code(precision, x)
    pin = bool(x.is_pinned())
    U = t.empty((m, n), dtype=x.dtype, pin_memory=pin)
    S = t.empty(n, dtype=L.real_dtype(x), pin_memory=pin)
    V = t.empty((n, n), dtype=x.dtype, pin_memory=pin)
    ws = L.workspace(L.load().plom_tsqr_svd_host_workspace(dt, prec, m, n))
    info = L.new_info()
    L.call("plom_tsqr_svd_host", dt, prec, L.ptr(x), m, n, ld, L.ptr(U), n, L.ptr(S), L.ptr(V),
           L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
    L.check_info(info, "tsqr_svd")
    return U, S, V


def tsqr_svd(Ai, *, precision=None):
    """U, S, V = tsqr_svd(A): A (m x n) = U diag(S) V with U m x n, S n
    descending, V n x n holding V^T (pyLOM/vmmath/svd.py:228).  A host
    matrix goes through the host-buffer entry (copies overlapped with the
    first pass); a device tensor through the device entry."""
    L.require_cuda()
    x = _host_rows(Ai)
    if x is not None:
        U, S, V = tsqr_svd_host(x, precision)
        if isinstance(Ai, L.torch().Tensor):
            return U, S, V
        return U.numpy(), S.numpy(), V.numpy()
    cv = L.to_device(Ai)
    x, ld = L.as_rows(cv.t)
    U, S, V = tsqr_svd_device(x, ld, precision)
    return cv.back(U), cv.back(S), cv.back(V)


def svd(A, method="gesdd", *, precision=None):
    """Thin SVD (pyLOM/vmmath/svd.py:39); computed with the TSQR-SVD."""
    return tsqr_svd(A, precision=precision)


def tsqr_device(x, ld, precision=None):
    """Q, R of a tall CUDA tensor (m >= n) with Householder QR's column signs."""
    t = L.torch()
    m, n = x.shape
    if x.dtype not in (t.float32, t.float64):
        raise TypeError("tsqr takes float32 or float64 data")
    if m < n:
        raise ValueError(f"tsqr needs m >= n, got {m} x {n}")
    dt = L.dtype_code(x)
    prec = L.precision_code(precision, x)
    Q = t.empty((m, n), dtype=x.dtype, device="cuda")
    R = t.empty((n, n), dtype=x.dtype, device="cuda")
    ws = L.workspace(L.load().plom_tsqr_workspace(dt, prec, m, n))
    info = L.new_info()
    L.call("plom_tsqr", dt, prec, L.ptr(x), m, n, ld, L.ptr(Q), n, L.ptr(R), L.ptr(ws), ws.numel(),
           L.ptr(info), L.stream_ptr())
    L.check_info(info, "tsqr")
    return Q, R


def tsqr(Ai, *, precision=None):
    """Q, R = tsqr(A): Q m x n orthonormal columns, R n x n upper triangular
    (pyLOM/vmmath/svd.py:50).  On one rank pyLOM's tsqr is LAPACK's
    Householder QR (svd.py:58 then QW = I), and so are these factors: R's
    diagonal carries Householder's signs (minus the sign of each pivot)."""
    cv = L.to_device(Ai)
    x, ld = L.as_rows(cv.t)
    Q, R = tsqr_device(x, ld, precision)
    return cv.back(Q), cv.back(R)


def qr(A, *, precision=None):
    """Reduced QR of any shape, numpy.linalg.qr's factors (pyLOM/vmmath/
    svd.py:29): m >= n -> Q m x n, R n x n; m < n -> Q m x m, R m x n
    (the QR of the leading m x m block, R's trailing columns Q^T A)."""
    cv = L.to_device(A)
    x, ld = L.as_rows(cv.t)
    m, n = x.shape
    if m >= n:
        Q, R = tsqr_device(x, ld, precision)
        return cv.back(Q), cv.back(R)
    Q, R1 = tsqr_device(x[:, :m], ld, precision)
    R2 = _matmul_dev(Q, m, 1, x[:, m:], ld, m, n - m, m, precision)
    return cv.back(Q), cv.back(L.torch().cat([R1, R2], dim=1))


def randomized_svd_device(x, ld, r, q, seed, precision=None):
    t = L.torch()
    m, n = x.shape
    dt = L.dtype_code(x)
    prec = L.precision_code(precision, x)
    U = t.empty((m, r), dtype=x.dtype, device="cuda")
    S = t.empty(r, dtype=x.dtype, device="cuda")
    V = t.empty((r, n), dtype=x.dtype, device="cuda")
    ws = L.workspace(L.load().plom_randomized_svd_workspace(dt, prec, m, n, r))
    info = L.new_info()
    L.call("plom_randomized_svd", dt, prec, L.ptr(x), m, n, ld, r, q, seed, L.ptr(U), r, L.ptr(S),
           L.ptr(V), L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
    L.check_info(info, "randomized_svd")
    return U, S, V


def randomized_svd(Ai, r, q, seed=-1, *, precision=None):
    """Randomized SVD with q power iterations (pyLOM/vmmath/svd.py:255).
    Returns U m x r, S r, V r x n.  The uniform [0,1) test matrix comes from
    a Philox counter stream keyed by ``seed`` (time-seeded when seed < 0, as
    in pyLOM)."""
    seed = int(time.time()) if seed < 0 else int(seed)
    cv = L.to_device(Ai)
    x, ld = L.as_rows(cv.t)
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("randomized_svd takes float32 or float64 data")
    U, S, V = randomized_svd_device(x, ld, int(r), int(q), seed, precision)
    return cv.back(U), cv.back(S), cv.back(V)


def randomized_qr_device(x, ld, r, q, seed, omega=None, precision=None):
    """Q (m x r), B = Q^T X (r x n) of the randomized range finder on a CUDA
    tensor (plom_randomized_qr); omega: an n x r CUDA tensor of x's dtype or
    None (Philox keyed by seed)."""
    t = L.torch()
    m, n = x.shape
    dt = L.dtype_code(x)
    prec = L.precision_code(precision, x)
    Q = t.empty((m, r), dtype=x.dtype, device="cuda")
    B = t.empty((r, n), dtype=x.dtype, device="cuda")
    if omega is not None:
        omega = omega.to(device="cuda", dtype=x.dtype).contiguous()
        if tuple(omega.shape) != (n, r):
            raise ValueError(f"omega must be {n} x {r}, got {tuple(omega.shape)}")
    ws = L.workspace(L.load().plom_randomized_qr_workspace(dt, prec, m, n, r))
    info = L.new_info()
    L.call("plom_randomized_qr", dt, prec, L.ptr(x), m, n, ld, r, q, seed & (2**64 - 1),
           L.ptr(omega), L.ptr(Q), r, L.ptr(B), L.ptr(ws), ws.numel(), L.ptr(info),
           L.stream_ptr())
    L.check_info(info, "randomized_qr")
    return Q, B


def randomized_qr(Ai, r, q, seed=-1, *, omega=None, precision=None):
    """Qi (m x r), B = Qi^T A (r x n) of the randomized range finder
    (pyLOM/vmmath/svd.py:121-144): Omega uniform [0, 1) (n x r), Y = A Omega,
    q times (Q = tsqr(Y); Y = A (A^T Q)), Q = tsqr(Y), B = Q^T A.  Q carries
    Householder QR's column signs, as the reference's tsqr gives them.
    Omega: the Philox4x32-10 stream keyed by ``seed`` (time-seeded when
    seed < 0, as in pyLOM), or ``omega`` when given (e.g. the reference's own
    numpy draw, for parity)."""
    seed = int(time.time()) if seed < 0 else int(seed)
    cv = L.to_device(Ai)
    x, ld = L.as_rows(cv.t)
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("randomized_qr takes float32 or float64 data")
    om = None if omega is None else _device_like(omega, x.dtype)
    Q, B = randomized_qr_device(x, ld, int(r), int(q), seed, om, precision)
    return cv.back(Q), cv.back(B)


def randomized_qr2(Ai, r, q, seed=-1, *, omega=None, precision=None):
    """pyLOM/vmmath/svd.py:147-173: the same range finder as randomized_qr
    (pyLOM runs its products on the host and only tsqr on the GPU; here every
    step is on the GPU), the same factors."""
    return randomized_qr(Ai, r, q, seed, omega=omega, precision=precision)


# --------------------------------------------------------------------------
# streaming range finder: pyLOM/vmmath/svd.py:175-225
# --------------------------------------------------------------------------

# Philox key of the last init_qr_streaming and the number of draws made from
# it (pyLOM's update_qr_streaming keeps drawing from numpy's global stream
# after the seeded init; here every update draws from the next key)
_QR_STREAM = {"seed": 0, "draws": 0}


def _uniform_device(rows, cols, seed, dtype):
    """rows x cols uniform [0, 1) from the Philox4x32-10 stream keyed by seed."""
    t = L.torch()
    out = t.empty((rows, cols), dtype=dtype, device="cuda")
    L.call("plom_fill_uniform", L.dtype_code(out), L.ptr(out), out.numel(), int(seed) & (2**64 - 1),
           L.stream_ptr())
    return out


def _tsqr_householder(Y, precision):
    """tsqr of a tall device matrix; its factors carry Householder QR's column
    signs (computed on the device), so sums of such factors across calls (the
    streaming update's Yo += Yn) follow the reference."""
    Yr, ld = L.as_rows(Y)
    return tsqr_device(Yr, ld, precision)


def _pack_dev(x):
    """Packed copy (plom_pack) of a float32 CUDA matrix with unit inner
    stride: the mixed form's tall operand, reusable across products."""
    m, N = x.shape
    ld = L.rows_ld(x)
    if ld is None:
        x = x.contiguous()
        ld = N
    buf = L.workspace(L.load().plom_packed_bytes(m, N))
    L.call("plom_pack", L.ptr(x), m, N, ld, L.ptr(buf), buf.numel(), L.stream_ptr())
    return buf, m, N


def _packed_apply(pk, W, infos):
    """X W (m x k float32) for a packed X and an FP64 W (N x k)."""
    t = L.torch()
    buf, m, N = pk
    W = W.to(t.float64).contiguous()
    k = W.shape[1]
    C = t.empty((m, k), dtype=t.float32, device="cuda")
    ws = L.workspace(L.load().plom_packed_apply_workspace(m, N, k))
    info = L.new_info()
    L.call("plom_packed_apply", L.ptr(buf), m, N, L.ptr(W), k, k, L.ptr(C), k, L.ptr(ws), ws.numel(),
           L.ptr(info), L.stream_ptr())
    infos.append(info)
    return C


def _packed_tn(pa, pb, infos):
    """Xa^T Xb (Na x Nb, FP64) for two packed matrices with the same rows."""
    t = L.torch()
    ba, m, Na = pa
    bb, _, Nb = pb
    C = t.empty((Na, Nb), dtype=t.float64, device="cuda")
    ws = L.workspace(L.load().plom_packed_tn_workspace(m, Na, Nb))
    info = L.new_info()
    L.call("plom_packed_tn", L.ptr(ba), Na, L.ptr(bb), Nb, m, L.ptr(C), Nb, L.ptr(ws), ws.numel(),
           L.ptr(info), L.stream_ptr())
    infos.append(info)
    return C


def _range_packed(xp, om, q, precision, infos):
    """Y = A Omega and q power steps Y = A (A^T tsqr(Y)) on a packed batch."""
    Y = _packed_apply(xp, om, infos)
    for _ in range(q):
        Q, _ = _tsqr_householder(Y, precision)
        Y = _packed_apply(xp, _packed_tn(xp, _pack_dev(Q), infos), infos)
    return Y


def _device_like(A, dtype):
    t = L.torch()
    if isinstance(A, t.Tensor):
        return A.to(device="cuda", dtype=dtype)
    return t.as_tensor(np.asarray(A), dtype=dtype, device="cuda")


def init_qr_streaming(Ai, r, q, seed=None, *, omega=None, precision=None):
    """First batch of the streaming randomized range finder
    (pyLOM/vmmath/svd.py:175-193): Omega uniform [0, 1) (n x r; the Philox
    stream keyed by ``seed``, time-seeded when None, or the given ``omega``),
    Y = A Omega, q times (Q = tsqr(Y); Y = A (A^T Q)), Q = tsqr(Y),
    B = Q^T A.  Returns Q (m x r), B (r x n), Y (m x r) of the input's kind."""
    t = L.torch()
    cv = L.to_device(Ai)
    x, _ = L.as_rows(cv.t)
    if x.dtype not in (t.float32, t.float64):
        raise TypeError("init_qr_streaming takes float32 or float64 data")
    n = x.shape[1]
    r, q = int(r), int(q)
    if omega is None:
        seed = int(time.time()) if seed is None else int(seed)
        _QR_STREAM.update(seed=seed, draws=1)
        om = _uniform_device(n, r, seed, x.dtype)
    else:
        om = _device_like(omega, x.dtype)
    if x.dtype == t.float32 and L.precision_code(precision, x) == L.PREC_MIXED:
        # mixed form: the batch is packed once and read by every product
        infos = []
        xp = _pack_dev(x)
        Y = _range_packed(xp, om, q, precision, infos)
        Q, _ = _tsqr_householder(Y, precision)
        B = _packed_tn(xp, _pack_dev(Q), infos).T.to(t.float32)
        for info in infos:
            L.check_info(info, "init_qr_streaming")
        return cv.back(Q), cv.back(B.contiguous()), cv.back(Y)
    Y = matmul(x, om, precision=precision)
    for _ in range(q):
        Q, _ = _tsqr_householder(Y, precision)
        Y = matmul(x, matmul(x.T, Q, precision=precision), precision=precision)
    Q, _ = _tsqr_householder(Y, precision)
    B = matmul(Q.T, x, precision=precision)
    return cv.back(Q), cv.back(B), cv.back(Y)


def update_qr_streaming(Ai, Q1, B1, Yo, r, q, *, omega=None, seed=None, precision=None):
    """Next batch of snapshots (pyLOM/vmmath/svd.py:196-225): Yn = A Omega
    with q power steps on the batch, Yo += Yn (in place, as the reference
    does), Q2 = tsqr(Yo), B2 = [(Q2^T Q1) B1, Q2^T A].  Omega: ``omega`` if
    given, else the Philox stream keyed by ``seed``, else the next key after
    the last init_qr_streaming.  Returns Q2, B2 and Yo."""
    t = L.torch()
    cv = L.to_device(Ai)
    x, _ = L.as_rows(cv.t)
    if x.dtype not in (t.float32, t.float64):
        raise TypeError("update_qr_streaming takes float32 or float64 data")
    n = x.shape[1]
    r, q = int(r), int(q)
    if omega is None:
        if seed is None:
            seed = _QR_STREAM["seed"] * 1000003 + _QR_STREAM["draws"]
            _QR_STREAM["draws"] += 1
        om = _uniform_device(n, r, seed, x.dtype)
    else:
        om = _device_like(omega, x.dtype)
    q1 = _device_like(Q1, x.dtype)
    b1 = _device_like(B1, x.dtype)
    if x.dtype == t.float32 and L.precision_code(precision, x) == L.PREC_MIXED:
        # mixed form: the batch is packed once and read by every product
        infos = []
        xp = _pack_dev(x)
        yo = _device_like(Yo, x.dtype) + _range_packed(xp, om, q, precision, infos)
        Q2, _ = _tsqr_householder(yo, precision)
        q2p = _pack_dev(Q2)
        Q2Q1 = _packed_tn(q2p, _pack_dev(q1), infos)
        B2o = matmul(Q2Q1, b1.to(t.float64), precision="fp64").to(t.float32)
        B2n = _packed_tn(xp, q2p, infos).T.to(t.float32)
        for info in infos:
            L.check_info(info, "update_qr_streaming")
    else:
        Yn = matmul(x, om, precision=precision)
        for _ in range(q):
            Qp, _ = _tsqr_householder(Yn, precision)
            Yn = matmul(x, matmul(x.T, Qp, precision=precision), precision=precision)
        yo = _device_like(Yo, x.dtype) + Yn
        Q2, _ = _tsqr_householder(yo, precision)
        B2o = matmul(matmul(Q2.T, q1, precision=precision), b1, precision=precision)
        B2n = matmul(Q2.T, x, precision=precision)
    B2 = t.cat([B2o, B2n], dim=1)
    # Yo += Yn in the caller's array
    if isinstance(Yo, t.Tensor):
        Yo.copy_(yo.to(device=Yo.device, dtype=Yo.dtype))
    else:
        np.copyto(Yo, yo.cpu().numpy().astype(np.asarray(Yo).dtype, copy=False))
    return cv.back(Q2), cv.back(B2), Yo


# --------------------------------------------------------------------------
# host-side helpers on small vectors
# --------------------------------------------------------------------------

def _host(v):
    t = L.torch()
    if isinstance(v, t.Tensor):
        return v.detach().cpu().numpy()
    return np.asarray(v)


def compute_truncation_residual(S, r):
    """Number of modes for a residual r > 0 or an energy fraction r < 0
    (pyLOM/vmmath/truncation.py:17; the float64 C version returns ii+1 in the
    energy branch, truncation.c:69, as the py path does)."""
    S = _host(S).astype(np.float64)
    N = 0
    if r > 0:
        # suffix norms ||S[ii:]|| / ||S|| computed once
        tail = np.sqrt(np.cumsum((S * S)[::-1])[::-1])
        normS = tail[0] if tail.size else 0.0
        for ii in range(S.shape[0]):
            if tail[ii] / normS < r:
                break
            N += 1
    else:
        r = abs(r)
        normS = np.sum(S)
        acc = 0.0
        for ii in range(S.shape[0]):
            acc += S[ii] / normS
            N += 1
            if acc > r:
                break
    return N


def energy(original, rec):
    """1 - ||orig - rec||^2 / ||orig||^2 (pyLOM/vmmath/truncation.py:42)."""
    t = L.torch()
    if isinstance(original, t.Tensor):
        return float(1.0 - ((original - rec) ** 2).sum() / (original ** 2).sum())
    o, r_ = np.asarray(original), np.asarray(rec)
    return float(1.0 - np.sum((o - r_) ** 2) / np.sum(o ** 2))


def RMSE(A, B, relative=True):
    """pyLOM/vmmath/stats.py:17."""
    t = L.torch()
    if isinstance(A, t.Tensor):
        d = A - B
        den = (A * A).sum() if relative else float(np.prod(A.shape))
        return float(t.sqrt((d * d).sum() / den))
    A, B = np.asarray(A), np.asarray(B)
    d = A - B
    den = np.sum(A * A) if relative else np.prod(A.shape)
    return float(np.sqrt(np.sum(d * d) / den))


def hammwin(N):
    """Hamming window 0.54 - 0.46 cos(2 pi i / (N-1)) (pyLOM/vmmath/fft.py:17)."""
    return 0.54 - 0.46 * np.cos(2 * np.pi * np.arange(N) / (N - 1))
