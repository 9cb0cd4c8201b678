"""CPU oracle for the pyLOM SVD hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy, the algorithms of pyLOM 3.2.8's Python
("py") path for tsqr_svd / randomized_svd / matmul and the POD / DMD / SPOD
models built on them.  It is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline and
``--impl reference`` legs) may import it.  The product package
``pyloworder_gb300`` never imports it and has no CPU fallback.

Parity of this restatement is pinned against the reference itself: the
fixtures under ``tests/golden/`` were produced by importing pyLOM's own py path
(with single-rank stand-ins for mpi4py/h5py/nfft/matplotlib) on seeded inputs,
and ``tests/test_oracle_golden.py`` checks every function here against them.

Each function cites the reference file:line (paths inside the pyLowOrder
project) whose behaviour it restates.  The dense kernels underneath (Householder
QR, SVD, eig, Cholesky, FFT) are LAPACK/FFT library calls in the reference too
(numpy.linalg / scipy.fft here, the same libraries the py path calls).
"""
from __future__ import annotations

import numpy as np
import scipy.fft

# ---------------------------------------------------------------------------
# averaging  (pyLOM/vmmath/averaging.py)
# ---------------------------------------------------------------------------


def temporal_mean(X):
    """Row mean over snapshots.  pyLOM/vmmath/averaging.py:18-29."""
    return np.mean(X, axis=1)


def subtract_mean(X, X_mean):
    """X - mean broadcast over columns.  pyLOM/vmmath/averaging.py:32-44."""
    return X - X_mean[:, None]


def temporal_variance(X, X_mean):
    """Row variance (population), shape (m,1).  pyLOM/vmmath/averaging.py:47-59."""
    return np.var(X, axis=1, keepdims=True)


def norm_variance(X, X_mean, X_var):
    """(X - mean) / variance (not std).  pyLOM/vmmath/averaging.py:62-75."""
    return subtract_mean(X, X_mean) / X_var


# ---------------------------------------------------------------------------
# maths  (pyLOM/vmmath/maths.py)
# ---------------------------------------------------------------------------


def matmul(A, B):
    """C = A @ B.  pyLOM/vmmath/maths.py:77-90."""
    return np.matmul(A, B)


def matmulp(A, B):
    """C = sum over ranks of A_i @ B_i; one rank -> plain matmul.  maths.py:93-110."""
    return np.matmul(A, B)


def vecmat(v, A):
    """Row scaling C[i,:] = v[i]*A[i,:].  pyLOM/vmmath/maths.py:113-130."""
    return v[:, None] * A


# pyLOM picks the complex type with ``real.dtype is p.double`` (maths.py:218,
# 241) and ``X.dtype is np.double`` (SPOD/wrapper.py:42).  A numpy dtype
# instance is never the ``np.double`` type object, so those tests are always
# False: the reference builds its Vandermonde matrices and the SPOD Fourier
# coefficients in complex64 even for float64 input.  ``REFERENCE_DTYPES=True``
# restates that behaviour (used to check against pyLOM's outputs); False gives
# the precision-consistent variant (complex128 for float64 input).
REFERENCE_DTYPES = True


def _cplx(real_dtype, faithful=None):
    faithful = REFERENCE_DTYPES if faithful is None else faithful
    if faithful:
        return np.complex64
    return np.complex128 if np.dtype(real_dtype) == np.float64 else np.complex64


def vandermonde(real, imag, m, n):
    """Vand[:, j] = mu**j.  pyLOM/vmmath/maths.py:203-223."""
    dtype = _cplx(real.dtype)
    mu = real + 1j * imag  # powers in the inputs' precision, stored as dtype
    V = np.zeros((m, n), dtype=dtype)
    for j in range(n):
        V[:, j] = mu ** j
    return V


def vandermondeTime(real, imag, m, t):
    """Vand[:, k] = mu**t_k.  pyLOM/vmmath/maths.py:225-247."""
    dtype = _cplx(real.dtype)
    mu = real + 1j * imag
    V = np.zeros((m, t.shape[0]), dtype=dtype)
    for k, tk in enumerate(t):
        V[:, k] = mu ** tk
    return V


def eigen(A):
    """General real eig, CPU (LAPACK geev).  pyLOM/vmmath/maths.py:161-183."""
    w, vecs = np.linalg.eig(A)
    return np.real(w), np.imag(w), vecs


def polar(real, imag):
    """pyLOM/vmmath/maths.py:185-201."""
    return np.sqrt(real * real + imag * imag), np.arctan2(imag, real)


# ---------------------------------------------------------------------------
# SVD family  (pyLOM/vmmath/svd.py)
# ---------------------------------------------------------------------------


def qr(A):
    """Householder QR, reduced.  pyLOM/vmmath/svd.py:29-36."""
    return np.linalg.qr(A)


def svd(A):
    """Thin SVD (gesdd).  pyLOM/vmmath/svd.py:39-47."""
    return np.linalg.svd(A, full_matrices=False)


def tsqr(Ai):
    """TSQR (Demmel et al. 2012, Alg. 1).  pyLOM/vmmath/svd.py:50-118.

    On one rank the butterfly has zero levels: Q = Q1 @ I, R from the local QR.
    """
    Q1, R = qr(Ai)
    n = Ai.shape[1]
    QW = np.eye(n, dtype=Ai.dtype)
    return matmul(Q1, QW), R


def householder_signs(Q):
    """Column signs s with Q diag(s), diag(s) R the Householder QR factors of
    the matrix whose CholeskyQR factors (R with a positive diagonal) are Q, R:
    s_k = minus the sign of the k-th pivot of the LU of Q's top n x n block
    shifted by diag(s) as it is built (Ballard, Demmel, Grigori, Jacquelin,
    Knight, Nguyen, J. Parallel Distrib. Comput. 85, 2015).  The sign rule the
    CUDA tsqr applies on the device; checked here against numpy/LAPACK's
    factors (the reference's qr, pyLOM/vmmath/svd.py:29-36).  For a square
    matrix LAPACK's last reflector is the identity (dlarfg of a 1-vector), so
    the last R entry keeps the pivot's own sign."""
    m, n = Q.shape
    A = np.array(Q[:n, :n], dtype=np.float64)
    s = np.empty(n)
    for k in range(n):
        if m == n and k == n - 1:
            s[k] = 1.0 if A[k, k] >= 0 else -1.0
            break
        s[k] = -1.0 if A[k, k] >= 0 else 1.0
        A[k, k] -= s[k]
        A[k + 1:, k] /= A[k, k]
        A[k + 1:, k + 1:] -= np.outer(A[k + 1:, k], A[k, k + 1:])
    return s


def tsqr_svd(Ai):
    """TSQR -> svd(R) -> U = Q @ Ur (Sayadi & Schmid 2016, Alg. 2).
    pyLOM/vmmath/svd.py:228-252.  Returns (U m x n, S n, V n x n) with V = V^T."""
    Q, R = tsqr(Ai)
    Ur, S, V = svd(R)
    return matmul(Q, Ur), S, V


def philox_uniform(shape, seed, dtype=np.float32):
    """Uniform [0,1) numbers from the Philox4x32-10 counter generator
    (Salmon et al., SC'11), counter = flat element index, key = seed.

    Restates the device generator the CUDA path uses for the randomized range
    finder so that the oracle can use the identical test matrix.  (The
    reference draws its Omega with numpy's MT19937 ``rand``:
    pyLOM/vmmath/svd.py:133; both are uniform [0,1).)"""
    count = int(np.prod(shape))
    idx = np.arange(count, dtype=np.uint64)
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    mask = np.uint64(0xFFFFFFFF)
    c0 = idx & mask
    c1 = idx >> np.uint64(32)
    c2 = np.zeros_like(idx)
    c3 = np.zeros_like(idx)
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    k0 = np.uint64(seed & 0xFFFFFFFF)
    k1 = np.uint64(seed >> 32)
    for rnd in range(10):
        if rnd > 0:
            k0 = (k0 + W0) & mask
            k1 = (k1 + W1) & mask
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & mask
        hi1, lo1 = p1 >> np.uint64(32), p1 & mask
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & mask, lo1, (hi0 ^ c3 ^ k1) & mask, lo0
    if np.dtype(dtype) == np.float64:
        bits = ((c0 << np.uint64(32)) | c1) >> np.uint64(11)
        out = bits.astype(np.float64) * (1.0 / 9007199254740992.0)
    else:
        out = (c0 >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    return out.reshape(shape).astype(dtype)


def randomized_qr(Ai, r, q, seed=-1, omega=None):
    """Randomized range finder.  pyLOM/vmmath/svd.py:121-144.

    ``omega`` (n x r) may be supplied; otherwise numpy's ``rand`` after
    ``np.random.seed(seed)`` exactly as the reference draws it."""
    n = Ai.shape[1]
    if omega is None:
        np.random.seed(seed=seed)
        omega = np.random.rand(n, r).astype(Ai.dtype)
    Y = matmul(Ai, omega)
    for _ in range(q):
        Q, _ = tsqr(Y)
        Q2 = matmulp(Ai.T, Q)
        Y = matmul(Ai, Q2)
    Q, _ = tsqr(Y)
    B = matmulp(Q.T, Ai)
    return Q, B


def randomized_svd(Ai, r, q, seed=-1, omega=None):
    """pyLOM/vmmath/svd.py:255-273.  Returns (U m x r, S r, V r x n)."""
    Q, B = randomized_qr(Ai, r, q, seed=seed, omega=omega)
    Ur, S, V = svd(B)
    return matmul(Q, Ur), S, V


def init_qr_streaming(Ai, r, q, seed=None, omega=None):
    """Streaming randomized range finder, first batch.
    pyLOM/vmmath/svd.py:175-193: Omega = rand(n, r) after seed(seed),
    Y = A Omega, q times (Q = tsqr(Y); Y = A (A^T Q)), Q = tsqr(Y), B = Q^T A.
    Returns (Q m x r, B r x n, Y m x r)."""
    n = Ai.shape[1]
    if omega is None:
        np.random.seed(seed=seed)
        omega = np.random.rand(n, r).astype(Ai.dtype)
    Y = matmul(Ai, omega)
    for _ in range(q):
        Q, _ = tsqr(Y)
        Q2 = matmulp(Ai.T, Q)
        Y = matmul(Ai, Q2)
    Q, _ = tsqr(Y)
    B = matmulp(Q.T, Ai)
    return Q, B, Y


def update_qr_streaming(Ai, Q1, B1, Yo, r, q, omega=None):
    """Streaming randomized range finder, next batch of snapshots.
    pyLOM/vmmath/svd.py:196-225: Omega = rand(n_new, r) (numpy's global
    stream, continuing), Yn = A Omega and q power steps on the new batch,
    Yo += Yn, Q2 = tsqr(Yo), B2 = [(Q2^T Q1) B1, Q2^T A].  Returns
    (Q2 m x r, B2 r x (n_old + n_new), Yo); the reference adds into the
    caller's Yo in place, this restatement returns a new array."""
    n = Ai.shape[1]
    if omega is None:
        omega = np.random.rand(n, r).astype(Ai.dtype)
    Yn = matmul(Ai, omega)
    for _ in range(q):
        Qp, _ = tsqr(Yn)
        O2 = matmulp(Ai.T, Qp)
        Yn = matmul(Ai, O2)
    Yo = Yo + Yn
    Q2, _ = tsqr(Yo)
    Q2Q1 = matmulp(Q2.T, Q1)
    B2o = matmul(Q2Q1, B1)
    B2n = matmulp(Q2.T, Ai)
    return Q2, np.hstack((B2o, B2n)), Yo


# ---------------------------------------------------------------------------
# truncation  (pyLOM/vmmath/truncation.py)
# ---------------------------------------------------------------------------


def compute_truncation_residual(S, r):
    """Mode count from a residual (r>0) or energy fraction (r<0).
    pyLOM/vmmath/truncation.py:17-39."""
    N = 0
    if r > 0:
        normS = np.linalg.norm(S, 2)
        for ii in range(S.shape[0]):
            if np.linalg.norm(S[ii:], 2) / normS < r:
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
    """1 - |orig-rec|^2/|orig|^2.  pyLOM/vmmath/truncation.py:42-58."""
    return 1.0 - np.sum((original - rec) ** 2) / np.sum(original ** 2)


def RMSE(A, B, relative=True):
    """pyLOM/vmmath/stats.py:17-34."""
    d = A - B
    den = np.sum(A * A) if relative else np.prod(A.shape)
    return float(np.sqrt(np.sum(d * d) / den))


# ---------------------------------------------------------------------------
# POD  (pyLOM/POD/wrapper.py)
# ---------------------------------------------------------------------------


def pod_run(X, remove_mean=True, divide_variance=False, randomized=False, r=1, q=3,
            seed=-1, omega=None):
    """pyLOM/POD/wrapper.py:17-51."""
    if remove_mean:
        X_mean = temporal_mean(X)
        if divide_variance:
            Y = norm_variance(X, X_mean, temporal_variance(X, X_mean))
        else:
            Y = subtract_mean(X, X_mean)
    else:
        Y = X.copy()
    if randomized:
        return randomized_svd(Y, r, q, seed=seed, omega=omega)
    return tsqr_svd(Y)


def pca_run(X, divide_variance=True, randomized=False, r=1, q=3, seed=-1):
    """pyLOM/PCA/wrapper.py:17-38: components U and scores (diag(S) V)^T of the
    POD of the mean-removed (variance-normalised) data."""
    U, S, V = pod_run(X, remove_mean=True, divide_variance=divide_variance, randomized=randomized,
                      r=r, q=q, seed=seed)
    return U, vecmat(S, V).T


def pod_truncate(U, S, V, r=1e-8):
    """pyLOM/POD/wrapper.py:56-82."""
    N = int(r) if r >= 1 else compute_truncation_residual(S, r)
    return U[:, :N], S[:N], V[:N, :]


def pod_reconstruct(U, S, V):
    """pyLOM/POD/wrapper.py:87-103."""
    return matmul(U, vecmat(S, V))


# ---------------------------------------------------------------------------
# DMD  (pyLOM/DMD/wrapper.py)
# ---------------------------------------------------------------------------


def dmd_order_modes(muReal, muImag, Phi, bJov):
    """Sort by |b| descending; a conjugate pair is put positive-imag first.
    pyLOM/DMD/wrapper.py:18-45 (including its exact imag-part reassignment)."""
    order = np.flip(np.abs(bJov).argsort())
    muReal = muReal[order].copy()
    muImag = muImag[order].copy()
    Phi = Phi[:, order].copy()
    bJov = bJov[order].copy()
    skip = False
    for ii in range(muImag.shape[0]):
        if skip:
            skip = False
            continue
        im = muImag[ii]
        if im < 0:
            muImag[ii] = muImag[ii + 1]
            muImag[ii + 1] = -muImag[ii]
            bJov.imag[ii] = bJov.imag[ii + 1]
            bJov.imag[ii + 1] = -bJov.imag[ii]
            Phi.imag[:, ii] = Phi.imag[:, ii + 1]
            Phi.imag[:, ii + 1] = -Phi.imag[:, ii + 1]
            skip = True
            continue
        if im > 0:
            skip = True
            continue
    return muReal, muImag, Phi, bJov


def dmd_run(X, r, remove_mean=True):
    """Exact DMD with Jovanovic amplitudes.  pyLOM/DMD/wrapper.py:49-117."""
    if remove_mean:
        Y = subtract_mean(X, temporal_mean(X))
    else:
        Y = X.copy()
    U, S, VT = tsqr_svd(Y[:, :-1])
    U, S, VT = pod_truncate(U, S, VT, r)
    aux1 = matmulp(U.T, Y[:, 1:])
    aux2 = vecmat(1.0 / S, VT).T
    Atilde = matmul(aux1, aux2)
    muReal, muImag, w = eigen(Atilde)
    Phi = matmul(matmul(matmul(Y[:, 1:], VT.T), np.diag(1 / S)), w) / (muReal + muImag * 1j)
    Vand = vandermonde(muReal, muImag, muReal.shape[0], Y.shape[1] - 1)
    P = matmul(np.conj(w).T, w) * np.conj(matmul(Vand, np.conj(Vand).T))
    Pl = np.linalg.cholesky(P)
    G = matmul(np.diag(S), VT)
    qv = np.conj(np.diag(matmul(matmul(Vand, np.conj(G).T), w)))
    bJov = matmul(np.linalg.inv(np.conj(Pl).T), matmul(np.linalg.inv(Pl), qv))
    return dmd_order_modes(muReal, muImag, Phi, bJov)


def dmd_frequency_damping(real, imag, dt):
    """pyLOM/DMD/wrapper.py:120-130."""
    mod, arg = polar(real, imag)
    return np.log(mod) / dt, arg / dt


def dmd_reconstruction_jovanovic(Phi, real, imag, t, bJov):
    """pyLOM/DMD/wrapper.py:141-146."""
    Vand = vandermondeTime(real, imag, real.shape[0], t)
    return matmul(Phi, matmul(np.diag(bJov), Vand)).real


# ---------------------------------------------------------------------------
# SPOD  (pyLOM/SPOD/wrapper.py, pyLOM/vmmath/fft.py)
# ---------------------------------------------------------------------------


def hammwin(N):
    """Hamming window 0.54-0.46cos(2 pi i/(N-1)).  pyLOM/vmmath/fft.py:17-27."""
    return np.transpose(0.54 - 0.46 * np.cos(2 * np.pi * np.arange(N) / (N - 1)))


def hannwin(N):
    """Symmetric Hann window 0.5-0.5cos(2 pi i/(N-1)) (the window a Hann run
    uses in place of the reference's Hamming; no reference counterpart)."""
    return 0.5 - 0.5 * np.cos(2 * np.pi * np.arange(N) / (N - 1))


def spod_run(X, t, nDFT=0, nolap=0, remove_mean=True, window="hamming", return_U=False):
    """Welch SPOD.  pyLOM/SPOD/wrapper.py:24-95 (``_fft`` at :18-20).
    With ``return_U`` the per-frequency complex left singular vectors
    (M x nBlks each, in the returned frequency order) come back as a fourth
    value: P = Re(U) depends on the arbitrary phase of each column, U up to
    that phase does not."""
    M, N = X.shape
    dt = t[1] - t[0]
    cdtype = _cplx(X.dtype)
    if nDFT == 0:
        nDFT = int(np.power(2, np.floor(np.log2(N / 10))))
    win = hammwin(nDFT) if window == "hamming" else hannwin(nDFT)
    if nolap == 0:
        nolap = int(np.floor(nDFT / 2))
    nBlks = int(np.floor((N - nolap) / (nDFT - nolap)))
    winWeight = 1 / np.mean(win)
    Y = subtract_mean(X, temporal_mean(X)) if remove_mean else X.copy()
    f = np.arange(np.ceil(nDFT / 2) + 1) / dt / nDFT
    nf = f.shape[0]
    qk = np.zeros((M, nf), cdtype)
    Q = np.zeros((M * nf, nBlks), cdtype)
    for iblk in range(nBlks):
        i0 = iblk * (nDFT - nolap)
        Xf = Y[:, i0:i0 + nDFT].copy() * win
        qk[:, :] = (winWeight / nDFT) * scipy.fft.fft2(Xf, axes=(-1,))[:, :nf]
        qk[:, 1:-1] *= 2
        Q[:, iblk] = qk.reshape((M * nf), order="F")
    L = np.zeros((nf, nBlks), X.dtype)
    P = np.zeros((M * nBlks, nf), X.dtype)
    Us = []
    for ifreq in range(nf):
        qf = Q[ifreq * M:(ifreq + 1) * M, :].copy() / np.sqrt(nBlks)
        U, S, V = tsqr_svd(qf)
        P[:, ifreq] = np.real(U.reshape((M * nBlks), order="F"))
        L[ifreq, :] = np.abs(S * S)
        if return_U:
            Us.append(U)
    order = np.argsort(L[:, 0])[::-1]
    if return_U:
        return L[order, :], P[:, order], f[order], [Us[i] for i in order]
    return L[order, :], P[:, order], f[order]


# ---------------------------------------------------------------------------
# error metrics used by the tests (not part of the reference)
# ---------------------------------------------------------------------------


def subspace_angle(U1, U2):
    """Largest principal angle (radians) between span(U1) and span(U2)."""
    Q1, _ = np.linalg.qr(U1)
    Q2, _ = np.linalg.qr(U2)
    s = np.linalg.svd(Q1.conj().T @ Q2, compute_uv=False)
    return float(np.arccos(np.clip(s.min(), -1.0, 1.0)))


def orthogonality(U):
    """||I - U^H U||_2."""
    k = U.shape[1]
    return float(np.linalg.norm(np.eye(k) - U.conj().T @ U, 2))
