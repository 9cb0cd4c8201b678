"""pyLOM.DMD hot path on GB300: run / frequency_damping / reconstruction_jovanovic.

DMD.run follows pyLOM/DMD/wrapper.py:49-117: mean removal, TSQR-SVD of
Y[:, :-1], truncation, U^T Y2 as a split-K product, then the reduced stage
(eigendecomposition, Vandermonde, Jovanovic amplitudes, ordering) in one FP64
kernel, and the modes as one tall product Phi = Y2 Mphi.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import vmmath as M

__all__ = ["run", "frequency_damping", "reconstruction_jovanovic"]


def run_device(x, ld, r, remove_mean=True, precision=None):
    t = L.torch()
    if remove_mean:
        Y, _, _ = M.remove_mean_device(x, ld)
        ldy = Y.shape[1]
    else:
        Y, ldy = x, ld
    m, n = Y.shape
    nt = n - 1
    Y1 = Y[:, :-1]
    U, S, VT = M.tsqr_svd_device(Y1, ldy, precision)
    N = int(r) if r >= 1 else M.compute_truncation_residual(S, r)
    N = max(1, min(N, S.shape[0]))
    U = U[:, :N]
    S = S[:N]
    VT = VT[:N, :]
    Y2 = Y[:, 1:]
    if Y.dtype == t.float32:
        # FP32 factors: aux1, S and V^T recomputed from span(U_r) with exact
        # products (plom_dmd_project), so the eigenvalues do not inherit the
        # mutual inconsistency of the FP32 / mixed-form U, S and V
        aux1 = t.empty((N, nt), dtype=t.float64, device="cuda")
        S64 = t.empty(N, dtype=t.float64, device="cuda")
        VT64 = t.empty((N, nt), dtype=t.float64, device="cuda")
        ws = L.workspace(L.load().plom_dmd_project_workspace(m, n, N))
        info = L.new_info()
        L.call("plom_dmd_project", L.ptr(U), U.stride(0), L.ptr(Y), ldy, m, n, N, L.ptr(aux1),
               L.ptr(S64), L.ptr(VT64), L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
        L.check_info(info, "DMD projection")
        del ws
    else:
        # aux1 = U^T Y2 (N x nt), reduction over the m points
        aux1 = M._matmul_dev(U, U.stride(0), 1, Y2, ldy, N, nt, m, precision)
        aux1 = aux1.to(t.float64).contiguous()
        S64 = S.to(t.float64).contiguous()
        VT64 = VT.to(t.float64).contiguous()
    muR = t.empty(N, dtype=t.float64, device="cuda")
    muI = t.empty(N, dtype=t.float64, device="cuda")
    b = t.empty(2 * N, dtype=t.float64, device="cuda")
    Mphi = t.empty((nt, 2 * N), dtype=t.float64, device="cuda")
    ws = L.workspace(L.load().plom_dmd_reduced_workspace(N, nt))
    info = L.new_info()
    L.call("plom_dmd_reduced", L.ptr(aux1), L.ptr(S64), L.ptr(VT64), N, nt, L.ptr(muR), L.ptr(muI),
           L.ptr(b), L.ptr(Mphi), L.ptr(ws), ws.numel(), L.ptr(info), L.stream_ptr())
    L.check_info(info, "DMD reduced stage")
    # Phi = Y2 Mphi : m x N complex as the interleaved real m x 2N result
    Mop = Mphi.to(Y.dtype).contiguous()
    Phi_r = M._matmul_dev(Y2, ldy, 0, Mop, 2 * N, m, 2 * N, nt, precision)
    cdt = t.complex128 if Y.dtype == t.float64 else t.complex64
    Phi = t.view_as_complex(Phi_r.reshape(m, N, 2))
    bc = t.view_as_complex(b.reshape(N, 2)).to(cdt)
    return muR.to(Y.dtype), muI.to(Y.dtype), Phi.to(cdt), bc


def run(X, r, remove_mean=True, *, precision=None):
    """DMD of X (points x snapshots) truncated at r (mode count if r >= 1,
    residual if r < 1).  Returns muReal, muImag, Phi (m x r complex) and the
    Jovanovic amplitudes bJov, ordered as pyLOM/DMD/wrapper.py:18-45."""
    cv = L.to_device(X)
    x, ld = L.as_rows(cv.t)
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("DMD.run takes float32 or float64 data")
    muR, muI, Phi, b = run_device(x, ld, r, remove_mean, precision)
    return cv.back(muR), cv.back(muI), cv.back(Phi), cv.back(b)


def frequency_damping(real, imag, dt):
    """delta = ln|mu| / dt, omega = arg(mu) / dt (pyLOM/DMD/wrapper.py:120-130)."""
    t = L.torch()
    if isinstance(real, t.Tensor):
        mod = t.sqrt(real * real + imag * imag)
        return t.log(mod) / dt, t.atan2(imag, real) / dt
    real, imag = np.asarray(real), np.asarray(imag)
    mod = np.sqrt(real * real + imag * imag)
    return np.log(mod) / dt, np.arctan2(imag, real) / dt


def reconstruction_jovanovic(Phi, real, imag, t, bJov, *, precision=None):
    """X_DMD = Re(Phi diag(b) Vand(t)) (pyLOM/DMD/wrapper.py:141-146): the
    Vandermonde in time is built on the device and the product is one tall
    GEMM of the interleaved real views."""
    tt = L.torch()
    is_np = not isinstance(Phi, tt.Tensor)
    Phi_d = tt.as_tensor(np.asarray(Phi), device="cuda") if is_np else Phi.to("cuda")
    rd = tt.as_tensor(np.asarray(real), device="cuda") if is_np else real.to("cuda")
    im = tt.as_tensor(np.asarray(imag), device="cuda") if is_np else imag.to("cuda")
    bb = tt.as_tensor(np.asarray(bJov), device="cuda") if is_np else bJov.to("cuda")
    ts = tt.as_tensor(np.asarray(t), device="cuda", dtype=tt.float64) if is_np else t.to("cuda", tt.float64)
    mu = tt.complex(rd.to(tt.float64), im.to(tt.float64))
    # Vand[i, k] = mu_i ** t_k, scaled by b_i:  D = diag(b) Vand   (r x nt)
    D = bb.to(tt.complex128)[:, None] * tt.exp(ts[None, :] * tt.log(mu)[:, None])
    # Re(Phi D) = Phi_r D_r - Phi_i D_i  ->  [Phi_r, Phi_i] @ [D_r; -D_i]
    rdt = tt.float64 if Phi_d.dtype == tt.complex128 else tt.float32
    Pr = tt.view_as_real(Phi_d.contiguous()).reshape(Phi_d.shape[0], -1).to(rdt)  # m x 2r
    Dm = tt.empty((2 * D.shape[0], D.shape[1]), dtype=tt.float64, device="cuda")
    Dm[0::2] = D.real
    Dm[1::2] = -D.imag
    Dm = Dm.to(rdt).contiguous()
    X = M._matmul_dev(Pr, Pr.shape[1], 0, Dm, Dm.shape[1], Pr.shape[0], Dm.shape[1], Dm.shape[0],
                      precision)
    return X.cpu().numpy() if is_np else X
