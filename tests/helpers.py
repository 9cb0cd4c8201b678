"""Comparison helpers shared by the parity tests."""
import numpy as np


def cols_up_to_phase(A, B, tol):
    """Column j of A equals column j of B up to a unit scalar (sign for real,
    phase for complex); max abs deviation <= tol * max|B|."""
    A = np.asarray(A)
    B = np.asarray(B)
    worst = 0.0
    for j in range(B.shape[1]):
        a, b = A[:, j], B[:, j]
        z = np.vdot(b, a)
        ph = z / abs(z) if abs(z) > 0 else 1.0
        worst = max(worst, float(np.max(np.abs(a - ph * b))))
    scale = max(1e-300, float(np.max(np.abs(B))))
    assert worst <= tol * scale, f"columns differ by {worst:.3e} (> {tol:.1e} x {scale:.3e})"
    return worst / scale


def sigma_rel(S, S_ref, k=None):
    S = np.asarray(S, dtype=np.float64)
    S_ref = np.asarray(S_ref, dtype=np.float64)
    k = len(S_ref) if k is None else k
    return float(np.max(np.abs(S[:k] - S_ref[:k]) / np.abs(S_ref[:k])))


def sigma_normwise(S, S_ref):
    S = np.asarray(S, dtype=np.float64)
    S_ref = np.asarray(S_ref, dtype=np.float64)
    return float(np.max(np.abs(S - S_ref)) / S_ref[0])


def orthogonality(U):
    U = np.asarray(U, dtype=np.complex128 if np.iscomplexobj(U) else np.float64)
    k = U.shape[1]
    return float(np.linalg.norm(np.eye(k) - U.conj().T @ U, 2))


def subspace_angle(U1, U2):
    Q1, _ = np.linalg.qr(np.asarray(U1, dtype=np.complex128))
    Q2, _ = np.linalg.qr(np.asarray(U2, dtype=np.complex128))
    s = np.linalg.svd(Q1.conj().T @ Q2, compute_uv=False)
    return float(np.arccos(np.clip(s.min(), -1.0, 1.0)))
