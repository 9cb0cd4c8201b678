"""Parity at the shapes of the large workloads, against the FP64 oracle on
the same inputs: a row-reduced POD field of the 8,388,608 x 1,024 headline
(262,144 x 1,024, the same generator, mean removed) through the mixed form,
and a row-reduced SPOD field of the 1,048,576 x 8,192 workload (32,768 x
8,192, nDFT 256, nolap 128: 63 blocks, 129 frequencies) with SPOD's modes P
pinned up to the phase of each complex singular vector.

Tolerances (mixed form against FP64): sigma 1e-5 relative on the 64
retained modes, subspace angle 1e-4 rad, ||I - U^T U|| 1e-5 on the retained
modes, sigma normwise 1e-5; SPOD energies 1e-4 relative on the three
leading modes of every frequency above 1e-3 of the largest energy, modes P
fitted to the oracle's Re(e^{i phi} U_f) with residual 1e-3.
"""
import numpy as np
import pytest

from oracle import plom_oracle as O
from tests.helpers import sigma_normwise, sigma_rel, subspace_angle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pyloworder_gb300 as P  # noqa: E402
from pyloworder_gb300 import datagen  # noqa: E402


class _fp64_oracle:
    """The oracle's precision-consistent variant (complex128 Fourier
    coefficients for float64 data; by default it restates pyLOM's complex64
    choice, which is right for checking pyLOM's own outputs)."""

    def __enter__(self):
        self.old = O.REFERENCE_DTYPES
        O.REFERENCE_DTYPES = False

    def __exit__(self, *a):
        O.REFERENCE_DTYPES = self.old


def phase_fit(p, u):
    """p (real) against Re(e^{i phi} u) = a Re(u) + c Im(u), a^2 + c^2 = 1:
    the least-squares (a, c), the relative residual and |a^2 + c^2 - 1|.
    When u is real up to one global phase (the zero and Nyquist bins), Re(u)
    and Im(u) are parallel and only p's direction is determined: the
    amplitude check is then 0."""
    Bm = np.stack([u.real, u.imag], axis=1)
    coef, *_ = np.linalg.lstsq(Bm, p, rcond=None)
    res = np.linalg.norm(p - Bm @ coef) / max(np.linalg.norm(u), 1e-300)
    sv = np.linalg.svd(Bm, compute_uv=False)
    if sv[1] < 1e-6 * sv[0]:
        return coef, res, 0.0
    return coef, res, abs(coef @ coef - 1.0)


def test_tsqr_svd_pod_field_row_reduced_vs_oracle():
    m, n, k = 262144, 1024, 64
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, k, seed=1002, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = P.vmmath.remove_mean_device(X, n)
    del X
    U, S, V = P.vmmath.tsqr_svd_device(Y, n, "mixed")
    Yh = Y.cpu().numpy().astype(np.float64)
    Uo, So, Vo = O.tsqr_svd(Yh)
    S = S.double().cpu().numpy()
    Uk = U[:, :k].double().cpu().numpy()
    assert sigma_rel(S, So, k) < 1e-5
    assert sigma_normwise(S, So) < 1e-5
    assert subspace_angle(Uk, Uo[:, :k]) < 1e-4
    assert np.linalg.norm(np.eye(k) - Uk.T @ Uk, 2) < 1e-5
    assert subspace_angle(V[:k].double().cpu().numpy().T, Vo[:k].T) < 1e-4


def _spod_leading_checks(Lm, Pm, f, Lo, Uo, fo, M, ltol, ptol, nfreq_p):
    """L and f against the oracle; P's leading modes (column b of U_f sits in
    rows b M .. (b + 1) M - 1 of P's column) fitted to the oracle's
    Re(e^{i phi} U_f[:, b]) for the three leading modes of the first nfreq_p
    frequencies that are separated from their neighbours (relative energy
    gap > 0.2) and above 1e-3 of the frequency's leading energy."""
    np.testing.assert_allclose(f, fo, rtol=1e-12)
    big = Lo[:, :3] > 1e-3 * Lo.max()
    rel = np.abs(Lm[:, :3] - Lo[:, :3]) / Lo[:, :3]
    assert rel[big].max() < ltol, rel[big].max()
    checked = 0
    nb = Lo.shape[1]
    for c in range(nfreq_p):
        for b in range(min(3, nb)):
            lb = Lo[c, b]
            if lb < 1e-3 * Lo[c, 0]:
                continue
            gaps = [abs(lb - Lo[c, j]) / lb for j in (b - 1, b + 1) if 0 <= j < nb]
            if min(gaps) < 0.2:
                continue
            p = Pm[b * M:(b + 1) * M, c].astype(np.float64)
            _, res, dn = phase_fit(p, Uo[c][:, b])
            tol = ptol * (1.0 if b == 0 else 10.0)
            assert res < tol and dn < 2 * tol, (c, b, res, dn)
            checked += 1
    assert checked >= 3, checked


@pytest.mark.parametrize("tag,precision,ltol,ptol", [("f64", "fp64", 1e-9, 1e-8),
                                                     ("f32", "mixed", 2e-4, 1e-3)])
def test_spod_modes_pinned_up_to_phase(golden, tag, precision, ltol, ptol):
    """SPOD's P = Re(U_f) against the FP64 oracle's complex U_f of the same
    Fourier coefficients, up to one phase per mode."""
    g = golden("spod_" + tag)
    X, t = g["X"], g["t"]
    nDFT, nolap = int(g["nDFT"]), int(g["nolap"])
    Lm, Pm, f = P.SPOD.run(X, t, nDFT=nDFT, nolap=nolap, precision=precision)
    with _fp64_oracle():
        Lo, Po, fo, Uo = O.spod_run(X.astype(np.float64), t.astype(np.float64), nDFT=nDFT,
                                    nolap=nolap, return_U=True)
    _spod_leading_checks(Lm, Pm, f, Lo, Uo, fo, X.shape[0], ltol, ptol, nfreq_p=Lm.shape[0])


def test_spod_field_row_reduced_vs_oracle():
    """32,768 x 8,192 rows of the SPOD workload's generator (8 narrow-band
    oscillators, AR(1) red noise), Hamming window, nDFT 256, nolap 128:
    63 blocks, 129 frequencies; mixed form against the FP64 oracle."""
    M, N = 32768, 8192
    X = datagen.spod_field_device(M, N)
    t = np.arange(N, dtype=np.float64)
    Lm, Pm, f = P.SPOD.run(X, t, nDFT=256, nolap=128, precision="mixed")
    assert Lm.shape == (129, 63) and Pm.shape == (M * 63, 129)
    Lm, Pm = Lm.double().cpu().numpy(), Pm.cpu().numpy()
    f = f.cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
    Xh = X.cpu().numpy().astype(np.float64)
    del X
    with _fp64_oracle():
        Lo, Po, fo, Uo = O.spod_run(Xh, t, nDFT=256, nolap=128, return_U=True)
    _spod_leading_checks(Lm, Pm, f, Lo, Uo, fo, M, 1e-4, 1e-3, nfreq_p=12)


def test_tsqr_svd_chunked_first_pass_matches_whole():
    """A large FP32 input takes the first pass in row chunks packed on a second
    stream beside the Gram (per-chunk column scales, one slab reduction that
    unscales each chunk in FP64); the result must match the whole-matrix
    packing (pass1_chunks = 1) to the mixed form's tolerances."""
    from pyloworder_gb300 import _lib as L
    lib = L.load()
    m, n, k = 2_097_152, 256, 32
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, k, seed=1203, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = P.vmmath.remove_mean_device(X, n)
    del X
    old = lib.plom_get_tuning(b"pass1_chunks")
    try:
        assert lib.plom_set_tuning(b"pass1_chunks", 8.0) == 0
        Uc, Sc, Vc = P.vmmath.tsqr_svd_device(Y, n, "mixed")
        assert lib.plom_set_tuning(b"pass1_chunks", 1.0) == 0
        Uw, Sw, Vw = P.vmmath.tsqr_svd_device(Y, n, "mixed")
    finally:
        lib.plom_set_tuning(b"pass1_chunks", old)
    Sc, Sw = Sc.double().cpu().numpy(), Sw.double().cpu().numpy()
    assert sigma_rel(Sc, Sw, k) < 1e-5
    assert sigma_normwise(Sc, Sw) < 1e-5
    assert subspace_angle(Uc[:, :k].double().cpu().numpy(), Uw[:, :k].double().cpu().numpy()) < 1e-4
    Ud = Uc.double()
    assert float((Ud.T @ Ud - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max()) < 1e-4
