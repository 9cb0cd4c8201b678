"""GPU parity of the SVD path (averaging, matmul, tsqr, tsqr_svd,
randomized_svd, POD) against the oracle and the golden fixtures produced by
pyLOM itself.

Tolerances: FP64 form 1e-10 relative on sigma (signal modes) and 1e-12
normwise (|dS|/S_1); mixed form 1e-5 relative on sigma for modes above
1e-3 S_1 and 1e-4 rad subspace angle.  Modes are compared up to sign/phase.
"""
import numpy as np
import pytest

from oracle import plom_oracle as O
from tests.helpers import cols_up_to_phase, orthogonality, sigma_normwise, sigma_rel, subspace_angle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU hosts, run on the GPU machine
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pyloworder_gb300 as P  # noqa: E402


def test_averaging_golden(golden):
    g = golden("averaging")
    m = P.math.temporal_mean(g["X"])
    np.testing.assert_allclose(m, g["mean"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(P.math.subtract_mean(g["X"], m), g["Y"], rtol=1e-13, atol=1e-14)
    v = P.math.temporal_variance(g["X"], m)
    np.testing.assert_allclose(v, g["var"], rtol=1e-12)
    np.testing.assert_allclose(P.math.norm_variance(g["X"], m, v), g["Yv"], rtol=1e-11)


@pytest.mark.parametrize("m,n", [(1000, 37), (4096, 256), (3, 1), (777, 1000)])
def test_averaging_f32_shapes(m, n):
    X = np.random.default_rng(m + n).standard_normal((m, n)).astype(np.float32) + 3.0
    mean = P.math.temporal_mean(X)
    ref = X.astype(np.float64).mean(axis=1)
    np.testing.assert_allclose(mean, ref, rtol=1e-6, atol=1e-6)
    Y = P.math.subtract_mean(X, mean)
    np.testing.assert_allclose(Y, X - mean[:, None], rtol=1e-6, atol=1e-6)


def test_kat_example_svd(golden):
    g = golden("kat_example_svd")
    U, S, V = P.math.tsqr_svd(g["A"])
    np.testing.assert_allclose(S, g["S"], rtol=1e-13)
    cols_up_to_phase(U, g["U"], 1e-12)
    cols_up_to_phase(V.T, g["V"].T, 1e-12)


def test_tsqr_svd_f64_golden(golden):
    g = golden("tsqr_svd_f64")
    U, S, V = P.math.tsqr_svd(g["A"])
    assert sigma_rel(S, g["S"]) < 1e-12
    cols_up_to_phase(U, g["U"], 1e-10)
    cols_up_to_phase(V.T, g["V"].T, 1e-10)
    assert orthogonality(U) < 1e-13


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_tsqr_svd_f32_golden(golden, precision):
    g = golden("tsqr_svd_f32")
    U, S, V = P.math.tsqr_svd(g["A"], precision=precision)
    assert U.dtype == np.float32 and S.dtype == np.float32
    ref = O.tsqr_svd(g["A"].astype(np.float64))
    assert sigma_rel(S, ref[1]) < 1e-5
    assert sigma_rel(S, g["S"]) < 2e-5
    cols_up_to_phase(U, ref[0], 1e-3)
    assert orthogonality(U) < 1e-5


def test_pod_cfg1_small_golden(golden):
    g = golden("pod_cfg1_small")
    U, S, V = P.POD.run(g["X"])
    k = 10
    assert sigma_rel(S, g["S"], k) < 1e-10
    assert sigma_normwise(S, g["S"]) < 1e-12
    cols_up_to_phase(U[:, :k], g["U"][:, :k], 1e-9)
    Ut, St, Vt = P.POD.truncate(U, S, V, r=1e-6)
    assert Ut.shape[1] == int(g["N_res"])
    assert P.POD.truncate(U, S, V, r=-0.99)[0].shape[1] == int(g["N_energy"])
    Xr = P.POD.reconstruct(Ut, St, Vt)
    np.testing.assert_allclose(Xr, g["Xr"], atol=1e-11)


def test_pod_divvar_golden(golden):
    g = golden("pod_divvar")
    U, S, V = P.POD.run(g["X"], remove_mean=True, divide_variance=True)
    assert sigma_rel(S, g["S"], 10) < 1e-10
    assert sigma_normwise(S, g["S"]) < 1e-12


def test_pod_f32_nomean_golden(golden):
    g = golden("pod_f32_nomean")
    U, S, V = P.POD.run(g["X"], remove_mean=False)
    ref = O.pod_run(g["X"].astype(np.float64), remove_mean=False)
    assert S.dtype == np.float32
    assert sigma_rel(S, ref[1], 9) < 1e-5
    # mode 10 (2.5e-3) sits on the noise floor (mode 11: 2.4e-3).  The mixed
    # form's tensor-core operands carry 22-23 significant bits of the FP32
    # input; rounding X in its 23rd-24th bits moves sigma_10 by 1e-6 to 1e-5
    # relative depending on the rounding pattern (measured on this matrix with
    # inputs perturbed by one ulp), so the noise-floor mode gets a wider
    # bound.  The 10-mode subspace is ill-conditioned even for pyLOM
    # (2.9e-5 rad); the 9 signal modes are well separated.
    assert sigma_rel(S, ref[1], 10) < 5e-5
    assert subspace_angle(U[:, :9], ref[0][:, :9]) < 1e-4


def test_mixed_mean_removed_u_orthonormal():
    """Mean-removed snapshots have an exact null vector (X 1 = 0), far below
    the mixed form's 22-bit operand precision; every column of U, including
    the null one, must still come out orthonormal."""
    from pyloworder_gb300 import datagen
    m, n = 262144, 256
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, 32, seed=77, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = P.vmmath.remove_mean_device(X, n)
    U, S, V = P.vmmath.tsqr_svd_device(Y, n, "mixed")
    Ud = U.double()
    D = Ud.T @ Ud - torch.eye(n, dtype=torch.float64, device="cuda")
    assert float(S[-1] / S[0]) < 1e-6          # the null direction is there
    assert float(D.abs().max()) < 1e-4
    Vd = V.double()
    assert float((Vd @ Vd.T - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max()) < 1e-6


@pytest.mark.parametrize("n", [1024, 517])
def test_mixed_large_n_fp32_presweeps(n):
    """256 <= n <= 1600 in the mixed form: the SVD of R starts with FP32 Jacobi sweeps,
    re-orthonormalises their rotation product and refines it with matrix
    products in double-float sums (simultaneous Jacobi angles plus
    Newton-Schulz steps).  The result must match the plain FP64 form within
    the mixed-form tolerances, with orthonormal U and V (n = 517: odd row
    quarters take the one-row-per-lane loops)."""
    from pyloworder_gb300 import _lib as L
    from pyloworder_gb300 import datagen
    m, k = 32768, 64
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, k, seed=91, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = P.vmmath.remove_mean_device(X, n)
    U, S, V = P.vmmath.tsqr_svd_device(Y, n, "mixed")
    info = list(L.last_info)
    print(f"FP32 sweeps {info[4]}, refinement steps {info[5]}")
    assert info[4] > 0 and info[5] > 0  # the FP32 phase and the refinement ran
    Ur, Sr, _ = P.vmmath.tsqr_svd_device(Y.double(), n, "fp64")
    S64, Sr64 = S.double().cpu().numpy(), Sr.cpu().numpy()
    assert sigma_rel(S64, Sr64, k) < 1e-5
    assert sigma_normwise(S64, Sr64) < 1e-5
    assert subspace_angle(U[:, :k].double().cpu().numpy(), Ur[:, :k].cpu().numpy()) < 1e-4
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    Ud, Vd = U.double(), V.double()
    assert float((Ud.T @ Ud - eye).abs().max()) < 1e-4
    assert float((Vd @ Vd.T - eye).abs().max()) < 1e-6


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("case", ["zero_col", "zero_cols3", "dup_cols", "rank3", "tiny_m", "n1",
                                  "wide_ragged"])
def test_degenerate_inputs(case, precision):
    """Inputs with exact null directions (zero columns, 20 duplicated columns,
    rank 3 of 64), few rows, one column, ragged sizes: finite outputs, sigma
    normwise, X = U S V, and every column of U orthonormal (LAPACK's U is,
    null directions included: an exact zero column's U column is completed
    to a unit vector orthogonal to the others)."""
    rng = np.random.default_rng(5)
    if case == "zero_col":
        X = rng.standard_normal((20000, 40))
        X[:, 7] = 0.0
    elif case == "zero_cols3":
        X = rng.standard_normal((20000, 40))
        X[:, [3, 17, 39]] = 0.0
    elif case == "dup_cols":
        X = rng.standard_normal((20000, 40))
        X[:, 20:] = X[:, :20]
    elif case == "rank3":
        X = rng.standard_normal((30000, 3)) @ rng.standard_normal((3, 64))
    elif case == "tiny_m":
        X = rng.standard_normal((70, 50))
    elif case == "n1":
        X = rng.standard_normal((5000, 1))
    else:
        X = rng.standard_normal((4097 * 3 + 5, 131))
    mixed = precision == "mixed"
    X = X.astype(np.float32 if mixed else np.float64)
    U, S, V = P.math.tsqr_svd(X, precision=precision)
    k = min(X.shape)
    assert U.shape == (X.shape[0], k) and S.shape == (k,) and V.shape == (k, X.shape[1])
    assert np.all(np.isfinite(U)) and np.all(np.isfinite(S)) and np.all(np.isfinite(V))
    Sr = np.linalg.svd(X.astype(np.float64), compute_uv=False)
    assert np.abs(S - Sr[:k]).max() <= (1e-5 if mixed else 1e-12) * Sr[0]
    A = (U.astype(np.float64) * S) @ V
    assert np.abs(A - X).max() <= (1e-4 if mixed else 1e-11) * np.abs(X).max()
    Ud = U.astype(np.float64)
    # FP64: 1e-11 (rank 3 of 64 leaves 61 renormalised null columns at ~1e-12)
    assert np.abs(Ud.T @ Ud - np.eye(k)).max() < (1e-4 if mixed else 1e-11)
    Vd = V.astype(np.float64)
    assert np.abs(Vd @ Vd.T - np.eye(k)).max() < (1e-5 if mixed else 1e-12)


@pytest.mark.parametrize("dtype,precision", [(np.float32, "mixed"), (np.float64, "fp64"),
                                             (np.complex64, "mixed")])
def test_tsqr_svd_host_entry(dtype, precision):
    """Host inputs go through plom_tsqr_svd_host: FP32 mixed streams X in 4
    row chunks of 75,008 rows (the last one ragged, padded with zero rows),
    each packed with its own column scales."""
    rng = np.random.default_rng(3)
    m, n, k = 300001, 40, 8
    X = (rng.standard_normal((m, k)) @ rng.standard_normal((k, n))) * np.logspace(0, -3, n)
    X += 1e-4 * rng.standard_normal((m, n))
    cplx = np.issubdtype(dtype, np.complexfloating)
    if cplx:
        X = X + 1j * ((rng.standard_normal((m, k)) @ rng.standard_normal((k, n))) * np.logspace(0, -3, n))
    X = X.astype(dtype)
    Xt = torch.from_numpy(X).pin_memory()
    Uh, Sh, Vh = P.math.tsqr_svd(Xt, precision=precision)
    assert Uh.device.type == "cpu" and Uh.is_pinned() and Uh.dtype == Xt.dtype
    ref = O.tsqr_svd(X.astype(np.complex128 if cplx else np.float64))
    U, S, V = Uh.numpy(), Sh.numpy(), Vh.numpy()
    if precision == "mixed":
        assert sigma_rel(S, ref[1], k) < 1e-5
        assert subspace_angle(U[:, :k], ref[0][:, :k]) < 1e-4
        assert orthogonality(U) < 1e-5
    else:
        assert sigma_rel(S, ref[1], k) < 1e-10
        assert sigma_normwise(S, ref[1]) < 1e-12
        cols_up_to_phase(U[:, :k], ref[0][:, :k], 1e-8)
        assert orthogonality(U) < 1e-12
    A = (U * S) @ V
    assert np.abs(A - X).max() <= (1e-4 if precision == "mixed" else 1e-11) * np.abs(X).max()
    # numpy in, numpy out, the same call path
    Un, Sn, Vn = P.math.tsqr_svd(X, precision=precision)
    assert isinstance(Un, np.ndarray) and Un.dtype == X.dtype
    np.testing.assert_array_equal(Sn, S)


def test_qr_streaming_matches_reference(golden):
    """init/update_qr_streaming with the reference's own Omegas reproduce its
    Q, B and Y (FP64 data, FP64 form); tsqr's factors carry Householder QR's
    column signs, so the update's Yo + Yn sums the same columns."""
    g = golden("qr_streaming")
    r, q = int(g["r"]), int(g["q"])
    Q1, B1, Y1 = P.math.init_qr_streaming(g["X1"], r, q, omega=g["om1"])
    assert isinstance(Q1, np.ndarray) and Q1.shape == g["Q1"].shape and B1.shape == g["B1"].shape
    np.testing.assert_allclose(Q1, g["Q1"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(B1, g["B1"], rtol=0, atol=1e-10 * np.abs(g["B1"]).max())
    np.testing.assert_allclose(Y1, g["Y1"], rtol=0, atol=1e-10 * np.abs(g["Y1"]).max())
    Yo = Y1.copy()
    Q2, B2, Y2 = P.math.update_qr_streaming(g["X2"], Q1, B1, Yo, r, q, omega=g["om2"])
    assert Y2 is Yo  # Yo += Yn in the caller's array, as the reference does
    np.testing.assert_allclose(Q2, g["Q2"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(B2, g["B2"], rtol=0, atol=1e-10 * np.abs(g["B2"]).max())
    np.testing.assert_allclose(Y2, g["Y2"], rtol=0, atol=1e-10 * np.abs(g["Y2"]).max())


def test_qr_streaming_f32_mixed_and_philox():
    """FP32 batches (mixed form) against the FP64 oracle with the same Omegas,
    and the Philox draws: a seeded init and its updates are deterministic."""
    from pyloworder_gb300 import datagen
    X1 = datagen.pod_field_np(64, 64, 40, 8, seed=31, noise=1e-6).astype(np.float32)
    X2 = datagen.pod_field_np(64, 64, 30, 8, seed=32, noise=1e-6).astype(np.float32)
    # one power step: Y = (A A^T) A Omega spans sigma^3 (3e5 down to 60 for
    # the six leading modes here), all above the 22-bit operand level of the
    # mixed form's tsqr; with q = 2 the spread sigma^5 puts the sixth mode at
    # the operand noise (an FP32 QR would lose it too)
    r, q = 8, 1
    om1 = O.philox_uniform((40, r), 5, np.float32)
    om2 = O.philox_uniform((30, r), 6, np.float32)
    Q1, B1, Y1 = P.math.init_qr_streaming(X1, r, q, omega=om1)
    Q2, B2, Y2 = P.math.update_qr_streaming(X2, Q1, B1, Y1.copy(), r, q, omega=om2)
    q1, b1, y1 = O.init_qr_streaming(X1.astype(np.float64), r, q, omega=om1.astype(np.float64))
    q2, b2, y2 = O.update_qr_streaming(X2.astype(np.float64), q1, b1, y1.copy(), r, q,
                                       omega=om2.astype(np.float64))
    # the leading modes of the streamed basis (U = Q2 Ur over svd(B2))
    Ur, S, _ = np.linalg.svd(B2.astype(np.float64), full_matrices=False)
    ur, s, _ = np.linalg.svd(b2, full_matrices=False)
    assert sigma_rel(S, s, 6) < 1e-4
    assert subspace_angle(Q2 @ Ur[:, :6], q2 @ ur[:, :6]) < 1e-4
    assert orthogonality(Q2) < 1e-5
    # Philox: same seed, same results
    a = P.math.init_qr_streaming(X1, r, q, seed=99)
    ua = P.math.update_qr_streaming(X2, a[0], a[1], a[2].copy(), r, q)
    b = P.math.init_qr_streaming(X1, r, q, seed=99)
    ub = P.math.update_qr_streaming(X2, b[0], b[1], b[2].copy(), r, q)
    np.testing.assert_array_equal(ua[1], ub[1])


def test_randomized_philox_matches_oracle():
    rng = np.random.default_rng(5)
    X = (rng.standard_normal((3000, 12)) @ rng.standard_normal((12, 120))
         + 1e-3 * rng.standard_normal((3000, 120)))
    r, q, seed = 16, 3, 1234
    U, S, V = P.math.randomized_svd(X, r, q, seed=seed)
    assert U.shape == (3000, r) and S.shape == (r,) and V.shape == (r, 120)
    omega = O.philox_uniform((120, r), seed, np.float64)
    Ur, Sr, Vr = O.randomized_svd(X, r, q, omega=omega)
    assert sigma_rel(S, Sr, 12) < 1e-10
    cols_up_to_phase(U[:, :12], Ur[:, :12], 1e-8)
    cols_up_to_phase(V[:12].T, Vr[:12].T, 1e-8)


def test_randomized_f32_mixed_tensor_core():
    """FP32 data take the packed tensor-core passes (A Omega, A^T Q, A Q2)."""
    rng = np.random.default_rng(15)
    X = (rng.standard_normal((20000, 12)) * np.logspace(0, -1.5, 12)) @ rng.standard_normal((12, 300))
    X = (X + 1e-4 * rng.standard_normal(X.shape)).astype(np.float32)
    r, q, seed = 24, 2, 99
    U, S, V = P.math.randomized_svd(X, r, q, seed=seed)
    assert U.dtype == np.float32 and U.shape == (20000, r) and V.shape == (r, 300)
    omega = O.philox_uniform((300, r), seed, np.float32).astype(np.float64)
    Ur, Sr, Vr = O.randomized_svd(X.astype(np.float64), r, q, omega=omega)
    assert sigma_rel(S, Sr, 12) < 1e-5
    assert subspace_angle(U[:, :12], Ur[:, :12]) < 1e-4
    assert subspace_angle(V[:12].T, Vr[:12].T) < 1e-4
    assert orthogonality(U) < 1e-5


def test_randomized_reference_omega_subspace(golden):
    # pyLOM draws Omega with numpy's MT19937; ours is Philox.  Both capture the
    # same dominant subspace: compare sigma and subspaces, not raw vectors.
    g = golden("pod_randomized")
    U, S, V = P.POD.run(g["X"], remove_mean=False, randomized=True, r=int(g["r"]), q=int(g["q"]),
                        seed=int(g["seed"]))
    # signal modes only: below 1e-2 S_1 the field is noise, whose captured
    # directions depend on the test matrix itself
    k = int(np.sum(g["S"] > 1e-2 * g["S"][0]))
    assert k >= 6
    assert sigma_rel(S, g["S"], k) < 1e-8
    assert subspace_angle(U[:, :k], g["U"][:, :k]) < 1e-6


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_matmul_and_matmulp(dtype):
    rng = np.random.default_rng(2)
    A = rng.standard_normal((5000, 96)).astype(dtype)
    B = rng.standard_normal((96, 40)).astype(dtype)
    Q = rng.standard_normal((5000, 40)).astype(dtype)
    tol = 1e-12 if dtype == np.float64 else 2e-5
    ref = A.astype(np.float64) @ B.astype(np.float64)
    np.testing.assert_allclose(P.math.matmul(A, B), ref, rtol=tol, atol=tol * np.abs(ref).max())
    ref2 = A.T.astype(np.float64) @ Q.astype(np.float64)
    got = P.math.matmulp(A.T, Q)
    assert got.shape == (96, 40)
    np.testing.assert_allclose(got, ref2, rtol=tol, atol=tol * np.abs(ref2).max())


def test_matmul_torch_transposed_view():
    rng = np.random.default_rng(3)
    A = torch.tensor(rng.standard_normal((3000, 64)), device="cuda")
    Q = torch.tensor(rng.standard_normal((3000, 8)), device="cuda")
    got = P.math.matmul(A.T, Q)
    assert isinstance(got, torch.Tensor) and got.is_cuda
    ref = A.T.cpu().numpy() @ Q.cpu().numpy()
    np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_tsqr(dtype):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((4000, 50)).astype(dtype)
    Q, R = P.math.tsqr(X)
    tol = 1e-12 if dtype == np.float64 else 5e-6
    assert orthogonality(Q) < tol * 10
    np.testing.assert_allclose(np.tril(R, -1), 0)
    np.testing.assert_allclose(Q.astype(np.float64) @ R, X, atol=tol * 10 * np.abs(X).max())


@pytest.mark.parametrize("tag", ["tall_f64", "tall_f32", "square_f64", "wide_f64", "tsqr_f64",
                                 "tsqr_f32"])
def test_qr_tsqr_reference_factors(golden, tag):
    """qr / tsqr return the reference's own factors (LAPACK Householder QR,
    pyLOM/vmmath/svd.py:29-36 and :50-118 on one rank), column by column with
    no sign freedom: R's diagonal signs are Householder's, computed on the
    device.  FP64 form 1e-10, mixed form (float32 data) 1e-5, both relative
    to the largest entry."""
    g = golden("qr")
    A, Qr, Rr = g[f"{tag}_A"], g[f"{tag}_Q"], g[f"{tag}_R"]
    Q, R = (P.math.tsqr if tag.startswith("tsqr") else P.math.qr)(A)
    assert isinstance(Q, np.ndarray) and Q.dtype == A.dtype and Q.shape == Qr.shape
    assert R.shape == Rr.shape
    tol = 1e-5 if A.dtype == np.float32 else 1e-10
    np.testing.assert_allclose(Q, Qr, rtol=0, atol=tol)
    np.testing.assert_allclose(R, Rr, rtol=0, atol=tol * np.abs(Rr).max())


@pytest.mark.parametrize("m,n", [(5000, 100), (3000, 300), (70, 70), (40000, 33)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_tsqr_householder_signs_multi_panel(m, n, dtype):
    """The device sign rule past its first 32-column panel (n = 33 .. 300,
    square included) gives numpy.linalg.qr's factors."""
    rng = np.random.default_rng(m + n)
    X = rng.standard_normal((m, n)).astype(dtype)
    Q, R = P.math.tsqr(X)
    Qr, Rr = O.qr(X.astype(np.float64))
    tol = 1e-4 if dtype == np.float32 else 1e-10
    assert np.array_equal(np.sign(np.diag(R)), np.sign(np.diag(Rr)))
    np.testing.assert_allclose(Q, Qr, rtol=0, atol=tol)
    np.testing.assert_allclose(R, Rr, rtol=0, atol=tol * np.abs(Rr).max())


@pytest.mark.parametrize("tag", ["f64", "f32"])
@pytest.mark.parametrize("fn", ["randomized_qr", "randomized_qr2"])
def test_randomized_qr_reference_factors(golden, tag, fn):
    """randomized_qr (pyLOM/vmmath/svd.py:121-144; randomized_qr2 at :147
    computes the same factors) with the reference's own Omega returns its Q
    (m x r, Householder signs) and B = Q^T A (r x n), column by column.  FP64:
    1e-10.  float32 (mixed form): 1e-5 on the 9 signal columns; the 10th sits
    on the noise floor (sigma_10 / sigma_11 = 1.03), where the reference's
    own float32 result differs from an FP64 evaluation of the same steps by
    1.3e-3, so it gets 5e-3."""
    g = golden("randomized_qr")
    r, q = int(g["r"]), int(g["q"])
    A = g[f"{tag}_A"]
    Q, B = getattr(P.math, fn)(A, r, q, omega=g[f"{tag}_omega"])
    assert Q.shape == (A.shape[0], r) and B.shape == (r, A.shape[1]) and Q.dtype == A.dtype
    Qr, Br = g[f"{tag}_Q"], g[f"{tag}_B"]
    bmax = np.abs(Br).max()
    if tag == "f64":
        np.testing.assert_allclose(Q, Qr, rtol=0, atol=1e-10)
        np.testing.assert_allclose(B, Br, rtol=0, atol=1e-10 * bmax)
    else:
        np.testing.assert_allclose(Q[:, :9], Qr[:, :9], rtol=0, atol=1e-5)
        np.testing.assert_allclose(B[:9], Br[:9], rtol=0, atol=1e-5 * bmax)
        np.testing.assert_allclose(Q[:, 9], Qr[:, 9], rtol=0, atol=5e-3)
    # the seeded Philox draw matches the oracle on the same Omega
    Qs, Bs = getattr(P.math, fn)(A, r, q, seed=77)
    om = O.philox_uniform((A.shape[1], r), 77, A.dtype)
    Qo, Bo = O.randomized_qr(A.astype(np.float64), r, q, omega=om.astype(np.float64))
    k = 10 if tag == "f64" else 9
    np.testing.assert_allclose(Qs[:, :k], Qo[:, :k], rtol=0, atol=1e-10 if tag == "f64" else 1e-5)


@pytest.mark.parametrize("n", [1024, 1700])
def test_mixed_repeated_calls_identical(n):
    """The same mean-removed input three times: bitwise-identical sigma, U and
    V.  The null direction of mean removal (sigma ~ 1e-8 sigma_1, below the
    22-bit operand level) makes R3^-1 long in a few directions; the columns
    renormalised for it are chosen by an ordered scan and every sum on that
    path is taken in a fixed order, so no run differs from another.
    ||I - U^T U|| is reported and held at the documented level: 1e-4 at
    n = 1,024, 1e-3 at n = 1,700 (32,768 points, noise floor 5e-7 sigma_1)."""
    from pyloworder_gb300 import datagen
    m, k = 32768, 64
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, k, seed=91, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = P.vmmath.remove_mean_device(X, n)
    runs = [P.vmmath.tsqr_svd_device(Y, n, "mixed") for _ in range(3)]
    U0, S0, V0 = runs[0]
    for U, S, V in runs[1:]:
        assert torch.equal(S, S0)
        assert torch.equal(U, U0)
        assert torch.equal(V, V0)
    Ud = U0.double()
    orth = float((Ud.T @ Ud - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max())
    print(f"n = {n}: max |U^T U - I| = {orth:.2e}")
    assert orth < (1e-4 if n <= 1600 else 1e-3)


@pytest.mark.parametrize("m,n,ld", [(1, 1, 1), (5, 1, 1), (64, 64, 64), (1000, 33, 40),
                                    (2049, 129, 129), (300, 500, 500)])
def test_tsqr_svd_shapes(m, n, ld):
    rng = np.random.default_rng(m * 7 + n)
    base = rng.standard_normal((m, ld))
    Xt = torch.tensor(base, device="cuda")[:, :n]  # strided view when ld > n
    U, S, V = P.math.tsqr_svd(Xt)
    X = base[:, :n]
    Sr = np.linalg.svd(X, compute_uv=False)
    k = min(m, n)
    assert U.shape == (m, k) and S.shape == (k,) and V.shape == (k, n)
    assert sigma_normwise(S.cpu().numpy(), Sr) < 1e-12
    Un, Sn, Vn = U.cpu().numpy(), S.cpu().numpy(), V.cpu().numpy()
    np.testing.assert_allclose((Un * Sn) @ Vn, X, atol=1e-11 * np.abs(X).max())


@pytest.mark.parametrize("dtype,precision,tol", [(np.complex128, "fp64", 1e-11),
                                                 (np.complex64, "mixed", 2e-5)])
def test_tsqr_svd_complex(dtype, precision, tol):
    rng = np.random.default_rng(9)
    X = (rng.standard_normal((2000, 24)) + 1j * rng.standard_normal((2000, 24))).astype(dtype)
    U, S, V = P.math.tsqr_svd(X, precision=precision)
    Ur, Sr, Vr = np.linalg.svd(X.astype(np.complex128), full_matrices=False)
    assert sigma_rel(S, Sr) < tol
    cols_up_to_phase(U, Ur, tol * 100)
    np.testing.assert_allclose((U.astype(np.complex128) * S) @ V, X, atol=tol * 10 * np.abs(X).max())


def test_pod_cfg1_full_fp64():
    """cfg1: 128x128 grid x 200 snapshots, FP64, mean removed, truncation at
    residual 1e-6; sigma within 1e-10 (signal modes) of the FP64 oracle."""
    from pyloworder_gb300 import datagen
    X = datagen.pod_field_np(128, 128, 200, 10, seed=1001)
    U, S, V = P.POD.run(X)
    Ur, Sr, Vr = O.pod_run(X)
    assert sigma_rel(S, Sr, 10) < 1e-10
    assert sigma_normwise(S, Sr) < 1e-12
    cols_up_to_phase(U[:, :10], Ur[:, :10], 1e-8)
    Ut, St, Vt = P.POD.truncate(U, S, V, r=1e-6)
    assert Ut.shape[1] == O.pod_truncate(Ur, Sr, Vr, r=1e-6)[0].shape[1]


def test_nonfinite_input_reports_error():
    X = np.ones((100, 4))
    X[3, 2] = np.nan
    with pytest.raises(RuntimeError):
        P.math.tsqr_svd(X)


def test_torch_in_torch_out():
    X = torch.randn(2000, 16, device="cuda", dtype=torch.float64)
    U, S, V = P.POD.run(X)
    assert all(isinstance(t, torch.Tensor) and t.is_cuda for t in (U, S, V))
    Xc = X - X.mean(dim=1, keepdim=True)
    np.testing.assert_allclose(((U * S) @ V).cpu().numpy(), Xc.cpu().numpy(), atol=1e-11)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_tsqr_svd_batched(cplx, precision):
    """Batched API: every problem of the batch against numpy's SVD."""
    rng = np.random.default_rng(21 + cplx)
    b, m, n = 5, 2500, 24
    spread = np.logspace(0, -2, n)
    A = rng.standard_normal((b, m, n)) * spread
    if cplx:
        A = A + 1j * rng.standard_normal((b, m, n)) * spread
    dt = (np.complex64 if cplx else np.float32) if precision == "mixed" else (
        np.complex128 if cplx else np.float64)
    A = A.astype(dt)
    x = torch.tensor(A, device="cuda")
    U, S, V = P.vmmath.tsqr_svd_batched_device(x, precision)
    U, S, V = U.cpu().numpy(), S.cpu().numpy(), V.cpu().numpy()
    tol = 1e-5 if precision == "mixed" else 1e-12
    for p in range(b):
        A64 = A[p].astype(np.complex128 if cplx else np.float64)
        Sr = np.linalg.svd(A64, compute_uv=False)
        assert sigma_rel(S[p], Sr) < tol
        assert orthogonality(U[p].astype(A64.dtype)) < tol * 10
        rec = (U[p].astype(A64.dtype) * S[p]) @ V[p].astype(A64.dtype)
        assert np.linalg.norm(rec - A64) / np.linalg.norm(A64) < tol * 10


def test_mixed_cholesky_of_near_identity_gram_in_closed_form():
    """The Gram of the last CholeskyQR factor sits next to the identity; its
    factor is written in closed form (R = I + triu(E, 1) + diag(E) / 2, exact
    for G perturbed by at most 1e-10 per element; info word 6 counts it) and
    the SVD keeps the mixed form's accuracy against the FP64 form."""
    from pyloworder_gb300 import _lib as L
    m, n = 65536, 384
    g = torch.Generator(device="cuda").manual_seed(4242)
    X = torch.randn(m, n, device="cuda", generator=g, dtype=torch.float32)
    X *= torch.logspace(0, -3, n, device="cuda")  # graded columns
    U, S, V = P.vmmath.tsqr_svd_device(X, n, "mixed")
    info = list(L.last_info)
    assert info[6] >= 1, info
    Ur, Sr, Vr = P.vmmath.tsqr_svd_device(X.double(), n, "fp64")
    s, sr = S.double().cpu().numpy(), Sr.cpu().numpy()
    assert sigma_normwise(s, sr) < 1e-6
    assert sigma_rel(s, sr, 64) < 1e-5
    Ud = U.double()
    assert float((Ud.T @ Ud - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max()) < 1e-5
    R = (Ud * S.double()) @ V.double() - X.double()
    assert float(R.abs().max()) / float(X.abs().max()) < 1e-5
