"""The CPU oracle against the fixtures produced by pyLOM's own py path.

These pin the oracle: every later GPU parity test trusts it only because these
pass.  Singular vectors are compared up to sign (real) and DMD modes up to the
ordering pyLOM itself produces.
"""
import numpy as np
import pytest

from oracle import plom_oracle as O


def _cols_match_up_to_sign(A, B, tol):
    for j in range(A.shape[1]):
        a, b = A[:, j], B[:, j]
        s = np.sign(np.vdot(a, b).real) or 1.0
        assert np.max(np.abs(a - s * b)) <= tol * max(1.0, np.max(np.abs(b))), j


def test_kat_example_svd(golden):
    g = golden("kat_example_svd")
    U, S, V = O.tsqr_svd(g["A"])
    np.testing.assert_allclose(S, g["S"], rtol=1e-14)
    _cols_match_up_to_sign(U, g["U"], 1e-13)
    _cols_match_up_to_sign(V.T, g["V"].T, 1e-13)
    np.testing.assert_allclose(S, [14.2690954, 0.62682823], rtol=1e-7)


@pytest.mark.parametrize("tag,rtol", [("f64", 1e-13), ("f32", 2e-5)])
def test_tsqr_svd(golden, tag, rtol):
    g = golden("tsqr_svd_" + tag)
    U, S, V = O.tsqr_svd(g["A"])
    assert U.dtype == g["U"].dtype and S.dtype == g["S"].dtype
    np.testing.assert_allclose(S, g["S"], rtol=rtol)
    _cols_match_up_to_sign(U, g["U"], 100 * rtol)


def test_averaging(golden):
    g = golden("averaging")
    m = O.temporal_mean(g["X"])
    np.testing.assert_allclose(m, g["mean"], rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(O.subtract_mean(g["X"], m), g["Y"], rtol=1e-15, atol=1e-15)
    v = O.temporal_variance(g["X"], m)
    np.testing.assert_allclose(v, g["var"], rtol=1e-14)
    np.testing.assert_allclose(O.norm_variance(g["X"], m, v), g["Yv"], rtol=1e-13)


def test_pod_cfg1_small(golden):
    g = golden("pod_cfg1_small")
    U, S, V = O.pod_run(g["X"])
    np.testing.assert_allclose(S, g["S"], rtol=1e-10, atol=1e-13 * S[0])
    k = 10
    _cols_match_up_to_sign(U[:, :k], g["U"][:, :k], 1e-8)
    Ut, St, Vt = O.pod_truncate(U, S, V, r=1e-6)
    assert Ut.shape[1] == int(g["N_res"])
    assert O.pod_truncate(U, S, V, r=-0.99)[0].shape[1] == int(g["N_energy"])
    Xr = O.pod_reconstruct(Ut, St, Vt)
    np.testing.assert_allclose(Xr, g["Xr"], atol=1e-12)


def test_pod_divvar_and_f32(golden):
    g = golden("pod_divvar")
    U, S, V = O.pod_run(g["X"], divide_variance=True)
    np.testing.assert_allclose(S, g["S"], rtol=1e-10, atol=1e-13 * S[0])
    g = golden("pod_f32_nomean")
    U, S, V = O.pod_run(g["X"], remove_mean=False)
    assert S.dtype == np.float32
    np.testing.assert_allclose(S[:10], g["S"][:10], rtol=1e-4)


def test_truncation(golden):
    g = golden("truncation")
    for r, N in zip(g["r"], g["N"]):
        assert O.compute_truncation_residual(g["S"], float(r)) == int(N)


def test_randomized_numpy_omega(golden):
    g = golden("pod_randomized")
    U, S, V = O.pod_run(g["X"], remove_mean=False, randomized=True, r=int(g["r"]), q=int(g["q"]),
                        seed=int(g["seed"]))
    np.testing.assert_allclose(S, g["S"], rtol=1e-10)
    _cols_match_up_to_sign(U, g["U"], 1e-8)


@pytest.mark.parametrize("tag", ["tall_f64", "tall_f32", "square_f64", "wide_f64", "tsqr_f64",
                                 "tsqr_f32"])
def test_qr_and_tsqr(golden, tag):
    """qr / tsqr reproduce the reference's Householder factors, signs
    included; the sign rule applied to CholeskyQR-signed factors (positive
    R diagonal) recovers them."""
    g = golden("qr")
    A, Qr, Rr = g[f"{tag}_A"], g[f"{tag}_Q"], g[f"{tag}_R"]
    tol = 1e-5 if A.dtype == np.float32 else 1e-12
    Q, R = (O.tsqr if tag.startswith("tsqr") else O.qr)(A)
    np.testing.assert_allclose(Q, Qr, rtol=0, atol=tol)
    np.testing.assert_allclose(R, Rr, rtol=0, atol=tol * np.abs(Rr).max())
    if A.shape[0] >= A.shape[1]:
        d = np.sign(np.diag(Rr))
        Qc = Qr * d  # CholeskyQR's factor: R with a positive diagonal
        s = O.householder_signs(Qc)
        np.testing.assert_array_equal(s, d)


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_randomized_qr(golden, tag):
    """randomized_qr with the reference's seed and with its Omega passed in;
    randomized_qr2 returns the same factors."""
    g = golden("randomized_qr")
    r, q, seed = int(g["r"]), int(g["q"]), int(g["seed"])
    A = g[f"{tag}_A"]
    tol = 2e-4 if tag == "f32" else 1e-10
    for kw in ({"seed": seed}, {"omega": g[f"{tag}_omega"]}):
        Q, B = O.randomized_qr(A, r, q, **kw)
        np.testing.assert_allclose(Q, g[f"{tag}_Q"], rtol=0, atol=tol)
        np.testing.assert_allclose(B, g[f"{tag}_B"], rtol=0, atol=tol * np.abs(g[f"{tag}_B"]).max())
    np.testing.assert_array_equal(g[f"{tag}_Q2"], g[f"{tag}_Q"])
    np.testing.assert_array_equal(g[f"{tag}_B2"], g[f"{tag}_B"])


def test_pca(golden):
    g = golden("pca")
    U, sc = O.pca_run(g["X"])
    _cols_match_up_to_sign(U[:, :10], g["U"][:, :10], 1e-8)
    _cols_match_up_to_sign(sc[:, :10], g["scores"][:, :10], 1e-8)
    U2, sc2 = O.pca_run(g["X"], divide_variance=False)
    _cols_match_up_to_sign(U2[:, :10], g["U_nv"][:, :10], 1e-8)
    _cols_match_up_to_sign(sc2[:, :10], g["scores_nv"][:, :10], 1e-8)


def test_qr_streaming(golden):
    """init/update_qr_streaming with the reference's own Omegas."""
    g = golden("qr_streaming")
    r, q = int(g["r"]), int(g["q"])
    Q1, B1, Y1 = O.init_qr_streaming(g["X1"], r, q, omega=g["om1"])
    np.testing.assert_allclose(Q1, g["Q1"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B1, g["B1"], rtol=0, atol=1e-10 * np.abs(g["B1"]).max())
    np.testing.assert_allclose(Y1, g["Y1"], rtol=0, atol=1e-10 * np.abs(g["Y1"]).max())
    Q2, B2, Y2 = O.update_qr_streaming(g["X2"], Q1, B1, Y1, r, q, omega=g["om2"])
    assert B2.shape == (r, g["X1"].shape[1] + g["X2"].shape[1])
    np.testing.assert_allclose(Q2, g["Q2"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(B2, g["B2"], rtol=0, atol=1e-10 * np.abs(g["B2"]).max())
    np.testing.assert_allclose(Y2, g["Y2"], rtol=0, atol=1e-10 * np.abs(g["Y2"]).max())
    # the seeded draw is the reference's: seed(7), then the global stream
    Qs, Bs, Ys = O.init_qr_streaming(g["X1"], r, q, seed=int(g["seed"]))
    np.testing.assert_allclose(Qs, g["Q1"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", ["dmd_small", "dmd_small_mean"])
def test_dmd(golden, name):
    g = golden(name)
    muR, muI, Phi, b = O.dmd_run(g["X"], float(g["r"]), remove_mean=(name == "dmd_small_mean"))
    np.testing.assert_allclose(muR, g["muReal"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(muI, g["muImag"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(np.abs(b), np.abs(g["bJov"]), rtol=1e-7)
    np.testing.assert_allclose(b * Phi, g["bJov"] * g["Phi"], rtol=1e-6, atol=1e-9 * np.abs(b[0] * Phi).max())


def test_dmd_small_true_eigs(golden):
    g = golden("dmd_small")
    lam = np.concatenate([g["lam"], np.conj(g["lam"])])
    mu = g["muReal"] + 1j * g["muImag"]
    for l in lam:
        assert np.min(np.abs(mu - l)) < 1e-4  # noise 1e-5 limits recovery
    d, w = O.dmd_frequency_damping(g["muReal"], g["muImag"], 0.1)
    np.testing.assert_allclose(d, g["delta"], rtol=1e-12)
    np.testing.assert_allclose(w, g["omega"], rtol=1e-12)
    Xr = O.dmd_reconstruction_jovanovic(g["Phi"], g["muReal"], g["muImag"], np.arange(48.0), g["bJov"])
    np.testing.assert_allclose(Xr, g["Xrec"], atol=1e-10)


@pytest.mark.parametrize("tag,rtol", [("f64", 1e-9), ("f32", 2e-3)])
def test_spod(golden, tag, rtol):
    g = golden("spod_" + tag)
    L, P, f = O.spod_run(g["X"], g["t"], nDFT=int(g["nDFT"]), nolap=int(g["nolap"]))
    np.testing.assert_allclose(f, g["f"], rtol=1e-12)
    np.testing.assert_allclose(L[:, :3], g["L"][:, :3], rtol=rtol, atol=rtol * 1e-3 * L.max())


def test_spod_defaults(golden):
    g = golden("spod_defaults")
    L, P, f = O.spod_run(g["X"], g["t"])
    assert L.shape == g["L"].shape and P.shape == g["P"].shape
    np.testing.assert_allclose(L, g["L"], rtol=1e-8, atol=1e-12 * L.max())


def test_hammwin(golden):
    g = golden("hammwin")
    np.testing.assert_allclose(O.hammwin(7), g["w7"], rtol=1e-15)
    np.testing.assert_allclose(O.hammwin(256), g["w256"], rtol=1e-15)


def test_philox_known_answer():
    # Philox4x32-10 known-answer vector (Salmon et al. Random123 kat_vectors:
    # counter = 0, key = 0 -> 6627e8d5 e169c58d bc57ac4c 9b00dbd8); our
    # mapping uses word 0 for float32.
    u = O.philox_uniform((1,), 0, np.float32)
    assert abs(float(u[0]) - (0x6627e8d5 >> 8) / 16777216.0) < 1e-12
