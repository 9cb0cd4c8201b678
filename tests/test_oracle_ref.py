"""pyLOM's own compiled tsqr_svd (pyLOM/vmmath/src/svd.c built by
oracle/build_ref.py into oracle/_ref/) against the fixtures pyLOM's py path
produced: the compiled build the CPU baseline times is the reference itself.
Skipped where the build is absent (no pyLOM sources staged, no bundled
OpenBLAS)."""
import numpy as np
import pytest

from oracle import plom_ref as R


def _built():
    if R.available():
        return True
    try:
        from oracle import build_ref
        build_ref.build()
        return R.available()
    except Exception:
        return False


pytestmark = pytest.mark.skipif(not _built(), reason="reference build not available here")


@pytest.mark.parametrize("tag,tol", [("f64", 1e-12), ("f32", 2e-6)])
def test_compiled_tsqr_svd_matches_py_path(golden, tag, tol):
    g = golden("tsqr_svd_" + tag)
    U, S, V = R.tsqr_svd(g["A"])
    assert U.dtype == g["A"].dtype
    np.testing.assert_allclose(S, g["S"], rtol=0, atol=tol * g["S"][0])
    # columns up to sign (LAPACK gesvd vs gesdd may choose other signs)
    for j in range(U.shape[1]):
        a, b = U[:, j].astype(np.float64), g["U"][:, j].astype(np.float64)
        s = np.sign(a @ b)
        assert np.abs(a - s * b).max() < 100 * tol


def test_compiled_kat_example_svd(golden):
    g = golden("kat_example_svd")
    U, S, V = R.tsqr_svd(g["A"])
    np.testing.assert_allclose(S, g["S"], rtol=1e-13)
    np.testing.assert_allclose(np.abs(U), np.abs(g["U"]), atol=1e-13)
