"""Tensor-core (tcgen05, fp16-pair) kernels of the mixed form against FP64
products: the tall apply (through math.matmul on float32) and the Gram
(through math.tsqr on float32, whose R^T R must reproduce X^T X).

Tolerance: 3e-6 relative to the product magnitude (|A||W| per entry), the
fp16 hi/lo operand pairs (22 significant bits, three products) being
FP32-accurate to ~2^-22."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pyloworder_gb300 as P  # noqa: E402


@pytest.mark.parametrize("m,K,n", [(128, 32, 128), (1000, 96, 40), (4097, 200, 130),
                                   (70000, 1024, 256), (333, 7, 3)])
def test_tc_apply_matches_fp64(m, K, n):
    rng = np.random.default_rng(m + K + n)
    A = rng.standard_normal((m, K)).astype(np.float32)
    B = rng.standard_normal((K, n)).astype(np.float32)
    C = P.math.matmul(A, B, precision="mixed")
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    err = np.max(np.abs(C - ref) / scale)
    assert err < 3e-6, err


@pytest.mark.parametrize("m,n", [(5000, 64), (9000, 130), (100000, 256), (4096 * 3 + 17, 300)])
def test_tc_gram_through_tsqr(m, n):
    rng = np.random.default_rng(m + n)
    X = rng.standard_normal((m, n)).astype(np.float32)
    Q, R = P.math.tsqr(X, precision="mixed")
    Q64 = Q.astype(np.float64)
    orth = np.linalg.norm(np.eye(n) - Q64.T @ Q64, 2)
    assert orth < 5e-6, orth
    rec = np.max(np.abs(Q64 @ R.astype(np.float64) - X)) / np.max(np.abs(X))
    assert rec < 5e-6, rec
