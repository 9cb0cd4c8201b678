"""plom_matmulp_static, the allocation-free variant of the reduction product
C = A^T B (matmulp(A.T, B)), for callers that cannot allocate device memory
(another framework owns the device's memory pool, or a loop must not pay the
device synchronisation of cudaMalloc/cudaFree).  It keeps its split-K
partials in a static device array instead of a caller workspace.

Checked through the C ABI against the existing entry point plom_matmul
(transA = 1, FP64 accumulation) on two calls in a row, with the tolerance the
other product tests use; a result too large for the static array must be
rejected before anything runs.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from pyloworder_gb300 import _lib as L  # noqa: E402

STATIC_BYTES = 32 << 20


def _existing(lib, dt, A, B, m, n, k):
    C = torch.empty((m, n), dtype=A.dtype, device="cuda")
    ws = L.workspace(lib.plom_matmul_workspace(dt, L.PREC_FP64, 1, m, n, k))
    st = lib.plom_matmul(dt, L.PREC_FP64, 1, L.ptr(A), m, L.ptr(B), n, L.ptr(C), n, m, n, k,
                         L.ptr(ws), ws.numel(), L.stream_ptr())
    assert st == 0, lib.plom_last_error_string()
    return C


def _static(lib, dt, A, B, m, n, k):
    C = torch.full((m, n), float("nan"), dtype=A.dtype, device="cuda")
    st = lib.plom_matmulp_static(dt, L.ptr(A), m, L.ptr(B), n, L.ptr(C), n, m, n, k, L.stream_ptr())
    assert st == 0, lib.plom_last_error_string()
    return C


@pytest.mark.parametrize("dtype,code,rtol", [(torch.float64, L.F64, 1e-12), (torch.float32, L.F32, 2e-5)])
def test_static_scratch_matches_existing_entry_point(dtype, code, rtol):
    lib = L.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    # two calls in a row, different shapes: the second must not see the first's leftovers
    for (m, n, k) in [(96, 40, 50000), (64, 80, 123457)]:
        A = torch.randn((k, m), dtype=dtype, device="cuda", generator=g)
        B = torch.randn((k, n), dtype=dtype, device="cuda", generator=g)
        ref = _existing(lib, code, A, B, m, n, k)
        got = _static(lib, code, A, B, m, n, k)
        torch.cuda.synchronize()
        scale = float(ref.abs().max())
        np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=rtol,
                                   atol=rtol * scale)


def _leading(lib, dt, dtype, m, n, k, lda, ldb, ldc, seed):
    """Operands with leading dimensions larger than the matrices; both entry
    points see the same padded buffers."""
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    A = torch.randn((max(k, 1), lda), dtype=dtype, device="cuda", generator=g)
    B = torch.randn((max(k, 1), ldb), dtype=dtype, device="cuda", generator=g)
    C1 = torch.full((m, ldc), 7.0, dtype=dtype, device="cuda")
    C2 = torch.full((m, ldc), 7.0, dtype=dtype, device="cuda")
    ws = L.workspace(lib.plom_matmul_workspace(dt, L.PREC_FP64, 1, m, n, k))
    st = lib.plom_matmul(dt, L.PREC_FP64, 1, L.ptr(A), lda, L.ptr(B), ldb, L.ptr(C1), ldc, m, n, k,
                         L.ptr(ws), ws.numel(), L.stream_ptr())
    assert st == 0, lib.plom_last_error_string()
    st = lib.plom_matmulp_static(dt, L.ptr(A), lda, L.ptr(B), ldb, L.ptr(C2), ldc, m, n, k,
                                 L.stream_ptr())
    assert st == 0, lib.plom_last_error_string()
    torch.cuda.synchronize()
    return C1, C2


def test_static_scratch_few_chunks_large_k():
    """m = n = 1024 and a long k: 8 MiB of partials per chunk, so only three
    chunks fit in the 32 MiB array and the split-K is lowered to fit it."""
    lib = L.load()
    m = n = 1024
    k = 300000
    C1, C2 = _leading(lib, L.F64, torch.float64, m, n, k, m, n, n, 5)
    scale = float(C1.abs().max())
    np.testing.assert_allclose(C2.cpu().numpy(), C1.cpu().numpy(), rtol=1e-12, atol=1e-12 * scale)


@pytest.mark.parametrize("dtype,code,rtol", [(torch.float64, L.F64, 1e-12), (torch.float32, L.F32, 2e-5)])
def test_static_scratch_padded_leading_dimensions(dtype, code, rtol):
    """lda > m, ldb > n and ldc > n: only the m x n block of C is written."""
    lib = L.load()
    m, n, k = 70, 45, 20011
    C1, C2 = _leading(lib, code, dtype, m, n, k, m + 13, n + 7, n + 9, 6)
    scale = float(C1[:, :n].abs().max())
    np.testing.assert_allclose(C2[:, :n].cpu().numpy(), C1[:, :n].cpu().numpy(), rtol=rtol,
                               atol=rtol * scale)
    assert torch.all(C2[:, n:] == 7.0)


def test_static_scratch_empty_sum():
    """k = 0: C is the empty sum, zero, whatever the array held before."""
    lib = L.load()
    m, n = 33, 17
    A = torch.randn((50, m), dtype=torch.float64, device="cuda")
    B = torch.randn((50, n), dtype=torch.float64, device="cuda")
    C = torch.empty((m, n), dtype=torch.float64, device="cuda")
    assert lib.plom_matmulp_static(L.F64, L.ptr(A), m, L.ptr(B), n, L.ptr(C), n, m, n, 50,
                                   L.stream_ptr()) == 0
    C.fill_(float("nan"))
    assert lib.plom_matmulp_static(L.F64, L.ptr(A), m, L.ptr(B), n, L.ptr(C), n, m, n, 0,
                                   L.stream_ptr()) == 0
    torch.cuda.synchronize()
    assert torch.all(C == 0.0)


def test_result_beyond_static_scratch_is_rejected():
    lib = L.load()
    m = n = 2048  # 2048 * 2048 * 8 bytes = 32 MiB of partials + tile list > the array
    A = torch.zeros((4, m), dtype=torch.float64, device="cuda")
    B = torch.zeros((4, n), dtype=torch.float64, device="cuda")
    C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    st = lib.plom_matmulp_static(L.F64, L.ptr(A), m, L.ptr(B), n, L.ptr(C), n, m, n, 4,
                                 L.stream_ptr())
    assert st == -2  # PLOM_ERR_WORKSPACE
    assert b"static scratch" in lib.plom_last_error_string()
