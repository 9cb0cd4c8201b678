"""Products on SM pairs (2-SM UMMA, tuning key apply_pair) against the single-SM
kernels.  Each output element takes the same products in the same K order in
both kernels (the pair only splits the rows and the W columns of a 256 x 256
tile between two SMs), so the results agree to the last bits; the tests allow
one FP32 rounding of slack."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    from pyloworder_gb300 import _lib as L
    return L, L.load()


class _Tuned:
    def __init__(self, key, value):
        self.key, self.value = key, value

    def __enter__(self):
        L, lib = _lib()
        self.old = lib.plom_get_tuning(self.key.encode())
        assert lib.plom_set_tuning(self.key.encode(), float(self.value)) == 0

    def __exit__(self, *exc):
        L, lib = _lib()
        lib.plom_set_tuning(self.key.encode(), self.old)


def _apply(pk, W):
    from pyloworder_gb300 import vmmath
    infos = []
    C = vmmath._packed_apply(pk, W, infos)
    torch.cuda.synchronize()
    L, _ = _lib()
    for info in infos:
        L.check_info(info, "packed_apply")
    return C


def _profiled(fn):
    L, _ = _lib()
    prof = L.Profiler()
    prof.start()
    try:
        out = fn()
    finally:
        names = prof.stop()
    return out, names


@pytest.mark.parametrize("m,N,k", [(262_344, 320, 300), (131_072, 1024, 1024), (70_000, 192, 1000),
                                   (100, 320, 300), (1, 192, 200)])
def test_packed_apply_pair_matches_single_sm(m, N, k):
    from pyloworder_gb300 import vmmath
    g = torch.Generator(device="cuda").manual_seed(m + N + k)
    X = torch.randn(m, N, device="cuda", generator=g, dtype=torch.float32)
    X[:, 3] *= 1e-3  # columns of different scales
    W = torch.randn(N, k, device="cuda", generator=g, dtype=torch.float64)
    pk = vmmath._pack_dev(X)
    with _Tuned("apply_pair", 0):
        C1, n1 = _profiled(lambda: _apply(pk, W))
    with _Tuned("apply_pair", 1):
        C2, n2 = _profiled(lambda: _apply(pk, W))
    assert "tc_apply_f16x3" in n1 and "tc_apply_f16x3_pair" not in n1
    assert "tc_apply_f16x3_pair" in n2, sorted(n2)
    scale = float(C1.abs().max())
    diff = float((C1 - C2).abs().max())
    assert diff <= 2 ** -22 * scale, (diff, scale)
    # and both against an FP64 product
    ref = (X.double() @ W)
    err = float((C2.double() - ref).abs().max()) / float(ref.abs().max())
    assert err < 1e-5


def test_tsqr_svd_pair_products_match_single_sm():
    """The triangular applies of the CholeskyQR passes and the dense final
    apply on SM pairs (apply_pair = 2) give the single-SM factors."""
    from pyloworder_gb300 import datagen, vmmath
    m, n = 262_144 + 128, 512
    nx, ny = datagen.grid_for_points(m)
    X = datagen.pod_field_device(nx, ny, n, 48, seed=77, noise=1e-5, amp_pow=1.5, m=m)
    Y, _, _ = vmmath.remove_mean_device(X, n)
    del X
    with _Tuned("apply_pair", 0):
        (U1, S1, V1), n1 = _profiled(lambda: vmmath.tsqr_svd_device(Y, n, "mixed"))
    with _Tuned("apply_pair", 2):
        (U2, S2, V2), n2 = _profiled(lambda: vmmath.tsqr_svd_device(Y, n, "mixed"))
    assert n2["tc_apply_f16x3_pair"]["count"] >= 3, sorted(n2)
    assert "tc_apply_f16x3_pair" not in n1
    s1, s2 = S1.double().cpu().numpy(), S2.double().cpu().numpy()
    assert np.max(np.abs(s1 - s2)) <= 1e-6 * s1[0]
    k = 48
    Ua, Ub = U1[:, :k].double(), U2[:, :k].double()
    assert float((Ua - Ub).abs().max()) < 1e-5
    Ud = U2.double()
    assert float((Ud.T @ Ud - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max()) < 1e-4

