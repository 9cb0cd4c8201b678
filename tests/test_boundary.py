"""The C ABI boundary without a GPU: the library builds/loads, exports every
symbol include/plom.h declares, answers workspace queries and rejects bad
arguments with an error status (no kernel is launched)."""
import ctypes
import os
import re

import pytest

from pyloworder_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"\b(plom_\w+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol():
    lib = L.load()
    names = declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_match_header():
    assert set(L.PROTOS) == set(declared_symbols())


def test_workspace_queries():
    lib = L.load()
    m, n = 8388608, 1024
    mixed = lib.plom_tsqr_svd_workspace(L.F32, L.PREC_MIXED, m, n)
    fp64 = lib.plom_tsqr_svd_workspace(L.F32, L.PREC_FP64, m, n)
    # mixed: one FP32 m x n buffer (Q1 lives in U) plus the Gram's FP32
    # sub-chunk slabs (20 tiles of 128 x 256 x 2,048 sub-chunks of 4,096 rows x
    # 128 KiB = 5 GiB) and their FP64 diagonals; FP64: two FP64 buffers
    slabs = 20 * (m // 4096) * 128 * 256 * 4
    assert 4 * m * n + slabs <= mixed < 4 * m * n + slabs + (2 << 30)
    assert 16 * m * n <= fp64 < 16 * m * n + (1 << 30)
    # mixed randomized: A packed once (4 m n bytes), Q packed (pitch 128), Y and
    # Q in FP32, and the packed CholeskyQR of the m x r sketch (two pitch-128
    # operands)
    rs = lib.plom_randomized_svd_workspace(L.F32, L.PREC_MIXED, m, n, 80)
    assert 4 * m * n <= rs < 4 * m * n + 4 * m * 128 * 3 + 8 * m * 80 + (1 << 30)
    assert lib.plom_matmul_workspace(L.F64, L.PREC_FP64, 1, 1024, 80, m) > 0
    # DMD projection on the 2,097,152 x 512 workload (r = 32): the point
    # reductions' chunk partials and the small FP64 factors, well under 1 GiB;
    # invalid shapes (r >= n, r > 1024) report 0
    dp = lib.plom_dmd_project_workspace(2097152, 512, 32)
    assert 0 < dp < (1 << 30)
    assert lib.plom_dmd_project_workspace(1000, 10, 10) == 0
    assert lib.plom_dmd_project_workspace(100000, 2000, 1025) == 0


@pytest.mark.parametrize("args", [
    dict(prec=7), dict(m=0), dict(n=0), dict(ldx=3), dict(ws_bytes=16),
])
def test_bad_arguments_rejected(args):
    lib = L.load()
    p = dict(dtype=L.F64, prec=L.PREC_FP64, m=100, n=8, ldx=8, ws_bytes=1 << 30)
    p.update(args)
    dummy = ctypes.c_void_p(16)
    st = lib.plom_tsqr_svd(p["dtype"], p["prec"], dummy, p["m"], p["n"], p["ldx"], dummy, 8, dummy,
                           dummy, dummy, p["ws_bytes"], dummy, None)
    assert st < 0
    assert lib.plom_last_error_string()


def test_matmul_rejects_bad_transA():
    lib = L.load()
    d = ctypes.c_void_p(16)
    assert lib.plom_matmul(L.F32, 1, 5, d, 4, d, 4, d, 4, 4, 4, 4, d, 0, None) == L.PLOM_ERR_ARG if hasattr(L, "PLOM_ERR_ARG") else -1


@pytest.mark.parametrize("dtype", [0, 1, 2, 3])
@pytest.mark.parametrize("prec", [0, 1])
def test_workspace_dry_runs_launch_nothing(dtype, prec):
    # A query walks the whole driver with a null arena; any kernel launch in
    # that walk fails here (no GPU) and the query reports 0.
    lib = L.load()
    for m, n in [(16384, 200), (8388608, 1024), (5, 1), (1000, 33), (300, 64)]:
        assert lib.plom_tsqr_svd_workspace(dtype, prec, m, n) > 0, lib.plom_last_error_string()
    for m, n in [(8388608, 1024), (100000, 50), (5, 1), (1000, 33)]:
        assert lib.plom_tsqr_svd_host_workspace(dtype, prec, m, n) > 0, lib.plom_last_error_string()
    for b, m, n in [(1, 2500, 24), (5, 2500, 24), (129, 65536, 63), (3, 5, 1)]:
        assert lib.plom_tsqr_svd_batched_workspace(dtype, prec, b, m, n) > 0, \
            lib.plom_last_error_string()
    if dtype in (0, 1):
        assert lib.plom_tsqr_workspace(dtype, prec, 4000, 50) > 0
        assert lib.plom_randomized_svd_workspace(dtype, prec, 3000, 120, 16) > 0
        for tA in (0, 1):
            assert lib.plom_matmul_workspace(dtype, prec, tA, 100, 20, 30) > 0


def test_tuning_parameters_round_trip_and_range():
    lib = L.load()
    keys = [b"gram_wave_mult", b"gram_wide_wave_mult", b"reduce_blocks_per_sm", b"apply_dense_tn", b"apply_dense_by_rows",
            b"pass1_chunks", b"apply_pair", b"apply_tri_by_rows"]
    old = {k: lib.plom_get_tuning(k) for k in keys}
    try:
        assert all(v >= 0 for v in old.values())
        assert lib.plom_set_tuning(b"gram_wave_mult", 2.0) == 0
        assert lib.plom_get_tuning(b"gram_wave_mult") == 2.0
        assert lib.plom_set_tuning(b"apply_dense_tn", 192.0) != 0  # 128 or 256 only
        assert lib.plom_set_tuning(b"gram_wave_mult", 2.5) != 0    # integers only
        assert lib.plom_set_tuning(b"apply_pair", 3.0) != 0        # 0, 1 or 2
        assert lib.plom_set_tuning(b"no_such_key", 1.0) != 0
        assert lib.plom_get_tuning(b"no_such_key") == -1.0
    finally:
        for k, v in old.items():
            lib.plom_set_tuning(k, v)


def test_committed_tuning_file_is_valid():
    import json
    with open(L.TUNING_FILE) as f:
        params = json.load(f)["params"]
    lib = L.load()
    old = {k: lib.plom_get_tuning(k.encode()) for k in params}
    try:
        for k, v in params.items():
            assert lib.plom_set_tuning(k.encode(), float(v)) == 0, (k, v)
    finally:
        for k, v in old.items():
            lib.plom_set_tuning(k.encode(), v)
