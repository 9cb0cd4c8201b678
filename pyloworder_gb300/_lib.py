"""ctypes binding of libplom.so and the tensor plumbing around it.

Device memory, streams and the caching allocator come from PyTorch; every
computation is a libplom kernel.  There is no CPU fallback: when the library
or a CUDA device is missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libplom.so")

F32, F64, C64, C128 = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
INFO_WORDS = 8
NUM_MESSAGES = {1: "Cholesky breakdown after all shift escalations",
                2: "one-sided Jacobi did not converge",
                3: "non-finite values in the input",
                4: "eigenvalue iteration did not converge",
                5: "a bounded device-side wait expired"}

_lock = threading.Lock()
_lib = None

c_i64 = ctypes.c_int64
c_vp = ctypes.c_void_p
c_int = ctypes.c_int
c_sz = ctypes.c_size_t

# name -> (restype, argtypes); mirrors include/plom.h
PROTOS = {
    "plom_last_error_string": (ctypes.c_char_p, []),
    "plom_version": (c_int, []),
    "plom_set_tuning": (c_int, [ctypes.c_char_p, ctypes.c_double]),
    "plom_get_tuning": (ctypes.c_double, [ctypes.c_char_p]),
    "plom_profile_begin": (c_int, []),
    "plom_profile_end": (c_int, [ctypes.c_char_p, c_sz]),
    "plom_temporal_mean": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp]),
    "plom_subtract_mean": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64, c_vp]),
    "plom_temporal_variance": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "plom_norm_variance": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "plom_remove_mean": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_int, c_vp, c_i64,
                                 c_vp]),
    "plom_matmul_workspace": (c_sz, [c_int, c_int, c_int, c_i64, c_i64, c_i64]),
    "plom_matmul": (c_int, [c_int, c_int, c_int, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_i64, c_i64,
                            c_i64, c_vp, c_sz, c_vp]),
    "plom_tsqr_workspace": (c_sz, [c_int, c_int, c_i64, c_i64]),
    "plom_tsqr": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_vp, c_sz,
                          c_vp, c_vp]),
    "plom_tsqr_svd_workspace": (c_sz, [c_int, c_int, c_i64, c_i64]),
    "plom_tsqr_svd": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp,
                              c_sz, c_vp, c_vp]),
    "plom_spod_modes": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp]),
    "plom_spod_assemble": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "plom_packed_bytes": (c_sz, [c_i64, c_i64]),
    "plom_pack": (c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_sz, c_vp]),
    "plom_packed_apply_workspace": (c_sz, [c_i64, c_i64, c_i64]),
    "plom_packed_apply": (c_int, [c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_vp, c_sz,
                                  c_vp, c_vp]),
    "plom_packed_tn_workspace": (c_sz, [c_i64, c_i64, c_i64]),
    "plom_packed_tn": (c_int, [c_vp, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_vp, c_sz, c_vp, c_vp]),
    "plom_tsqr_svd_host_workspace": (c_sz, [c_int, c_int, c_i64, c_i64]),
    "plom_tsqr_svd_host": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, c_vp,
                                   c_vp, c_sz, c_vp, c_vp]),
    "plom_tsqr_svd_batched_workspace": (c_sz, [c_int, c_int, c_i64, c_i64, c_i64]),
    "plom_tsqr_svd_batched": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp,
                                      c_i64, c_i64, c_vp, c_vp, c_vp, c_sz, c_vp, c_vp]),
    "plom_randomized_svd_workspace": (c_sz, [c_int, c_int, c_i64, c_i64, c_i64]),
    "plom_randomized_svd": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_int,
                                    ctypes.c_uint64, c_vp, c_i64, c_vp, c_vp, c_vp, c_sz, c_vp,
                                    c_vp]),
    "plom_randomized_qr_workspace": (c_sz, [c_int, c_int, c_i64, c_i64, c_i64]),
    "plom_randomized_qr": (c_int, [c_int, c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_int,
                                   ctypes.c_uint64, c_vp, c_vp, c_i64, c_vp, c_vp, c_sz, c_vp,
                                   c_vp]),
    "plom_fill_uniform": (c_int, [c_int, c_vp, c_i64, ctypes.c_uint64, c_vp]),
    "plom_spod_fft": (c_int, [c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_i64, c_i64, c_i64,
                              c_vp, c_vp, c_vp, ctypes.c_double, c_vp, c_vp]),
    "plom_matmulp_static": (c_int, [c_int, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_i64, c_i64, c_i64,
                                    c_vp]),
    "plom_dmd_project_workspace": (c_sz, [c_i64, c_i64, c_i64]),
    "plom_dmd_project": (c_int, [c_vp, c_i64, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp,
                                 c_vp, c_sz, c_vp, c_vp]),
    "plom_dmd_reduced_workspace": (c_sz, [c_i64, c_i64]),
    "plom_dmd_reduced": (c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_sz,
                                 c_vp, c_vp]),
}


class PlomError(RuntimeError):
    pass


def load(build_if_missing: bool = True):
    """Load libplom.so (building it in-tree first when absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIBPATH):
            if not build_if_missing:
                raise PlomError(f"{LIBPATH} missing: run pyloworder_gb300._build.build()")
            from . import _build
            _build.build()
        lib = ctypes.CDLL(LIBPATH)
        for name, (res, args) in PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _apply_tuning(lib)
        _lib = lib
        return lib


TUNING_FILE = os.path.join(HERE, "tuning", "gb300.json")


def _apply_tuning(lib, path=None):
    """Set the kernels' tuning parameters from the tuning file (written by
    pyloworder_gb300.autotune); PLOM_TUNING names another file, and an empty
    PLOM_TUNING keeps the library's defaults."""
    import json
    path = path or os.environ.get("PLOM_TUNING", TUNING_FILE)
    if not path or not os.path.exists(path):
        return {}
    with open(path) as f:
        params = json.load(f).get("params", {})
    for key, value in params.items():
        if lib.plom_set_tuning(key.encode(), float(value)) != 0:
            raise PlomError(f"tuning file {path}: {lib.plom_last_error_string().decode()}")
    return params


def call(name, *args):
    lib = load()
    status = getattr(lib, name)(*args)
    if status != 0:
        msg = lib.plom_last_error_string().decode(errors="replace")
        raise PlomError(f"{name} failed (status {status}): {msg}")
    return status


# --------------------------------------------------------------------------
# tensors
# --------------------------------------------------------------------------

def torch():
    import torch as _t
    return _t


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise PlomError("pyloworder_gb300 needs a CUDA GPU (GB300, sm_103a); none is available")
    return t


class Converted:
    """Input array moved to the device, plus how to hand results back.

    Results for a host torch tensor in page-locked memory come back in
    page-locked memory too (torch's pinned-memory cache: repeated calls of
    the same size reuse the same blocks, and device-to-host copies run at the
    DMA rate instead of the first-touch rate of fresh pageable pages)."""

    def __init__(self, tensor, kind, device, pinned=False):
        self.t = tensor
        self.kind = kind      # 'numpy' | 'torch'
        self.device = device  # original torch device for kind == 'torch'
        self.pinned = pinned

    def back(self, x):
        if self.kind == "numpy":
            return x.cpu().numpy()
        if x.device == self.device:
            return x
        if self.device.type == "cpu" and self.pinned:
            out = torch().empty(x.shape, dtype=x.dtype, pin_memory=True)
            out.copy_(x)
            return out
        return x.to(self.device)


def to_device(A, dtype=None):
    """numpy array / torch tensor -> CUDA torch tensor (no copy when already
    a CUDA tensor of the right dtype with unit inner stride)."""
    t = require_cuda()
    pinned = False
    if isinstance(A, t.Tensor):
        kind, dev = "torch", A.device
        x = A
        if x.device.type != "cuda":
            pinned = bool(x.is_pinned())
            x = x.to("cuda")
    else:
        kind, dev = "numpy", None
        arr = np.asarray(A)
        x = t.from_numpy(np.ascontiguousarray(arr)).to("cuda")
    if dtype is not None and x.dtype != dtype:
        x = x.to(dtype)
    return Converted(x, kind, dev, pinned)


def dtype_code(x):
    t = torch()
    return {t.float32: F32, t.float64: F64, t.complex64: C64, t.complex128: C128}[x.dtype]


def real_dtype(x):
    t = torch()
    return {t.float32: t.float32, t.float64: t.float64, t.complex64: t.float32,
            t.complex128: t.float64}[x.dtype]


def rows_ld(x):
    """Leading dimension of a 2-D tensor with unit inner stride (else None)."""
    if x.dim() != 2:
        return None
    if x.shape[1] <= 1:
        return max(1, x.shape[1]) if x.stride(0) >= x.shape[1] or x.shape[0] <= 1 else None
    if x.stride(1) != 1:
        return None
    return x.stride(0)


def as_rows(x):
    """(tensor, ld) with unit inner stride; copies only when needed."""
    ld = rows_ld(x)
    if ld is None or ld < x.shape[1]:
        x = x.contiguous()
        ld = max(1, x.shape[1])
    if x.data_ptr() % 16 and x.element_size() >= 4:
        pass  # kernels handle unaligned rows on their scalar paths
    return x, ld


def stream_ptr():
    t = torch()
    return ctypes.c_void_p(t.cuda.current_stream().cuda_stream)


def ptr(x):
    return ctypes.c_void_p(x.data_ptr()) if x is not None else ctypes.c_void_p(0)


def workspace(nbytes):
    t = torch()
    return t.empty(max(int(nbytes), 256), dtype=t.uint8, device="cuda")


def new_info():
    t = torch()
    return t.zeros(INFO_WORDS, dtype=t.int32, device="cuda")


last_info = None  # info words of the most recent checked call (diagnostics)


def check_info(info, what):
    global last_info
    v = info.cpu().tolist()
    last_info = v
    if v[0] != 0:
        raise PlomError(f"{what}: {NUM_MESSAGES.get(v[0], 'numerical failure')} (info={v})")
    return v


class Profiler:
    """Per-kernel CUDA-event timings of libplom launches made on this thread
    (plom_profile_begin / plom_profile_end)."""

    def start(self):
        call("plom_profile_begin")

    def stop(self):
        buf = ctypes.create_string_buffer(1 << 16)
        call("plom_profile_end", buf, len(buf))
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms, fl, by, nl = line.split()
            out[name] = {"name": name, "count": int(cnt), "ms_total": float(ms),
                         "flops": float(fl), "bytes": float(by), "launches": int(nl)}
        return out


def precision_code(precision, x):
    t = torch()
    if precision is None:
        return PREC_FP64 if x.dtype in (t.float64, t.complex128) else PREC_MIXED
    p = str(precision).lower()
    if p in ("fp64", "double", "float64"):
        return PREC_FP64
    if p in ("mixed", "fp32"):
        return PREC_MIXED
    raise ValueError(f"precision must be 'fp64' or 'mixed', got {precision!r}")
