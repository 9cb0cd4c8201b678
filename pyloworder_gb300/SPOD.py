"""pyLOM.SPOD hot path on GB300.

SPOD.run follows pyLOM/SPOD/wrapper.py:24-95: mean removal, Welch blocks
(nDFT, nolap), window, FFT along time with pyLOM's scaling and one-sided
doubling, one TSQR-SVD per frequency of the M x nBlks block matrix, P = Re(U)
laid out as pyLOM lays it out, L = |S|^2, frequencies sorted by L[:, 0].

``window='hamming'`` (default) is the reference's window
(pyLOM/vmmath/fft.py:17); ``window='hann'`` is the symmetric Hann window.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L
from . import vmmath as M

__all__ = ["run"]

SVD_BATCH_MAX = 64  # frequencies per batched SVD


def _window(name, n):
    i = np.arange(n)
    if name == "hamming":
        return 0.54 - 0.46 * np.cos(2 * np.pi * i / (n - 1))
    if name == "hann":
        return 0.5 - 0.5 * np.cos(2 * np.pi * i / (n - 1))
    raise ValueError("window must be 'hamming' or 'hann'")


def spod_fft_device(Y, ldy, nDFT, nolap, nBlks, nf, win, scale, mean=None):
    """Q[f] (M x nBlks complex) for every frequency bin, as one device array;
    `mean` (M values on the device) is subtracted from each point's samples
    as they are loaded."""
    t = L.torch()
    Mrows, N = Y.shape
    rdt = Y.dtype
    cdt = t.complex128 if rdt == t.float64 else t.complex64
    Q = t.empty((nf, Mrows, nBlks), dtype=cdt, device="cuda")
    j = np.arange(nDFT)
    wd = t.tensor(win, dtype=rdt, device="cuda")
    twr = t.tensor(np.cos(2 * np.pi * j / nDFT), dtype=rdt, device="cuda")
    twi = t.tensor(-np.sin(2 * np.pi * j / nDFT), dtype=rdt, device="cuda")
    L.call("plom_spod_fft", L.dtype_code(Y), L.ptr(Y), Mrows, N, ldy, L.ptr(mean), nDFT,
           nDFT - nolap, nBlks, nf, L.ptr(wd), L.ptr(twr), L.ptr(twi), float(scale), L.ptr(Q),
           L.stream_ptr())
    return Q


def _svd_batch(Q, nBlks, precision):
    """Frequencies per batched SVD: half of the free device memory (the
    driver's free memory plus what torch's caching allocator holds unused)
    over the per-frequency footprint (workspace + U), at most SVD_BATCH_MAX."""
    t = L.torch()
    nf, Mrows = Q.shape[0], Q.shape[1]
    dt = L.dtype_code(Q)
    prec = L.precision_code(precision, Q)
    per = (L.load().plom_tsqr_svd_batched_workspace(dt, prec, 2, Mrows, nBlks)
           - L.load().plom_tsqr_svd_batched_workspace(dt, prec, 1, Mrows, nBlks))
    per = max(per, 1) + Q[0].numel() * Q.element_size()
    free = t.cuda.mem_get_info()[0] + t.cuda.memory_reserved() - t.cuda.memory_allocated()
    return int(max(1, min(nf, SVD_BATCH_MAX, (free // 2) // per)))


def run_device(x, ld, t_host, nDFT=0, nolap=0, remove_mean=True, window="hamming", precision=None):
    t = L.torch()
    Mrows, N = x.shape
    dt = float(t_host[1] - t_host[0])
    if nDFT == 0:
        nDFT = int(np.power(2, np.floor(np.log2(N / 10))))
    win = _window(window, nDFT)
    if nolap == 0:
        nolap = int(np.floor(nDFT / 2))
    nBlks = int(np.floor((N - nolap) / (nDFT - nolap)))
    if nBlks < 1:
        raise ValueError("SPOD: not enough snapshots for one block")
    winWeight = 1 / np.mean(win)
    # the temporal mean is removed as the FFT stage loads the samples (no
    # centred copy of the snapshots)
    mean = M.temporal_mean_device(x, ld) if remove_mean else None
    f = np.arange(np.ceil(nDFT / 2) + 1) / dt / nDFT
    nf = f.shape[0]
    Q = spod_fft_device(x, ld, nDFT, nolap, nBlks, nf, win, winWeight / nDFT / math.sqrt(nBlks),
                        mean=mean)
    del mean
    Lm = t.empty((nf, nBlks), dtype=x.dtype, device="cuda")
    rows = Mrows * nBlks
    P = t.empty((rows, nf), dtype=x.dtype, device="cuda")
    # P[i + M*b, f] = Re U_f[i, b]
    # the per-frequency SVDs run as batches of frequencies (one launch per
    # stage for the whole batch), as many per batch as device memory allows
    group = _svd_batch(Q, nBlks, precision)
    # the mode-layout kernel stages group x nBlks real parts per point
    group = max(1, min(group, (48 * 1024) // (x.element_size() * (nBlks | 1))))
    # a batch's modes are written densely (rows x G_k, G_k frequencies per
    # row) into the Fourier coefficients the batch has just consumed; one
    # gather then writes P whole rows at a time in the final column order
    Qr = t.view_as_real(Q).reshape(-1)
    for f0 in range(0, nf, group):
        f1 = min(nf, f0 + group)
        U, S, _ = M.tsqr_svd_batched_device(Q[f0:f1], precision)
        L.call("plom_spod_modes", L.dtype_code(P), L.ptr(U), f1 - f0, Mrows, nBlks,
               U.stride(0) if f1 - f0 > 1 else Mrows * nBlks, L.ptr(Qr[2 * f0 * rows:]), f1 - f0, 0,
               L.stream_ptr())
        Lm[f0:f1] = (S * S).to(x.dtype)
        del U, S
    order = np.argsort(Lm[:, 0].cpu().numpy())[::-1].copy()
    od = t.as_tensor(order, device="cuda")
    od32 = t.as_tensor(order.astype(np.int32), device="cuda")
    L.call("plom_spod_assemble", L.dtype_code(P), L.ptr(Qr), rows, nf, group, 2 * group * rows,
           L.ptr(od32), L.ptr(P), L.stream_ptr())
    del Qr, Q
    return Lm.index_select(0, od), P, f[order]


def run(X, t, nDFT: int = 0, nolap: int = 0, remove_mean: bool = True, *, window="hamming",
        precision=None):
    """Spectral POD of X (points x snapshots) sampled at times t.  Returns L
    (nf x nBlks modal energies), P ((M nBlks) x nf real modes) and f."""
    cv = L.to_device(X)
    x, ld = L.as_rows(cv.t)
    if x.dtype not in (L.torch().float32, L.torch().float64):
        raise TypeError("SPOD.run takes float32 or float64 data")
    th = t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)
    Lm, P, f = run_device(x, ld, th, nDFT, nolap, remove_mean, window, precision)
    if cv.kind == "numpy":
        return Lm.cpu().numpy(), P.cpu().numpy(), f
    return cv.back(Lm), cv.back(P), L.torch().as_tensor(f, device=cv.device)
