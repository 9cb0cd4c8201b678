"""Seeded synthetic snapshot matrices for the benchmark configurations.

No dataset is shipped with the reference for these workloads, so inputs are
synthetic, seeded and described here:

* POD field (configs 1 and 2): X[i, t] = sum_k a_k sin(kx_k x_i) sin(ky_k y_i)
  cos(w_k t + th_k) + noise, on an nx x ny grid over [0, 2 pi]^2 (endpoints
  included), dt = 1.  w_k ~ U[0.1, 2], th_k ~ U[0, 2 pi].  Config 1 uses 10
  modes, a_k = 2^-k, (kx, ky) ~ U{1..8}, noise 1e-4.  Config 2 uses 64 modes
  with a_k = k^-1.5 and 1e-5 noise; its (kx, ky) pairs are drawn WITHOUT
  replacement from {1..16}^2 so that the 64 spatial modes are distinct (with
  replacement from {1..8}^2 colliding pairs would merge modes and lower the
  rank).
* DMD field (config 3) and SPOD field (config 4): see dmd_field / spod_field.

Host (numpy) generators serve the small parity cases; the device generators
build the large matrices directly in HBM with torch in row chunks.
"""
from __future__ import annotations

import math

import numpy as np


def _pod_params(nmodes, seed, distinct, kmax):
    rng = np.random.default_rng(seed)
    if distinct:
        pairs = rng.choice(kmax * kmax, size=nmodes, replace=False)
        kx, ky = pairs // kmax + 1, pairs % kmax + 1
    else:
        kx = np.empty(nmodes, dtype=np.int64)
        ky = np.empty(nmodes, dtype=np.int64)
    w = np.empty(nmodes)
    th = np.empty(nmodes)
    for k in range(nmodes):
        if not distinct:
            kx[k], ky[k] = rng.integers(1, 9, size=2)
        w[k] = rng.uniform(0.1, 2.0)
        th[k] = rng.uniform(0, 2 * np.pi)
    return rng, kx, ky, w, th


def pod_field_np(nx, ny, nt, nmodes, seed, noise=1e-4, amp_pow=None, dtype=np.float64,
                 distinct=False, kmax=16):
    """Config-1 style field on the host (float64 math, cast at the end)."""
    rng, kx, ky, w, th = _pod_params(nmodes, seed, distinct, kmax)
    x = np.linspace(0, 2 * np.pi, nx)
    y = np.linspace(0, 2 * np.pi, ny)
    XX, YY = np.meshgrid(x, y, indexing="ij")
    xs, ys = XX.ravel(), YY.ravel()
    t = np.arange(nt, dtype=np.float64)
    amps = np.array([2.0 ** (-k) if amp_pow is None else k ** (-amp_pow) for k in range(1, nmodes + 1)])
    Phi = np.sin(np.outer(xs, kx)) * np.sin(np.outer(ys, ky))          # m x K
    T = amps[:, None] * np.cos(np.outer(w, t) + th[:, None])           # K x n
    X = Phi @ T
    X += noise * rng.standard_normal(X.shape)
    return X.astype(dtype)


def pod_field_device(nx, ny, nt, nmodes, seed, noise=1e-5, amp_pow=1.5, dtype="float32",
                     distinct=True, kmax=16, chunk_rows=1 << 20, m=None, compute="float64"):
    """Config-2 style field generated in HBM (torch, row chunks).  With `m`
    given, the first m points of the nx x ny grid (row by row) are used, so
    any point count fits a grid with nx * ny >= m.  `compute`: the arithmetic
    of the generator (float64 by default; float32 makes the per-job fields of
    the serving mix cheap to build, GB300 running FP64 at a small fraction of
    its FP32 rate)."""
    import torch
    tdt = getattr(torch, dtype) if isinstance(dtype, str) else dtype
    cdt = getattr(torch, compute) if isinstance(compute, str) else compute
    rng, kx, ky, w, th = _pod_params(nmodes, seed, distinct, kmax)
    if m is None:
        m = nx * ny
    if not (0 < m <= nx * ny) or nx < 2 or ny < 2:
        raise ValueError("pod_field_device: need nx, ny >= 2 and 0 < m <= nx * ny")
    amps = np.array([2.0 ** (-k) if amp_pow is None else k ** (-amp_pow)
                     for k in range(1, nmodes + 1)])
    t = np.arange(nt, dtype=np.float64)
    T = torch.tensor(amps[:, None] * np.cos(np.outer(w, t) + th[:, None]), device="cuda",
                     dtype=cdt)
    kxt = torch.tensor(kx, device="cuda", dtype=cdt)
    kyt = torch.tensor(ky, device="cuda", dtype=cdt)
    X = torch.empty((m, nt), dtype=tdt, device="cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    hx = 2 * math.pi / (nx - 1)
    hy = 2 * math.pi / (ny - 1)
    for r0 in range(0, m, chunk_rows):
        r1 = min(m, r0 + chunk_rows)
        idx = torch.arange(r0, r1, device="cuda", dtype=torch.int64)
        xs = (idx // ny).to(cdt) * hx
        ys = (idx % ny).to(cdt) * hy
        Phi = torch.sin(xs[:, None] * kxt[None, :]) * torch.sin(ys[:, None] * kyt[None, :])
        blk = Phi @ T
        blk += noise * torch.randn(blk.shape, device="cuda", dtype=cdt, generator=g)
        X[r0:r1].copy_(blk)
        del Phi, blk
    return X


def grid_for_points(m):
    """nx, ny with nx >= ny >= 2 covering m points: nx * ny = m for powers of
    two, otherwise ny = floor(sqrt(m)) and nx * ny >= m (the last grid row is
    partly used)."""
    if m & (m - 1) == 0:
        ny = max(2, 1 << (int(math.log2(m)) // 2))
    else:
        ny = max(2, int(math.isqrt(m)))
    return max(2, -(-m // ny)), ny


def dmd_field_device(m, n, npairs=16, seed=1003, dt=0.1, noise=1e-5, width=32.0,
                     dtype="float32", chunk_rows=1 << 20):
    """Config-3 field: 16 conjugate eigenvalue pairs lambda_j = exp((s_j + i w_j) dt),
    s_j ~ U[-0.05, 0], w_j ~ U[0.05, 3], spatial modes complex Gaussian fields
    smoothed along the point index by a Gaussian filter of standard deviation
    `width` points, plus `noise` white noise.  X = 2 Re(Phi diag(lambda^t)).
    Returns (X on the device, lambda)."""
    import torch
    tdt = getattr(torch, dtype) if isinstance(dtype, str) else dtype
    rng = np.random.default_rng(seed)
    sig = rng.uniform(-0.05, 0.0, npairs)
    om = rng.uniform(0.05, 3.0, npairs)
    lam = np.exp((sig + 1j * om) * dt)
    t = np.arange(n)
    T = lam[:, None] ** t[None, :]                       # npairs x n
    Tr = torch.tensor(np.concatenate([T.real, -T.imag]), device="cuda", dtype=torch.float64)
    half = int(4 * width)
    ker = np.exp(-0.5 * (np.arange(-half, half + 1) / width) ** 2)
    ker /= np.sqrt(np.sum(ker ** 2))
    kt = torch.tensor(ker, device="cuda", dtype=torch.float32).reshape(1, 1, -1)
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    X = torch.empty((m, n), dtype=tdt, device="cuda")
    for r0 in range(0, m, chunk_rows):
        r1 = min(m, r0 + chunk_rows)
        rows = r1 - r0
        # white complex fields with a halo so chunks join smoothly in distribution
        w = torch.randn((2 * npairs, 1, rows + 2 * half), device="cuda", dtype=torch.float32,
                        generator=g)
        ph = torch.nn.functional.conv1d(w, kt).reshape(2 * npairs, rows).T.to(torch.float64)
        blk = 2.0 * (ph @ Tr)                            # 2 Re(Phi T)
        blk += noise * torch.randn(blk.shape, device="cuda", dtype=torch.float64, generator=g)
        X[r0:r1].copy_(blk)
        del w, ph, blk
    return X, lam


def spod_field_device(M, N, noscill=8, seed=1004, fs=1.0, bw=0.002, phi=0.9, ncomp=16,
                      noise_amp=0.1, dtype="float32", chunk_rows=1 << 16):
    """Config-4 field: `noscill` narrow-band oscillators (centre frequency
    ~ U[0.01, 0.4] fs, bandwidth 0.002 fs, each a sum of `ncomp` sinusoids with
    random frequencies inside its band and random phases) with random smooth
    spatial shapes, plus AR(1) red noise x_t = phi x_{t-1} + e_t (phi = 0.9),
    realised per row by filtering white noise with 1/(1 - phi e^{-i w}) in the
    Fourier domain (circular AR(1))."""
    import torch
    tdt = getattr(torch, dtype) if isinstance(dtype, str) else dtype
    rng = np.random.default_rng(seed)
    t = np.arange(N) / fs
    S = np.zeros((noscill, N))
    for j in range(noscill):
        fc = rng.uniform(0.01, 0.4) * fs
        fr = fc + rng.uniform(-0.5, 0.5, ncomp) * bw * fs
        phs = rng.uniform(0, 2 * np.pi, ncomp)
        S[j] = np.cos(2 * np.pi * fr[:, None] * t[None, :] + phs[:, None]).sum(0) / np.sqrt(ncomp)
    St = torch.tensor(S, device="cuda", dtype=torch.float32)
    kx = rng.uniform(0.5, 4.0, noscill)
    ph0 = rng.uniform(0, 2 * np.pi, noscill)
    amp = 1.0 / (1 + np.arange(noscill))
    kxt = torch.tensor(kx, device="cuda", dtype=torch.float32)
    pht = torch.tensor(ph0, device="cuda", dtype=torch.float32)
    ampt = torch.tensor(amp, device="cuda", dtype=torch.float32)
    freqs = torch.fft.rfftfreq(N, device="cuda")
    H = 1.0 / (1.0 - phi * torch.exp(-2j * np.pi * freqs))
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    X = torch.empty((M, N), dtype=tdt, device="cuda")
    for r0 in range(0, M, chunk_rows):
        r1 = min(M, r0 + chunk_rows)
        x = torch.arange(r0, r1, device="cuda", dtype=torch.float32) / M * 2 * np.pi
        shapes = ampt * torch.sin(x[:, None] * kxt[None, :] + pht[None, :])
        blk = shapes @ St
        e = torch.randn((r1 - r0, N), device="cuda", dtype=torch.float32, generator=g)
        red = torch.fft.irfft(torch.fft.rfft(e, dim=1) * H, n=N, dim=1)
        blk += noise_amp * red
        X[r0:r1].copy_(blk)
        del blk, e, red, shapes
    return X
