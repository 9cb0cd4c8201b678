"""Generate the golden fixtures in this folder by running pyLOM's OWN py path.

Run in a container where the pyLowOrder sources are available (read-only):

    python tests/golden/make_golden.py /path/to/pyLowOrder

pyLOM's imports of mpi4py, h5py, nfft and matplotlib are replaced by
single-rank stand-ins (COMM_WORLD of size 1, reductions = identity), which is
exactly the one-rank configuration the hot path runs in.  Inputs are seeded
synthetic matrices; every fixture stores the inputs next to the reference's
outputs so the tests never need the reference at run time.
"""
from __future__ import annotations

import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    def stub(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    class _Comm:
        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

        def Barrier(self):
            pass

        def allreduce(self, x, op=None):
            return x

        def reduce(self, x, op=None, root=0):
            return x

        def bcast(self, x, root=0):
            return x

        def gather(self, x, root=0):
            return [x]

        def scatter(self, x, root=0):
            return x[0]

        def Abort(self, c):
            raise SystemExit(c)

        def send(self, *a, **k):
            raise RuntimeError("single-rank stand-in: no point-to-point traffic")

        recv = send

    class _Op:
        @staticmethod
        def Create(f, commute=True):
            return f

    mpi = stub("mpi4py.MPI", COMM_WORLD=_Comm(), Status=object, ANY_TAG=-1, ANY_SOURCE=-1,
               MODE_RDONLY=0, MODE_WRONLY=1, MODE_CREATE=2, Op=_Op, Wtime=time.perf_counter,
               File=types.SimpleNamespace(Open=None), SUM="sum", MAX="max", MIN="min",
               DOUBLE=None, FLOAT=None, INT=None, IN_PLACE=None)
    stub("mpi4py", MPI=mpi, rc=types.SimpleNamespace(recv_mprobe=False))
    stub("h5py")
    stub("nfft")

    class _Dummy:
        def __call__(self, *a, **k):
            return _Dummy()

        def __getattr__(self, k):
            return _Dummy()

    class _Any(types.ModuleType):
        def __getattr__(self, k):
            if k.startswith("__"):
                raise AttributeError(k)
            return _Dummy()

    for nm in ["matplotlib", "matplotlib.pyplot", "matplotlib.colors", "matplotlib.animation",
               "matplotlib.cm", "matplotlib.tri", "matplotlib.gridspec", "mpl_toolkits",
               "mpl_toolkits.mplot3d"]:
        sys.modules[nm] = _Any(nm)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]


def pod_field(nx, ny, nt, nmodes, seed, noise=1e-4, amp_pow=None, dtype=np.float64):
    """Sum of separable modes 2^-k sin(kx x) sin(ky y) cos(w t + th) + noise."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2 * np.pi, nx)
    y = np.linspace(0, 2 * np.pi, ny)
    XX, YY = np.meshgrid(x, y, indexing="ij")
    xs, ys = XX.ravel(), YY.ravel()
    t = np.arange(nt, dtype=np.float64)
    X = np.zeros((nx * ny, nt))
    for k in range(1, nmodes + 1):
        kx, ky = rng.integers(1, 9, size=2)
        w = rng.uniform(0.1, 2.0)
        th = rng.uniform(0, 2 * np.pi)
        a = 2.0 ** (-k) if amp_pow is None else k ** (-amp_pow)
        X += a * np.outer(np.sin(kx * xs) * np.sin(ky * ys), np.cos(w * t + th))
    X += noise * rng.standard_normal(X.shape)
    return X.astype(dtype)


def dmd_field(m, n, npairs, seed, dt=0.1, noise=1e-5, dtype=np.float64):
    rng = np.random.default_rng(seed)
    sig = rng.uniform(-0.05, 0.0, npairs)
    om = rng.uniform(0.05, 3.0, npairs)
    lam = np.exp((sig + 1j * om) * dt)
    t = np.arange(n)
    X = np.zeros((m, n))
    for j in range(npairs):
        phi = rng.standard_normal(m) + 1j * rng.standard_normal(m)
        amp = 1.0 / (1 + j)
        X += 2 * amp * np.real(np.outer(phi, lam[j] ** t))
    X += noise * rng.standard_normal(X.shape)
    return X.astype(dtype), lam


def spod_field(M, N, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    X = np.zeros((M, N))
    t = np.arange(N)
    for j in range(4):
        f0 = rng.uniform(0.02, 0.4)
        shape = np.convolve(rng.standard_normal(M), np.ones(16) / 16, mode="same")
        X += np.outer(shape, np.cos(2 * np.pi * f0 * t + rng.uniform(0, 6.28)))
    e = np.zeros((M, N))
    for k in range(1, N):
        e[:, k] = 0.9 * e[:, k - 1] + 0.1 * rng.standard_normal(M)
    return (X + e).astype(dtype)


def main(refroot):
    _install_stubs()
    sys.path.insert(0, refroot)
    import pyLOM  # noqa: E402

    # KAT: the 4x2 matrix of Examples/example_SVD.py
    A = np.array([[1, 2], [3, 4], [5, 6], [7, 8]], dtype=np.double, order="C")
    U, S, V = pyLOM.math.tsqr_svd(A)
    np.savez_compressed(os.path.join(HERE, "kat_example_svd.npz"), A=A, U=U, S=S, V=V)

    # tsqr_svd, f64 and f32
    rng = np.random.default_rng(11)
    for dt, tag, (m, n) in [(np.float64, "f64", (400, 24)), (np.float32, "f32", (300, 16))]:
        A = rng.standard_normal((m, n)).astype(dt)
        U, S, V = pyLOM.math.tsqr_svd(A)
        np.savez_compressed(os.path.join(HERE, f"tsqr_svd_{tag}.npz"), A=A, U=U, S=S, V=V)

    # qr (numpy.linalg.qr's Householder factors) and tsqr (one rank: the same
    # factors), tall, square and wide; randomized_qr / randomized_qr2 with the
    # Omega the reference draws (np.random.seed(seed); rand(n, r))
    rq = np.random.default_rng(21)
    cases = {"tall_f64": rq.standard_normal((300, 20)),
             "tall_f32": rq.standard_normal((200, 12)).astype(np.float32),
             "square_f64": rq.standard_normal((16, 16)),
             "wide_f64": rq.standard_normal((12, 30))}
    out = {}
    for tag, A in cases.items():
        Q, R = pyLOM.math.qr(A)
        out[f"{tag}_A"], out[f"{tag}_Q"], out[f"{tag}_R"] = A, Q, R
    for tag, A in [("tsqr_f64", rq.standard_normal((500, 30))),
                   ("tsqr_f32", rq.standard_normal((400, 16)).astype(np.float32))]:
        Q, R = pyLOM.math.tsqr(A)
        out[f"{tag}_A"], out[f"{tag}_Q"], out[f"{tag}_R"] = A, Q, R
    np.savez_compressed(os.path.join(HERE, "qr.npz"), **out)
    out = {}
    for tag, dt in [("f64", np.float64), ("f32", np.float32)]:
        A = pod_field(16, 16, 48, 10, seed=1008, dtype=dt)
        r, q, seed = 10, 2, 13
        Q, B = pyLOM.math.randomized_qr(A, r, q, seed=seed)
        Q2, B2 = pyLOM.math.randomized_qr2(A, r, q, seed=seed)
        np.random.seed(seed=seed)
        om = np.random.rand(A.shape[1], r).astype(A.dtype)
        out.update({f"{tag}_A": A, f"{tag}_Q": Q, f"{tag}_B": B, f"{tag}_Q2": Q2, f"{tag}_B2": B2,
                    f"{tag}_omega": om})
    np.savez_compressed(os.path.join(HERE, "randomized_qr.npz"), r=10, q=2, seed=13, **out)

    # averaging
    X = pod_field(16, 16, 30, 5, seed=3)
    mean = pyLOM.math.temporal_mean(X)
    Y = pyLOM.math.subtract_mean(X, mean)
    var = pyLOM.math.temporal_variance(X, mean)
    Yv = pyLOM.math.norm_variance(X, mean, var)
    np.savez_compressed(os.path.join(HERE, "averaging.npz"), X=X, mean=mean, Y=Y, var=var, Yv=Yv)

    # POD: tsqr path, truncation by residual and energy, reconstruct, RMSE
    X = pod_field(20, 20, 40, 10, seed=1001)
    U, S, V = pyLOM.POD.run(X, remove_mean=True)
    Ut, St, Vt = pyLOM.POD.truncate(U, S, V, r=1e-6)
    Ue, Se, Ve = pyLOM.POD.truncate(U, S, V, r=-0.99)
    Xr = pyLOM.POD.reconstruct(Ut, St, Vt)
    rmse = pyLOM.math.RMSE(Xr, X - X.mean(axis=1, keepdims=True))
    np.savez_compressed(os.path.join(HERE, "pod_cfg1_small.npz"), X=X, U=U, S=S, V=V, N_res=Ut.shape[1],
             N_energy=Ue.shape[1], Xr=Xr, rmse=rmse)
    U2, S2, V2 = pyLOM.POD.run(X, remove_mean=True, divide_variance=True)
    np.savez_compressed(os.path.join(HERE, "pod_divvar.npz"), X=X, U=U2, S=S2, V=V2)
    Xf = X.astype(np.float32)
    U3, S3, V3 = pyLOM.POD.run(Xf, remove_mean=False)
    np.savez_compressed(os.path.join(HERE, "pod_f32_nomean.npz"), X=Xf, U=U3, S=S3, V=V3)

    # PCA: components and scores, variance normalised (the default) and not
    Uc, Sc = pyLOM.PCA.run(X)
    Uc2, Sc2 = pyLOM.PCA.run(X, divide_variance=False)
    np.savez_compressed(os.path.join(HERE, "pca.npz"), X=X, U=Uc, scores=Sc, U_nv=Uc2, scores_nv=Sc2)

    # truncation residual cases
    Ss = np.sort(np.abs(rng.standard_normal(50)))[::-1] ** 3
    rs = np.array([1e-1, 1e-2, 1e-4, 1e-8, -0.5, -0.9, -0.99, -1.0])
    Ns = np.array([pyLOM.math.compute_truncation_residual(Ss, float(r)) for r in rs])
    np.savez_compressed(os.path.join(HERE, "truncation.npz"), S=Ss, r=rs, N=Ns)

    # randomized POD with the reference's own numpy Omega (seed fixed)
    X = pod_field(16, 16, 48, 10, seed=1002)
    U, S, V = pyLOM.POD.run(X, remove_mean=False, randomized=True, r=12, q=3, seed=25)
    np.savez_compressed(os.path.join(HERE, "pod_randomized.npz"), X=X, U=U, S=S, V=V, r=12, q=3, seed=25)

    # streaming range finder: two batches of snapshots; the Omegas the
    # reference draws (seed 7, then numpy's global stream) are stored too
    Xs1 = pod_field(16, 16, 40, 10, seed=1006)
    Xs2 = pod_field(16, 16, 24, 10, seed=1007)
    Q1, B1, Y1 = pyLOM.math.init_qr_streaming(Xs1, 8, 2, seed=7)
    Y1 = Y1.copy()
    Q2, B2, Y2 = pyLOM.math.update_qr_streaming(Xs2, Q1, B1, Y1.copy(), 8, 2)
    np.random.seed(seed=7)
    om1 = np.random.rand(Xs1.shape[1], 8).astype(Xs1.dtype)
    om2 = np.random.rand(Xs2.shape[1], 8).astype(Xs2.dtype)
    np.savez_compressed(os.path.join(HERE, "qr_streaming.npz"), X1=Xs1, X2=Xs2, Q1=Q1, B1=B1, Y1=Y1,
                        Q2=Q2, B2=B2, Y2=Y2, om1=om1, om2=om2, r=8, q=2, seed=7)

    # DMD
    Xd, lam = dmd_field(500, 48, 4, seed=1003)
    muR, muI, Phi, b = pyLOM.DMD.run(Xd, 8, remove_mean=False)
    delta, omega = pyLOM.DMD.frequency_damping(muR, muI, 0.1)
    tt = np.arange(48, dtype=np.float64)
    Xrec = pyLOM.DMD.reconstruction_jovanovic(Phi, muR, muI, tt, b)
    np.savez_compressed(os.path.join(HERE, "dmd_small.npz"), X=Xd, lam=lam, muReal=muR, muImag=muI, Phi=Phi,
             bJov=b, delta=delta, omega=omega, Xrec=Xrec, r=8)
    muR2, muI2, Phi2, b2 = pyLOM.DMD.run(Xd, 1e-6, remove_mean=True)
    np.savez_compressed(os.path.join(HERE, "dmd_small_mean.npz"), X=Xd, muReal=muR2, muImag=muI2, Phi=Phi2,
             bJov=b2, r=1e-6)

    # SPOD (Hamming window, the reference's)
    for dt, tag in [(np.float64, "f64"), (np.float32, "f32")]:
        Xs = spod_field(96, 320, seed=1004, dtype=dt)
        ts = np.arange(320, dtype=dt) * 0.5
        L, P, f = pyLOM.SPOD.run(Xs, ts, nDFT=32, nolap=16, remove_mean=True)
        np.savez_compressed(os.path.join(HERE, f"spod_{tag}.npz"), X=Xs, t=ts, L=L, P=P, f=f, nDFT=32, nolap=16)
    Xs = spod_field(48, 400, seed=1005)
    ts = np.arange(400, dtype=np.float64)
    L, P, f = pyLOM.SPOD.run(Xs, ts)  # default nDFT / nolap
    np.savez_compressed(os.path.join(HERE, "spod_defaults.npz"), X=Xs, t=ts, L=L, P=P, f=f)

    # Hamming window
    np.savez_compressed(os.path.join(HERE, "hammwin.npz"), w7=pyLOM.math.hammwin(7), w256=pyLOM.math.hammwin(256))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the pyLowOrder sources>")
    main(sys.argv[1])
