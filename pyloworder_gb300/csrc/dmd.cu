// DMD reduced stage on the GPU, all in FP64, one CTA (the reduced operator
// is r x r with r up to a few hundred):
//
//   Atilde = (U^T Y2) (S^-1 VT)^T                     pyLOM/DMD/wrapper.py:84-87
//   eig(Atilde) -> mu, W                              wrapper.py:93 (LAPACK dgeev
//                                                     on the host in pyLOM)
//   Vand[i][t] = mu_i^t, P = (W^H W) o conj(Vand Vand^H),
//   q = conj(diag(Vand (S VT)^H W)), b = P^-1 q       wrapper.py:103-109
//   order by |b| descending, conjugate pairs positive-imag first
//                                                     wrapper.py:18-45, 113-114
//   Mphi = VT^T S^-1 W diag(1/mu) (ordered, with the pair fix-up), so that the
//   modes are one tall product Phi = Y2 Mphi         wrapper.py:99
//
// Eigen-solver: Householder reduction to Hessenberg form, Francis double-
// shift QR to real Schur form T = Z^T A Z (Golub & Van Loan, Matrix
// Computations, Alg. 7.4.2 and 7.5.2), eigenvectors by complex back
// substitution on T, back-transformed by Z and normalised as LAPACK's dgeev
// normalises them (unit 2-norm; the largest component of a complex vector made
// real).  Phi_j * b_j does not depend on that normalisation.
#include <algorithm>
#include <cmath>

#include "plom_common.cuh"
#include "plom_kernels.cuh"

namespace plom {

struct cplx {
  double re, im;
};
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cplx cconj(cplx a) { return {a.re, -a.im}; }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
  // Smith's algorithm
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  double r = b.re / b.im, d = b.im + b.re * r;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
__device__ __forceinline__ double cabs2(cplx a) { return a.re * a.re + a.im * a.im; }

struct DmdBufs {
  double* A;    // N x N  Atilde, then T (real Schur form)
  double* Z;    // N x N  Schur vectors
  double* wr;   // N
  double* wi;   // N
  double* Wv;   // N x N complex (eigenvectors, columns), interleaved
  double* Y;    // N x N complex (eigenvectors of T), interleaved
  double* Pm;   // N x N complex (P, then its Cholesky factor)
  double* qv;   // N complex
  double* bv;   // N complex
  double* babs; // N
  int* order;   // N
  double* Vr;   // N x nt complex Vandermonde
  int* flip;    // N conjugate-pair fix-up flags of the ordered modes
};

// -------------------------------------------------------------------------
// Hessenberg + Francis QR (one CTA).  A (N x N, row-major) is overwritten
// with T, Z accumulates the orthogonal transformations.
// -------------------------------------------------------------------------
__device__ void hessenberg(double* A, double* Z, int N, double* sh) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < N * N; e += nt) Z[e] = ((e / N) == (e % N)) ? 1.0 : 0.0;
  __syncthreads();
  double* v = sh;        // N
  double* w = sh + N;    // N
  for (int k = 0; k + 2 < N; ++k) {
    // reflector for x = A[k+1:N, k]
    if (tid == 0) {
      double s = 0.0;
      for (int i = k + 1; i < N; ++i) s += A[i * N + k] * A[i * N + k];
      double nrm = sqrt(s);
      double x0 = A[(k + 1) * N + k];
      double alpha = (x0 >= 0.0) ? -nrm : nrm;
      for (int i = 0; i < N; ++i) v[i] = 0.0;
      double vv = 0.0;
      if (nrm > 0.0) {
        v[k + 1] = x0 - alpha;
        for (int i = k + 2; i < N; ++i) v[i] = A[i * N + k];
        for (int i = k + 1; i < N; ++i) vv += v[i] * v[i];
      }
      w[0] = (vv > 0.0) ? 2.0 / vv : 0.0;  // tau
    }
    __syncthreads();
    const double tau = w[0];
    __syncthreads();
    if (tau != 0.0) {
      // A = (I - tau v v^T) A : column j update
      for (int j = tid; j < N; j += nt) {
        double s = 0.0;
        for (int i = k + 1; i < N; ++i) s += v[i] * A[i * N + j];
        s *= tau;
        for (int i = k + 1; i < N; ++i) A[i * N + j] -= s * v[i];
      }
      __syncthreads();
      // A = A (I - tau v v^T), Z = Z (I - tau v v^T): row updates
      for (int i = tid; i < 2 * N; i += nt) {
        double* M = (i < N) ? A : Z;
        const int r = (i < N) ? i : i - N;
        double s = 0.0;
        for (int j = k + 1; j < N; ++j) s += M[r * N + j] * v[j];
        s *= tau;
        for (int j = k + 1; j < N; ++j) M[r * N + j] -= s * v[j];
      }
      __syncthreads();
      if (tid == 0)
        for (int i = k + 2; i < N; ++i) A[i * N + k] = 0.0;
    }
    __syncthreads();
  }
}

// apply the reflector I - tau v v^T (v of length len at rows/cols k..k+len-1)
// to rows k.. of A over columns [c0, N), to columns k.. of A over rows
// [0, r1], and to columns k.. of Z (all rows)
__device__ void apply_reflector(double* A, double* Z, int N, int k, int len, const double* v,
                                double tau, int c0, int r1) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int j = c0 + tid; j < N; j += nt) {
    double s = 0.0;
    for (int q = 0; q < len; ++q) s += v[q] * A[(k + q) * N + j];
    s *= tau;
    for (int q = 0; q < len; ++q) A[(k + q) * N + j] -= s * v[q];
  }
  __syncthreads();
  for (int i = tid; i < (r1 + 1) + N; i += nt) {
    double* M = (i <= r1) ? A : Z;
    const int r = (i <= r1) ? i : i - (r1 + 1);
    double s = 0.0;
    for (int q = 0; q < len; ++q) s += M[r * N + k + q] * v[q];
    s *= tau;
    for (int q = 0; q < len; ++q) M[r * N + k + q] -= s * v[q];
  }
  __syncthreads();
}

// plane rotation [c s; -s c] applied on rows/cols p, p+1
__device__ void apply_rotation(double* A, double* Z, int N, int p, double c, double s) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int j = p + tid; j < N; j += nt) {  // rows p, p+1 : G^T A
    double x = A[p * N + j], y = A[(p + 1) * N + j];
    A[p * N + j] = c * x + s * y;
    A[(p + 1) * N + j] = -s * x + c * y;
  }
  __syncthreads();
  for (int i = tid; i < 2 * N; i += nt) {  // cols p, p+1 : A G and Z G
    if (i < N && i > p + 1) continue;
    double* M = (i < N) ? A : Z;
    const int r = (i < N) ? i : i - N;
    double x = M[r * N + p], y = M[r * N + p + 1];
    M[r * N + p] = c * x + s * y;
    M[r * N + p + 1] = -s * x + c * y;
  }
  __syncthreads();
}

// Francis double-shift QR on the Hessenberg A; returns false on non-convergence
__device__ bool francis(double* A, double* Z, double* wr, double* wi, int N, double* sh) {
  const int tid = threadIdx.x;
  volatile int* ctl = reinterpret_cast<volatile int*>(sh + 8);  // [0]=l, [1]=action
  double* v = sh;                                                 // 3 + tau at v[3]
  const double eps = 2.220446049250313e-16;
  int nn = N - 1;
  int its = 0, total = 0;
  const int max_total = 60 * N + 60;
  while (nn >= 0) {
    if (total > max_total) return false;
    if (tid == 0) {
      int l = nn;
      for (; l > 0; --l) {
        double s = fabs(A[(l - 1) * N + l - 1]) + fabs(A[l * N + l]);
        if (s == 0.0) s = 1.0;
        if (fabs(A[l * N + l - 1]) <= eps * s) {
          A[l * N + l - 1] = 0.0;
          break;
        }
      }
      ctl[0] = l;
    }
    __syncthreads();
    const int l = ctl[0];
    __syncthreads();
    if (l == nn) {  // one real root
      if (tid == 0) {
        wr[nn] = A[nn * N + nn];
        wi[nn] = 0.0;
      }
      --nn;
      its = 0;
      __syncthreads();
      continue;
    }
    if (l == nn - 1) {  // 2 x 2 block
      const double a = A[(nn - 1) * N + nn - 1], b = A[(nn - 1) * N + nn];
      const double c = A[nn * N + nn - 1], d = A[nn * N + nn];
      const double p = 0.5 * (a - d), q = p * p + b * c;
      __syncthreads();  // every thread has read the block before it is rotated
      if (q >= 0.0) {
        // real pair: rotate the block to upper triangular form
        const double z = p + copysign(sqrt(q), p);
        const double l1 = d + z;
        // eigenvector of the block for l1: (b, l1 - a) or (l1 - d, c)
        double x0 = l1 - d, x1 = c;
        if (fabs(b) + fabs(l1 - a) > fabs(x0) + fabs(x1)) {
          x0 = b;
          x1 = l1 - a;
        }
        const double r = hypot(x0, x1);
        const double cs = (r > 0.0) ? x0 / r : 1.0, sn = (r > 0.0) ? x1 / r : 0.0;
        apply_rotation(A, Z, N, nn - 1, cs, sn);
        if (tid == 0) {
          A[nn * N + nn - 1] = 0.0;
          wr[nn - 1] = A[(nn - 1) * N + nn - 1];
          wr[nn] = A[nn * N + nn];
          wi[nn - 1] = wi[nn] = 0.0;
        }
      } else if (tid == 0) {
        const double re = d + p, im = sqrt(-q);
        wr[nn - 1] = wr[nn] = re;
        wi[nn - 1] = im;
        wi[nn] = -im;
      }
      nn -= 2;
      its = 0;
      __syncthreads();
      continue;
    }
    // double-shift QR sweep on the window l..nn
    ++its;
    ++total;
    double s, t;
    if (its % 11 == 10) {  // exceptional shift
      const double e = fabs(A[nn * N + nn - 1]) + fabs(A[(nn - 1) * N + nn - 2]);
      s = 1.5 * e;
      t = e * e;
    } else {
      s = A[(nn - 1) * N + nn - 1] + A[nn * N + nn];
      t = A[(nn - 1) * N + nn - 1] * A[nn * N + nn] - A[(nn - 1) * N + nn] * A[nn * N + nn - 1];
    }
    double x = A[l * N + l] * A[l * N + l] + A[l * N + l + 1] * A[(l + 1) * N + l] -
               s * A[l * N + l] + t;
    double y = A[(l + 1) * N + l] * (A[l * N + l] + A[(l + 1) * N + l + 1] - s);
    double z = A[(l + 1) * N + l] * A[(l + 2) * N + l + 1];
    for (int k = l; k <= nn - 1; ++k) {
      const int len = (k < nn - 1) ? 3 : 2;
      if (tid == 0) {
        const double nrm = (len == 3) ? sqrt(x * x + y * y + z * z) : hypot(x, y);
        const double alpha = (x >= 0.0) ? -nrm : nrm;
        v[0] = x - alpha;
        v[1] = y;
        v[2] = (len == 3) ? z : 0.0;
        const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        v[3] = (nrm > 0.0 && vv > 0.0) ? 2.0 / vv : 0.0;
        v[4] = alpha;
      }
      __syncthreads();
      const double tau = v[3];
      if (tau != 0.0) {
        const int c0 = (k > l) ? k - 1 : l;
        const int r1 = (k + 3 <= nn) ? k + 3 : nn;
        apply_reflector(A, Z, N, k, len, v, tau, c0, r1);
        if (tid == 0 && k > l) {
          A[k * N + k - 1] = v[4];
          A[(k + 1) * N + k - 1] = 0.0;
          if (len == 3) A[(k + 2) * N + k - 1] = 0.0;
        }
      }
      __syncthreads();
      if (k < nn - 1) {
        x = A[(k + 1) * N + k];
        y = A[(k + 2) * N + k];
        z = (k < nn - 2) ? A[(k + 3) * N + k] : 0.0;
      }
      __syncthreads();
    }
  }
  return true;
}

// eigenvectors of the quasi-triangular T (complex back substitution), then
// W = Z Y, normalised like dgeev
__device__ void schur_vectors(const double* T, const double* Z, const double* wr, const double* wi,
                              int N, double* Y, double* W, double* sh) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const double eps = 2.220446049250313e-16;
  double tnorm = 0.0;
  for (int e = 0; e < N * N; ++e) tnorm = fmax(tnorm, fabs(T[e]));
  const double smin = fmax(eps * tnorm, 1e-300);
  // one thread per eigenvalue column k (sequential solve, N^2)
  for (int k = tid; k < N; k += nt) {
    cplx* y = reinterpret_cast<cplx*>(Y) + (size_t)k * N;  // row k of Y holds y_k
    for (int i = 0; i < N; ++i) y[i] = {0.0, 0.0};
    const cplx lam = {wr[k], wi[k]};
    int top;  // highest row of the eigen-block
    if (wi[k] == 0.0) {
      y[k] = {1.0, 0.0};
      top = k;
    } else if (wi[k] > 0.0) {  // block rows k, k+1
      const double c = T[(k + 1) * N + k];
      y[k + 1] = {1.0, 0.0};
      y[k] = cdiv({lam.re - T[(k + 1) * N + k + 1], lam.im}, {c, 0.0});
      top = k;
    } else {  // second of a pair (rows k-1, k)
      const double c = T[k * N + k - 1];
      y[k] = {1.0, 0.0};
      y[k - 1] = cdiv({lam.re - T[k * N + k], lam.im}, {c, 0.0});
      top = k - 1;
    }
    const int bottom = (wi[k] > 0.0) ? k + 1 : k;
    int i = top - 1;
    while (i >= 0) {
      const bool pair = (i > 0) && (T[i * N + i - 1] != 0.0);
      if (!pair) {
        cplx r = {0.0, 0.0};
        for (int j = i + 1; j <= bottom; ++j) {
          r.re += T[i * N + j] * y[j].re;
          r.im += T[i * N + j] * y[j].im;
        }
        cplx den = {T[i * N + i] - lam.re, -lam.im};
        if (cabs2(den) < smin * smin) den = {smin, 0.0};
        y[i] = cdiv({-r.re, -r.im}, den);
        i -= 1;
      } else {
        // rows i-1, i jointly
        cplx r0 = {0.0, 0.0}, r1 = {0.0, 0.0};
        for (int j = i + 1; j <= bottom; ++j) {
          r0.re += T[(i - 1) * N + j] * y[j].re;
          r0.im += T[(i - 1) * N + j] * y[j].im;
          r1.re += T[i * N + j] * y[j].re;
          r1.im += T[i * N + j] * y[j].im;
        }
        const cplx a11 = {T[(i - 1) * N + i - 1] - lam.re, -lam.im};
        const cplx a12 = {T[(i - 1) * N + i], 0.0};
        const cplx a21 = {T[i * N + i - 1], 0.0};
        const cplx a22 = {T[i * N + i] - lam.re, -lam.im};
        cplx det = cmul(a11, a22);
        cplx t2 = cmul(a12, a21);
        det.re -= t2.re;
        det.im -= t2.im;
        if (cabs2(det) < smin * smin) det = {smin, 0.0};
        // [y_{i-1}; y_i] = A^-1 (-r)
        cplx u0 = cmul(a22, {-r0.re, -r0.im});
        cplx u1 = cmul(a12, {-r1.re, -r1.im});
        cplx w0 = cmul(a11, {-r1.re, -r1.im});
        cplx w1 = cmul(a21, {-r0.re, -r0.im});
        y[i - 1] = cdiv({u0.re - u1.re, u0.im - u1.im}, det);
        y[i] = cdiv({w0.re - w1.re, w0.im - w1.im}, det);
        i -= 2;
      }
    }
  }
  __syncthreads();
  // W[:, k] = Z y_k
  cplx* Wc = reinterpret_cast<cplx*>(W);
  const cplx* Yc = reinterpret_cast<const cplx*>(Y);
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, k = e % N;
    cplx s = {0.0, 0.0};
    for (int j = 0; j < N; ++j) {
      s.re += Z[i * N + j] * Yc[(size_t)k * N + j].re;
      s.im += Z[i * N + j] * Yc[(size_t)k * N + j].im;
    }
    Wc[(size_t)i * N + k] = s;
  }
  __syncthreads();
  // normalise each column: unit 2-norm; complex: largest component real >= 0
  for (int k = tid; k < N; k += nt) {
    double s = 0.0;
    int imax = 0;
    double best = -1.0;
    for (int i = 0; i < N; ++i) {
      const double a = cabs2(Wc[(size_t)i * N + k]);
      s += a;
      if (a > best) {
        best = a;
        imax = i;
      }
    }
    const double inv = (s > 0.0) ? 1.0 / sqrt(s) : 0.0;
    cplx ph = {inv, 0.0};
    if (wi[k] != 0.0 && best > 0.0) {
      const cplx c = Wc[(size_t)imax * N + k];
      const double a = sqrt(best);
      ph = {c.re / a * inv, -c.im / a * inv};  // conj(c)/|c| / ||w||
    }
    for (int i = 0; i < N; ++i) Wc[(size_t)i * N + k] = cmul(Wc[(size_t)i * N + k], ph);
  }
  __syncthreads();
}

// -------------------------------------------------------------------------
// the reduced stage: Atilde, its eigenpairs (Hessenberg + Francis, the Schur
// vectors) and the Vandermonde rows in one CTA; P, q and the mode matrix in
// kernels spread over the GPU (their FP64 sums over the snapshots were 57 %
// of the one-CTA version's cycles); the amplitude solve in one CTA
// -------------------------------------------------------------------------
__global__ void __launch_bounds__(256) dmd_eig_kernel(const double* __restrict__ aux1,
                                                          const double* __restrict__ S,
                                                          const double* __restrict__ VT, int N,
                                                          int nt, DmdBufs B, double* muR,
                                                          double* muI, double* bJov, double* Mphi,
                                                          int* info) {
  (void)muR;
  (void)muI;
  (void)bJov;
  (void)Mphi;
  extern __shared__ double sh[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  // Atilde[i][j] = sum_t aux1[i][t] VT[j][t] / S[j]
  for (int e = tid; e < N * N; e += nthr) {
    const int i = e / N, j = e % N;
    double s = 0.0;
    for (int t = 0; t < nt; ++t) s += aux1[(size_t)i * nt + t] * VT[(size_t)j * nt + t];
    B.A[e] = s / S[j];
  }
  __syncthreads();
  hessenberg(B.A, B.Z, N, sh);
  if (!francis(B.A, B.Z, B.wr, B.wi, N, sh)) {
    if (tid == 0) atomicMax(&info[ST_FAIL], PLOM_NUM_EIG);
    return;
  }
  __syncthreads();
  schur_vectors(B.A, B.Z, B.wr, B.wi, N, B.Y, B.Wv, sh);
  cplx* V = reinterpret_cast<cplx*>(B.Vr);
  // Vandermonde rows mu_i^t by repeated multiplication
  for (int i = tid; i < N; i += nthr) {
    const cplx mu = {B.wr[i], B.wi[i]};
    cplx p = {1.0, 0.0};
    for (int t = 0; t < nt; ++t) {
      V[(size_t)i * nt + t] = p;
      p = cmul(p, mu);
    }
  }
  __syncthreads();
}

// P = (W^H W) o conj(Vand Vand^H) (one warp per element) and
// q_i = conj( sum_t Vand[i][t] sum_k S_k VT[k][t] W[k][i] ) (one block per i,
// the blocks after the P warps'): FP64 sums over t and k spread over the GPU
__global__ void __launch_bounds__(256) dmd_pq_kernel(const double* __restrict__ S,
                                                     const double* __restrict__ VT, int N, int nt,
                                                     DmdBufs B, const int* __restrict__ info) {
  if (info[ST_FAIL]) return;
  const cplx* W = reinterpret_cast<const cplx*>(B.Wv);
  const cplx* V = reinterpret_cast<const cplx*>(B.Vr);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pblocks = (N * N + 7) / 8;
  if ((int)blockIdx.x < pblocks) {
    const int e = blockIdx.x * 8 + warp;
    if (e >= N * N) return;
    const int i = e / N, j = e % N;
    cplx g = {0.0, 0.0}, vv = {0.0, 0.0};
    for (int k = lane; k < N; k += 32) {
      const cplx ab = cmul(cconj(W[(size_t)k * N + i]), W[(size_t)k * N + j]);
      g.re += ab.re;
      g.im += ab.im;
    }
    for (int t = lane; t < nt; t += 32) {
      const cplx ab = cmul(V[(size_t)i * nt + t], cconj(V[(size_t)j * nt + t]));
      vv.re += ab.re;
      vv.im += ab.im;
    }
    g.re = warp_sum(g.re);
    g.im = warp_sum(g.im);
    vv.re = warp_sum(vv.re);
    vv.im = warp_sum(vv.im);
    if (lane == 0) reinterpret_cast<cplx*>(B.Pm)[e] = cmul(g, cconj(vv));
    return;
  }
  const int i = (int)blockIdx.x - pblocks;
  if (i >= N) return;
  cplx acc = {0.0, 0.0};
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    cplx gw = {0.0, 0.0};
    for (int k = 0; k < N; ++k) {
      const double gk = S[k] * VT[(size_t)k * nt + t];
      gw.re += gk * W[(size_t)k * N + i].re;
      gw.im += gk * W[(size_t)k * N + i].im;
    }
    const cplx ab = cmul(V[(size_t)i * nt + t], gw);
    acc.re += ab.re;
    acc.im += ab.im;
  }
  __shared__ double red[8][2];
  acc.re = warp_sum(acc.re);
  acc.im = warp_sum(acc.im);
  if (lane == 0) {
    red[warp][0] = acc.re;
    red[warp][1] = acc.im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cplx t = {0.0, 0.0};
    for (int w = 0; w < 8; ++w) {
      t.re += red[w][0];
      t.im += red[w][1];
    }
    reinterpret_cast<cplx*>(B.qv)[i] = cconj(t);
  }
}

// Cholesky solve for the amplitudes, the ordering and the conjugate-pair
// fix-up flags (one CTA)
__global__ void __launch_bounds__(256) dmd_amp_kernel(int N, DmdBufs B, double* muR, double* muI,
                                                      double* bJov, int* info) {
  if (info[ST_FAIL]) return;
  const int tid = threadIdx.x, nthr = blockDim.x;
  cplx* P = reinterpret_cast<cplx*>(B.Pm);
  cplx* q = reinterpret_cast<cplx*>(B.qv);
  // Cholesky P = L L^H (in place, lower), then solve L L^H b = q
  cplx* b = reinterpret_cast<cplx*>(B.bv);
  __shared__ int bad;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < N; ++j) {
    if (tid == 0) {
      double d = P[(size_t)j * N + j].re;
      for (int k = 0; k < j; ++k) d -= cabs2(P[(size_t)j * N + k]);
      if (!(d > 0.0) || !isfinite(d)) {
        bad = 1;
        d = 1e-300;
      }
      P[(size_t)j * N + j] = {sqrt(d), 0.0};
    }
    __syncthreads();
    const double ljj = P[(size_t)j * N + j].re;
    for (int i = j + 1 + tid; i < N; i += nthr) {
      cplx s = P[(size_t)i * N + j];
      for (int k = 0; k < j; ++k) {
        const cplx ab = cmul(P[(size_t)i * N + k], cconj(P[(size_t)j * N + k]));
        s.re -= ab.re;
        s.im -= ab.im;
      }
      P[(size_t)i * N + j] = {s.re / ljj, s.im / ljj};
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (bad) atomicMax(&info[ST_FAIL], PLOM_NUM_CHOLESKY);
    // forward: L z = q
    for (int i = 0; i < N; ++i) {
      cplx s = q[i];
      for (int k = 0; k < i; ++k) {
        const cplx ab = cmul(P[(size_t)i * N + k], b[k]);
        s.re -= ab.re;
        s.im -= ab.im;
      }
      b[i] = {s.re / P[(size_t)i * N + i].re, s.im / P[(size_t)i * N + i].re};
    }
    // backward: L^H b = z
    for (int i = N - 1; i >= 0; --i) {
      cplx s = b[i];
      for (int k = i + 1; k < N; ++k) {
        const cplx ab = cmul(cconj(P[(size_t)k * N + i]), b[k]);
        s.re -= ab.re;
        s.im -= ab.im;
      }
      b[i] = {s.re / P[(size_t)i * N + i].re, s.im / P[(size_t)i * N + i].re};
    }
    // order: |b| descending (ties: larger index first, as flip(argsort))
    for (int i = 0; i < N; ++i) B.babs[i] = sqrt(cabs2(b[i]));
    for (int i = 0; i < N; ++i) {
      int rank = 0;
      for (int k = 0; k < N; ++k)
        rank += (B.babs[k] > B.babs[i]) || (B.babs[k] == B.babs[i] && k > i);
      B.order[rank] = i;
    }
  }
  __syncthreads();
  // ordered eigenvalues / amplitudes and the pair fix-up flags
  int* flip_tab = B.flip;
  if (tid == 0) {
    for (int j = 0; j < N; ++j) {
      const int o = B.order[j];
      muR[j] = B.wr[o];
      muI[j] = B.wi[o];
      bJov[2 * j] = b[o].re;
      bJov[2 * j + 1] = b[o].im;
      if (j < 1024) flip_tab[j] = 0;
    }
    bool skip = false;
    for (int j = 0; j < N; ++j) {
      if (skip) {
        skip = false;
        continue;
      }
      if (muI[j] < 0.0 && j + 1 < N) {
        // pyLOM/DMD/wrapper.py:31-38: take the partner's imag parts
        muI[j] = muI[j + 1];
        muI[j + 1] = -muI[j];
        bJov[2 * j + 1] = bJov[2 * (j + 1) + 1];
        bJov[2 * (j + 1) + 1] = -bJov[2 * j + 1];
        if (j < 1024) flip_tab[j] = 1;
        skip = true;
      } else if (muI[j] > 0.0) {
        skip = true;
      }
    }
  }
  __syncthreads();
}

// Mphi[t][j] = sum_k VT[k][t] / S_k * W[k][o_j] / mu_{o_j} (one thread per
// element), then the conjugate-pair fix-up of its imaginary parts per row
__global__ void __launch_bounds__(256) dmd_mphi_kernel(const double* __restrict__ S,
                                                       const double* __restrict__ VT, int N,
                                                       int nt, DmdBufs B, double* Mphi,
                                                       const int* __restrict__ info) {
  if (info[ST_FAIL]) return;
  const cplx* W = reinterpret_cast<const cplx*>(B.Wv);
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)nt * N) return;
  const int t = (int)(e / N), j = (int)(e % N);
  const int o = B.order[j];
  const cplx mu = {B.wr[o], B.wi[o]};
  cplx s = {0.0, 0.0};
  for (int k = 0; k < N; ++k) {
    const double g = VT[(size_t)k * nt + t] / S[k];
    s.re += g * W[(size_t)k * N + o].re;
    s.im += g * W[(size_t)k * N + o].im;
  }
  s = cdiv(s, mu);
  Mphi[(size_t)t * 2 * N + 2 * j] = s.re;
  Mphi[(size_t)t * 2 * N + 2 * j + 1] = s.im;
}

// Phi.imag[:, j] = Phi.imag[:, j+1]; Phi.imag[:, j+1] = -Phi.imag[:, j+1]
__global__ void dmd_flip_kernel(int N, int nt, DmdBufs B, double* Mphi,
                                const int* __restrict__ info) {
  if (info[ST_FAIL]) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double* row = Mphi + (size_t)t * 2 * N;
  for (int j = 0; j + 1 < N; ++j) {
    if (!B.flip[j]) continue;
    const double im1 = row[2 * (j + 1) + 1];
    row[2 * j + 1] = im1;
    row[2 * (j + 1) + 1] = -im1;
  }
}

size_t dmd_reduced_workspace(int N, int nt) {
  Arena a(nullptr, 0);
  a.take<double>((size_t)N * N);
  a.take<double>((size_t)N * N);
  a.take<double>(N);
  a.take<double>(N);
  a.take<double>((size_t)2 * N * N);
  a.take<double>((size_t)2 * N * N);
  a.take<double>((size_t)2 * N * N);
  a.take<double>((size_t)2 * N);
  a.take<double>((size_t)2 * N);
  a.take<double>(N);
  a.take<int>(N);
  a.take<double>((size_t)2 * N * nt);
  a.take<int>(N);
  return a.off + 1024;
}

}  // namespace plom

using namespace plom;

extern "C" size_t plom_dmd_reduced_workspace(int64_t r, int64_t nt) {
  if (r < 1 || nt < 1 || r > 1024) return 0;
  return dmd_reduced_workspace((int)r, (int)nt);
}

extern "C" int plom_dmd_reduced(const double* aux1, const double* S, const double* VT, int64_t r,
                                int64_t nt, double* muReal, double* muImag, double* bJov,
                                double* Mphi, void* ws, size_t ws_bytes, int* info, void* stream) {
  PLOM_REQUIRE(r >= 1 && r <= 1024 && nt >= 1, PLOM_ERR_ARG,
               "dmd_reduced: need 1 <= r <= 1024 and nt >= 1");
  PLOM_REQUIRE(aux1 && S && VT && muReal && muImag && bJov && Mphi && ws && info, PLOM_ERR_ARG,
               "dmd_reduced: null pointer");
  const int N = (int)r, T = (int)nt;
  PLOM_REQUIRE(ws_bytes >= dmd_reduced_workspace(N, T), PLOM_ERR_WORKSPACE,
               "dmd_reduced: workspace too small");
  Arena a(ws, ws_bytes);
  DmdBufs B;
  B.A = a.take<double>((size_t)N * N);
  B.Z = a.take<double>((size_t)N * N);
  B.wr = a.take<double>(N);
  B.wi = a.take<double>(N);
  B.Wv = a.take<double>((size_t)2 * N * N);
  B.Y = a.take<double>((size_t)2 * N * N);
  B.Pm = a.take<double>((size_t)2 * N * N);
  B.qv = a.take<double>((size_t)2 * N);
  B.bv = a.take<double>((size_t)2 * N);
  B.babs = a.take<double>(N);
  B.order = a.take<int>(N);
  B.Vr = a.take<double>((size_t)2 * N * T);
  B.flip = a.take<int>(N);
  cudaStream_t st = (cudaStream_t)stream;
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, st));
  const size_t shbytes = sizeof(double) * (2 * (size_t)N + 16);
  PLOM_REQUIRE(shbytes <= 48 * 1024, PLOM_ERR_ARG, "dmd_reduced: r too large for one CTA");
  ProfScope prof("dmd_reduced_fp64", st, 0.0, 0.0, 5);
  // eigenpairs of Atilde and the Vandermonde rows (one CTA), P and q (spread
  // over the GPU), the amplitude solve and ordering (one CTA), the mode matrix
  dmd_eig_kernel<<<1, 256, shbytes, st>>>(aux1, S, VT, N, T, B, muReal, muImag, bJov, Mphi, info);
  PLOM_CHECK_LAUNCH();
  dmd_pq_kernel<<<(unsigned)((N * N + 7) / 8 + N), 256, 0, st>>>(S, VT, N, T, B, info);
  PLOM_CHECK_LAUNCH();
  dmd_amp_kernel<<<1, 256, 0, st>>>(N, B, muReal, muImag, bJov, info);
  PLOM_CHECK_LAUNCH();
  dmd_mphi_kernel<<<(unsigned)cdiv((int64_t)T * N, 256), 256, 0, st>>>(S, VT, N, T, B, Mphi, info);
  PLOM_CHECK_LAUNCH();
  dmd_flip_kernel<<<(unsigned)cdiv((int64_t)T, 256), 256, 0, st>>>(N, T, B, Mphi, info);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}
