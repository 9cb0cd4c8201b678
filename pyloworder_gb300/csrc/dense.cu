// FP64 small dense linear algebra on the GPU for the n x n stage of the SVD
// path: shifted Cholesky, triangular inverse and one-sided Jacobi SVD.
//
// Every routine takes a batch of equally sized problems (batch = 1 for the
// n = 1024 TSQR-SVD of the snapshot matrix, batch = 129 for SPOD's
// per-frequency problems) and runs as ONE cooperative launch whose blocks
// advance in lock-step through grid-wide barriers: the panel/trailing steps
// of the blocked Cholesky and the parallel (round-robin) rotation steps of
// Jacobi.  GB300's FP64 rate is ~1/64 of FP32, so the work is spread over
// all SMs rather than one CTA per problem.
//
// Reference counterparts (pyLowOrder): dsvd -> LAPACKE_dgesdd
// (pyLOM/vmmath/src/svd.c:83-139) for the SVD of R; the Cholesky/inverse are
// the n x n pieces of the CholeskyQR form of the TSQR R-factor merge that
// replaces dtsqr's per-rank dgeqrf (svd.c:565-676).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "plom_common.cuh"
#include "plom_kernels.cuh"

namespace cg = cooperative_groups;

namespace plom {

constexpr int NB = 32;  // block size of the blocked Cholesky
constexpr int CHOL_ROUNDS = 8;
constexpr int JACOBI_MAX_SWEEPS = 40;

// ---------------------------------------------------------------------------
// Cholesky
// ---------------------------------------------------------------------------
struct CholState {
  double* trace;  // [batch]
  double* shift;  // [batch]
  int* status;    // [batch]: 0 pending, 1 done, 2 failed in this round
  int* shifts_used;
  int* pending;   // [CHOL_ROUNDS] counters
};

__global__ void __launch_bounds__(256) chol_coop_kernel(const double* __restrict__ G,
                                                        double* __restrict__ R,
                                                        double* __restrict__ Dinv, int n,
                                                        int batch, double rel0, double relfail,
                                                        CholState stt, int* info) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double S[NB][NB + 1];
  __shared__ double P[NB][NB + 1];
  __shared__ int sflag;
  const int tid = threadIdx.x;
  const int T = (n + NB - 1) / NB;
  const int64_t nn = (int64_t)n * n;

  // per-problem trace and initial shift
  for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    double s = 0.0;
    for (int i = tid; i < n; i += blockDim.x) s += G[b * nn + (int64_t)i * n + i];
    s = warp_sum(s);
    __shared__ double red[8];
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      stt.trace[b] = t;
      stt.shift[b] = rel0 * t / n;
      stt.status[b] = (isfinite(t) && t > 0.0) ? 0 : 3;  // 3 = bad input
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && tid < CHOL_ROUNDS) stt.pending[tid] = 0;
  grid.sync();

  for (int round = 0; round < CHOL_ROUNDS; ++round) {
    // R = upper(G) + shift I for pending problems
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + tid; e < nn * batch;
         e += (int64_t)gridDim.x * blockDim.x) {
      int64_t b = e / nn, r = e % nn;
      if (stt.status[b] != 0) continue;
      int i = (int)(r / n), j = (int)(r % n);
      double v = (i <= j) ? G[e] : 0.0;
      if (i == j) v += stt.shift[b];
      R[e] = v;
    }
    grid.sync();
    for (int k = 0; k < T; ++k) {
      const int k0 = k * NB, nbk = min(NB, n - k0);
      // (1) diagonal block: factor + invert, one CTA per problem
      for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        if (stt.status[b] != 0) continue;
        double* Rb = R + b * nn;
        for (int e = tid; e < NB * NB; e += blockDim.x) {
          int i = e / NB, j = e % NB;
          S[i][j] = (i < nbk && j < nbk) ? Rb[(int64_t)(k0 + i) * n + k0 + j] : 0.0;
        }
        __syncthreads();
        for (int j = 0; j < nbk; ++j) {
          if (tid == 0) {
            double d = S[j][j];
            bool ok = (d > 0.0) && isfinite(d);
            sflag = ok ? 1 : 0;
            S[j][j] = ok ? sqrt(d) : 1.0;
          }
          __syncthreads();
          if (!sflag) break;
          const double piv = S[j][j];
          for (int i = j + 1 + tid; i < nbk; i += blockDim.x) S[j][i] /= piv;
          __syncthreads();
          const int w = nbk - j - 1;
          for (int e = tid; e < w * w; e += blockDim.x) {
            int a = j + 1 + e / w, c = j + 1 + e % w;
            if (a <= c) S[a][c] -= S[j][a] * S[j][c];
          }
          __syncthreads();
        }
        if (!sflag) {
          if (tid == 0) stt.status[b] = 2;
          __syncthreads();
          continue;
        }
        // write back upper block, zero strict lower part
        for (int e = tid; e < nbk * nbk; e += blockDim.x) {
          int i = e / nbk, j = e % nbk;
          Rb[(int64_t)(k0 + i) * n + k0 + j] = (i <= j) ? S[i][j] : 0.0;
        }
        // inverse of the upper triangular block: thread c -> column c
        double* Db = Dinv + (int64_t)b * NB * NB;
        if (tid < nbk) {
          const int c = tid;
          double x[NB];
#pragma unroll
          for (int i = 0; i < NB; ++i) x[i] = 0.0;
          x[c] = 1.0 / S[c][c];
          for (int i = c - 1; i >= 0; --i) {
            double acc = 0.0;
            for (int t = i + 1; t <= c; ++t) acc += S[i][t] * x[t];
            x[i] = -acc / S[i][i];
          }
          for (int i = 0; i < NB; ++i) Db[i * NB + c] = (i <= c) ? x[i] : 0.0;
        }
        __syncthreads();
      }
      grid.sync();
      // (2) panel: R_kj = Dinv_k^T R_kj for j > k
      const int ntask_p = (T - k - 1) * batch;
      for (int t = blockIdx.x; t < ntask_p; t += gridDim.x) {
        int b = t / (T - k - 1), j = k + 1 + t % (T - k - 1);
        if (stt.status[b] != 0) continue;
        const int j0 = j * NB, nbj = min(NB, n - j0);
        double* Rb = R + b * nn;
        const double* Db = Dinv + (int64_t)b * NB * NB;
        for (int e = tid; e < NB * NB; e += blockDim.x) {
          int i = e / NB, c = e % NB;
          S[i][c] = Db[i * NB + c];
          P[i][c] = (i < nbk && c < nbj) ? Rb[(int64_t)(k0 + i) * n + j0 + c] : 0.0;
        }
        __syncthreads();
        for (int e = tid; e < nbk * nbj; e += blockDim.x) {
          int r = e / nbj, c = e % nbj;
          double acc = 0.0;
          for (int q = 0; q <= r; ++q) acc += S[q][r] * P[q][c];
          Rb[(int64_t)(k0 + r) * n + j0 + c] = acc;
        }
        __syncthreads();
      }
      grid.sync();
      // (3) trailing update R_ac -= R_ka^T R_kc for k < a <= c
      const int w = T - k - 1;
      const int ntask_t = w * (w + 1) / 2 * batch;
      for (int t = blockIdx.x; t < ntask_t; t += gridDim.x) {
        int b = t / (w * (w + 1) / 2);
        int r = t % (w * (w + 1) / 2);
        // map r -> (a, c) with 0 <= a <= c < w
        int a = 0;
        while (r >= w - a) {
          r -= w - a;
          ++a;
        }
        int c = a + r;
        a += k + 1;
        c += k + 1;
        if (stt.status[b] != 0) continue;
        const int a0 = a * NB, c0 = c * NB, nba = min(NB, n - a0), nbc = min(NB, n - c0);
        double* Rb = R + b * nn;
        for (int e = tid; e < NB * NB; e += blockDim.x) {
          int i = e / NB, q = e % NB;
          S[i][q] = (i < nbk && q < nba) ? Rb[(int64_t)(k0 + i) * n + a0 + q] : 0.0;
          P[i][q] = (i < nbk && q < nbc) ? Rb[(int64_t)(k0 + i) * n + c0 + q] : 0.0;
        }
        __syncthreads();
        for (int e = tid; e < nba * nbc; e += blockDim.x) {
          int r2 = e / nbc, s2 = e % nbc;
          double acc = 0.0;
#pragma unroll 8
          for (int q = 0; q < NB; ++q) acc += S[q][r2] * P[q][s2];
          Rb[(int64_t)(a0 + r2) * n + c0 + s2] -= acc;
        }
        __syncthreads();
      }
      grid.sync();
    }
    // evaluate the round
    for (int b = blockIdx.x * blockDim.x + tid; b < batch; b += gridDim.x * blockDim.x) {
      int s = stt.status[b];
      if (s == 0) {
        stt.status[b] = 1;
      } else if (s == 2) {
        double base = relfail * stt.trace[b] / n;
        stt.shift[b] = fmax(stt.shift[b] * 100.0, base);
        stt.status[b] = 0;
        atomicAdd(&stt.pending[round], 1);
        atomicMax(stt.shifts_used, round + 1);
      }
    }
    grid.sync();
    if (stt.pending[round] == 0) break;
  }
  // problems still pending after all rounds, or with bad input
  for (int b = blockIdx.x * blockDim.x + tid; b < batch; b += gridDim.x * blockDim.x) {
    int s = stt.status[b];
    if (s == 0 || s == 2) atomicMax(&info[ST_FAIL], PLOM_NUM_CHOLESKY);
    if (s == 3) atomicMax(&info[ST_FAIL], PLOM_NUM_NONFINITE);
  }
  if (blockIdx.x == 0 && tid == 0) atomicMax(&info[ST_SHIFTS], *stt.shifts_used);
}

static int coop_blocks(const void* kern, int threads, size_t smem, int want) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (per_sm < 1) per_sm = 1;
  int cap = per_sm * num_sms();
  return std::max(1, std::min(cap, want));
}

int chol_shifted(const double* G, double* R, int n, int batch, double rel0, double relfail,
                 int* info, Arena& ws, cudaStream_t st) {
  CholState s;
  s.trace = ws.take<double>(batch);
  s.shift = ws.take<double>(batch);
  s.status = ws.take<int>(batch);
  s.shifts_used = ws.take<int>(1);
  s.pending = ws.take<int>(CHOL_ROUNDS);
  double* Dinv = ws.take<double>((size_t)batch * NB * NB);
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "chol: workspace too small");
  PLOM_REQUIRE(G && R && info, PLOM_ERR_ARG, "chol: null pointer");
  PLOM_CHECK_CUDA(cudaMemsetAsync(s.shifts_used, 0, sizeof(int), st));
  const int T = (n + NB - 1) / NB;
  int want = std::max(batch * std::max(1, T * (T + 1) / 2), 1);
  int blocks = coop_blocks((const void*)chol_coop_kernel, 256, 0, want);
  ProfScope prof("chol_fp64", st, (double)n * n * n / 3.0 * batch, 16.0 * n * n * batch);
  void* args[] = {(void*)&G, (void*)&R, (void*)&Dinv, (void*)&n, (void*)&batch,
                  (void*)&rel0, (void*)&relfail, (void*)&s, (void*)&info};
  PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void*)chol_coop_kernel, dim3(blocks),
                                              dim3(256), args, 0, st));
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// triangular inverse: W = R^{-1}, R upper (batch).  One CTA per column
// (column-oriented back substitution on R^T rows, one barrier per step).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) trtri_col_kernel(const double* __restrict__ Rt,
                                                         double* __restrict__ W, int n,
                                                         int batch) {
  __shared__ double wk[2];
  const int tid = threadIdx.x;
  const int64_t nn = (int64_t)n * n;
  constexpr int PER = 4;  // rows per thread: n <= 4 * blockDim
  for (int64_t task = blockIdx.x; task < (int64_t)n * batch; task += gridDim.x) {
    const int64_t b = task / n;
    const int j = (int)(task % n);
    const double* Rb = Rt + b * nn;  // Rb[k*n + i] = R[i][k]
    double w[PER];
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      int i = tid + p * blockDim.x;
      w[p] = (i == j) ? 1.0 : 0.0;
    }
    for (int k = j; k >= 0; --k) {
      const int owner = k % blockDim.x, slot = k / blockDim.x;
      if (tid == owner) {
        double v = 0.0;
#pragma unroll
        for (int p = 0; p < PER; ++p)
          if (p == slot) v = w[p] / Rb[(int64_t)k * n + k];
#pragma unroll
        for (int p = 0; p < PER; ++p)
          if (p == slot) w[p] = v;
        wk[k & 1] = v;
      }
      __syncthreads();
      const double x = wk[k & 1];
      const double* col = Rb + (int64_t)k * n;
#pragma unroll
      for (int p = 0; p < PER; ++p) {
        int i = tid + p * blockDim.x;
        if (i < k) w[p] -= col[i] * x;
      }
    }
    __syncthreads();
    double* Wb = W + b * nn;
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      int i = tid + p * blockDim.x;
      if (i < n) Wb[(int64_t)i * n + j] = (i <= j) ? w[p] : 0.0;
    }
    __syncthreads();
  }
}

__global__ void transpose_f64_kernel(const double* __restrict__ in, double* __restrict__ out,
                                     int64_t rows, int64_t cols, int batch) {
  __shared__ double tile[32][33];
  const int64_t rc = rows * cols;
  for (int b = blockIdx.z; b < batch; b += gridDim.z) {
    int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t r = r0 + i, c = c0 + threadIdx.x;
      if (r < rows && c < cols) tile[i][threadIdx.x] = in[b * rc + r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t c = c0 + i, r = r0 + threadIdx.x;
      if (r < rows && c < cols) out[b * rc + c * rows + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}

int transpose_f64(const double* in, double* out, int64_t rows, int64_t cols, int batch,
                  cudaStream_t st) {
  if (rows == 0 || cols == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(in && out, PLOM_ERR_ARG, "transpose: null pointer");
  dim3 grid((unsigned)cdiv(cols, 32), (unsigned)cdiv(rows, 32), (unsigned)std::min(batch, 65535));
  transpose_f64_kernel<<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

int trtri_upper(const double* R, double* W, int n, int batch, Arena& ws, cudaStream_t st) {
  double* Rt = ws.take<double>((size_t)n * n * batch);
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "trtri: workspace too small");
  PLOM_REQUIRE(R && W, PLOM_ERR_ARG, "trtri: null pointer");
  PLOM_REQUIRE(n <= 4096, PLOM_ERR_UNSUPPORTED, "trtri: n > 4096");
  PLOM_TRY(transpose_f64(R, Rt, n, n, batch, st));
  int threads = std::min(1024, std::max(32, (int)cdiv(n, 4 * 32) * 32));
  while ((int64_t)threads * 4 < n) threads += 32;
  int64_t tasks = (int64_t)n * batch;
  int blocks = (int)std::min<int64_t>(tasks, (int64_t)num_sms() * 2);
  ProfScope prof("trtri_fp64", st, (double)n * n * n / 3.0 * batch, 16.0 * n * n * batch);
  trtri_col_kernel<<<blocks, threads, 0, st>>>(Rt, W, n, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// one-sided Jacobi SVD (Hestenes), real or complex, cooperative
// ---------------------------------------------------------------------------
template <typename T>
struct JacState {
  T* At;        // batch x n x (n*cw): rows = columns of A
  T* Vt;        // batch x n x (n*cw): rows = columns of V
  int* counts;  // [JACOBI_MAX_SWEEPS]
  int* perm;    // batch x n
  T* nrm;       // batch x n
};

__device__ __forceinline__ void rr_pair(int step, int k, int np, int& a, int& b) {
  // round-robin (circle method) over np (even) players; np-1 steps
  const int m = np - 1;
  if (k == 0) {
    a = 0;
    b = 1 + (step % m);
  } else {
    a = 1 + (step + k) % m;
    b = 1 + (step - k + m) % m;
  }
}

// T = double: the SVD itself.  T = float: a fast pass whose accumulated
// rotations (js.Vt) precondition the FP64 pass; with S == nullptr the output
// stage is skipped.
template <typename T>
__global__ void __launch_bounds__(128) jacobi_coop_kernel(const double* __restrict__ A, int n,
                                                          int batch, int cplx, JacState<T> js,
                                                          double* __restrict__ S,
                                                          double* __restrict__ U,
                                                          double* __restrict__ VH, int* info) {
  cg::grid_group grid = cg::this_grid();
  const int cw = cplx ? 2 : 1;
  const int64_t rl = (int64_t)n * cw;  // doubles per row
  const int64_t mat = (int64_t)n * rl;
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;

  // init: At[j][i] = A[i][j] (complex: element-wise, no conjugation), Vt = I
  for (int64_t e = gtid; e < (int64_t)batch * n * n; e += gthreads) {
    int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    int i = (int)(r / n), j = (int)(r % n);
    const double* src = A + b * mat + (int64_t)i * rl + (int64_t)j * cw;
    T* dst = js.At + b * mat + (int64_t)j * rl + (int64_t)i * cw;
    dst[0] = (T)src[0];
    if (cplx) dst[1] = (T)src[1];
    T* v = js.Vt + b * mat + (int64_t)i * rl + (int64_t)j * cw;
    v[0] = (i == j) ? T(1) : T(0);
    if (cplx) v[1] = T(0);
  }
  if (gtid < JACOBI_MAX_SWEEPS) js.counts[gtid] = 0;
  grid.sync();

  const int np = n + (n & 1);
  const int pairs = np / 2;
  // rotate while |a_p^H a_q| > n eps ||a_p|| ||a_q||: below that the pair is
  // orthogonal to working precision (one-sided Jacobi stopping rule)
  const T tol = (sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07)) * (T)n;
  int sweep = 0;
  for (; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    int myrot = 0;
    for (int step = 0; step < np - 1; ++step) {
      for (int64_t task = gwarp; task < (int64_t)pairs * batch; task += nwarps) {
        const int64_t b = task / pairs;
        int p, q;
        rr_pair(step, (int)(task % pairs), np, p, q);
        if (p >= n || q >= n) continue;
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        T* ap = js.At + b * mat + (int64_t)p * rl;
        T* aq = js.At + b * mat + (int64_t)q * rl;
        T alpha = 0, beta = 0, gr = 0, gi = 0;
        if (!cplx) {
          for (int64_t i = lane; i < n; i += 32) {
            T x = ap[i], y = aq[i];
            alpha = fma(x, x, alpha);
            beta = fma(y, y, beta);
            gr = fma(x, y, gr);
          }
        } else {
          for (int64_t i = lane; i < n; i += 32) {
            T xr = ap[2 * i], xi = ap[2 * i + 1], yr = aq[2 * i], yi = aq[2 * i + 1];
            alpha += xr * xr + xi * xi;
            beta += yr * yr + yi * yi;
            gr += xr * yr + xi * yi;  // conj(x) * y
            gi += xr * yi - xi * yr;
          }
        }
        alpha = warp_sum(alpha);
        beta = warp_sum(beta);
        gr = warp_sum(gr);
        if (cplx) gi = warp_sum(gi);
        const T gabs = cplx ? hypot(gr, gi) : fabs(gr);
        if (!(alpha > T(0) && beta > T(0)) || !(gabs > tol * sqrt(alpha) * sqrt(beta))) continue;
        ++myrot;
        const T zeta = (beta - alpha) / (T(2) * gabs);
        const T t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + t * t), s = c * t;
        // phase e^{i phi} = gamma/|gamma| (real: sign of gamma)
        const T er = cplx ? gr / gabs : copysign(T(1), gr), ei = cplx ? gi / gabs : T(0);
        T* vp = js.Vt + b * mat + (int64_t)p * rl;
        T* vq = js.Vt + b * mat + (int64_t)q * rl;
        // a' = c a - s e^{-i phi} b ;  b' = s e^{i phi} a + c b
        for (int side = 0; side < 2; ++side) {
          T* x = side ? vp : ap;
          T* y = side ? vq : aq;
          if (!cplx) {
            for (int64_t i = lane; i < n; i += 32) {
              T xv = x[i], yv = y[i];
              x[i] = c * xv - s * er * yv;
              y[i] = s * er * xv + c * yv;
            }
          } else {
            for (int64_t i = lane; i < n; i += 32) {
              T xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
              // e^{-i phi} y = (er - i ei)(yr + i yi)
              T zr = er * yr + ei * yi, zi = er * yi - ei * yr;
              // e^{i phi} x = (er + i ei)(xr + i xi)
              T wr = er * xr - ei * xi, wi = er * xi + ei * xr;
              x[2 * i] = c * xr - s * zr;
              x[2 * i + 1] = c * xi - s * zi;
              y[2 * i] = s * wr + c * yr;
              y[2 * i + 1] = s * wi + c * yi;
            }
          }
        }
      }
      grid.sync();
    }
    if (lane == 0 && myrot) atomicAdd(&js.counts[sweep], myrot);
    grid.sync();
    if (js.counts[sweep] == 0) break;
  }
  if (S == nullptr) return;  // preconditioning pass: only js.Vt is wanted
  if (gtid == 0) {
    info[ST_SWEEPS] = sweep + 1;
    if (sweep >= JACOBI_MAX_SWEEPS) atomicMax(&info[ST_FAIL], PLOM_NUM_JACOBI);
  }
  // column norms
  for (int64_t task = gwarp; task < (int64_t)batch * n; task += nwarps) {
    const T* a = js.At + (task / n) * mat + (task % n) * rl;
    double s = 0.0;
    for (int64_t i = lane; i < rl; i += 32) s = fma((double)a[i], (double)a[i], s);
    s = warp_sum(s);
    if (lane == 0) js.nrm[task] = (T)sqrt(s);
  }
  grid.sync();
  // descending order: rank of each column (ties broken by index)
  for (int64_t e = gtid; e < (int64_t)batch * n; e += gthreads) {
    const int64_t b = e / n;
    const int j = (int)(e % n);
    const T sj = js.nrm[e];
    int rank = 0;
    for (int k = 0; k < n; ++k) {
      T sk = js.nrm[b * n + k];
      rank += (sk > sj) || (sk == sj && k < j);
    }
    js.perm[b * n + rank] = j;
  }
  grid.sync();
  // outputs: S, U[i][k] = At[perm k][i] / s, VH[k][:] = conj(Vt[perm k][:])
  for (int64_t e = gtid; e < (int64_t)batch * n * n; e += gthreads) {
    const int64_t b = e / ((int64_t)n * n);
    const int64_t r = e % ((int64_t)n * n);
    const int k = (int)(r / n), i = (int)(r % n);
    const int src = js.perm[b * n + k];
    const double sk = (double)js.nrm[b * n + src];
    if (i == 0) S[b * n + k] = sk;
    const double inv = sk > 0.0 ? 1.0 / sk : 0.0;
    const T* a = js.At + b * mat + (int64_t)src * rl + (int64_t)i * cw;
    double* u = U + b * mat + (int64_t)i * rl + (int64_t)k * cw;
    u[0] = (double)a[0] * inv;
    if (cplx) u[1] = (double)a[1] * inv;
    const T* v = js.Vt + b * mat + (int64_t)src * rl + (int64_t)i * cw;
    double* vh = VH + b * mat + (int64_t)k * rl + (int64_t)i * cw;
    vh[0] = (double)v[0];
    if (cplx) vh[1] = -(double)v[1];
  }
}

// FP32 pre-pass + FP64 finish is used for real matrices from this size on
constexpr int JACOBI_PRECOND_MIN_N = 128;

template <typename T>
static int jacobi_launch(const double* A, int n, int batch, int cplx, JacState<T>& js, double* S,
                         double* U, double* VH, int* info, cudaStream_t st) {
  const int np = n + (n & 1);
  // one warp per column pair, 4 warps per CTA: spreads the FP64 work over
  // as many SMs as there are pairs / 4
  int want = (int)std::max<int64_t>(1, cdiv((int64_t)np / 2 * batch, 4));
  int blocks = coop_blocks((const void*)jacobi_coop_kernel<T>, 128, 0, want);
  void* args[] = {(void*)&A, (void*)&n, (void*)&batch, (void*)&cplx, (void*)&js,
                  (void*)&S, (void*)&U, (void*)&VH, (void*)&info};
  ProfScope prof(sizeof(T) == 8 ? "jacobi_svd_fp64" : "jacobi_pass_fp32", st, 0.0,
                 (double)sizeof(T) * 3.0 * n * n * batch * (cplx ? 2 : 1));
  PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_coop_kernel<T>, dim3(blocks),
                                              dim3(128), args, 0, st));
  return PLOM_OK;
}

template <typename T>
static void carve_jac(Arena& ws, JacState<T>& js, int n, int batch, int cplx) {
  const size_t mat = (size_t)n * n * (cplx ? 2 : 1);
  js.At = ws.take<T>(mat * batch);
  js.Vt = ws.take<T>(mat * batch);
  js.counts = ws.take<int>(JACOBI_MAX_SWEEPS);
  js.perm = ws.take<int>((size_t)batch * n);
  js.nrm = ws.take<T>((size_t)batch * n);
}

size_t dense_workspace(int n, int batch, int cplx) {
  Arena a(nullptr, 0);
  JacState<double> js;
  carve_jac(a, js, n, batch, cplx);
  return a.off + 256;
}

// Real n x n SVD with an FP32 pre-pass: one-sided Jacobi in FP32 yields V0;
// V0 is re-orthogonalised in FP64 (one CholeskyQR step), A1 = A V0 has
// nearly orthogonal columns, and the FP64 Jacobi on A1 converges in a few
// sweeps; V = V0 V1.
static int jacobi_svd_precond(const double* A, int n, double* S, double* U, double* VH, int* info,
                              Arena& ws, cudaStream_t st) {
  const size_t nn = (size_t)n * n;
  JacState<float> j32;
  carve_jac(ws, j32, n, 1, 0);
  double* V0 = ws.take<double>(nn);
  double* G = ws.take<double>(nn);
  double* Rv = ws.take<double>(nn);
  double* Wv = ws.take<double>(nn);
  double* V0n = ws.take<double>(nn);
  double* A1 = ws.take<double>(nn);
  double* VH1 = ws.take<double>(nn);
  double* V0nT = ws.take<double>(nn);
  const size_t mark = ws.off;
  size_t need = mark;
  // FP64 pass state (reuses the scratch after the small FP64 products)
  JacState<double> j64;
  carve_jac(ws, j64, n, 1, 0);
  need = std::max(need, ws.off);
  ws.off = mark;
  if (ws.measuring()) {
    gemm_tn<double, double, double, double>(V0, n, V0, n, G, n, n, n, n, true, ws, st);
    need = std::max(need, ws.off);
    ws.off = mark;
    chol_shifted(G, Rv, n, 1, 0.0, 1e-12, info, ws, st);
    need = std::max(need, ws.off);
    ws.off = mark;
    trtri_upper(Rv, Wv, n, 1, ws, st);
    ws.off = std::max(need, ws.off);
    return PLOM_OK;
  }
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi: workspace too small");
  PLOM_TRY(jacobi_launch<float>(A, n, 1, 0, j32, nullptr, nullptr, nullptr, info, st));
  {
    double* Vt64 = A1;  // temporarily: rows = v_k in FP64
    PLOM_TRY((convert<float, double>(j32.Vt, Vt64, (int64_t)nn, st)));
    PLOM_TRY(transpose_f64(Vt64, V0, n, n, 1, st));  // columns = v_k
  }
  PLOM_TRY((gemm_tn<double, double, double, double>(V0, n, V0, n, G, n, n, n, n, true, ws, st)));
  need = std::max(need, ws.off);
  ws.off = mark;
  PLOM_TRY(chol_shifted(G, Rv, n, 1, 0.0, 1e-12, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  PLOM_TRY(trtri_upper(Rv, Wv, n, 1, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  PLOM_TRY((gemm_nn<double, double, double, double>(V0, n, Wv, n, V0n, n, n, n, n, st)));
  PLOM_TRY((gemm_nn<double, double, double, double>(A, n, V0n, n, A1, n, n, n, n, st)));
  carve_jac(ws, j64, n, 1, 0);
  PLOM_TRY(jacobi_launch<double>(A1, n, 1, 0, j64, S, U, VH1, info, st));
  // VH = VH1 V0n^T  (row k = (V0n v1_k)^T)
  PLOM_TRY(transpose_f64(V0n, V0nT, n, n, 1, st));
  PLOM_TRY((gemm_nn<double, double, double, double>(VH1, n, V0nT, n, VH, n, n, n, n, st)));
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

int jacobi_svd(const double* A, int n, int batch, int cplx, double* S, double* U, double* VH,
               int* info, Arena& ws, cudaStream_t st) {
  if (!cplx && batch == 1 && n >= JACOBI_PRECOND_MIN_N)
    return jacobi_svd_precond(A, n, S, U, VH, info, ws, st);
  JacState<double> js;
  carve_jac(ws, js, n, batch, cplx);
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi: workspace too small");
  PLOM_REQUIRE(A && S && U && VH && info, PLOM_ERR_ARG, "jacobi: null pointer");
  return jacobi_launch<double>(A, n, batch, cplx, js, S, U, VH, info, st);
}

// ---------------------------------------------------------------------------
// complex <-> real embedding helpers (interleaved ordering re0, im0, re1, ...)
// real_embed(c) block = [[re, -im], [im, re]]
// ---------------------------------------------------------------------------
__global__ void complexify_gram_kernel(const double* __restrict__ H, double* __restrict__ G,
                                       int n, int batch) {
  const int64_t N2 = 2 * (int64_t)n;
  const int64_t mat = N2 * N2;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)batch * n * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    int64_t a = r / n, c = r % n;
    const double* h = H + b * mat;
    double h00 = h[(2 * a) * N2 + 2 * c], h11 = h[(2 * a + 1) * N2 + 2 * c + 1];
    double h01 = h[(2 * a) * N2 + 2 * c + 1], h10 = h[(2 * a + 1) * N2 + 2 * c];
    double re = h00 + h11, im = h01 - h10;  // (Z^H Z)_{ac}
    double* g = G + b * mat;
    g[(2 * a) * N2 + 2 * c] = re;
    g[(2 * a) * N2 + 2 * c + 1] = -im;
    g[(2 * a + 1) * N2 + 2 * c] = im;
    g[(2 * a + 1) * N2 + 2 * c + 1] = re;
  }
}

__global__ void embed_rowform_kernel(const double* __restrict__ E, double* __restrict__ F, int n,
                                     int batch) {
  const int64_t N2 = 2 * (int64_t)n;
  const int64_t mat = N2 * N2;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)batch * n * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    int64_t a = r / n, c = r % n;
    const double* s = E + b * mat;
    double re = s[(2 * a) * N2 + 2 * c], im = s[(2 * a + 1) * N2 + 2 * c];
    double* d = F + b * mat;
    d[(2 * a) * N2 + 2 * c] = re;
    d[(2 * a) * N2 + 2 * c + 1] = im;
    d[(2 * a + 1) * N2 + 2 * c] = -im;
    d[(2 * a + 1) * N2 + 2 * c + 1] = re;
  }
}

__global__ void complex_to_embed_kernel(const double* __restrict__ C, double* __restrict__ E,
                                        int n, int batch) {
  const int64_t N2 = 2 * (int64_t)n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)batch * n * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    int64_t a = r / n, c = r % n;
    double re = C[2 * e], im = C[2 * e + 1];
    double* d = E + b * N2 * N2;
    d[(2 * a) * N2 + 2 * c] = re;
    d[(2 * a) * N2 + 2 * c + 1] = -im;
    d[(2 * a + 1) * N2 + 2 * c] = im;
    d[(2 * a + 1) * N2 + 2 * c + 1] = re;
  }
}

__global__ void embed_to_complex_kernel(const double* __restrict__ E, double* __restrict__ C,
                                        int n, int batch) {
  const int64_t N2 = 2 * (int64_t)n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)batch * n * n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    int64_t a = r / n, c = r % n;
    const double* s = E + b * N2 * N2;
    C[2 * e] = s[(2 * a) * N2 + 2 * c];
    C[2 * e + 1] = s[(2 * a + 1) * N2 + 2 * c];
  }
}

static int grid_for(int64_t work) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(work, 256), (int64_t)num_sms() * 16));
}

int complexify_gram(const double* H, double* G, int n, int batch, cudaStream_t st) {
  PLOM_REQUIRE(H && G, PLOM_ERR_ARG, "complexify: null pointer");
  complexify_gram_kernel<<<grid_for((int64_t)n * n * batch), 256, 0, st>>>(H, G, n, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}
int embed_to_rowform(const double* E, double* F, int n, int batch, cudaStream_t st) {
  PLOM_REQUIRE(E && F, PLOM_ERR_ARG, "rowform: null pointer");
  embed_rowform_kernel<<<grid_for((int64_t)n * n * batch), 256, 0, st>>>(E, F, n, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}
int complex_to_embed(const double* C, double* E, int n, int batch, cudaStream_t st) {
  PLOM_REQUIRE(C && E, PLOM_ERR_ARG, "embed: null pointer");
  complex_to_embed_kernel<<<grid_for((int64_t)n * n * batch), 256, 0, st>>>(C, E, n, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}
int embed_to_complex(const double* E, double* C, int n, int batch, cudaStream_t st) {
  PLOM_REQUIRE(E && C, PLOM_ERR_ARG, "unembed: null pointer");
  embed_to_complex_kernel<<<grid_for((int64_t)n * n * batch), 256, 0, st>>>(E, C, n, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

}  // namespace plom
