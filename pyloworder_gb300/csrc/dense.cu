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
  double* colsq;  // [CHOL_NEAR_GROUPS x n]: partial column sums of the near-identity test
};

// Unshifted factorisation of one Gram close to the identity, G = I + E (the
// later CholeskyQR passes): R = I + X with X = triu(E, 1) + diag(E) / 2 gives
// R^T R = G + X^T X exactly, and |(X^T X)_ij| <= max_j ||X e_j||^2.  When the
// caller allows a perturbation of G (near_tol > 0: the mixed form, whose
// operands carry 22 bits) and that bound is at most near_tol, R is written
// directly and the blocked factorisation is skipped.
constexpr int CHOL_NEAR_GROUPS = 8;   // row groups of the column sums

__global__ void __launch_bounds__(256) chol_coop_kernel(const double* __restrict__ G,
                                                        double* __restrict__ R,
                                                        double* __restrict__ Dinv, int n,
                                                        int batch, double rel0, double relfail,
                                                        double near_tol, CholState stt, int* info) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double S[NB][NB + 1];
  __shared__ double P[NB][NB + 1];
  __shared__ double rpiv;
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
  if (batch == 1 && rel0 == 0.0 && stt.colsq) {
    // near-identity test: partial sums of X's squared columns over
    // CHOL_NEAR_GROUPS row groups (thread per column, coalesced rows), summed
    // per column in group order and compared with the bound (every block
    // reaches the same answer from the same partials)
    const int rows_g = (n + CHOL_NEAR_GROUPS - 1) / CHOL_NEAR_GROUPS;
    const int cblocks = (n + blockDim.x - 1) / blockDim.x;
    for (int task = blockIdx.x; task < cblocks * CHOL_NEAR_GROUPS; task += gridDim.x) {
      const int g = task / cblocks, j = (task % cblocks) * blockDim.x + tid;
      if (j >= n) continue;
      double acc = 0.0;
      const int i1 = min(min(n, (g + 1) * rows_g), j + 1);
      for (int i = g * rows_g; i < i1; ++i) {
        const double e = G[(int64_t)i * n + j];
        const double x = (i == j) ? 0.5 * (e - 1.0) : e;
        acc = fma(x, x, acc);
      }
      stt.colsq[(int64_t)g * n + j] = acc;
    }
    grid.sync();
    int ok = 1;
    for (int j = tid; j < n; j += blockDim.x) {
      double c = 0.0;
      for (int g = 0; g < CHOL_NEAR_GROUPS; ++g) c += stt.colsq[(int64_t)g * n + j];
      if (!(c <= near_tol)) ok = 0;  // (a NaN fails the test)
    }
    const bool near = __syncthreads_and(ok) && stt.status[0] == 0;
    if (near) {
      for (int64_t e = (int64_t)blockIdx.x * blockDim.x + tid; e < nn;
           e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e % n);
        R[e] = (i < j) ? G[e] : (i == j ? 1.0 + 0.5 * (G[e] - 1.0) : 0.0);
      }
      if (blockIdx.x == 0 && tid == 0) atomicAdd(&info[ST_NEAR], 1);
      return;  // every block takes the same branch: no grid barrier follows
    }
  }
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
    // (1) diagonal block of problem b at block step k, by one CTA: the factor
    // and Z = R_kk^-T row by row in the same steps (forward substitution of
    // R^T Z = I):
    //   piv = sqrt(S_jj), R_j. = S_j. / piv, Z_j. = P_j. / piv,
    //   S_ac -= R_ja R_jc (j < a <= c),  P_a. -= R_ja Z_j. (a > j),  P = I at start
    // Block step k + 1's diagonal block is factored inside step k's trailing
    // update, by the CTA that updates it (look-ahead: one grid barrier less
    // per block step, and the factorisation overlaps the other CTAs' updates)
    auto diag_block = [&](int b, int k) {
      const int k0 = k * NB, nbk = min(NB, n - k0);
      if (stt.status[b] != 0) return;
      double* Rb = R + b * nn;
      for (int e = tid; e < NB * NB; e += blockDim.x) {
        int i = e / NB, j = e % NB;
        S[i][j] = (i < nbk && j < nbk) ? Rb[(int64_t)(k0 + i) * n + k0 + j] : 0.0;
        P[i][j] = (i == j) ? 1.0 : 0.0;
      }
      __syncthreads();
      for (int j = 0; j < nbk; ++j) {
        if (tid == 0) {
          double d = S[j][j];
          bool ok = (d > 0.0) && isfinite(d);
          if (!ok && rel0 == 0.0 && isfinite(d)) {
            // unshifted factorization (a CholeskyQR pass after the first):
            // a non-positive pivot is a null direction of G, e.g. an exact
            // zero column of the tall matrix.  Floor this pivot alone (its
            // row's remaining entries are at the rounding level of G);
            // a shift of the whole diagonal would bias every other column
            d = relfail * stt.trace[b] / n;
            ok = d > 0.0;
          }
          sflag = ok ? 1 : 0;
          const double piv = ok ? sqrt(d) : 1.0;
          S[j][j] = piv;
          rpiv = 1.0 / piv;
        }
        __syncthreads();
        if (!sflag) break;
        const double rp = rpiv;
        for (int i = tid; i < nbk; i += blockDim.x) {
          if (i > j) S[j][i] *= rp;
          else P[j][i] *= rp;
        }
        __syncthreads();
        const int w = nbk - j - 1;
        const int ns = w * w, np = w * (j + 1);
        for (int e = tid; e < ns + np; e += blockDim.x) {
          if (e < ns) {
            const int a = j + 1 + e / w, c = j + 1 + e % w;
            if (a <= c) S[a][c] -= S[j][a] * S[j][c];
          } else {
            const int e2 = e - ns;
            const int a = j + 1 + e2 / (j + 1), q = e2 % (j + 1);
            P[a][q] -= S[j][a] * P[j][q];
          }
        }
        __syncthreads();
      }
      if (!sflag) {
        if (tid == 0) stt.status[b] = 2;
        __syncthreads();
        return;
      }
      // write back upper block, zero strict lower part
      for (int e = tid; e < nbk * nbk; e += blockDim.x) {
        int i = e / nbk, j = e % nbk;
        Rb[(int64_t)(k0 + i) * n + k0 + j] = (i <= j) ? S[i][j] : 0.0;
      }
      // R_kk^-1 = Z^T
      double* Db = Dinv + (int64_t)b * NB * NB;
      for (int e = tid; e < NB * NB; e += blockDim.x) {
        int i = e / NB, c = e % NB;
        Db[e] = (i <= c && c < nbk) ? P[c][i] : 0.0;
      }
      __syncthreads();
    };
    for (int b = blockIdx.x; b < batch; b += gridDim.x) diag_block(b, 0);
    grid.sync();
    for (int k = 0; k < T; ++k) {
      const int k0 = k * NB, nbk = min(NB, n - k0);
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
      const int per = w * (w + 1) / 2;
      const int ntask_t = per * batch;
      for (int t = blockIdx.x; t < ntask_t; t += gridDim.x) {
        // the problems' (k + 1, k + 1) blocks first (task b, so that the CTA
        // of problem b's next diagonal block updates it), then the others
        int b, r;
        if (t < batch) {
          b = t;
          r = 0;
        } else {
          const int u = t - batch;
          b = u / (per - 1);
          r = 1 + u % (per - 1);
        }
        const int r_task = r;
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
        if (r_task == 0) diag_block(b, k + 1);  // look-ahead: final after this update
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
                 int* info, Arena& ws, cudaStream_t st, double near_tol) {
  CholState s;
  s.trace = ws.take<double>(batch);
  s.shift = ws.take<double>(batch);
  s.status = ws.take<int>(batch);
  s.shifts_used = ws.take<int>(1);
  s.pending = ws.take<int>(CHOL_ROUNDS);
  s.colsq = (batch == 1 && rel0 == 0.0 && near_tol > 0.0)
                ? ws.take<double>((size_t)CHOL_NEAR_GROUPS * n)
                : nullptr;
  double* Dinv = ws.take<double>((size_t)batch * NB * NB);
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "chol: workspace too small");
  PLOM_REQUIRE(G && R && info, PLOM_ERR_ARG, "chol: null pointer");
  PLOM_CHECK_CUDA(cudaMemsetAsync(s.shifts_used, 0, sizeof(int), st));
  const int T = (n + NB - 1) / NB;
  int want = std::max(batch * std::max(1, T * (T + 1) / 2), 1);
  // one problem: one CTA per SM (the FP64 pipe of an SM is shared by its
  // CTAs, and fewer CTAs make each grid barrier cheaper: 9.8 -> 8.1 ms for the
  // three factorisations of the 1,024 x 1,024 headline Grams)
  if (batch == 1) want = std::min(want, num_sms());
  int blocks = coop_blocks((const void*)chol_coop_kernel, 256, 0, want);
  ProfScope prof("chol_fp64", st, (double)n * n * n / 3.0 * batch, 16.0 * n * n * batch);
  void* args[] = {(void*)&G,       (void*)&R,       (void*)&Dinv,     (void*)&n,
                  (void*)&batch,   (void*)&rel0,    (void*)&relfail,  (void*)&near_tol,
                  (void*)&s,       (void*)&info};
  PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void*)chol_coop_kernel, dim3(blocks),
                                              dim3(256), args, 0, st));
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// triangular inverse: W = R^{-1}, R upper (batch), by recursive halving:
//   [A B; 0 C]^{-1} = [A^{-1}, -A^{-1} (B C^{-1}); 0, C^{-1}]
// The 32 x 32 diagonal blocks are inverted first (one warp each, back
// substitution per column); each level s = 32, 64, ... then joins the pairs
// of s x s inverses along the diagonal with two batched products that skip
// the triangular zero bands (n^3/6 FMAs in all, spread over every SM).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) trtri_leaf_kernel(const double* __restrict__ R,
                                                        double* __restrict__ W, int n) {
  __shared__ double S[32][33];
  __shared__ double X[32][33];
  __shared__ double dinv[32];
  const int64_t nn = (int64_t)n * n;
  const double* Rb = R + (int64_t)blockIdx.y * nn;
  double* Wb = W + (int64_t)blockIdx.y * nn;
  const int j0 = blockIdx.x * 32, nb = min(32, n - j0);
  const int c = threadIdx.x;
  for (int i = 0; i < 32; ++i) {
    S[i][c] = (i < nb && c < nb) ? Rb[(int64_t)(j0 + i) * n + j0 + c] : (i == c ? 1.0 : 0.0);
    X[i][c] = 0.0;
  }
  __syncwarp();
  dinv[c] = 1.0 / S[c][c];
  __syncwarp();
  X[c][c] = dinv[c];
  for (int i = c - 1; i >= 0; --i) {
    double acc = 0.0;
    for (int t = i + 1; t <= c; ++t) acc = fma(S[i][t], X[t][c], acc);
    X[i][c] = -acc * dinv[i];
  }
  __syncwarp();
  if (c < nb)
    for (int i = 0; i < nb; ++i) Wb[(int64_t)(j0 + i) * n + j0 + c] = X[i][c];
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
  double* T = ws.take<double>((size_t)n * n * batch);  // B C^{-1} blocks
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "trtri: workspace too small");
  PLOM_REQUIRE(R && W, PLOM_ERR_ARG, "trtri: null pointer");
  PLOM_REQUIRE(batch <= 65535, PLOM_ERR_ARG, "trtri: batch too large");
  const int64_t nn = (int64_t)n * n;
  int launches = 1;
  for (int s = 32; s < n; s *= 2) launches += 2 * ((n / (2 * s) > 0) + (2 * (n / (2 * s)) * s + s < n));
  ProfScope prof("trtri_fp64", st, (double)n * n * n / 3.0 * batch, 16.0 * n * n * batch, launches);
  PLOM_CHECK_CUDA(cudaMemsetAsync(W, 0, sizeof(double) * nn * batch, st));
  trtri_leaf_kernel<<<dim3((unsigned)cdiv(n, 32), (unsigned)batch), 32, 0, st>>>(R, W, n);
  PLOM_CHECK_LAUNCH();
  for (int s = 32; s < n; s *= 2) {
    // sub-block t: rows [2ts, 2ts + s) hold A^{-1}, columns [2ts + s, 2ts + 2s) C^{-1}
    const int64_t step = 2 * (int64_t)s * (n + 1);
    const int nfull = n / (2 * s);
    const int tail_c0 = 2 * nfull * s + s;  // a last, narrower sub-block
    for (int part = 0; part < 2; ++part) {
      const int nsub = part == 0 ? nfull : (tail_c0 < n ? 1 : 0);
      if (nsub == 0) continue;
      const int64_t off = part == 0 ? 0 : (int64_t)nfull * step;
      const int cols = part == 0 ? s : n - tail_c0;
      const int64_t ab = off + s;                  // row r0, column c0 = r0 + s
      const int64_t cc = off + (int64_t)s * n + s; // C^{-1} at (c0, c0)
      // T = B C^{-1}
      PLOM_TRY(gemm_sq(R + ab, n, nn, step, W + cc, n, nn, step, T + ab, n, nn, step, s, cols,
                       cols, batch, nsub, 1.0, 2, st, nullptr));
      // W12 = -A^{-1} T
      PLOM_TRY(gemm_sq(W + off, n, nn, step, T + ab, n, nn, step, W + ab, n, nn, step, s, cols, s,
                       batch, nsub, -1.0, 1, st, nullptr));
    }
  }
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// one-sided Jacobi SVD (Hestenes), real or complex, cooperative
//
// The columns of A (rows of At) are rotated in pairs until every pair is
// orthogonal to the tolerance.  GB300 runs FP64 at a small fraction of its
// FP32 rate, so the kernels keep the FP64 instructions per row and pair low:
//  * squared column norms are carried from rotation to rotation
//    (a'^2 = a^2 - t|g|, b'^2 = b^2 + t|g|), recomputed exactly once per
//    sweep and after cancellation, so each pair needs one dot product;
//  * rotations are applied in scaled form (column = d * stored row):
//    x' = x - t (dq/dp) e^{-i phi} y,  y' = y + t (dp/dq) e^{i phi} x,
//    d' = c d: two FMAs per row; a scale is folded back into its row when it
//    falls below 2^-40 (|t| <= 1 bounds the growth of a stored row to
//    sqrt(2) per rotation);
//  * the angle t is computed in FP32: every t gives an exactly orthogonal
//    rotation as long as c = (1 + t^2)^-1/2 is exact for that t, and c comes
//    from an FP32 estimate refined by two Newton steps in FP64;
//  * the matrix is first scaled by a power of two so that max |a_ij| < 1.
// Block ordering (jacobi_block_kernel): the columns are grouped in blocks of
// 4; one CTA holds a pair of blocks (8 rows of At and of Vt) in shared
// memory for one round-robin step over the blocks, applies the 16 cross
// rotations in 4 rounds of 4 disjoint pairs (plus the 6 + 6 rotations inside
// the two blocks at the first step of a sweep) and writes the rows back: one
// grid barrier per block step instead of one per column step.  Problems
// whose 8 rows do not fit in shared memory use jacobi_pair_kernel (one warp
// per column pair, one grid barrier per column step).
// ---------------------------------------------------------------------------
constexpr double JAC_FOLD_BELOW = 9.094947017729282e-13;  // 2^-40

struct JacState {
  double* At;     // batch x n x pitch: rows = columns of A (times dsc)
  double* Vt;     // batch x n x pitch: rows = columns of V (times dsc)
  double* nrm2;   // batch x n: squared column norms; < 0 = recompute
  double* dsc;    // batch x n: column scales
  int* counts;    // [JACOBI_MAX_SWEEPS] rotations per sweep
  int* perm;      // batch x n
  unsigned long long* amax;  // [batch] bits of max |a_ij|
  int64_t pitch;  // doubles per row (n * cw rounded up to even)
  const double* V0;  // real, batch 1: starting rotation product (n x n row-major); null = I
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

// Rotation of a pair with squared norms al, be and |a_p^H a_q| = gabs.
// False when the pair is orthogonal to the tolerance (gabs^2 <= tol2 al be).
__device__ __forceinline__ bool jac_angle(double al, double be, double gabs, double tol2,
                                          double& t, double& c, double& sq) {
  if (!(al > 0.0 && be > 0.0) || !(gabs * gabs > tol2 * (al * be))) return false;
  const double diff = be - al;
  const float gf = (float)gabs;
  if (gf >= 1e-30f) {
    const float z = (float)diff / (2.0f * gf);
    const float az = fabsf(z);
    t = (double)(az > 1e18f ? 0.5f / z : copysignf(1.0f, z) / (az + sqrtf(fmaf(z, z, 1.0f))));
  } else {
    const double z = diff / (2.0 * gabs);
    const double az = fabs(z);
    t = az > 1e150 ? 0.5 / z : copysign(1.0, z) / (az + sqrt(fma(z, z, 1.0)));
  }
  const double x = fma(t, t, 1.0);
  double y = (double)rsqrtf((float)x);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double r = fma(-x * y, y, 1.0);
    y = fma(0.5 * y, r, y);
  }
  c = y;
  sq = x * y;
  return true;
}

// x^H y over rows [0, len) of the warp's pair (+ |x|^2, |y|^2 when SQ)
template <int CW, bool SQ>
__device__ __forceinline__ void jac_dots(const double* x, const double* y, int64_t len, int lane,
                                         double& gr, double& gi, double& sa, double& sb) {
  double g0 = 0, g1 = 0, h0 = 0, a0 = 0, a1 = 0, b0 = 0, b1 = 0;
  if (CW == 1) {
    int64_t i = lane;
    for (; i + 96 < len; i += 128) {
      const double x0 = x[i], x1 = x[i + 32], x2 = x[i + 64], x3 = x[i + 96];
      const double y0 = y[i], y1 = y[i + 32], y2 = y[i + 64], y3 = y[i + 96];
      g0 = fma(x0, y0, g0);
      g1 = fma(x1, y1, g1);
      g0 = fma(x2, y2, g0);
      g1 = fma(x3, y3, g1);
      if (SQ) {
        a0 = fma(x0, x0, a0);
        a1 = fma(x1, x1, a1);
        a0 = fma(x2, x2, a0);
        a1 = fma(x3, x3, a1);
        b0 = fma(y0, y0, b0);
        b1 = fma(y1, y1, b1);
        b0 = fma(y2, y2, b0);
        b1 = fma(y3, y3, b1);
      }
    }
    for (; i < len; i += 32) {
      const double x0 = x[i], y0 = y[i];
      g0 = fma(x0, y0, g0);
      if (SQ) {
        a0 = fma(x0, x0, a0);
        b0 = fma(y0, y0, b0);
      }
    }
  } else {
    for (int64_t i = lane; i < len; i += 32) {
      const double xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
      g0 = fma(xr, yr, g0);  // conj(x) * y
      g0 = fma(xi, yi, g0);
      h0 = fma(xr, yi, h0);
      h0 = fma(-xi, yr, h0);
      if (SQ) {
        a0 = fma(xr, xr, a0);
        a0 = fma(xi, xi, a0);
        b0 = fma(yr, yr, b0);
        b0 = fma(yi, yi, b0);
      }
    }
  }
  gr = warp_sum(g0 + g1);
  gi = (CW == 2) ? warp_sum(h0) : 0.0;
  if (SQ) {
    sa = warp_sum(a0 + a1);
    sb = warp_sum(b0 + b1);
  } else {
    sa = sb = 0.0;
  }
}

// x <- x - w y, y <- y + v x (old x) over rows [0, len); real: w, v real
template <int CW>
__device__ __forceinline__ void jac_rotate(double* x, double* y, int64_t len, int lane, double wr,
                                           double wi, double vr, double vi) {
  if (CW == 1) {
    int64_t i = lane;
    for (; i + 96 < len; i += 128) {
      double xv[4], yv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        xv[u] = x[i + 32 * u];
        yv[u] = y[i + 32 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        x[i + 32 * u] = fma(-wr, yv[u], xv[u]);
        y[i + 32 * u] = fma(vr, xv[u], yv[u]);
      }
    }
    for (; i < len; i += 32) {
      const double xv = x[i], yv = y[i];
      x[i] = fma(-wr, yv, xv);
      y[i] = fma(vr, xv, yv);
    }
  } else {
    for (int64_t i = lane; i < len; i += 32) {
      const double xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
      x[2 * i] = xr - (wr * yr - wi * yi);
      x[2 * i + 1] = xi - (wr * yi + wi * yr);
      y[2 * i] = yr + (vr * xr - vi * xi);
      y[2 * i + 1] = yi + (vr * xi + vi * xr);
    }
  }
}

// One pair (rows x, y of At; xv, yv of Vt) by one warp.  nrm/d/e point at
// the pair's norm and scale slots.  Returns 1 when the pair was rotated.
template <int CW>
__device__ __forceinline__ int jac_pair(double* x, double* y, double* xv, double* yv, int64_t n,
                                        double* na_, double* nb_, double* da_, double* db_,
                                        double* ea_, double* eb_, double tol2, int lane) {
  double al = *na_, be = *nb_;
  const double da = *da_, db = *db_, ea = *ea_, eb = *eb_;
  const bool need = (al < 0.0) || (be < 0.0);
  double gr, gi, sa, sb;
  if (need)
    jac_dots<CW, true>(x, y, n, lane, gr, gi, sa, sb);
  else
    jac_dots<CW, false>(x, y, n, lane, gr, gi, sa, sb);
  if (al < 0.0) al = da * da * sa;
  if (be < 0.0) be = db * db * sb;
  const double dd = da * db;
  gr *= dd;
  gi *= dd;
  const double gabs = (CW == 1) ? fabs(gr) : sqrt(fma(gr, gr, gi * gi));
  double t, c, sq;
  if (!jac_angle(al, be, gabs, tol2, t, c, sq)) {
    if (lane == 0 && need) {
      *na_ = al;
      *nb_ = be;
    }
    return 0;
  }
  const double tp = t * (db * ea), tq = t * (da * eb);  // t dq/dp, t dp/dq
  if (CW == 1) {
    const double e = copysign(1.0, gr);  // phase of gamma
    jac_rotate<1>(x, y, n, lane, tp * e, 0.0, tq * e, 0.0);
    jac_rotate<1>(xv, yv, n, lane, tp * e, 0.0, tq * e, 0.0);
  } else {
    const double ig = 1.0 / gabs;
    const double er = gr * ig, ei = gi * ig;
    jac_rotate<2>(x, y, n, lane, tp * er, -tp * ei, tq * er, tq * ei);
    jac_rotate<2>(xv, yv, n, lane, tp * er, -tp * ei, tq * er, tq * ei);
  }
  __syncwarp();
  if (lane == 0) {
    // carried norms; a large relative drop is recomputed next time
    const double na = fma(-t, gabs, al), nb = fma(t, gabs, be);
    *na_ = (na > 0.125 * al) ? na : -1.0;
    *nb_ = (nb > 0.125 * be) ? nb : -1.0;
    *da_ = da * c;
    *db_ = db * c;
    *ea_ = ea * sq;
    *eb_ = eb * sq;
  }
  return 1;
}

// ---------------------------------------------------------------------------
// Double-float storage (mixed form, real): each element of At and Vt is an
// unevaluated sum hi + lo of two FP32 numbers (~48 significant bits) held in
// the 8-byte slot of a double.  Dots and rotations run on the FP32 pipe with
// error-free transformations (Knuth's two-sum, FMA two-product); the scalar
// pair parameters stay in FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_split(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_val(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
  const float s = a + b;
  return make_float2(s, b - (s - a));
}
// a - t b
__device__ __forceinline__ float2 df_fms(float2 a, float2 t, float2 b) {
  const float ph = t.x * b.x;
  float pe = fmaf(t.x, b.x, -ph);
  pe = fmaf(t.x, b.y, pe);
  pe = fmaf(t.y, b.x, pe);
  const float2 sm = two_sum(a.x, -ph);
  return fast_two_sum(sm.x, sm.y + (a.y - pe));
}
// acc += x y (acc.y collects the low-order parts)
__device__ __forceinline__ void df_dot_acc(float2& acc, float2 x, float2 y) {
  const float ph = x.x * y.x;
  float pe = fmaf(x.x, y.x, -ph);
  pe = fmaf(x.x, y.y, pe);
  pe = fmaf(x.y, y.x, pe);
  const float2 sm = two_sum(acc.x, ph);
  acc.x = sm.x;
  acc.y += sm.y + pe;
}
__device__ __forceinline__ double df_warp_sum(float2 v) {
  v = fast_two_sum(v.x, v.y);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, v.x, o);
    const float l = __shfl_xor_sync(0xffffffffu, v.y, o);
    const float2 sm = two_sum(v.x, h);
    v = fast_two_sum(sm.x, sm.y + (v.y + l));
  }
  return df_val(v);
}

template <bool SQ>
__device__ __forceinline__ void jac_dots_df(const float2* x, const float2* y, int64_t len,
                                            int lane, double& gr, double& sa, double& sb) {
  float2 g0 = make_float2(0.f, 0.f), g1 = g0, a0 = g0, b0 = g0;
  int64_t i = lane;
  for (; i + 32 < len; i += 64) {
    const float2 x0 = x[i], x1 = x[i + 32], y0 = y[i], y1 = y[i + 32];
    df_dot_acc(g0, x0, y0);
    df_dot_acc(g1, x1, y1);
    if (SQ) {
      df_dot_acc(a0, x0, x0);
      df_dot_acc(a0, x1, x1);
      df_dot_acc(b0, y0, y0);
      df_dot_acc(b0, y1, y1);
    }
  }
  for (; i < len; i += 32) {
    const float2 x0 = x[i], y0 = y[i];
    df_dot_acc(g0, x0, y0);
    if (SQ) {
      df_dot_acc(a0, x0, x0);
      df_dot_acc(b0, y0, y0);
    }
  }
  const float2 sm = two_sum(g0.x, g1.x);
  gr = df_warp_sum(make_float2(sm.x, sm.y + g0.y + g1.y));
  if (SQ) {
    sa = df_warp_sum(a0);
    sb = df_warp_sum(b0);
  } else {
    sa = sb = 0.0;
  }
}

// x <- x - tp y, y <- y - tqn x (old x)
__device__ __forceinline__ void jac_rotate_df(float2* x, float2* y, int64_t len, int lane,
                                              float2 tp, float2 tqn) {
  int64_t i = lane;
  for (; i + 32 < len; i += 64) {
    const float2 x0 = x[i], x1 = x[i + 32], y0 = y[i], y1 = y[i + 32];
    x[i] = df_fms(x0, tp, y0);
    x[i + 32] = df_fms(x1, tp, y1);
    y[i] = df_fms(y0, tqn, x0);
    y[i + 32] = df_fms(y1, tqn, x1);
  }
  for (; i < len; i += 32) {
    const float2 x0 = x[i], y0 = y[i];
    x[i] = df_fms(x0, tp, y0);
    y[i] = df_fms(y0, tqn, x0);
  }
}

// x <- x - tp y, y <- y - tqn x over rows [h0, h1) of the warp
__device__ __forceinline__ void jac_rotate_df_range(float2* x, float2* y, int64_t h0, int64_t h1,
                                                    int lane, float2 tp, float2 tqn) {
  int64_t i = h0 + lane;
  for (; i + 32 < h1; i += 64) {
    const float2 x0 = x[i], x1 = x[i + 32], y0 = y[i], y1 = y[i + 32];
    x[i] = df_fms(x0, tp, y0);
    x[i + 32] = df_fms(x1, tp, y1);
    y[i] = df_fms(y0, tqn, x0);
    y[i + 32] = df_fms(y1, tqn, x1);
  }
  for (; i < h1; i += 32) {
    const float2 x0 = x[i], y0 = y[i];
    x[i] = df_fms(x0, tp, y0);
    y[i] = df_fms(y0, tqn, x0);
  }
}

// jac_pair on double-float rows (real)
__device__ __forceinline__ int jac_pair_df(float2* x, float2* y, float2* xv, float2* yv,
                                           int64_t n, double* na_, double* nb_, double* da_,
                                           double* db_, double* ea_, double* eb_, double tol2,
                                           int lane) {
  double al = *na_, be = *nb_;
  const double da = *da_, db = *db_, ea = *ea_, eb = *eb_;
  const bool need = (al < 0.0) || (be < 0.0);
  double gr, sa, sb;
  if (need)
    jac_dots_df<true>(x, y, n, lane, gr, sa, sb);
  else
    jac_dots_df<false>(x, y, n, lane, gr, sa, sb);
  if (al < 0.0) al = da * da * sa;
  if (be < 0.0) be = db * db * sb;
  gr *= da * db;
  const double gabs = fabs(gr);
  double t, c, sq;
  if (!jac_angle(al, be, gabs, tol2, t, c, sq)) {
    if (lane == 0 && need) {
      *na_ = al;
      *nb_ = be;
    }
    return 0;
  }
  const double e = copysign(1.0, gr);
  const float2 tp = df_split(t * (db * ea) * e), tqn = df_split(-t * (da * eb) * e);
  jac_rotate_df(x, y, n, lane, tp, tqn);
  jac_rotate_df(xv, yv, n, lane, tp, tqn);
  __syncwarp();
  if (lane == 0) {
    const double na = fma(-t, gabs, al), nb = fma(t, gabs, be);
    *na_ = (na > 0.125 * al) ? na : -1.0;
    *nb_ = (nb > 0.125 * be) ? nb : -1.0;
    *da_ = da * c;
    *db_ = db * c;
    *ea_ = ea * sq;
    *eb_ = eb * sq;
  }
  return 1;
}

// jac_pair on double-float rows (complex: element i is slots 2i (re) and
// 2i + 1 (im)).  Dots x^H y and the rotation x' = x - w y, y' = y + v x with
// w = t dq/dp e^{-i phi}, v = t dp/dq e^{i phi} on the FP32 pipe; the pair's
// scalars in FP64 as in jac_pair.
__device__ __forceinline__ int jac_pair_df_c(float2* x, float2* y, float2* xv, float2* yv,
                                             int64_t n, double* na_, double* nb_, double* da_,
                                             double* db_, double* ea_, double* eb_, double tol2,
                                             int lane) {
  double al = *na_, be = *nb_;
  const double da = *da_, db = *db_, ea = *ea_, eb = *eb_;
  const bool need = (al < 0.0) || (be < 0.0);
  float2 g = make_float2(0.f, 0.f), h = g, a2 = g, b2 = g;
  for (int64_t i = lane; i < n; i += 32) {
    const float2 xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
    df_dot_acc(g, xr, yr);  // conj(x) y
    df_dot_acc(g, xi, yi);
    df_dot_acc(h, xr, yi);
    df_dot_acc(h, make_float2(-xi.x, -xi.y), yr);
    if (need) {
      df_dot_acc(a2, xr, xr);
      df_dot_acc(a2, xi, xi);
      df_dot_acc(b2, yr, yr);
      df_dot_acc(b2, yi, yi);
    }
  }
  double gr = df_warp_sum(g), gi = df_warp_sum(h);
  if (need) {
    const double sa = df_warp_sum(a2), sb = df_warp_sum(b2);
    if (al < 0.0) al = da * da * sa;
    if (be < 0.0) be = db * db * sb;
  }
  const double dd = da * db;
  gr *= dd;
  gi *= dd;
  const double gabs = sqrt(fma(gr, gr, gi * gi));
  double t, c, sq;
  if (!jac_angle(al, be, gabs, tol2, t, c, sq)) {
    if (lane == 0 && need) {
      *na_ = al;
      *nb_ = be;
    }
    return 0;
  }
  const double tp = t * (db * ea), tq = t * (da * eb);
  const double ig = 1.0 / gabs;
  const double er = gr * ig, ei = gi * ig;
  // w = tp (er - i ei), v = tq (er + i ei)
  const float2 wr = df_split(tp * er), wi = df_split(-tp * ei), nwi = df_split(tp * ei);
  const float2 nvr = df_split(-tq * er), vi = df_split(tq * ei), nvi = df_split(-tq * ei);
  auto rot = [&](float2* p, float2* q) {
    for (int64_t i = lane; i < n; i += 32) {
      const float2 pr = p[2 * i], pi = p[2 * i + 1], qr = q[2 * i], qi = q[2 * i + 1];
      p[2 * i] = df_fms(df_fms(pr, wr, qr), nwi, qi);       // pr - wr qr + wi qi
      p[2 * i + 1] = df_fms(df_fms(pi, wr, qi), wi, qr);    // pi - wr qi - wi qr
      q[2 * i] = df_fms(df_fms(qr, nvr, pr), vi, pi);       // qr + vr pr - vi pi
      q[2 * i + 1] = df_fms(df_fms(qi, nvr, pi), nvi, pr);  // qi + vr pi + vi pr
    }
  };
  rot(x, y);
  rot(xv, yv);
  __syncwarp();
  if (lane == 0) {
    const double na = fma(-t, gabs, al), nb = fma(t, gabs, be);
    *na_ = (na > 0.125 * al) ? na : -1.0;
    *nb_ = (nb > 0.125 * be) ? nb : -1.0;
    *da_ = da * c;
    *db_ = db * c;
    *ea_ = ea * sq;
    *eb_ = eb * sq;
  }
  return 1;
}

template <int CW, bool DF>
__device__ __forceinline__ int jac_pair_any(double* x, double* y, double* xv, double* yv,
                                            int64_t n, double* na_, double* nb_, double* da_,
                                            double* db_, double* ea_, double* eb_, double tol2,
                                            int lane) {
  if constexpr (DF && CW == 2)
    return jac_pair_df_c(reinterpret_cast<float2*>(x), reinterpret_cast<float2*>(y),
                         reinterpret_cast<float2*>(xv), reinterpret_cast<float2*>(yv), n, na_,
                         nb_, da_, db_, ea_, eb_, tol2, lane);
  else if constexpr (DF)
    return jac_pair_df(reinterpret_cast<float2*>(x), reinterpret_cast<float2*>(y),
                       reinterpret_cast<float2*>(xv), reinterpret_cast<float2*>(yv), n, na_, nb_,
                       da_, db_, ea_, eb_, tol2, lane);
  else
    return jac_pair<CW>(x, y, xv, yv, n, na_, nb_, da_, db_, ea_, eb_, tol2, lane);
}

// element i of a stored row as FP64 (double or double-float storage)
template <bool DF>
__device__ __forceinline__ double jac_get(const double* row, int64_t i) {
  if (DF) return df_val(reinterpret_cast<const float2*>(row)[i]);
  return row[i];
}
template <bool DF>
__device__ __forceinline__ void jac_put(double* row, int64_t i, double v) {
  if (DF)
    reinterpret_cast<float2*>(row)[i] = df_split(v);
  else
    row[i] = v;
}

// Shared prologue: scale by a power of two (max |a_ij| < 1), At = A^T,
// Vt = I, unit scales, norms flagged for recomputation.
template <int CW, bool DF>
__device__ void jac_init(const double* __restrict__ A, int n, int batch, JacState& js,
                         cg::grid_group& grid) {
  const int64_t rl = (int64_t)n * CW;
  const int64_t P = js.pitch;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = gtid; e < batch; e += gthreads) js.amax[e] = 0ull;
  if (gtid < JACOBI_MAX_SWEEPS) js.counts[gtid] = 0;
  grid.sync();
  for (int64_t e = gtid; e < (int64_t)batch * n * rl; e += gthreads) {
    const double v = fabs(A[e]);
    if (v > 0.0) atomicMax(&js.amax[e / ((int64_t)n * rl)], (unsigned long long)__double_as_longlong(v));
  }
  grid.sync();
  for (int64_t e = gtid; e < (int64_t)batch * n * n; e += gthreads) {
    const int64_t b = e / ((int64_t)n * n), r = e % ((int64_t)n * n);
    const int i = (int)(r / n), j = (int)(r % n);
    int ex = 0;
    frexp(__longlong_as_double((long long)js.amax[b]), &ex);
    const double sc = ldexp(1.0, -ex);
    const double* src = A + b * n * rl + (int64_t)i * rl + (int64_t)j * CW;
    double* dst = js.At + b * n * P + (int64_t)j * P;
    jac_put<DF>(dst, (int64_t)i * CW, src[0] * sc);
    if (CW == 2) jac_put<DF>(dst, (int64_t)i * CW + 1, src[1] * sc);
    double* v = js.Vt + b * n * P + (int64_t)i * P;
    // row i of Vt = column i of the starting rotation product
    const double v0 = (CW == 1 && js.V0) ? js.V0[(int64_t)j * n + i] : ((i == j) ? 1.0 : 0.0);
    jac_put<DF>(v, (int64_t)j * CW, v0);
    if (CW == 2) jac_put<DF>(v, (int64_t)j * CW + 1, 0.0);
    if (j == 0) {
      for (int64_t p = rl; p < P; ++p) {  // row padding stays zero
        js.At[b * n * P + (int64_t)i * P + p] = 0.0;
        js.Vt[b * n * P + (int64_t)i * P + p] = 0.0;
      }
      js.nrm2[b * n + i] = -1.0;
      js.dsc[b * n + i] = 1.0;
    }
  }
  grid.sync();
}

// Shared epilogue: exact norms, descending order, outputs
//   S = sigma, U[i][k] = a_perm(k)[i] / sigma, VH[k][:] = conj(v_perm(k)).
template <int CW, bool DF>
__device__ void jac_finish(int n, int batch, JacState& js, int sweep, double* __restrict__ S,
                           double* __restrict__ U, double* __restrict__ VH, int* info,
                           cg::grid_group& grid) {
  const int64_t rl = (int64_t)n * CW;
  const int64_t P = js.pitch;
  const int lane = threadIdx.x & 31;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t gwarp = gtid >> 5, nwarps = gthreads >> 5;
  if (gtid == 0) {
    info[ST_SWEEPS] = sweep + 1;
    if (sweep >= JACOBI_MAX_SWEEPS) atomicMax(&info[ST_FAIL], PLOM_NUM_JACOBI);
  }
  for (int64_t task = gwarp; task < (int64_t)batch * n; task += nwarps) {
    const double* a = js.At + (task / n) * n * P + (task % n) * P;
    double s = 0.0;
    for (int64_t i = lane; i < rl; i += 32) {
      const double x = jac_get<DF>(a, i);
      s = fma(x, x, s);
    }
    s = warp_sum(s);
    if (lane == 0) js.nrm2[task] = js.dsc[task] * js.dsc[task] * s;
  }
  grid.sync();
  for (int64_t e = gtid; e < (int64_t)batch * n; e += gthreads) {
    const int64_t b = e / n;
    const int j = (int)(e % n);
    const double sj = js.nrm2[e];
    int rank = 0;
    for (int k = 0; k < n; ++k) {
      const double sk = js.nrm2[b * n + k];
      rank += (sk > sj) || (sk == sj && k < j);
    }
    js.perm[b * n + rank] = j;
  }
  grid.sync();
  for (int64_t e = gtid; e < (int64_t)batch * n * n; e += gthreads) {
    const int64_t b = e / ((int64_t)n * n);
    const int64_t r = e % ((int64_t)n * n);
    const int k = (int)(r / n), i = (int)(r % n);
    const int src = js.perm[b * n + k];
    const double s2 = js.nrm2[b * n + src];
    const double sk = sqrt(s2);
    int ex = 0;
    frexp(__longlong_as_double((long long)js.amax[b]), &ex);
    if (i == 0) S[b * n + k] = ldexp(sk, ex);
    const double d = js.dsc[b * n + src];
    const double f = sk > 0.0 ? d / sk : 0.0;
    const double* a = js.At + b * n * P + (int64_t)src * P;
    double* u = U + b * n * rl + (int64_t)i * rl + (int64_t)k * CW;
    u[0] = jac_get<DF>(a, (int64_t)i * CW) * f;
    if (CW == 2) u[1] = jac_get<DF>(a, (int64_t)i * CW + 1) * f;
    const double* v = js.Vt + b * n * P + (int64_t)src * P;
    double* vh = VH + b * n * rl + (int64_t)k * rl + (int64_t)i * CW;
    vh[0] = jac_get<DF>(v, (int64_t)i * CW) * d;
    if (CW == 2) vh[1] = -jac_get<DF>(v, (int64_t)i * CW + 1) * d;
  }
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
      : "memory");
}

// rounds of the 6 pairs inside a block of 4: (0,1)(2,3) / (0,2)(1,3) / (0,3)(1,2)
__device__ __forceinline__ void intra_pair(int round, int which, int& a, int& b) {
  if (round == 0) {
    a = which ? 2 : 0;
    b = which ? 3 : 1;
  } else if (round == 1) {
    a = which ? 1 : 0;
    b = which ? 3 : 2;
  } else {
    a = which ? 1 : 0;
    b = which ? 2 : 3;
  }
}

constexpr uint64_t JAC_WAIT_NS = 2000000000ull;

template <int CW, bool DF>
__global__ void __launch_bounds__(128) jacobi_block_kernel(const double* __restrict__ A, int n,
                                                           int batch, JacState js, double tol2,
                                                           double* __restrict__ S,
                                                           double* __restrict__ U,
                                                           double* __restrict__ VH, int* info) {
  extern __shared__ __align__(16) double jsm[];  // [8][pitch] At rows, [8][pitch] Vt rows
  __shared__ double snrm[8], sd[8], se[8];
  __shared__ int scol[8];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_sh;
  cg::grid_group grid = cg::this_grid();
  const int64_t P = js.pitch;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* cA = jsm;
  double* cV = jsm + 8 * P;
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
  }
  jac_init<CW, DF>(A, n, batch, js, grid);  // ends with a grid barrier

  const int nb = (n + 3) / 4;
  const int nbp = (nb + (nb & 1) < 2) ? 2 : nb + (nb & 1);  // even, >= 2
  const int bpairs = nbp / 2;
  const int64_t tasks = (int64_t)bpairs * batch;
  uint32_t phase = 0;
  int sweep = 0;
  for (; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    int myrot = 0;
    for (int step = 0; step < nbp - 1; ++step) {
      for (int64_t task = blockIdx.x; task < tasks; task += gridDim.x) {
        const int64_t b = task / bpairs;
        int bi, bj;
        rr_pair(step, (int)(task % bpairs), nbp, bi, bj);
        double* At = js.At + b * n * P;
        double* Vt = js.Vt + b * n * P;
        if (threadIdx.x < 8) {
          const int col = 4 * (threadIdx.x < 4 ? bi : bj) + (threadIdx.x & 3);
          const bool v = col < n;
          scol[threadIdx.x] = v ? col : -1;
          snrm[threadIdx.x] = v ? js.nrm2[b * n + col] : 0.0;
          const double d = v ? js.dsc[b * n + col] : 1.0;
          sd[threadIdx.x] = d;
          se[threadIdx.x] = 1.0 / d;  // exact inverse once per block step (no drift of d e)
        }
        __syncthreads();
        // rows in: bulk copies (pitch is even, so every row is 16-byte aligned)
        if (threadIdx.x == 0 && !abort_sh) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          uint32_t bytes = 0;
          for (int s8 = 0; s8 < 8; ++s8)
            if (scol[s8] >= 0) bytes += 2u * (uint32_t)(P * 8);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s),
                       "r"(bytes)
                       : "memory");
          for (int s8 = 0; s8 < 8; ++s8) {
            const int col = scol[s8];
            if (col < 0) continue;
            bulk_load((uint32_t)__cvta_generic_to_shared(cA + s8 * P), At + (int64_t)col * P,
                      (uint32_t)(P * 8), bar_s);
            bulk_load((uint32_t)__cvta_generic_to_shared(cV + s8 * P), Vt + (int64_t)col * P,
                      (uint32_t)(P * 8), bar_s);
          }
        }
        if (!abort_sh) {
          // bounded wait for the rows
          uint32_t ok = 0;
          uint64_t t0 = 0;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
          while (true) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(bar_s), "r"(phase)
                : "memory");
            if (ok) break;
            uint64_t t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            if (t1 - t0 > JAC_WAIT_NS) {
              abort_sh = 1;
              break;
            }
          }
          phase ^= 1u;
        }
        __syncthreads();
        if (abort_sh) {
          // rows never arrived: report and do no more work (every later task
          // of this block skips too; the barriers stay uniform)
          if (threadIdx.x == 0) atomicMax(&info[ST_FAIL], PLOM_NUM_TIMEOUT);
          __syncthreads();
          continue;
        }
        if (step == 0) {
          // exact squared norms once per sweep
          for (int s8 = warp; s8 < 8; s8 += 4) {
            double acc = 0.0;
            if (scol[s8] >= 0) {
              const double* x = cA + s8 * P;
              for (int64_t i = lane; i < (int64_t)n * CW; i += 32) {
                const double v = jac_get<DF>(x, i);
                acc = fma(v, v, acc);
              }
              acc = warp_sum(acc);
            }
            if (lane == 0) snrm[s8] = sd[s8] * sd[s8] * acc;
          }
          __syncthreads();
          for (int r = 0; r < 3; ++r) {
            int a, c;
            intra_pair(r, warp & 1, a, c);
            const int off = (warp >> 1) * 4;
            a += off;
            c += off;
            if (scol[a] >= 0 && scol[c] >= 0)
              myrot += jac_pair_any<CW, DF>(cA + a * P, cA + c * P, cV + a * P, cV + c * P, n,
                                            &snrm[a], &snrm[c], &sd[a], &sd[c], &se[a], &se[c],
                                            tol2, lane);
            __syncthreads();
          }
        }
        for (int u = 0; u < 4; ++u) {
          const int a = warp, c = 4 + ((warp + u) & 3);
          if (scol[a] >= 0 && scol[c] >= 0)
            myrot += jac_pair_any<CW, DF>(cA + a * P, cA + c * P, cV + a * P, cV + c * P, n,
                                          &snrm[a], &snrm[c], &sd[a], &sd[c], &se[a], &se[c],
                                          tol2, lane);
          __syncthreads();
        }
        // rows out; a scale below 2^-40 is folded into its rows
        for (int s8 = 0; s8 < 8; ++s8) {
          const int col = scol[s8];
          if (col < 0) continue;
          double* ga = At + (int64_t)col * P;
          double* gv = Vt + (int64_t)col * P;
          const double* sa = cA + s8 * P;
          const double* sv = cV + s8 * P;
          const double f = sd[s8];
          if (f < JAC_FOLD_BELOW) {
            for (int64_t i = threadIdx.x; i < P; i += 128) {
              jac_put<DF>(ga, i, jac_get<DF>(sa, i) * f);
              jac_put<DF>(gv, i, jac_get<DF>(sv, i) * f);
            }
          } else {
            for (int64_t i = threadIdx.x; i < P; i += 128) {
              ga[i] = sa[i];
              gv[i] = sv[i];
            }
          }
        }
        if (threadIdx.x < 8 && scol[threadIdx.x] >= 0) {
          const int col = scol[threadIdx.x];
          const bool fold = sd[threadIdx.x] < JAC_FOLD_BELOW;
          js.nrm2[b * n + col] = snrm[threadIdx.x];
          js.dsc[b * n + col] = fold ? 1.0 : sd[threadIdx.x];
        }
        __syncthreads();
      }
      grid.sync();
    }
    if (lane == 0 && myrot) atomicAdd(&js.counts[sweep], myrot);
    grid.sync();
    if (js.counts[sweep] == 0) break;
  }
  if (S == nullptr) return;
  jac_finish<CW, DF>(n, batch, js, sweep, S, U, VH, info, grid);
}

// ---------------------------------------------------------------------------
// Double-float block kernel with 16 warps per CTA (mixed form, real): the 4
// pairs of a round get 4 warps each (a quarter of the rows per warp), and the
// pair parameters are computed once per pair, by one lane, in double-float
// FP32 arithmetic (no FP64 instructions inside the sweep loop):
//   t from zeta in FP32 (any t is exact for the rotation it defines),
//   c = (1 + t^2)^-1/2 from an FP32 estimate and one Newton step in
//   double-float, scales d, 1/d, carried norms and t dq/dp in double-float.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ float2 df_add2(float2 a, float2 b) {
  const float2 s = two_sum(a.x, b.x);
  return fast_two_sum(s.x, s.y + (a.y + b.y));
}
__device__ __forceinline__ float2 df_mulf(float2 a, float t) {
  const float p = a.x * t;
  const float e = fmaf(a.x, t, -p);
  return fast_two_sum(p, fmaf(a.y, t, e));
}
// 1 / d in double-float
__device__ __forceinline__ float2 df_recip(float2 d) {
  const float h = 1.0f / d.x;
  const float r = fmaf(-d.x, h, 1.0f) - d.y * h;
  return fast_two_sum(h, r * h);
}

struct DfPair {
  float2 tp, tqn;  // x -= tp y ; y -= tqn x
  int rot;
};

// Pair parameters (one lane).  al/be: squared norms (x < 0: recompute from
// sa/sb), g: a_p^T a_q of the stored rows, d/e: scales and their inverses.
__device__ __forceinline__ DfPair df_params(float2& al, float2& be, float2 sa, float2 sb, float2 g,
                                            float2& dp, float2& dq, float2& ep, float2& eq,
                                            float tol) {
  DfPair out;
  out.rot = 0;
  out.tp = out.tqn = make_float2(0.f, 0.f);
  if (al.x < 0.f) al = df_mul(df_mul(dp, dp), sa);
  if (be.x < 0.f) be = df_mul(df_mul(dq, dq), sb);
  g = df_mul(df_mul(dp, dq), g);
  const float sg = (g.x < 0.f) ? -1.f : 1.f;
  const float2 ga = make_float2(fabsf(g.x), sg * g.y);
  if (!(al.x > 0.f && be.x > 0.f) || !(ga.x > tol * sqrtf(al.x) * sqrtf(be.x))) return out;
  // zeta = (be - al) / (2 |g|) with the difference in double-float
  const float2 s = two_sum(be.x, -al.x);
  const float diff = s.x + (s.y + (be.y - al.y));
  const float z = diff / (2.0f * ga.x);
  const float az = fabsf(z);
  const float t = az > 1e18f ? 0.5f / z : copysignf(1.0f, z) / (az + sqrtf(fmaf(z, z, 1.0f)));
  // x = 1 + t^2 (double-float), c = x^-1/2, sq = x^1/2
  const float p = t * t;
  float2 x = fast_two_sum(1.0f, p);
  x.y += fmaf(t, t, -p);
  const float y0 = rsqrtf(x.x);
  const float q = y0 * y0, qe = fmaf(y0, y0, -q);
  const float r = fmaf(-x.x, q, 1.0f) - fmaf(x.x, qe, x.y * q);
  const float2 c = fast_two_sum(y0, 0.5f * y0 * r);
  const float2 sq = df_mul(x, c);
  out.tp = df_mulf(df_mul(dq, ep), t * sg);
  out.tqn = df_mulf(df_mul(dp, eq), -t * sg);
  // carried norms: al - t|g|, be + t|g|; a large relative drop is recomputed
  const float2 tg = df_mulf(ga, t);
  const float2 na = df_add2(al, make_float2(-tg.x, -tg.y));
  const float2 nb = df_add2(be, tg);
  al = (na.x > 0.125f * al.x) ? na : make_float2(-1.f, 0.f);
  be = (nb.x > 0.125f * be.x) ? nb : make_float2(-1.f, 0.f);
  dp = df_mul(dp, c);
  dq = df_mul(dq, c);
  ep = df_mul(ep, sq);
  eq = df_mul(eq, sq);
  out.rot = 1;
  return out;
}

// dots of rows [h0, h1) of the warp; SQ adds |x|^2 and |y|^2
template <bool SQ>
__device__ __forceinline__ void df16_dots(const float2* x, const float2* y, int64_t h0, int64_t h1,
                                          int lane, float2& g, float2& a2, float2& b2) {
  float2 g0 = make_float2(0.f, 0.f), g1 = g0, aa = g0, bb = g0;
  int64_t i = h0 + lane;
  for (; i + 32 < h1; i += 64) {
    const float2 x0 = x[i], x1 = x[i + 32], y0 = y[i], y1 = y[i + 32];
    df_dot_acc(g0, x0, y0);
    df_dot_acc(g1, x1, y1);
    if (SQ) {
      df_dot_acc(aa, x0, x0);
      df_dot_acc(aa, x1, x1);
      df_dot_acc(bb, y0, y0);
      df_dot_acc(bb, y1, y1);
    }
  }
  for (; i < h1; i += 32) {
    const float2 x0 = x[i], y0 = y[i];
    df_dot_acc(g0, x0, y0);
    if (SQ) {
      df_dot_acc(aa, x0, x0);
      df_dot_acc(bb, y0, y0);
    }
  }
  g = df_add2(g0, g1);
  a2 = aa;
  b2 = bb;
}

__device__ __forceinline__ float2 df_warp_sum2(float2 v) {
  v = fast_two_sum(v.x, v.y);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, v.x, o);
    const float l = __shfl_xor_sync(0xffffffffu, v.y, o);
    const float2 sm = two_sum(v.x, h);
    v = fast_two_sum(sm.x, sm.y + (v.y + l));
  }
  return v;
}

__global__ void __launch_bounds__(512, 1)
    jacobi_block_df16_kernel(const double* __restrict__ A, int n, int batch, JacState js,
                             float tol, double* __restrict__ S, double* __restrict__ U,
                             double* __restrict__ VH, int* info) {
  extern __shared__ __align__(16) double jsm[];  // [8][pitch] At rows, [8][pitch] Vt rows
  __shared__ float2 snrm[8], sd[8], se[8];
  __shared__ float2 red[4][4][3];                 // [pair][quarter][g a2 b2]
  __shared__ DfPair prm[4];
  __shared__ int scol[8];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_sh;
  cg::grid_group grid = cg::this_grid();
  const int64_t P = js.pitch;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pk = warp >> 2, qtr = warp & 3;       // pair slot, row quarter
  const int64_t h0 = (int64_t)n * qtr / 4, h1 = (int64_t)n * (qtr + 1) / 4;
  float2* cA = reinterpret_cast<float2*>(jsm);
  float2* cV = reinterpret_cast<float2*>(jsm + 8 * P);
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
  }
  jac_init<1, true>(A, n, batch, js, grid);  // ends with a grid barrier

  const int nb = (n + 3) / 4;
  const int nbp = (nb + (nb & 1) < 2) ? 2 : nb + (nb & 1);  // even, >= 2
  const int bpairs = nbp / 2;
  const int64_t tasks = (int64_t)bpairs * batch;
  uint32_t phase = 0;
  int sweep = 0;
  for (; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    int myrot = 0;
    for (int step = 0; step < nbp - 1; ++step) {
      for (int64_t task = blockIdx.x; task < tasks; task += gridDim.x) {
        const int64_t b = task / bpairs;
        int bi, bj;
        rr_pair(step, (int)(task % bpairs), nbp, bi, bj);
        double* At = js.At + b * n * P;
        double* Vt = js.Vt + b * n * P;
        if (threadIdx.x < 8) {
          const int col = 4 * (threadIdx.x < 4 ? bi : bj) + (threadIdx.x & 3);
          const bool v = col < n;
          scol[threadIdx.x] = v ? col : -1;
          const double nr = v ? js.nrm2[b * n + col] : 0.0;
          snrm[threadIdx.x] = nr < 0.0 ? make_float2(-1.f, 0.f) : df_split(nr);
          const float2 d = df_split(v ? js.dsc[b * n + col] : 1.0);
          sd[threadIdx.x] = d;
          se[threadIdx.x] = df_recip(d);  // exact inverse once per block step
        }
        __syncthreads();
        if (threadIdx.x == 0 && !abort_sh) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          uint32_t bytes = 0;
          for (int s8 = 0; s8 < 8; ++s8)
            if (scol[s8] >= 0) bytes += 2u * (uint32_t)(P * 8);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s),
                       "r"(bytes)
                       : "memory");
          for (int s8 = 0; s8 < 8; ++s8) {
            const int col = scol[s8];
            if (col < 0) continue;
            bulk_load((uint32_t)__cvta_generic_to_shared(cA + s8 * P), At + (int64_t)col * P,
                      (uint32_t)(P * 8), bar_s);
            bulk_load((uint32_t)__cvta_generic_to_shared(cV + s8 * P), Vt + (int64_t)col * P,
                      (uint32_t)(P * 8), bar_s);
          }
        }
        if (!abort_sh) {
          uint32_t ok = 0;
          uint64_t t0 = 0;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
          while (true) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(bar_s), "r"(phase)
                : "memory");
            if (ok) break;
            uint64_t t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            if (t1 - t0 > JAC_WAIT_NS) {
              abort_sh = 1;
              break;
            }
          }
          phase ^= 1u;
        }
        __syncthreads();
        if (abort_sh) {
          if (threadIdx.x == 0) atomicMax(&info[ST_FAIL], PLOM_NUM_TIMEOUT);
          __syncthreads();
          continue;
        }
        if (step == 0) {
          // exact squared norms once per sweep: 2 warps per row
          const int s8 = warp >> 1, half = warp & 1;
          float2 acc = make_float2(0.f, 0.f);
          if (scol[s8] >= 0) {
            const float2* x = cA + s8 * P;
            for (int64_t i = (int64_t)n * half / 2 + lane; i < (int64_t)n * (half + 1) / 2; i += 32)
              df_dot_acc(acc, x[i], x[i]);
          }
          acc = df_warp_sum2(acc);
          if (lane == 0) red[s8 >> 1][(s8 & 1) * 2 + half][0] = acc;
          __syncthreads();
          if (threadIdx.x < 8) {
            const int r8 = threadIdx.x;
            const float2 sum = df_add2(red[r8 >> 1][(r8 & 1) * 2][0], red[r8 >> 1][(r8 & 1) * 2 + 1][0]);
            snrm[r8] = df_mul(df_mul(sd[r8], sd[r8]), sum);
          }
          __syncthreads();
        }
        const int nrounds = (step == 0) ? 7 : 4;
        for (int rd = 0; rd < nrounds; ++rd) {
          // pair of this warp's slot pk in round rd
          int a, c;
          if (step == 0 && rd < 3) {
            intra_pair(rd, pk & 1, a, c);
            const int off = (pk >> 1) * 4;
            a += off;
            c += off;
          } else {
            const int u = (step == 0) ? rd - 3 : rd;
            a = pk;
            c = 4 + ((pk + u) & 3);
          }
          const bool live = scol[a] >= 0 && scol[c] >= 0;
          const bool need = live && (snrm[a].x < 0.f || snrm[c].x < 0.f);
          if (live) {
            float2 g, a2, b2;
            if (need)
              df16_dots<true>(cA + a * P, cA + c * P, h0, h1, lane, g, a2, b2);
            else
              df16_dots<false>(cA + a * P, cA + c * P, h0, h1, lane, g, a2, b2);
            g = df_warp_sum2(g);
            if (need) {
              a2 = df_warp_sum2(a2);
              b2 = df_warp_sum2(b2);
            }
            if (lane == 0) {
              red[pk][qtr][0] = g;
              red[pk][qtr][1] = a2;
              red[pk][qtr][2] = b2;
            }
          }
          __syncthreads();
          if (qtr == pk && lane == 0) {
            // one lane per pair, on four different warps (SM sub-partitions)
            DfPair pr;
            pr.rot = 0;
            if (live) {
              float2 g = red[pk][0][0], a2 = red[pk][0][1], b2 = red[pk][0][2];
#pragma unroll
              for (int w = 1; w < 4; ++w) {
                g = df_add2(g, red[pk][w][0]);
                a2 = df_add2(a2, red[pk][w][1]);
                b2 = df_add2(b2, red[pk][w][2]);
              }
              pr = df_params(snrm[a], snrm[c], a2, b2, g, sd[a], sd[c], se[a], se[c], tol);
            }
            prm[pk] = pr;
            myrot += pr.rot;
          }
          __syncthreads();
          const DfPair pr = prm[pk];
          if (pr.rot) {
            jac_rotate_df_range(cA + a * P, cA + c * P, h0, h1, lane, pr.tp, pr.tqn);
            jac_rotate_df_range(cV + a * P, cV + c * P, h0, h1, lane, pr.tp, pr.tqn);
          }
          __syncthreads();
        }
        // rows out; a scale below 2^-40 is folded into its rows
        for (int s8 = 0; s8 < 8; ++s8) {
          const int col = scol[s8];
          if (col < 0) continue;
          double* ga = At + (int64_t)col * P;
          double* gv = Vt + (int64_t)col * P;
          const double* sa = jsm + s8 * P;
          const double* sv = jsm + (8 + s8) * P;
          // the fold test on the FP32 head of the scale: no FP64 instruction
          // per thread and row on the common path (GB300 runs FP64 at 1/64)
          if (sd[s8].x < (float)JAC_FOLD_BELOW) {
            const double f = df_val(sd[s8]);
            for (int64_t i = threadIdx.x; i < P; i += 512) {
              jac_put<true>(ga, i, jac_get<true>(sa, i) * f);
              jac_put<true>(gv, i, jac_get<true>(sv, i) * f);
            }
          } else {
            for (int64_t i = threadIdx.x; i < P; i += 512) {
              ga[i] = sa[i];
              gv[i] = sv[i];
            }
          }
        }
        if (threadIdx.x < 8 && scol[threadIdx.x] >= 0) {
          const int col = scol[threadIdx.x];
          const bool fold = sd[threadIdx.x].x < (float)JAC_FOLD_BELOW;
          js.nrm2[b * n + col] = snrm[threadIdx.x].x < 0.f ? -1.0 : df_val(snrm[threadIdx.x]);
          js.dsc[b * n + col] = fold ? 1.0 : df_val(sd[threadIdx.x]);
        }
        __syncthreads();
      }
      grid.sync();
    }
    if (lane == 0 && myrot) atomicAdd(&js.counts[sweep], myrot);
    grid.sync();
    if (js.counts[sweep] == 0) break;
  }
  if (S == nullptr) return;
  jac_finish<1, true>(n, batch, js, sweep, S, U, VH, info, grid);
}

// ---------------------------------------------------------------------------
// FP32 sweeps of large real Jacobi problems at the mixed form's tolerance.
// Block schedule with J32B-column blocks: one CTA per pair of blocks holds
// their 2 J32B rows of At and Vt in shared memory for one round-robin block
// step (the J32B^2 cross rotations in J32B rounds of J32B disjoint pairs,
// plus the rotations inside the two blocks at the first step of a sweep),
// one grid barrier per block step; 16 warps, 16 / J32B per pair, each over
// a share of the rows.  J32B = 4 (255 steps a sweep at n = 1,024, 128 CTAs):
// 8-column blocks halve the barriers but double each warp's rows per round
// and halve the CTAs, 4.0 against 3.2 ms a sweep measured on the headline R.
// Explicit (c, s) rotations: a dot costs one FMA per row, a rotation four
// FMAs.  The sweeps stop when every pair is orthogonal to `tol`, when the
// pairs above the floor have converged (see JAC_PRE32_TSTOP), or after
// max_sweeps.  Output: the rotation product J32 (n x n row-major FP32, J32 =
// the accumulated V); the host re-orthonormalises it to Jo and refines the
// SVD of B Jo (jacobi_pre32).
// ---------------------------------------------------------------------------
constexpr int JAC_PRE32_MIN_N = 256;       // real, batch 1, n from here on (see use_pre32)
constexpr int J32B = 4;                    // columns per block of the FP32 kernel
constexpr int J32W = 16 / J32B;            // warps per column pair (of 16)
constexpr float JAC_PRE32_TOL = 2e-6f;     // pair orthogonality of the FP32 phase
// The FP32 phase also ends after a sweep in which every rotated pair with a
// column above JAC_PRE32_FLOOR of the largest turned by less than
// JAC_PRE32_TSTOP: those pairs are then well inside the refinement's
// quadratic range, and the pairs of smaller columns (a noise floor, which
// the Jacobi ordering keeps rotating for several more sweeps) are only used
// at the FP32 phase's accuracy.  The floor matches the refinement's, and the
// refinement's first step takes angles of 3e-3 down to ~1e-5 (measured on two
// 8,388,608 x 1,024 POD fields: 8 and 9 sweeps with 3e-3, 10 with 1e-4, the
// same sigma, subspace angle and orthogonality after the refinement).
constexpr float JAC_PRE32_FLOOR = 1e-5f;
constexpr float JAC_PRE32_TSTOP = 3e-3f;
constexpr int JAC_PRE32_MAX_SWEEPS = 30;

struct Jac32State {
  float* At;      // n x pitch: rows = columns of B (scaled by a power of two)
  float* Vt;      // n x pitch: rows = columns of the rotation product
  float* nrm2;    // n squared column norms; < 0 = recompute
  int* counts;    // [JACOBI_MAX_SWEEPS] rotations per sweep
  unsigned* cmax; // [JACOBI_MAX_SWEEPS] bits of the largest squared column norm (sweep start)
  unsigned* tmax; // [JACOBI_MAX_SWEEPS] bits of the largest |t| of the pairs above the floor
  int* bflag;     // [blocks] block steps through which a block's rows are final
  int* abortf;    // set by a CTA whose wait ran out: every CTA stops waiting
  unsigned long long* amax;  // bits of max |b_ij|
  int64_t pitch;  // floats per row: n rounded up to 4 (16-byte bulk copies)
};

// (c, s) of the rotation of a pair with squared norms al, be and dot g;
// c = 0 when the pair is orthogonal to tol.  Carried norms al - t g, be + t g
// (a drop below 1/8 is flagged for recomputation from the rows).
__device__ __forceinline__ float2 f32_params(float& al, float& be, float g, float tol) {
  if (!(al > 0.f && be > 0.f) || !(fabsf(g) > tol * sqrtf(al) * sqrtf(be)))
    return make_float2(0.f, 0.f);
  const float z = (be - al) / (2.0f * g);
  const float az = fabsf(z);
  const float t = az > 1e18f ? 0.5f / z : copysignf(1.0f, z) / (az + sqrtf(fmaf(z, z, 1.0f)));
  const float c = 1.0f / sqrtf(fmaf(t, t, 1.0f));
  const float tg = t * g;
  const float na = al - tg, nb = be + tg;
  al = (na > 0.125f * al) ? na : -1.f;
  be = (nb > 0.125f * be) ? nb : -1.f;
  return make_float2(c, c * t);
}

// dots over rows [h0, h1) of the warp (+ squared norms when sq); two rows per
// lane and access when both bounds are even (8-byte shared loads, 32-bit
// indices: the loop is issue-bound)
__device__ __forceinline__ void f32_dots(const float* x, const float* y, int h0, int h1,
                                         int lane, bool sq, float& g, float& a2, float& b2) {
  float g0 = 0.f, g1 = 0.f, aa = 0.f, bb = 0.f;
  if (((h0 | h1) & 1) == 0) {
    const float2* x2 = reinterpret_cast<const float2*>(x);
    const float2* y2 = reinterpret_cast<const float2*>(y);
    for (int i = (h0 >> 1) + lane; i < (h1 >> 1); i += 32) {
      const float2 xv = x2[i], yv = y2[i];
      g0 = fmaf(xv.x, yv.x, g0);
      g1 = fmaf(xv.y, yv.y, g1);
      if (sq) {
        aa = fmaf(xv.x, xv.x, fmaf(xv.y, xv.y, aa));
        bb = fmaf(yv.x, yv.x, fmaf(yv.y, yv.y, bb));
      }
    }
  } else {
    for (int i = h0 + lane; i < h1; i += 32) {
      const float x0 = x[i], y0 = y[i];
      g0 = fmaf(x0, y0, g0);
      if (sq) {
        aa = fmaf(x0, x0, aa);
        bb = fmaf(y0, y0, bb);
      }
    }
  }
  g = warp_sum(g0 + g1);
  a2 = sq ? warp_sum(aa) : 0.f;
  b2 = sq ? warp_sum(bb) : 0.f;
}

// x' = c x - s y, y' = s x + c y over rows [h0, h1)
__device__ __forceinline__ void f32_rotate(float* x, float* y, int h0, int h1, int lane, float c,
                                           float s) {
  if (((h0 | h1) & 1) == 0) {
    float2* x2 = reinterpret_cast<float2*>(x);
    float2* y2 = reinterpret_cast<float2*>(y);
    for (int i = (h0 >> 1) + lane; i < (h1 >> 1); i += 32) {
      const float2 a = x2[i], b = y2[i];
      x2[i] = make_float2(fmaf(c, a.x, -s * b.x), fmaf(c, a.y, -s * b.y));
      y2[i] = make_float2(fmaf(s, a.x, c * b.x), fmaf(s, a.y, c * b.y));
    }
  } else {
    for (int i = h0 + lane; i < h1; i += 32) {
      const float a = x[i], b = y[i];
      x[i] = fmaf(c, a, -s * b);
      y[i] = fmaf(s, a, c * b);
    }
  }
}

__global__ void __launch_bounds__(512, 1)
    jacobi_block_f32_kernel(const double* __restrict__ B, int n, Jac32State js, float tol,
                            int max_sweeps, float* __restrict__ J, int* info) {
  extern __shared__ __align__(16) float jsm32[];  // [2 J32B][pitch] At rows, then Vt rows
  __shared__ float snrm[2 * J32B];
  __shared__ float red[J32B][J32W][3];  // [pair][row part][g a2 b2]
  __shared__ int scol[2 * J32B];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_sh;
  cg::grid_group grid = cg::this_grid();
  const int64_t P = js.pitch;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pk = warp / J32W, qtr = warp % J32W;  // pair slot, row part
  const int h0 = n * qtr / J32W, h1 = n * (qtr + 1) / J32W;
  float* cA = jsm32;
  float* cV = jsm32 + 2 * J32B * P;
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_sh = 0;
  }
  // prologue: power-of-two scale (max |b_ij| < 1), At = B^T in FP32, Vt = I
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
  if (gtid == 0) js.amax[0] = 0ull;
  if (gtid < JACOBI_MAX_SWEEPS) {
    js.counts[gtid] = 0;
    js.cmax[gtid] = 0u;
    js.tmax[gtid] = 0u;
  }
  grid.sync();
  {
    unsigned long long mx = 0ull;  // non-negative doubles order as their bits
    for (int64_t e = gtid; e < (int64_t)n * n; e += gthreads) {
      const unsigned long long v = (unsigned long long)__double_as_longlong(fabs(B[e]));
      mx = v > mx ? v : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long w = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = w > mx ? w : mx;
    }
    if (lane == 0 && mx) atomicMax(js.amax, mx);
  }
  grid.sync();
  {
    int ex = 0;
    frexp(__longlong_as_double((long long)js.amax[0]), &ex);
    const double sc = ldexp(1.0, -ex);
    for (int64_t e = gtid; e < (int64_t)n * P; e += gthreads) {
      const int64_t i = e / P, j = e % P;  // row i of At / Vt, entry j
      js.At[e] = (j < n) ? (float)(B[j * n + i] * sc) : 0.f;
      js.Vt[e] = (j == i) ? 1.f : 0.f;
    }
    for (int64_t e = gtid; e < n; e += gthreads) js.nrm2[e] = -1.f;
  }
  const int nb = (n + J32B - 1) / J32B;
  const int nbp = (nb + (nb & 1) < 2) ? 2 : nb + (nb & 1);  // even, >= 2
  const int bpairs = nbp / 2;
  for (int64_t e = gtid; e < nbp; e += gthreads) js.bflag[e] = 0;
  if (gtid == 0) *js.abortf = 0;
  grid.sync();
  int gstep = 0;  // block steps since the first sweep
  uint32_t phase = 0;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    int myrot = 0;
    float mytmax = 0.f;  // |t| of this thread's rotated pairs above the floor
    // floor from the previous sweep's largest squared column norm (none in
    // the first sweep)
    const float floor2 = sweep > 0 ? JAC_PRE32_FLOOR * JAC_PRE32_FLOOR *
                                         __uint_as_float(js.cmax[sweep - 1])
                                   : 3.0e38f;
    for (int step = 0; step < nbp - 1; ++step) {
      for (int task = blockIdx.x; task < bpairs; task += gridDim.x) {
        int bi, bj;
        rr_pair(step, task, nbp, bi, bj);
        // the two blocks' rows and norms are final once the CTAs that held
        // them in the previous block step have released their flags (a
        // release/acquire pair per block instead of a grid-wide barrier per
        // step); threads 0 .. 2 J32B - 1 each acquire them, as they read
        // the norms below, and thread 0 then issues the row loads
        if (threadIdx.x < 2 * J32B && !abort_sh) {
          uint64_t t0 = 0;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
          for (int q = 0; q < 2; ++q) {
            const int* fl = js.bflag + (q ? bj : bi);
            while (true) {
              int v;
              asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(fl) : "memory");
              if (v >= gstep) break;
              if (*(volatile int*)js.abortf) {
                abort_sh = 1;
                break;
              }
              uint64_t t1;
              asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
              if (t1 - t0 > JAC_WAIT_NS) {
                abort_sh = 1;
                atomicExch(js.abortf, 1);
                break;
              }
            }
          }
        }
        __syncthreads();
        // the row loads go out first (their columns follow from the schedule
        // alone); the carried norms are read while they are in flight
        if (threadIdx.x == 0 && !abort_sh) {
          asm volatile("fence.proxy.async.global;" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          uint32_t bytes = 0;
          for (int s8 = 0; s8 < 2 * J32B; ++s8)
            if (J32B * (s8 < J32B ? bi : bj) + (s8 % J32B) < n) bytes += 2u * (uint32_t)(P * 4);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s),
                       "r"(bytes)
                       : "memory");
          for (int s8 = 0; s8 < 2 * J32B; ++s8) {
            const int col = J32B * (s8 < J32B ? bi : bj) + (s8 % J32B);
            if (col >= n) continue;
            bulk_load((uint32_t)__cvta_generic_to_shared(cA + s8 * P), js.At + (int64_t)col * P,
                      (uint32_t)(P * 4), bar_s);
            bulk_load((uint32_t)__cvta_generic_to_shared(cV + s8 * P), js.Vt + (int64_t)col * P,
                      (uint32_t)(P * 4), bar_s);
          }
        }
        if (threadIdx.x < 2 * J32B) {
          const int col = J32B * (threadIdx.x < J32B ? bi : bj) + (threadIdx.x % J32B);
          const bool v = col < n;
          scol[threadIdx.x] = v ? col : -1;
          snrm[threadIdx.x] = v ? js.nrm2[col] : 0.f;
        }
        if (!abort_sh) {
          uint32_t ok = 0;
          uint64_t t0 = 0;
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
          while (true) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(bar_s), "r"(phase)
                : "memory");
            if (ok) break;
            uint64_t t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            if (t1 - t0 > JAC_WAIT_NS) {
              abort_sh = 1;
              atomicExch(js.abortf, 1);
              break;
            }
          }
          phase ^= 1u;
        }
        __syncthreads();
        if (abort_sh) {
          if (threadIdx.x == 0) atomicMax(&info[ST_FAIL], PLOM_NUM_TIMEOUT);
          __syncthreads();
          continue;
        }
        if (step == 0) {
          // exact squared norms once per sweep: one warp per row (warps
          // 0 .. 2 J32B - 1)
          if (warp < 2 * J32B) {
            const int s16 = warp;
            float acc = 0.f;
            if (scol[s16] >= 0) {
              const float* x = cA + s16 * P;
              for (int i = lane; i < n; i += 32) acc = fmaf(x[i], x[i], acc);
            }
            acc = warp_sum(acc);
            if (lane == 0) {
              snrm[s16] = acc;
              if (scol[s16] >= 0) atomicMax(&js.cmax[sweep], __float_as_uint(acc));
            }
          }
          __syncthreads();
        }
        // rounds: at a sweep's first step the 28 pairs inside each block (7
        // rounds of the circle method, 4 + 4 pairs), then the 64 cross pairs
        // (8 rounds of 8: column pk of the first block with column
        // (pk + u) mod 8 of the second)
        const int nintra = (step == 0) ? J32B - 1 : 0;
        const int nrounds = nintra + J32B;
        for (int rd = 0; rd < nrounds; ++rd) {
          int a, c;
          if (rd < nintra) {
            rr_pair(rd, pk % (J32B / 2), J32B, a, c);
            const int off = (pk / (J32B / 2)) * J32B;
            a += off;
            c += off;
          } else {
            const int u = rd - nintra;
            a = pk;
            c = J32B + ((pk + u) % J32B);
          }
          const bool live = scol[a] >= 0 && scol[c] >= 0;
          float al = snrm[a], be = snrm[c];  // read before the owner updates them
          const bool need = live && (al < 0.f || be < 0.f);
          if (live) {
            float g, a2, b2;
            f32_dots(cA + a * P, cA + c * P, h0, h1, lane, need, g, a2, b2);
            if (lane == 0) {
              red[pk][qtr][0] = g;
              red[pk][qtr][1] = a2;
              red[pk][qtr][2] = b2;
            }
          }
          __syncthreads();
          // every lane of the pair's warps derives the same (c, s) from the
          // same sums in the same order; the first warp stores the norms
          float2 cs = make_float2(0.f, 0.f);
          if (live) {
            float g = 0.f, sa = 0.f, sb = 0.f;
#pragma unroll
            for (int w = 0; w < J32W; ++w) {
              g += red[pk][w][0];
              sa += red[pk][w][1];
              sb += red[pk][w][2];
            }
            if (al < 0.f) al = sa;
            if (be < 0.f) be = sb;
            const float big = fmaxf(al, be);
            cs = f32_params(al, be, g, tol);
            if (qtr == 0 && lane == 0) {
              snrm[a] = al;
              snrm[c] = be;
              myrot += cs.x > 0.f ? 1 : 0;
              if (cs.x > 0.f && big > floor2) mytmax = fmaxf(mytmax, fabsf(cs.y / cs.x));
            }
          }
          if (cs.x > 0.f) {
            f32_rotate(cA + a * P, cA + c * P, h0, h1, lane, cs.x, cs.y);
            f32_rotate(cV + a * P, cV + c * P, h0, h1, lane, cs.x, cs.y);
          }
          __syncthreads();
        }
        // rows out (16-byte vectors: the pitch is a multiple of 4 floats)
        for (int s8 = 0; s8 < 2 * J32B; ++s8) {
          const int col = scol[s8];
          if (col < 0) continue;
          float4* ga = reinterpret_cast<float4*>(js.At + (int64_t)col * P);
          float4* gv = reinterpret_cast<float4*>(js.Vt + (int64_t)col * P);
          const float4* sa = reinterpret_cast<const float4*>(cA + s8 * P);
          const float4* sv = reinterpret_cast<const float4*>(cV + s8 * P);
          for (int64_t i = threadIdx.x; i < P / 4; i += 512) {
            ga[i] = sa[i];
            gv[i] = sv[i];
          }
        }
        if (threadIdx.x < 2 * J32B && scol[threadIdx.x] >= 0)
          js.nrm2[scol[threadIdx.x]] = snrm[threadIdx.x];
        __syncthreads();
        if (threadIdx.x == 0) {
          __threadfence();
          asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(js.bflag + bi), "r"(gstep + 1)
                       : "memory");
          asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(js.bflag + bj), "r"(gstep + 1)
                       : "memory");
        }
      }
      ++gstep;
    }
    if (lane == 0 && myrot) atomicAdd(&js.counts[sweep], myrot);
    if (lane == 0 && mytmax > 0.f) atomicMax(&js.tmax[sweep], __float_as_uint(mytmax));
    grid.sync();
    if (*(volatile int*)js.abortf) break;
    if (js.counts[sweep] == 0) break;
    if (sweep > 0 && __uint_as_float(js.tmax[sweep]) <= JAC_PRE32_TSTOP) break;
  }
  if (gtid == 0) info[ST_SWEEPS32] = sweep < max_sweeps ? sweep + 1 : sweep;
  // J32 (row-major): column k = row k of Vt
  for (int64_t e = gtid; e < (int64_t)n * n; e += gthreads) {
    const int64_t k = e / n, i = e % n;
    J[i * n + k] = js.Vt[k * P + i];
  }
}

// one warp per column pair, 4 pairs per 128-thread block, rows in global memory
template <int CW>
__global__ void __launch_bounds__(128) jacobi_pair_kernel(const double* __restrict__ A, int n,
                                                          int batch, JacState js, double tol2,
                                                          double* __restrict__ S,
                                                          double* __restrict__ U,
                                                          double* __restrict__ VH, int* info) {
  cg::grid_group grid = cg::this_grid();
  const int64_t P = js.pitch;
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  jac_init<CW, false>(A, n, batch, js, grid);
  const int np = n + (n & 1);
  const int pairs = np / 2;
  const int64_t total = (int64_t)pairs * batch;
  int sweep = 0;
  for (; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    int myrot = 0;
    // exact squared norms once per sweep
    for (int64_t task = gwarp; task < (int64_t)batch * n; task += nwarps) {
      const double* a = js.At + (task / n) * n * P + (task % n) * P;
      double s = 0.0;
      for (int64_t i = lane; i < (int64_t)n * CW; i += 32) s = fma(a[i], a[i], s);
      s = warp_sum(s);
      if (lane == 0) js.nrm2[task] = js.dsc[task] * js.dsc[task] * s;
    }
    grid.sync();
    for (int step = 0; step < np - 1; ++step) {
      for (int64_t task = gwarp; task < total; task += nwarps) {
        const int64_t b = task / pairs;
        int p, q;
        rr_pair(step, (int)(task % pairs), np, p, q);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        if (q >= n) continue;
        double* At = js.At + b * n * P;
        double* Vt = js.Vt + b * n * P;
        const int64_t ip = b * n + p, iq = b * n + q;
        double ep = 1.0 / js.dsc[ip], eq = 1.0 / js.dsc[iq];
        if (jac_pair<CW>(At + (int64_t)p * P, At + (int64_t)q * P, Vt + (int64_t)p * P,
                         Vt + (int64_t)q * P, n, &js.nrm2[ip], &js.nrm2[iq], &js.dsc[ip],
                         &js.dsc[iq], &ep, &eq, tol2, lane)) {
          ++myrot;
          __syncwarp();
          const double dp = js.dsc[ip], dq = js.dsc[iq];
          __syncwarp();
          // fold a small scale into its rows
          for (int side = 0; side < 2; ++side) {
            const double f = side ? dq : dp;
            if (f >= JAC_FOLD_BELOW) continue;
            const int col = side ? q : p;
            double* ga = At + (int64_t)col * P;
            double* gv = Vt + (int64_t)col * P;
            for (int64_t i = lane; i < P; i += 32) {
              ga[i] *= f;
              gv[i] *= f;
            }
            __syncwarp();
            if (lane == 0) js.dsc[b * n + col] = 1.0;
          }
        }
      }
      grid.sync();
    }
    if (lane == 0 && myrot) atomicAdd(&js.counts[sweep], myrot);
    grid.sync();
    if (js.counts[sweep] == 0) break;
  }
  if (S == nullptr) return;
  jac_finish<CW, false>(n, batch, js, sweep, S, U, VH, info, grid);
}

// real matrices from this size on are solved through their transpose
constexpr int JACOBI_TRANSPOSED_MIN_N = 64;
constexpr size_t JAC_BLOCK_SMEM_MAX = 200 * 1024;

static int64_t jac_pitch(int n, int cplx) {
  const int64_t rl = (int64_t)n * (cplx ? 2 : 1);
  return rl + (rl & 1);
}

template <int CW>
static int jacobi_launch_cw(const double* A, int n, int batch, JacState& js, double tol2,
                            bool df, double* S, double* U, double* VH, int* info,
                            cudaStream_t st) {
  void* args[] = {(void*)&A,    (void*)&n, (void*)&batch, (void*)&js, (void*)&tol2,
                  (void*)&S,    (void*)&U, (void*)&VH,    (void*)&info};
  const size_t smem = (size_t)16 * js.pitch * sizeof(double);
  const bool use_df = df && CW == 1 && smem <= JAC_BLOCK_SMEM_MAX;
  const bool block_df = df && CW == 2;  // complex: the generic block kernel on double-float rows
  ProfScope prof(use_df || (block_df && smem <= JAC_BLOCK_SMEM_MAX) ? "jacobi_svd_df"
                                                                    : "jacobi_svd_fp64",
                 st, 0.0, 8.0 * 3.0 * n * n * batch * CW);
  if (use_df) {
    const void* k = (const void*)jacobi_block_df16_kernel;
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int nb = (n + 3) / 4;
    const int nbp = std::max(2, nb + (nb & 1));
    const int want = (int)std::max<int64_t>(1, (int64_t)nbp / 2 * batch);
    const int blocks = coop_blocks(k, 512, smem, want);
    float tolf = (float)sqrt(tol2);
    void* args16[] = {(void*)&A,    (void*)&n, (void*)&batch, (void*)&js, (void*)&tolf,
                      (void*)&S,    (void*)&U, (void*)&VH,    (void*)&info};
    PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(512), args16, smem, st));
    return PLOM_OK;
  }
  if (smem <= JAC_BLOCK_SMEM_MAX) {
    const void* k = block_df ? (const void*)jacobi_block_kernel<CW, true>
                             : (const void*)jacobi_block_kernel<CW, false>;
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int nb = (n + 3) / 4;
    const int nbp = std::max(2, nb + (nb & 1));
    const int want = (int)std::max<int64_t>(1, (int64_t)nbp / 2 * batch);
    const int blocks = coop_blocks(k, 128, smem, want);
    PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(128), args, smem, st));
  } else {
    const void* k = (const void*)jacobi_pair_kernel<CW>;
    const int want = (int)std::max<int64_t>(1, cdiv((int64_t)(n + (n & 1)) / 2 * batch, 4));
    const int blocks = coop_blocks(k, 128, 0, want);
    PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(128), args, 0, st));
  }
  return PLOM_OK;
}

// Tolerances at or above this level (the mixed form's) run on double-float rows
constexpr double JAC_DF_TOL = 1e-10;

static int jacobi_launch(const double* A, int n, int batch, int cplx, JacState& js, double tol,
                         double* S, double* U, double* VH, int* info, cudaStream_t st) {
  const double tol2 = tol * tol;
  const bool df = tol >= JAC_DF_TOL;
  return cplx ? jacobi_launch_cw<2>(A, n, batch, js, tol2, df, S, U, VH, info, st)
              : jacobi_launch_cw<1>(A, n, batch, js, tol2, df, S, U, VH, info, st);
}

static void carve_jac(Arena& ws, JacState& js, int n, int batch, int cplx) {
  js.pitch = jac_pitch(n, cplx);
  const size_t mat = (size_t)n * js.pitch;
  js.At = ws.take<double>(mat * batch);
  js.Vt = ws.take<double>(mat * batch);
  js.nrm2 = ws.take<double>((size_t)batch * n);
  js.dsc = ws.take<double>((size_t)batch * n);
  js.counts = ws.take<int>(JACOBI_MAX_SWEEPS);
  js.perm = ws.take<int>((size_t)batch * n);
  js.amax = ws.take<unsigned long long>((size_t)batch);
  js.V0 = nullptr;
}

// ---- FP32 pre-sweeps, host side -------------------------------------------
// After the FP32 sweeps, J32 (FP32) is orthonormal to ~1e-5.  One
// Newton-Schulz step of its polar factor, Jo = J32 (3 I - J32^T J32) / 2 =
// J32 + J32 (I - G) / 2, brings that to ~1e-10 (G from exact FP32 products
// with double-float sums; the correction term is ~1e-5 and needs FP32 only).
// B' = B Jo is formed at double-float accuracy as one sum over 3n rows,
// [Bh; Bh; Bl]^T [Joh; Jol; Joh] (hi/lo FP32 splits, B scaled by the power
// of two of the FP32 phase), and the double-float kernel starts from
// V = Jo, so its accumulated rotations are the V of B itself.
__global__ void pre32_residual_kernel(const double* __restrict__ G, float* __restrict__ E, int n) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    E[e] = (float)(((e / n == e % n) ? 1.0 : 0.0) - G[e]);
}

__global__ void pre32_operands_kernel(const float* __restrict__ J32, const float* __restrict__ C,
                                      const double* __restrict__ A,
                                      const unsigned long long* __restrict__ amax,
                                      double* __restrict__ Jo, float* __restrict__ Jcat,
                                      float* __restrict__ Rcat, int n) {
  const int64_t nn = (int64_t)n * n;
  int ex = 0;
  frexp(__longlong_as_double((long long)*amax), &ex);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double jo = (double)J32[e] + 0.5 * (double)C[e];
    Jo[e] = jo;
    if (Jcat) {
      const float jh = (float)jo;
      const float jl = (float)(jo - (double)jh);
      Jcat[e] = jh;
      Jcat[nn + e] = jl;
      Jcat[2 * nn + e] = jh;
    }
    const double a = ldexp(A[e], -ex);
    const float ah = (float)a;
    const float al = (float)(a - (double)ah);
    Rcat[e] = ah;
    Rcat[nn + e] = ah;
    Rcat[2 * nn + e] = al;
  }
}

__global__ void pre32_unscale_kernel(double* __restrict__ S, int n,
                                     const unsigned long long* __restrict__ amax) {
  int ex = 0;
  frexp(__longlong_as_double((long long)*amax), &ex);
  for (int i = threadIdx.x; i < n; i += blockDim.x) S[i] = ldexp(S[i], ex);
}

// ---- refinement of the FP32 phase ----------------------------------------
// The FP32 sweeps leave the rotation product Jo accurate to ~1e-5 with
// respect to B itself.  B' = B Jo is formed once (double-float sums of exact
// FP32 products, operands split x = xh + xl:  X^T Y ~ [Xh; Xh; Xl]^T
// [Yh; Yl; Yh]), and its right singular vectors V' = I + D are found close
// to the identity: with W = B' (I + D) and C = W^T W, the simultaneous
// one-sided Jacobi angles of all pairs
//     Om_ij = C_ij / (C_jj - C_ii)  (skew),   I + D <- (I + D)(I + Om),
// followed by Newton-Schulz steps that keep I + D orthogonal
// (E = I - (I + D)^T (I + D) = -(D + D^T) - D^T D,  D <- D + (I + D) E / 2).
// Only D, Om and E are products of small matrices, so W = B' + B' D keeps
// every column of B' to its own relative accuracy (the small singular
// values included) and the iteration converges to the SVD of the fixed B'
// (the same matrix a double-float Jacobi finish would decompose), the error
// of a separated pair squaring at each step (two steps from the FP32 phase's
// end, where every pair above the floor turned by less than 1e-4).  Pairs whose angle would
// exceed 0.1 (singular values closer than the remaining error) and pairs of
// columns both below JAC_REFINE_FLOOR of the largest are not rotated, and a
// step whose angles have a Frobenius norm above 0.25 is shortened to it.
// Finally V = Jo (I + D), sigma_k = ||W e_k||, and the columns of
// Ut = W diag(sigma)^-1 are orthonormalised in descending sigma order
// (graded: the leading, accurate columns keep their directions).
// (T. Ogita and K. Aishima refine SVDs by matrix products in the same
// spirit, J. Comput. Appl. Math. 369 (2020); this is a one-sided form.)
constexpr int JAC_REFINE_STEPS = 2;
constexpr int JAC_REFINE_NS = 2;           // Newton-Schulz steps after the first refinement step
                                           // (one after the later, smaller ones)
constexpr double JAC_REFINE_MAX_ANGLE = 0.1;
constexpr double JAC_REFINE_NULL = 1e-8;   // sigma_k / sigma_1 below this: a null column
constexpr double JAC_REFINE_FLOOR = 1e-5;  // pairs of columns both below this fraction: kept
constexpr int JAC_REFINE_GS = 3;           // graded orthonormalisation steps of Ut

// a3 = [Xh; Xh; Xl], b3 = [Xh; Xl; Xh] (3n x n FP32 each; either may be null)
__global__ void rf_split3_kernel(const double* __restrict__ X, int64_t nn, float* __restrict__ a3,
                                 float* __restrict__ b3) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double x = X[e];
    const float h = (float)x;
    const float l = (float)(x - (double)h);
    if (a3) {
      a3[e] = h;
      a3[nn + e] = h;
      a3[2 * nn + e] = l;
    }
    if (b3) {
      b3[e] = h;
      b3[nn + e] = l;
      b3[2 * nn + e] = h;
    }
  }
}

// t = the transposed split of X (so that t^T Y = X Y): nparts = 2 gives
// [Xh^T; Xl^T] (against [Y; Y]), nparts = 3 gives [Xh^T; Xh^T; Xl^T]
// (against [Yh; Yl; Yh])
__global__ void rf_tsplit_kernel(const double* __restrict__ X, int n, int nparts,
                                 float* __restrict__ t) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e % n;
    const double x = X[j * n + i];
    const float h = (float)x;
    const float l = (float)(x - (double)h);
    t[e] = h;
    if (nparts == 2) {
      t[nn + e] = l;
    } else {
      t[nn + e] = h;
      t[2 * nn + e] = l;
    }
  }
}

// cmax[0] = max_i C_ii (one block)
__global__ void rf_cmax_kernel(const double* __restrict__ C, int n, double* __restrict__ cmax) {
  __shared__ double red[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = fmax(v, C[(int64_t)i * n + i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
    cmax[0] = t;
  }
}

// om (FP32): Om_ij = C_ij / (C_jj - C_ii) with C symmetrised; 0 on the
// diagonal, where |Om_ij| would exceed JAC_REFINE_MAX_ANGLE and for pairs of
// columns both below JAC_REFINE_FLOOR of the largest
__global__ void __launch_bounds__(256) rf_omega_kernel(const double* __restrict__ C, int n,
                                                       const double* __restrict__ cmax,
                                                       float* __restrict__ om,
                                                       double* __restrict__ part) {
  const int64_t nn = (int64_t)n * n;
  const double floor2 = JAC_REFINE_FLOOR * JAC_REFINE_FLOOR * cmax[0];
  double sq = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e % n;
    double o = 0.0;
    const double ci = C[i * n + i], cj = C[j * n + j];
    if (i != j && fmax(ci, cj) > floor2) {
      const double c = 0.5 * (C[e] + C[j * n + i]);
      const double d = cj - ci;
      if (fabs(d) * JAC_REFINE_MAX_ANGLE > fabs(c)) o = c / d;
    }
    const float of = (float)o;
    om[e] = of;
    sq = fma((double)of, (double)of, sq);
  }
  // this block's share of ||om||_F^2, warps in a fixed order
  __shared__ double red[8];
  sq = warp_sum(sq);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// om *= min(1, JAC_REFINE_MAX_NORM / ||om||_F): a step that would leave
// I + D far from orthogonal (many unresolved pairs at the angle bound at
// once) is shortened so that the Newton-Schulz steps stay convergent.  The
// sum of squares: per-block partials (rf_omega_kernel), then one block sums
// them, both in a fixed order.
constexpr double JAC_REFINE_MAX_NORM = 0.25;
__global__ void rf_omnorm_kernel(const double* __restrict__ part, int nparts,
                                 double* __restrict__ g) {
  __shared__ double red[32];
  double v = 0.0;
  for (int e = threadIdx.x; e < nparts; e += blockDim.x) v += part[e];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    const double f = sqrt(t);
    g[0] = (f > JAC_REFINE_MAX_NORM) ? JAC_REFINE_MAX_NORM / f : 1.0;
  }
}

__global__ void rf_omscale_kernel(float* __restrict__ om, int64_t nn, const double* __restrict__ g) {
  const float f = (float)g[0];
  if (f == 1.f) return;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    om[e] *= f;
}

// D += om + P  ((I + D)(I + Om) - I with P = D Om)
__global__ void rf_rotate_kernel(double* __restrict__ D, const float* __restrict__ om,
                                 const double* __restrict__ P, int64_t nn) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    D[e] += (double)om[e] + P[e];
}

// E = -(D + D^T) - G  (G = D^T D): FP64 and FP32 copies
__global__ void rf_ns_residual_kernel(const double* __restrict__ D, const double* __restrict__ G,
                                      int n, double* __restrict__ E, float* __restrict__ E32) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e % n;
    const double v = -(D[e] + D[j * n + i]) - G[e];
    E[e] = v;
    E32[e] = (float)v;
  }
}

// D += (E + P) / 2  (P = D E)
__global__ void rf_ns_update_kernel(double* __restrict__ D, const double* __restrict__ E,
                                    const double* __restrict__ P, int64_t nn) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    D[e] += 0.5 * (E[e] + P[e]);
}

// out = X + P
__global__ void rf_add_kernel(double* __restrict__ out, const double* __restrict__ X,
                              const double* __restrict__ P, int64_t nn) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = X[e] + P[e];
}

// f = strict upper triangle of G (the first-order Gram-Schmidt coefficients)
__global__ void rf_upper_kernel(const double* __restrict__ G, int n, float* __restrict__ f) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    f[e] = (e % n > e / n) ? (float)G[e] : 0.f;
}

// X -= P, then (separately) columns to unit norm
__global__ void rf_sub_kernel(double* __restrict__ X, const double* __restrict__ P, int64_t nn) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x)
    X[e] -= P[e];
}

// s[c] = ||X e_c||: 32 columns per block, 8 row groups per column (each
// thread sums every 8th row of its group in order), the 8 partials combined
// in a fixed order
__global__ void __launch_bounds__(256) rf_colnorm_kernel(const double* __restrict__ W, int n,
                                                         double* __restrict__ s) {
  __shared__ double red[8][33];
  const int cl = threadIdx.x & 31, rg = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + cl;
  double acc = 0.0;
  if (c < n)
    for (int r = rg; r < n; r += 8) {
      const double w = W[(int64_t)r * n + c];
      acc = fma(w, w, acc);
    }
  red[rg][cl] = acc;
  __syncthreads();
  if (rg == 0 && c < n) {
    double t = 0.0;
    for (int g = 0; g < 8; ++g) t += red[g][cl];
    s[c] = sqrt(t);
  }
}

// columns of X to unit norm; a column whose norm fell below 1e-3 (it
// depended on the earlier ones) becomes zero and is completed later
__global__ void rf_colscale_kernel(double* __restrict__ X, int n, const double* __restrict__ s,
                                   int* __restrict__ zero) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = s[e % n];
    X[e] = (v > 1e-3) ? X[e] / v : 0.0;
    if (e < n && !(v > 1e-3)) zero[e] = 1;
  }
}

// rank of column c in descending sigma (ties: lower index first)
__global__ void rf_order_kernel(const double* __restrict__ s, int n, int* __restrict__ perm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double v = s[c];
  int rank = 0;
  for (int k = 0; k < n; ++k) rank += (s[k] > v) || (s[k] == v && k < c);
  perm[rank] = c;
}

// sorted outputs: S[k] = s[p], Ut e_k = W e_p / s[p] (zero for a null
// column, flagged for completion), VHt row k = V e_p (p = perm[k])
__global__ void rf_output_kernel(const double* __restrict__ W, const double* __restrict__ V,
                                 const double* __restrict__ s, const int* __restrict__ perm, int n,
                                 double* __restrict__ S, double* __restrict__ Ut,
                                 double* __restrict__ VHt, int* __restrict__ zero) {
  const int64_t nn = (int64_t)n * n;
  const double s1 = s[perm[0]];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, k = e % n;
    const int p = perm[k];
    const double sp = s[p];
    const bool live = sp > JAC_REFINE_NULL * s1;
    Ut[e] = live ? W[i * n + p] / sp : 0.0;
    VHt[k * n + i] = V[i * n + p];
    if (i == 0) {
      S[k] = sp;
      zero[k] = live ? 0 : 1;
    }
  }
}

// Orthonormal completion of the zero columns of Ut (null singular values, or
// columns that the orthonormalisation found dependent): column k becomes
// e_r - Ut (Ut^T e_r), twice, normalised, for the first row r (from k on,
// cyclically) whose projection keeps at least half its norm.  One CTA; only
// exactly rank-deficient problems have such columns.
__global__ void __launch_bounds__(256) rf_complete_kernel(double* __restrict__ Ut, int n,
                                                          const int* __restrict__ zero) {
  extern __shared__ double cw[];  // [n] coefficients, [n] the new column
  double* coef = cw;
  double* col = cw + n;
  __shared__ double red[8];
  __shared__ double tot;
  for (int k = 0; k < n; ++k) {
    if (!zero[k]) continue;
    for (int tries = 0; tries < n; ++tries) {
      const int r = (k + tries) % n;
      for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = (i == r) ? 1.0 : 0.0;
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        // coef_l = col . Ut e_l (the columns not yet completed are zero)
        for (int l = threadIdx.x; l < n; l += blockDim.x) {
          double a = 0.0;
          for (int i = 0; i < n; ++i) a = fma(Ut[(int64_t)i * n + l], col[i], a);
          coef[l] = a;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
          double a = col[i];
          for (int l = 0; l < n; ++l) a = fma(-Ut[(int64_t)i * n + l], coef[l], a);
          col[i] = a;
        }
        __syncthreads();
      }
      double q = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) q = fma(col[i], col[i], q);
      q = warp_sum(q);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = q;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        tot = t;
      }
      __syncthreads();
      if (tot >= 0.25) {
        const double f = 1.0 / sqrt(tot);
        for (int i = threadIdx.x; i < n; i += blockDim.x) Ut[(int64_t)i * n + k] = col[i] * f;
        __syncthreads();
        break;
      }
      __syncthreads();
    }
  }
}

__global__ void rf_info_kernel(int* info, int slot, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) info[slot] = v;
}

struct RefineBufs {
  double *Bp, *Dl, *W, *C, *P, *G, *E, *s, *cmax, *part;
  float *a3, *b3, *bt3, *t2, *om, *E32;
  int* perm;
  int* zero;  // [n] 1 = column of Ut to be completed
};

static void carve_refine(Arena& ws, RefineBufs& b, int n) {
  const size_t nn = (size_t)n * n;
  b.Bp = ws.take<double>(nn);
  b.Dl = ws.take<double>(nn);
  b.W = ws.take<double>(nn);
  b.C = ws.take<double>(nn);
  b.P = ws.take<double>(nn);
  b.G = ws.take<double>(nn);
  b.E = ws.take<double>(nn);
  b.s = ws.take<double>(n);
  b.cmax = ws.take<double>(2);  // max C_ii, the step's scale
  b.part = ws.take<double>((size_t)num_sms() * 16);  // per-block sums of squares of the angles
  b.a3 = ws.take<float>(3 * nn);
  b.b3 = ws.take<float>(3 * nn);
  b.bt3 = ws.take<float>(3 * nn);
  b.t2 = ws.take<float>(2 * nn);
  b.om = ws.take<float>(nn);
  b.E32 = ws.take<float>(nn);
  b.perm = ws.take<int>(n);
  b.zero = ws.take<int>(n);
}

// gemm_tn_df (C = A^T B, K x n operands) whose row-chunk partials go back to
// the arena after the call
static int rf_prod(const float* A, const float* B, double* C, int n, int64_t K, Arena& ws,
                   cudaStream_t st) {
  const size_t mark = ws.off;
  const int r = gemm_tn_df(A, n, B, n, C, n, n, n, K, ws, st);
  ws.off = mark;
  return r;
}

static int rf_grid(int64_t nn) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(nn, 256), (int64_t)num_sms() * 16));
}

// Graded orthonormalisation of X's columns in their order: the first-order
// Gram-Schmidt step X <- X - X triu(X^T X, 1) (column k loses its components
// along the columns before it; the leading columns are not rotated), then
// every column to unit norm.  Quadratic in the departure from
// orthonormality, like Newton-Schulz, but the accurate leading columns keep
// their directions (the symmetric polar step would spread the small columns'
// errors onto them).
static int rf_graded(double* X, int n, RefineBufs& b, Arena& ws, cudaStream_t st) {
  const int64_t nn = (int64_t)n * n;
  const int eg = rf_grid(nn);
  rf_split3_kernel<<<eg, 256, 0, st>>>(X, nn, b.a3, b.b3);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY(rf_prod(b.a3, b.b3, b.G, n, 3 * (int64_t)n, ws, st));  // X^T X
  rf_upper_kernel<<<eg, 256, 0, st>>>(b.G, n, b.E32);
  PLOM_CHECK_LAUNCH();
  rf_tsplit_kernel<<<eg, 256, 0, st>>>(X, n, 2, b.t2);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY(rf_prod(b.t2, b.E32, b.P, n, n, ws, st));  // X F (the coefficients are small)
  rf_sub_kernel<<<eg, 256, 0, st>>>(X, b.P, nn);
  PLOM_CHECK_LAUNCH();
  rf_colnorm_kernel<<<(unsigned)cdiv(n, 32), 256, 0, st>>>(X, n, b.s);
  PLOM_CHECK_LAUNCH();
  rf_colscale_kernel<<<eg, 256, 0, st>>>(X, n, b.s, b.zero);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// C = A B (n x n FP64): [Ah^T; Ah^T; Al^T]^T [Bh; Bl; Bh] by gemm_tn_df
int gemm_nn_df(const double* A, const double* B, double* C, int n, Arena& ws, cudaStream_t st) {
  const int64_t nn = (int64_t)n * n;
  float* at = ws.take<float>((size_t)(3 * nn));
  float* b3 = ws.take<float>((size_t)(3 * nn));
  if (ws.measuring()) return gemm_tn_df(nullptr, n, nullptr, n, nullptr, n, n, n, 3 * (int64_t)n, ws, st);
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gemm_nn_df: workspace too small");
  PLOM_REQUIRE(A && B && C && n >= 1, PLOM_ERR_ARG, "gemm_nn_df: bad arguments");
  const int eg = rf_grid(nn);
  rf_tsplit_kernel<<<eg, 256, 0, st>>>(A, n, 3, at);
  PLOM_CHECK_LAUNCH();
  rf_split3_kernel<<<eg, 256, 0, st>>>(B, nn, nullptr, b3);
  PLOM_CHECK_LAUNCH();
  return gemm_tn_df(at, n, b3, n, C, n, n, n, 3 * (int64_t)n, ws, st);
}

// SVD of the scaled B (Rcat = [Ah; Ah; Al], A = B^T) from the orthonormal
// starting product Jo: S (scaled), Ut (columns = left vectors), VHt (rows =
// right vectors)
static int jacobi_refine(const float* Rcat, const double* Jo, int n, double* S, double* Ut,
                         double* VHt, int* info, Arena& ws, cudaStream_t st) {
  RefineBufs b;
  carve_refine(ws, b, n);
  const int64_t nn = (int64_t)n * n;
  if (ws.measuring())  // the largest row-chunk partials of the products (K = 3n)
    return gemm_tn_df(nullptr, n, nullptr, n, nullptr, n, n, n, 3 * (int64_t)n, ws, st);
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi refine: workspace too small");
  const int eg = rf_grid(nn);
  const int64_t K3 = 3 * (int64_t)n;
  ProfScope prof("jacobi_refine", st, 2.0 * (7.0 + 8.0 * JAC_REFINE_STEPS) * (double)nn * n, 0.0);
  // B' = B Jo, fixed; its transposed split for the W updates
  rf_split3_kernel<<<eg, 256, 0, st>>>(Jo, nn, nullptr, b.b3);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY(rf_prod(Rcat, b.b3, b.Bp, n, K3, ws, st));
  rf_tsplit_kernel<<<eg, 256, 0, st>>>(b.Bp, n, 3, b.bt3);
  PLOM_CHECK_LAUNCH();
  PLOM_CHECK_CUDA(cudaMemsetAsync(b.Dl, 0, sizeof(double) * nn, st));
  PLOM_CHECK_CUDA(cudaMemcpyAsync(b.W, b.Bp, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
  for (int it = 0; it < JAC_REFINE_STEPS; ++it) {
    // C = W^T W and the angles
    rf_split3_kernel<<<eg, 256, 0, st>>>(b.W, nn, b.a3, b.b3);
    PLOM_CHECK_LAUNCH();
    PLOM_TRY(rf_prod(b.a3, b.b3, b.C, n, K3, ws, st));
    rf_cmax_kernel<<<1, 256, 0, st>>>(b.C, n, b.cmax);
    PLOM_CHECK_LAUNCH();
    rf_omega_kernel<<<eg, 256, 0, st>>>(b.C, n, b.cmax, b.om, b.part);
    PLOM_CHECK_LAUNCH();
    rf_omnorm_kernel<<<1, 1024, 0, st>>>(b.part, eg, b.cmax + 1);
    PLOM_CHECK_LAUNCH();
    rf_omscale_kernel<<<eg, 256, 0, st>>>(b.om, nn, b.cmax + 1);
    PLOM_CHECK_LAUNCH();
    // D <- D + Om + D Om
    rf_tsplit_kernel<<<eg, 256, 0, st>>>(b.Dl, n, 2, b.t2);
    PLOM_CHECK_LAUNCH();
    PLOM_TRY(rf_prod(b.t2, b.om, b.P, n, n, ws, st));
    rf_rotate_kernel<<<eg, 256, 0, st>>>(b.Dl, b.om, b.P, nn);
    PLOM_CHECK_LAUNCH();
    for (int k = 0; k < (it == 0 ? JAC_REFINE_NS : 1); ++k) {
      // E = -(D + D^T) - D^T D;  D <- D + (E + D E) / 2
      rf_split3_kernel<<<eg, 256, 0, st>>>(b.Dl, nn, b.a3, nullptr);
      PLOM_CHECK_LAUNCH();
      PLOM_TRY(rf_prod(b.a3, b.a3, b.G, n, n, ws, st));
      rf_ns_residual_kernel<<<eg, 256, 0, st>>>(b.Dl, b.G, n, b.E, b.E32);
      PLOM_CHECK_LAUNCH();
      rf_tsplit_kernel<<<eg, 256, 0, st>>>(b.Dl, n, 2, b.t2);
      PLOM_CHECK_LAUNCH();
      PLOM_TRY(rf_prod(b.t2, b.E32, b.P, n, n, ws, st));
      rf_ns_update_kernel<<<eg, 256, 0, st>>>(b.Dl, b.E, b.P, nn);
      PLOM_CHECK_LAUNCH();
    }
    // W = B' + B' D
    rf_split3_kernel<<<eg, 256, 0, st>>>(b.Dl, nn, nullptr, b.b3);
    PLOM_CHECK_LAUNCH();
    PLOM_TRY(rf_prod(b.bt3, b.b3, b.P, n, K3, ws, st));
    rf_add_kernel<<<eg, 256, 0, st>>>(b.W, b.Bp, b.P, nn);
    PLOM_CHECK_LAUNCH();
  }
  // V = Jo + Jo D (into C)
  rf_tsplit_kernel<<<eg, 256, 0, st>>>(Jo, n, 3, b.bt3);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY(rf_prod(b.bt3, b.b3, b.P, n, K3, ws, st));  // b3 still holds D's split
  rf_add_kernel<<<eg, 256, 0, st>>>(b.C, Jo, b.P, nn);
  PLOM_CHECK_LAUNCH();
  rf_colnorm_kernel<<<(unsigned)cdiv(n, 32), 256, 0, st>>>(b.W, n, b.s);
  PLOM_CHECK_LAUNCH();
  rf_order_kernel<<<(unsigned)cdiv(n, 128), 128, 0, st>>>(b.s, n, b.perm);
  PLOM_CHECK_LAUNCH();
  rf_output_kernel<<<eg, 256, 0, st>>>(b.W, b.C, b.s, b.perm, n, S, Ut, VHt, b.zero);
  PLOM_CHECK_LAUNCH();
  for (int k = 0; k < JAC_REFINE_GS; ++k) PLOM_TRY(rf_graded(Ut, n, b, ws, st));
  rf_complete_kernel<<<1, 256, sizeof(double) * 2 * n, st>>>(Ut, n, b.zero);
  PLOM_CHECK_LAUNCH();
  rf_info_kernel<<<1, 1, 0, st>>>(info, ST_REFINE, JAC_REFINE_STEPS);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// Real problems from n = 256 on at the mixed form's tolerance, up to the size
// whose FP32 block kernel rows fit in shared memory (the double-float kernel's
// bound, kept for the larger sizes' workspace estimates).
static bool use_pre32(int n, double tol) {
  return n >= JAC_PRE32_MIN_N && tol >= JAC_DF_TOL &&
         (size_t)16 * jac_pitch(n, 0) * sizeof(double) <= JAC_BLOCK_SMEM_MAX;
}

// SVD of B = A^T (At holds B, A is B^T) through the FP32 pre-sweeps and the
// refinement of their rotation product: B = Ut diag(S) VHt.
static int jacobi_pre32(const double* A, const double* At, int n, double tol, double* S,
                        double* Ut, double* VHt, int* info, Arena& ws, cudaStream_t st) {
  (void)tol;
  const size_t nn = (size_t)n * n;
  Jac32State j32;
  j32.pitch = ((int64_t)n + 3) / 4 * 4;
  j32.At = ws.take<float>((size_t)n * j32.pitch);
  j32.Vt = ws.take<float>((size_t)n * j32.pitch);
  j32.nrm2 = ws.take<float>(n);
  j32.counts = ws.take<int>(JACOBI_MAX_SWEEPS);
  j32.cmax = ws.take<unsigned>(JACOBI_MAX_SWEEPS);
  j32.tmax = ws.take<unsigned>(JACOBI_MAX_SWEEPS);
  j32.bflag = ws.take<int>((size_t)n / J32B + 2);
  j32.abortf = ws.take<int>(1);
  j32.amax = ws.take<unsigned long long>(1);
  float* J32 = ws.take<float>(nn);
  float* E = ws.take<float>(nn);
  float* C = ws.take<float>(nn);
  double* G = ws.take<double>(nn);
  double* Jo = ws.take<double>(nn);
  float* Rcat = ws.take<float>(3 * nn);
  const size_t mark = ws.off;
  if (ws.measuring()) {  // the partials of G's product, then the refinement's needs
    PLOM_TRY(gemm_tn_df(nullptr, n, nullptr, n, nullptr, n, n, n, n, ws, st));
    size_t need = ws.off;
    ws.off = mark;
    PLOM_TRY(jacobi_refine(nullptr, nullptr, n, nullptr, nullptr, nullptr, nullptr, ws, st));
    ws.off = std::max(need, ws.off);
    return PLOM_OK;
  }
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi: workspace too small");
  {
    const void* k = (const void*)jacobi_block_f32_kernel;
    const size_t smem = (size_t)4 * J32B * j32.pitch * sizeof(float);
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int nb = (n + J32B - 1) / J32B;
    const int nbp = std::max(2, nb + (nb & 1));
    const int blocks = coop_blocks(k, 512, smem, nbp / 2);
    float tolf = JAC_PRE32_TOL;
    int maxs = JAC_PRE32_MAX_SWEEPS;
    const double* Bin = At;
    void* args[] = {(void*)&Bin,  (void*)&n,   (void*)&j32, (void*)&tolf,
                    (void*)&maxs, (void*)&J32, (void*)&info};
    ProfScope prof("jacobi_svd_f32", st, 0.0, 4.0 * 3.0 * n * n);
    PLOM_CHECK_CUDA(cudaLaunchCooperativeKernel(k, dim3(blocks), dim3(512), args, smem, st));
  }
  const int eg = (int)std::max<int64_t>(1, std::min<int64_t>(cdiv((int64_t)nn, 256),
                                                             (int64_t)num_sms() * 16));
  PLOM_TRY(rf_prod(J32, J32, G, n, n, ws, st));  // G = J32^T J32
  pre32_residual_kernel<<<eg, 256, 0, st>>>(G, E, n);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY((gemm_nn<float, float, float, float>(J32, n, E, n, C, n, n, n, n, st)));
  pre32_operands_kernel<<<eg, 256, 0, st>>>(J32, C, A, j32.amax, Jo, nullptr, Rcat, n);
  PLOM_CHECK_LAUNCH();
  PLOM_TRY(jacobi_refine(Rcat, Jo, n, S, Ut, VHt, info, ws, st));
  pre32_unscale_kernel<<<1, 256, 0, st>>>(S, n, j32.amax);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

size_t dense_workspace(int n, int batch, int cplx) {
  // the larger of the two forms' needs (the mixed form's tolerance may take
  // the FP32 pre-sweeps)
  Arena a(nullptr, 0), b(nullptr, 0);
  jacobi_svd(nullptr, n, batch, cplx, 1e-8, nullptr, nullptr, nullptr, nullptr, a, nullptr);
  jacobi_svd(nullptr, n, batch, cplx, 0.0, nullptr, nullptr, nullptr, nullptr, b, nullptr);
  return std::max(a.off, b.off) + 256;
}

// Real n x n SVD through the transpose: one-sided Jacobi on A^T (whose
// columns are the rows of A) needs fewer sweeps than on A for the
// triangular factors of the TSQR.  A^T = Ut S Vt^T  ->  A = Vt S Ut^T.
static int jacobi_svd_transposed(const double* A, int n, double tol, double* S, double* U,
                                 double* VH, int* info, Arena& ws, cudaStream_t st) {
  const size_t nn = (size_t)n * n;
  double* At = ws.take<double>(nn);
  double* Ut = ws.take<double>(nn);
  double* VHt = ws.take<double>(nn);
  const bool pre32 = use_pre32(n, tol);
  JacState js;
  if (!pre32) carve_jac(ws, js, n, 1, 0);
  if (ws.measuring())
    return pre32 ? jacobi_pre32(A, At, n, tol, S, Ut, VHt, info, ws, st) : PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi: workspace too small");
  PLOM_REQUIRE(A && S && U && VH && info, PLOM_ERR_ARG, "jacobi: null pointer");
  PLOM_TRY(transpose_f64(A, At, n, n, 1, st));
  if (pre32)
    PLOM_TRY(jacobi_pre32(A, At, n, tol, S, Ut, VHt, info, ws, st));
  else
    PLOM_TRY(jacobi_launch(At, n, 1, 0, js, tol, S, Ut, VHt, info, st));
  PLOM_TRY(transpose_f64(VHt, U, n, n, 1, st));   // U of A = Vt (columns)
  PLOM_TRY(transpose_f64(Ut, VH, n, n, 1, st));   // rows of V^T of A = columns of Ut
  return PLOM_OK;
}

int jacobi_svd(const double* A, int n, int batch, int cplx, double tol, double* S, double* U,
               double* VH, int* info, Arena& ws, cudaStream_t st) {
  if (!(tol > 0.0)) tol = 2.220446049250313e-16 * (double)std::max(n, 1);
  if (!cplx && batch == 1 && n >= JACOBI_TRANSPOSED_MIN_N)
    return jacobi_svd_transposed(A, n, tol, S, U, VH, info, ws, st);
  JacState js;
  carve_jac(ws, js, n, batch, cplx);
  if (ws.measuring() || n == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "jacobi: workspace too small");
  PLOM_REQUIRE(A && S && U && VH && info, PLOM_ERR_ARG, "jacobi: null pointer");
  return jacobi_launch(A, n, batch, cplx, js, tol, S, U, VH, info, st);
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
