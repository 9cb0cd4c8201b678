// CUDA-core (SIMT) GEMMs for the tall-skinny shapes of the SVD path.
//
//  * gemm_nn:  C(M x N) = A(M x K) B(K x N), A tall (M = points), B small.
//              Used for Q = X R^-1, U = Q Ur, Y = A Omega, Phi = Y2 (...).
//  * gemm_tn:  C(M x N) = A(K x M)^T B(K x N) with K = points (huge): a
//              split-K reduction over row chunks, partial tiles written to
//              a workspace slab and summed in FP64 in a fixed order (the
//              in-GPU replacement of the TSQR butterfly / MPI_Allreduce of
//              pyLOM/vmmath/src/svd.c:565-676 and vector_matrix.c:330-356).
//              sym=true computes only the upper block triangle (Gram).
//
// These are the plain-FP64 GPU form's products (GB300's FP64 rate bounds
// them), the n x n FP64 products of the small factorizations, and the
// fallback of the mixed form for operand shapes the tensor-core kernels do
// not take.
#include "plom_common.cuh"
#include "plom_kernels.cuh"

#include <algorithm>
#include <memory>

namespace plom {

// ----------------------------------------------------------------------------
// NN: BM x BN block tile, BK deep; 256 threads as 16 x 16, TM x TN per thread.
// ----------------------------------------------------------------------------
template <typename TA, typename TB, typename TC, typename Acc, int BM, int BN, int BK, int TM,
          int TN>
__global__ void __launch_bounds__(256) gemm_nn_kernel(const TA* __restrict__ A, int64_t lda,
                                                      int64_t sA, const TB* __restrict__ B,
                                                      int64_t ldb, int64_t sB, TC* __restrict__ C,
                                                      int64_t ldc, int64_t sC, int64_t M,
                                                      int64_t N, int64_t K, int b_upper) {
  static_assert(BM == 16 * TM && BN == 16 * TN, "tile/thread mismatch");
  A += (int64_t)blockIdx.z * sA;
  B += (int64_t)blockIdx.z * sB;
  C += (int64_t)blockIdx.z * sC;
  __shared__ Acc As[BK][BM + 1];
  __shared__ Acc Bs[BK][BN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  Acc acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = Acc(0);

  // B upper triangular (B[k][j] = 0 for k > j): this column block needs k < n0 + BN
  const int64_t kend = b_upper ? min(K, n0 + BN) : K;
  for (int64_t k0 = 0; k0 < kend; k0 += BK) {
    // A tile: BM rows x BK cols
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      int r = e / BK, c = e % BK;
      int64_t gr = m0 + r, gc = k0 + c;
      As[c][r] = (gr < M && gc < kend) ? (Acc)A[gr * lda + gc] : Acc(0);
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      int r = e / BN, c = e % BN;
      int64_t gr = k0 + r, gc = n0 + c;
      Bs[r][c] = (gr < kend && gc < N) ? (Acc)B[gr * ldb + gc] : Acc(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      Acc a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int64_t gr = m0 + ty + 16 * i;
    if (gr >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t gc = n0 + tx + 16 * j;
      if (gc < N) C[gr * ldc + gc] = (TC)acc[i][j];
    }
  }
}

template <typename TA, typename TB, typename TC, typename Acc>
int gemm_nn_batched(const TA* A, int64_t lda, int64_t sA, const TB* B, int64_t ldb, int64_t sB,
                    TC* C, int64_t ldc, int64_t sC, int64_t M, int64_t N, int64_t K, int batch,
                    cudaStream_t st, bool b_upper) {
  if (M == 0 || N == 0 || batch == 0) return PLOM_OK;
  PLOM_REQUIRE(A && B && C, PLOM_ERR_ARG, "gemm_nn: null operand");
  constexpr int BM = 128, BN = 64, BK = 8;
  dim3 grid((unsigned)cdiv(M, BM), (unsigned)cdiv(N, BN), (unsigned)batch);
  PLOM_REQUIRE(grid.y <= 65535 && batch <= 65535, PLOM_ERR_ARG, "gemm_nn: N or batch too large");
  const double fl = b_upper && N == K ? (double)M * N * (N + 1) : 2.0 * M * N * K;
  ProfScope prof(sizeof(Acc) == 8 ? "gemm_nn_fp64" : "gemm_nn_fp32", st, fl * batch,
                 (double)batch * ((double)M * K * sizeof(TA) + (double)M * N * sizeof(TC)));
  gemm_nn_kernel<TA, TB, TC, Acc, BM, BN, BK, 8, 4><<<grid, 256, 0, st>>>(
      A, lda, sA, B, ldb, sB, C, ldc, sC, M, N, K, b_upper ? 1 : 0);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

template <typename TA, typename TB, typename TC, typename Acc>
int gemm_nn(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc, int64_t M,
            int64_t N, int64_t K, cudaStream_t st, bool b_upper) {
  return gemm_nn_batched<TA, TB, TC, Acc>(A, lda, 0, B, ldb, 0, C, ldc, 0, M, N, K, 1, st, b_upper);
}

// ----------------------------------------------------------------------------
// Small FP64 products of the n x n stage: C = alpha A B on 32 x 32 tiles.  A
// tile's K range is clipped to the band where triangular operands are
// non-zero (tri bit 0: A upper, A[i][k] = 0 for k < i; bit 1: B upper,
// B[k][j] = 0 for k > j), so a triangular x triangular product costs n^3/6
// FMAs and triangular x dense n^3/2.  FP64 throughput per SM bounds these
// products on GB300, so the tiles are small enough (1,024 for n = 1,024) that
// the longest tile is a small share of the whole.  grid.z enumerates
// (problem b, sub-block t): operands sit at b*s + t*tstride.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) gemm_sq_kernel(const double* __restrict__ A, int64_t lda,
                                                      int64_t sA, int64_t tA,
                                                      const double* __restrict__ B, int64_t ldb,
                                                      int64_t sB, int64_t tB, double* __restrict__ C,
                                                      int64_t ldc, int64_t sC, int64_t tC, int M,
                                                      int N, int K, int nsub, double alpha, int tri) {
  const int64_t b = blockIdx.z / nsub, t = blockIdx.z % nsub;
  A += b * sA + t * tA;
  B += b * sB + t * tB;
  C += b * sC + t * tC;
  __shared__ double As[32][33];  // [k][row]
  __shared__ double Bs[32][33];  // [k][col]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
  const int kbeg = (tri & 1) ? m0 : 0;
  const int kend = (tri & 2) ? min(K, n0 + 32) : K;
  double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
  for (int k0 = kbeg; k0 < kend; k0 += 32) {
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      const int r = e >> 5, c = e & 31;
      const int ga = m0 + r, gk = k0 + c;
      As[c][r] = (ga < M && gk < kend) ? A[(int64_t)ga * lda + gk] : 0.0;
      const int gb = k0 + r, gn = n0 + c;
      Bs[r][c] = (gb < kend && gn < N) ? B[(int64_t)gb * ldb + gn] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const double a0 = As[kk][ty], a1 = As[kk][ty + 16];
      const double b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
      c00 = fma(a0, b0, c00);
      c01 = fma(a0, b1, c01);
      c10 = fma(a1, b0, c10);
      c11 = fma(a1, b1, c11);
    }
    __syncthreads();
  }
  const int r0 = m0 + ty, r1 = r0 + 16, q0 = n0 + tx, q1 = q0 + 16;
  if (r0 < M && q0 < N) C[(int64_t)r0 * ldc + q0] = alpha * c00;
  if (r0 < M && q1 < N) C[(int64_t)r0 * ldc + q1] = alpha * c01;
  if (r1 < M && q0 < N) C[(int64_t)r1 * ldc + q0] = alpha * c10;
  if (r1 < M && q1 < N) C[(int64_t)r1 * ldc + q1] = alpha * c11;
}

int gemm_sq(const double* A, int64_t lda, int64_t sA, int64_t tA, const double* B, int64_t ldb,
            int64_t sB, int64_t tB, double* C, int64_t ldc, int64_t sC, int64_t tC, int M, int N,
            int K, int batch, int nsub, double alpha, int tri, cudaStream_t st, const char* tag) {
  if (M <= 0 || N <= 0 || batch <= 0 || nsub <= 0) return PLOM_OK;
  PLOM_REQUIRE(A && B && C, PLOM_ERR_ARG, "gemm_sq: null operand");
  PLOM_REQUIRE((int64_t)batch * nsub <= 65535, PLOM_ERR_ARG, "gemm_sq: batch too large");
  const dim3 grid((unsigned)cdiv(M, 32), (unsigned)cdiv(N, 32), (unsigned)(batch * nsub));
  // FMAs of the band the kernel visits, counted as flops (2 per FMA)
  double fl = 2.0 * M * N * K;
  if ((tri & 3) == 3) fl = 2.0 * M * (double)N * K / 6.0;
  else if (tri & 3) fl = 2.0 * M * (double)N * K / 2.0;
  // tag == nullptr: timed by the caller's region
  std::unique_ptr<ProfScope> prof;
  if (tag)
    prof.reset(new ProfScope(tag, st, fl * batch * nsub,
                             8.0 * batch * nsub * ((double)M * K + (double)K * N + (double)M * N)));
  gemm_sq_kernel<<<grid, 256, 0, st>>>(A, lda, sA, tA, B, ldb, sB, tB, C, ldc, sC, tC, M, N, K,
                                       nsub, alpha, tri);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// ----------------------------------------------------------------------------
// TN split-K: partial[b][c](M x N) = sum_{k in chunk c} A_b[k][i] B_b[k][j]
// ----------------------------------------------------------------------------
template <typename TA, typename TB, typename Acc, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_tn_kernel(const TA* __restrict__ A, int64_t lda,
                                                      int64_t sA, const TB* __restrict__ B,
                                                      int64_t ldb, int64_t sB,
                                                      Acc* __restrict__ part, int64_t M, int64_t N,
                                                      int64_t K, int64_t kchunk, int nchunks,
                                                      const int2* __restrict__ tiles) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ Acc As[BK][BM];
  __shared__ Acc Bs[BK][BN];
  const int bz = blockIdx.z;
  A += (int64_t)bz * sA;
  B += (int64_t)bz * sB;
  const int2 t = tiles[blockIdx.x];
  const int64_t i0 = (int64_t)t.x * BM, j0 = (int64_t)t.y * BN;
  const int64_t kbeg = (int64_t)blockIdx.y * kchunk;
  const int64_t kend = min(K, kbeg + kchunk);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  Acc acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = Acc(0);
  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
    for (int e = threadIdx.x; e < BK * BM; e += 256) {
      int r = e / BM, c = e % BM;
      int64_t gk = k0 + r, gi = i0 + c;
      As[r][c] = (gk < kend && gi < M) ? (Acc)A[gk * lda + gi] : Acc(0);
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      int r = e / BN, c = e % BN;
      int64_t gk = k0 + r, gj = j0 + c;
      Bs[r][c] = (gk < kend && gj < N) ? (Acc)B[gk * ldb + gj] : Acc(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      Acc a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  Acc* P = part + ((int64_t)bz * nchunks + blockIdx.y) * M * N;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int64_t gi = i0 + ty + 16 * i;
    if (gi >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t gj = j0 + tx + 16 * j;
      if (gj < N) P[gi * N + gj] = acc[i][j];
    }
  }
}

// Sum the chunk partials in a fixed order (deterministic), mirror the upper
// block triangle for sym, and write C (batch stride sC) in TC.
template <typename Acc, typename TC>
__global__ void reduce_partials_kernel(const Acc* __restrict__ part, int nchunks, int64_t M,
                                       int64_t N, int sym, int bm, int bn, TC* __restrict__ C,
                                       int64_t ldc, int64_t sC, int batch) {
  const int64_t total = M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total * batch;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = e / total, r = e % total;
    int64_t i = r / N, j = r % N;
    int64_t si = i, sj = j;
    if (sym && (i / bm) > (j / bn)) {  // lower block triangle: read the mirror
      si = j;
      sj = i;
    }
    const Acc* p = part + b * nchunks * total + si * N + sj;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += (double)p[(int64_t)c * total];
    C[b * sC + i * ldc + j] = (TC)s;
  }
}

__global__ void make_tiles_kernel(int2* tiles, int tm, int tn, int sym) {
  int idx = 0;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = 0; i < tm; ++i)
    for (int j = 0; j < tn; ++j)
      if (!sym || i <= j) tiles[idx++] = make_int2(i, j);
}

static int tn_chunks(int64_t ntiles, int64_t K, int BK, int batch) {
  int64_t target = (int64_t)num_sms() * 4;
  int64_t c = cdiv(target, ntiles * batch);
  int64_t maxc = cdiv(K, (int64_t)BK * 64);  // at least 64 k-steps per chunk
  if (c > maxc) c = maxc;
  if (c < 1) c = 1;
  if (c > 512) c = 512;
  return (int)c;
}

struct TnPlan {
  int64_t tm, tn, ntiles, kchunk;
  int chunks;
};
static TnPlan tn_plan(int64_t M, int64_t N, int64_t K, bool sym, int batch) {
  constexpr int BM = 64, BN = 64, BK = 16;
  TnPlan p;
  p.tm = cdiv(M, BM);
  p.tn = cdiv(N, BN);
  p.ntiles = sym ? p.tm * (p.tm + 1) / 2 : p.tm * p.tn;
  int c = tn_chunks(p.ntiles, K, BK, batch);
  int64_t kc = cdiv(std::max<int64_t>(K, 1), c);
  kc = cdiv(kc, BK) * BK;
  p.kchunk = kc;
  p.chunks = (int)std::max<int64_t>(1, cdiv(K, kc));
  return p;
}

size_t gemm_tn_workspace_batched(int64_t M, int64_t N, int64_t K, bool sym, size_t acc_bytes,
                                 int batch) {
  TnPlan p = tn_plan(M, N, K, sym, batch);
  Arena a(nullptr, 0);
  a.take<char>((size_t)batch * p.chunks * M * N * acc_bytes);
  a.take<int2>((size_t)p.tm * p.tn);
  return a.off + 256;
}
size_t gemm_tn_workspace(int64_t M, int64_t N, int64_t K, bool sym, size_t acc_bytes) {
  return gemm_tn_workspace_batched(M, N, K, sym, acc_bytes, 1);
}

template <typename TA, typename TB, typename Acc, typename TC>
int gemm_tn_batched(const TA* A, int64_t lda, int64_t sA, const TB* B, int64_t ldb, int64_t sB,
                    TC* C, int64_t ldc, int64_t sC, int64_t M, int64_t N, int64_t K, bool sym,
                    int batch, Arena& ws, cudaStream_t st) {
  if (M == 0 || N == 0 || batch == 0) return PLOM_OK;
  constexpr int BM = 64, BN = 64, BK = 16;
  PLOM_REQUIRE(!sym || M == N, PLOM_ERR_ARG, "gemm_tn: sym needs a square result");
  PLOM_REQUIRE(batch <= 65535, PLOM_ERR_ARG, "gemm_tn: batch too large");
  TnPlan p = tn_plan(M, N, K, sym, batch);
  Acc* part = ws.take<Acc>((size_t)batch * p.chunks * M * N);
  int2* tiles = ws.take<int2>((size_t)p.tm * p.tn);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gemm_tn: workspace too small");
  PLOM_REQUIRE(A && B && C && part, PLOM_ERR_ARG, "gemm_tn: null operand");
  make_tiles_kernel<<<1, 1, 0, st>>>(tiles, (int)p.tm, (int)p.tn, sym ? 1 : 0);
  PLOM_CHECK_LAUNCH();
  if (K > 0) {
    dim3 grid((unsigned)p.ntiles, (unsigned)p.chunks, (unsigned)batch);
    ProfScope prof(sizeof(Acc) == 8 ? "gemm_tn_fp64" : "gemm_tn_fp32", st,
                   (sym ? 1.0 : 2.0) * M * N * K * batch,
                   (double)batch * K * ((double)M * sizeof(TA) + (sym ? 0.0 : (double)N * sizeof(TB))));
    gemm_tn_kernel<TA, TB, Acc, BM, BN, BK><<<grid, 256, 0, st>>>(A, lda, sA, B, ldb, sB, part, M,
                                                                  N, K, p.kchunk, p.chunks, tiles);
    PLOM_CHECK_LAUNCH();
  } else {
    PLOM_CHECK_CUDA(cudaMemsetAsync(part, 0, sizeof(Acc) * M * N * batch * p.chunks, st));
  }
  int64_t total = M * N * batch;
  int blocks = (int)std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16);
  reduce_partials_kernel<Acc, TC><<<blocks, 256, 0, st>>>(part, p.chunks, M, N, sym ? 1 : 0, BM, BN,
                                                          C, ldc, sC, batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

template <typename TA, typename TB, typename Acc, typename TC>
int gemm_tn(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc, int64_t M,
            int64_t N, int64_t K, bool sym, Arena& ws, cudaStream_t st) {
  return gemm_tn_batched<TA, TB, Acc, TC>(A, lda, 0, B, ldb, 0, C, ldc, 0, M, N, K, sym, 1, ws, st);
}

// The split-K product of gemm_tn (non-symmetric, one matrix) computed in a
// caller-given scratch region of `cap` bytes instead of an arena: the chunk
// count is lowered until the FP64 partials and the tile list fit.  Returns
// PLOM_ERR_WORKSPACE (and launches nothing) when one chunk does not fit.
template <typename TA, typename TB, typename TC>
int gemm_tn_in_scratch(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc,
                       int64_t M, int64_t N, int64_t K, void* scratch, size_t cap,
                       cudaStream_t st) {
  if (M == 0 || N == 0) return PLOM_OK;
  constexpr int BM = 64, BN = 64, BK = 16;
  PLOM_REQUIRE(A && B && C && scratch, PLOM_ERR_ARG, "null operand");
  TnPlan p = tn_plan(M, N, K, false, 1);
  const size_t tiles_bytes = ((size_t)p.tm * p.tn * sizeof(int2) + 255) / 256 * 256;
  const size_t per_chunk = (size_t)M * N * sizeof(double);
  PLOM_REQUIRE(cap > tiles_bytes && (cap - tiles_bytes) / per_chunk >= 1, PLOM_ERR_WORKSPACE,
               "result %lld x %lld needs %zu bytes of scratch; the static scratch holds %zu",
               (long long)M, (long long)N, per_chunk + tiles_bytes, cap);
  int64_t chunks = std::min<int64_t>(p.chunks, (int64_t)((cap - tiles_bytes) / per_chunk));
  int64_t kchunk = cdiv(std::max<int64_t>(K, 1), chunks);
  kchunk = cdiv(kchunk, BK) * BK;
  chunks = std::max<int64_t>(1, cdiv(K, kchunk));
  int2* tiles = reinterpret_cast<int2*>(scratch);
  double* part = reinterpret_cast<double*>(static_cast<char*>(scratch) + tiles_bytes);
  make_tiles_kernel<<<1, 1, 0, st>>>(tiles, (int)p.tm, (int)p.tn, 0);
  PLOM_CHECK_LAUNCH();
  if (K > 0) {
    dim3 grid((unsigned)p.ntiles, (unsigned)chunks, 1u);
    gemm_tn_kernel<TA, TB, double, BM, BN, BK><<<grid, 256, 0, st>>>(A, lda, 0, B, ldb, 0, part, M,
                                                                     N, K, kchunk, (int)chunks,
                                                                     tiles);
    PLOM_CHECK_LAUNCH();
  } else {
    PLOM_CHECK_CUDA(cudaMemsetAsync(part, 0, per_chunk, st));  // empty sum
    chunks = 1;
  }
  int64_t total = M * N;
  int blocks = (int)std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16);
  reduce_partials_kernel<double, TC><<<blocks, 256, 0, st>>>(part, (int)chunks, M, N, 0, BM, BN, C,
                                                             ldc, 0, 1);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}
template int gemm_tn_in_scratch<float, float, float>(const float*, int64_t, const float*, int64_t,
                                                     float*, int64_t, int64_t, int64_t, int64_t,
                                                     void*, size_t, cudaStream_t);
template int gemm_tn_in_scratch<double, double, double>(const double*, int64_t, const double*,
                                                        int64_t, double*, int64_t, int64_t,
                                                        int64_t, int64_t, void*, size_t,
                                                        cudaStream_t);

// ----------------------------------------------------------------------------
// TN with blocked double-float sums:
//   C(M x N, FP64) = A(K x M)^T B(K x N), A and B FP32, K = points.
// Each thread sums 32 rows of products with FP32 FMAs (round-to-nearest, so
// the block errors are unbiased, at most ~32 u of the block's |terms|) and
// folds the block sum into a double-float accumulator with TwoSum; the
// accumulator carries ~44 bits across the whole row chunk.  The relative
// error of a chunk sum is then ~u / sqrt(blocks) instead of the ~u K drift
// (and, on the tensor cores, the ~1e-5 truncation bias) of one long FP32
// accumulation, at ~1.2 FP32 instructions per product (GB300 runs FP64 at
// 1/64 of its FP32 rate).  Row-chunk partials are summed in FP64 in a fixed
// order.  Used where a reduction over the points must be FP64-accurate (DMD's
// projection onto span(U_r)).
// 128 threads as 8 x 16, 4 x 8 outputs each (rows ty*4.., columns tx*4.. and
// 64 + tx*4..), operands from shared memory as 16-byte vectors, the next
// 32-row tile prefetched into registers while the current one is summed.
// ----------------------------------------------------------------------------
constexpr int DF_BM = 32, DF_BN = 128, DF_BK = 32, DF_THREADS = 128;

__global__ void __launch_bounds__(DF_THREADS) gemm_tn_df_kernel(const float* __restrict__ A,
                                                                int64_t lda,
                                                                const float* __restrict__ B,
                                                                int64_t ldb,
                                                                double* __restrict__ part,
                                                                int64_t M, int64_t N, int64_t K,
                                                                int64_t kchunk, int64_t tm) {
  constexpr int TM = 4, TN = 8;
  constexpr int LA = DF_BK * DF_BM / DF_THREADS, LB = DF_BK * DF_BN / DF_THREADS;
  static_assert(DF_BM == 8 * TM && DF_BN == 16 * TN, "tile / thread layout");
  __shared__ __align__(16) float As[DF_BK][DF_BM];
  __shared__ __align__(16) float Bs[DF_BK][DF_BN];
  const int64_t i0 = (int64_t)(blockIdx.x % tm) * DF_BM, j0 = (int64_t)(blockIdx.x / tm) * DF_BN;
  const int64_t kbeg = (int64_t)blockIdx.y * kchunk;
  const int64_t kend = min(K, kbeg + kchunk);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float hi[TM][TN], lo[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) hi[i][j] = lo[i][j] = 0.f;
  float ra[LA], rb[LB];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + q * DF_THREADS;
      const int64_t gk = k0 + e / DF_BM, gi = i0 + e % DF_BM;
      ra[q] = (gk < kend && gi < M) ? A[gk * lda + gi] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + q * DF_THREADS;
      const int64_t gk = k0 + e / DF_BN, gj = j0 + e % DF_BN;
      rb[q] = (gk < kend && gj < N) ? B[gk * ldb + gj] : 0.f;
    }
  };
  if (kbeg < kend) load(kbeg);
  for (int64_t k0 = kbeg; k0 < kend; k0 += DF_BK) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      const int e = threadIdx.x + q * DF_THREADS;
      As[e / DF_BM][e % DF_BM] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      const int e = threadIdx.x + q * DF_THREADS;
      Bs[e / DF_BN][e % DF_BN] = rb[q];
    }
    __syncthreads();
    if (k0 + DF_BK < kend) load(k0 + DF_BK);
    float s[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) s[i][j] = 0.f;
#pragma unroll 8
    for (int kk = 0; kk < DF_BK; ++kk) {
      const float4 av = *reinterpret_cast<const float4*>(&As[kk][ty * TM]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + tx * 4]);
      const float a[TM] = {av.x, av.y, av.z, av.w};
      const float b[TN] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) s[i][j] = fmaf(a[i], b[j], s[i][j]);
    }
    // fold the block sums: (hi, lo) += s with TwoSum
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const float t = hi[i][j] + s[i][j];
        const float bb = t - hi[i][j];
        lo[i][j] += (hi[i][j] - (t - bb)) + (s[i][j] - bb);
        hi[i][j] = t;
      }
    __syncthreads();
  }
  double* P = part + (int64_t)blockIdx.y * M * N;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t gi = i0 + ty * TM + i;
    if (gi >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t gj = j0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
      if (gj < N) P[gi * N + gj] = (double)hi[i][j] + (double)lo[i][j];
    }
  }
}

struct DfPlan {
  int64_t tm, tn, kchunk;
  int chunks;
};
static DfPlan df_plan(int64_t M, int64_t N, int64_t K) {
  DfPlan p;
  p.tm = cdiv(M, DF_BM);
  p.tn = cdiv(N, DF_BN);
  int c = tn_chunks(p.tm * p.tn, K, DF_BK, 1);
  int64_t kc = cdiv(std::max<int64_t>(K, 1), c);
  kc = cdiv(kc, DF_BK) * DF_BK;
  p.kchunk = kc;
  p.chunks = (int)std::max<int64_t>(1, cdiv(K, kc));
  return p;
}

int gemm_tn_df(const float* A, int64_t lda, const float* B, int64_t ldb, double* C, int64_t ldc,
               int64_t M, int64_t N, int64_t K, Arena& ws, cudaStream_t st) {
  if (M == 0 || N == 0) return PLOM_OK;
  const DfPlan p = df_plan(M, N, K);
  double* part = ws.take<double>((size_t)p.chunks * M * N);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gemm_tn_df: workspace too small");
  PLOM_REQUIRE(A && B && C && part, PLOM_ERR_ARG, "gemm_tn_df: null operand");
  PLOM_REQUIRE(p.tm * p.tn <= INT32_MAX && p.chunks <= 65535, PLOM_ERR_ARG,
               "gemm_tn_df: result too large");
  ProfScope prof("gemm_tn_df", st, 2.0 * M * N * K, (double)K * (M + N) * sizeof(float),
                 K > 0 ? 2 : 1);
  if (K > 0) {
    dim3 grid((unsigned)(p.tm * p.tn), (unsigned)p.chunks, 1u);
    gemm_tn_df_kernel<<<grid, DF_THREADS, 0, st>>>(A, lda, B, ldb, part, M, N, K, p.kchunk, p.tm);
    PLOM_CHECK_LAUNCH();
  } else {
    PLOM_CHECK_CUDA(cudaMemsetAsync(part, 0, sizeof(double) * M * N, st));
  }
  const int64_t total = M * N;
  const int blocks = (int)std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16);
  reduce_partials_kernel<double, double><<<blocks, 256, 0, st>>>(part, K > 0 ? p.chunks : 1, M, N,
                                                                 0, DF_BM, DF_BN, C, ldc, 0, 1);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// explicit instantiations used across the library
#define NN(TA, TB, TC, ACC)                                                                  \
  template int gemm_nn<TA, TB, TC, ACC>(const TA*, int64_t, const TB*, int64_t, TC*, int64_t, \
                                        int64_t, int64_t, int64_t, cudaStream_t, bool);       \
  template int gemm_nn_batched<TA, TB, TC, ACC>(const TA*, int64_t, int64_t, const TB*, int64_t, \
                                                int64_t, TC*, int64_t, int64_t, int64_t, int64_t, \
                                                int64_t, int, cudaStream_t, bool);
NN(float, float, float, float)
NN(float, double, double, double)
NN(float, double, float, double)
NN(double, double, double, double)
NN(double, double, float, double)
NN(float, double, float, float)
NN(float, float, float, double)
#undef NN
#define TN(TA, TB, ACC, TC)                                                                    \
  template int gemm_tn<TA, TB, ACC, TC>(const TA*, int64_t, const TB*, int64_t, TC*, int64_t,   \
                                        int64_t, int64_t, int64_t, bool, Arena&, cudaStream_t); \
  template int gemm_tn_batched<TA, TB, ACC, TC>(const TA*, int64_t, int64_t, const TB*, int64_t, \
                                                int64_t, TC*, int64_t, int64_t, int64_t, int64_t, \
                                                int64_t, bool, int, Arena&, cudaStream_t);
TN(float, float, float, double)
TN(float, float, double, double)
TN(double, double, double, double)
TN(float, float, float, float)
TN(float, float, double, float)
TN(double, double, double, float)
TN(float, double, double, double)
TN(double, float, double, double)
#undef TN

}  // namespace plom
