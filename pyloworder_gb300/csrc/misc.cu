// Small utility kernels: type conversion, strided 2-D copies and the Philox
// uniform generator for the randomized range finder's test matrix.
#include <algorithm>

#include "plom_common.cuh"
#include "plom_kernels.cuh"

namespace plom {

static int grid1d(int64_t work) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(work, 256), (int64_t)num_sms() * 32));
}

template <typename TI, typename TO>
__global__ void convert_kernel(const TI* __restrict__ in, TO* __restrict__ out, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (TO)in[i];
}

template <typename TI, typename TO>
int convert(const TI* in, TO* out, int64_t count, cudaStream_t st) {
  if (count == 0) return PLOM_OK;
  PLOM_REQUIRE(in && out, PLOM_ERR_ARG, "convert: null pointer");
  convert_kernel<TI, TO><<<grid1d(count), 256, 0, st>>>(in, out, count);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

template <typename TI, typename TO>
__global__ void copy2d_kernel(const TI* __restrict__ in, int64_t ldi, TO* __restrict__ out,
                              int64_t ldo, int64_t rows, int64_t cols) {
  const int64_t total = rows * cols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e / cols, c = e % cols;
    out[r * ldo + c] = (TO)in[r * ldi + c];
  }
}

template <typename TI, typename TO>
int copy2d(const TI* in, int64_t ldi, TO* out, int64_t ldo, int64_t rows, int64_t cols,
           cudaStream_t st) {
  if (rows == 0 || cols == 0) return PLOM_OK;
  PLOM_REQUIRE(in && out, PLOM_ERR_ARG, "copy2d: null pointer");
  copy2d_kernel<TI, TO><<<grid1d(rows * cols), 256, 0, st>>>(in, ldi, out, ldo, rows, cols);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

#define INST(TI, TO)                                                                   \
  template int convert<TI, TO>(const TI*, TO*, int64_t, cudaStream_t);                 \
  template int copy2d<TI, TO>(const TI*, int64_t, TO*, int64_t, int64_t, int64_t, cudaStream_t);
INST(float, double)
INST(double, float)
INST(double, double)
INST(float, float)
#undef INST

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter = element index,
// key = seed.  float: top 24 bits of word 0; double: 53 bits of words 0,1.
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

template <typename T>
__global__ void uniform_kernel(T* __restrict__ out, int64_t count, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)(uint64_t)i, (uint32_t)((uint64_t)i >> 32), 0u, 0u};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    if (sizeof(T) == 8) {
      uint64_t bits = (((uint64_t)c[0] << 32) | c[1]) >> 11;
      out[i] = (T)((double)bits * (1.0 / 9007199254740992.0));
    } else {
      out[i] = (T)((float)(c[0] >> 8) * (1.0f / 16777216.0f));
    }
  }
}

int fill_uniform_dispatch(int dtype, void* out, int64_t count, uint64_t seed, cudaStream_t st) {
  if (count == 0) return PLOM_OK;
  if (dtype == PLOM_F32)
    uniform_kernel<float><<<grid1d(count), 256, 0, st>>>((float*)out, count, seed);
  else if (dtype == PLOM_F64)
    uniform_kernel<double><<<grid1d(count), 256, 0, st>>>((double*)out, count, seed);
  else {
    set_error("fill_uniform: dtype must be F32 or F64");
    return PLOM_ERR_UNSUPPORTED;
  }
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// Orthonormal completion of U's null columns (real, one problem).  An exact
// zero column of the tall matrix leaves an exact zero column in every
// CholeskyQR factor Q, so U = Q M gets a zero column for that singular value
// (sigma ~ 0), where LAPACK returns a unit vector orthogonal to the other
// columns.  Candidates are the columns with sigma <= 1e-6 sigma_1 (at most
// NC_MAX, smallest first); those whose norm is below 1/2 are replaced one at
// a time by u = e_i - U (U^T e_i), normalised, with a different row i for
// each (U^T e_i is row i of U, with the columns still to be completed left
// out).  The candidates' norms come from the factors, not from U (which may
// be mapped host memory): U = F M with F the tall factor of Gram G, so
// ||U e_c||^2 = m_c^T G m_c.  Without null columns U is not touched.
// ---------------------------------------------------------------------------
constexpr int NC_MAX = 8;

__global__ void nc_candidates_kernel(const double* __restrict__ S, int n, int* __restrict__ list,
                                     int* __restrict__ count) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int c = 0;
  const double thr = 1e-6 * S[0];
  for (int j = n - 1; j >= 0 && c < NC_MAX; --j) {
    if (!(S[j] <= thr)) break;
    list[c++] = j;
  }
  *count = c;
}

// part[q gn + blockIdx.x] = sum over the 32 rows k of this block of
// m_c[k] (G m_c)[k] (c = list[q]); the 8 warps' shares summed in a fixed order
__global__ void __launch_bounds__(256) nc_norms_kernel(const double* __restrict__ G,
                                                       const double* __restrict__ Mf, int N,
                                                       const int* __restrict__ list,
                                                       const int* __restrict__ count,
                                                       double* __restrict__ part) {
  const int q = blockIdx.y;
  if (q >= *count) return;
  const int c = list[q];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  __shared__ double red[8];
  double mine = 0.0;
  for (int k = blockIdx.x * 32 + wib; k < min(N, (int)blockIdx.x * 32 + 32); k += 8) {
    double acc = 0.0;
    for (int l = lane; l < N; l += 32) acc = fma(G[(int64_t)k * N + l], Mf[(int64_t)l * N + c], acc);
    acc = warp_sum(acc);
    mine = fma(Mf[(int64_t)k * N + c], acc, mine);
  }
  if (lane == 0) red[wib] = mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[(int64_t)q * gridDim.x + blockIdx.x] = t;
  }
}

// out[q] = sum of the g partials of candidate q, in a fixed order (one warp
// per candidate)
__global__ void __launch_bounds__(32 * NC_MAX) nc_sum_kernel(const double* __restrict__ part,
                                                             int g, double* __restrict__ out) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double t = 0.0;
  for (int k = lane; k < g; k += 32) t += part[(int64_t)q * g + k];
  t = warp_sum(t);
  if (lane == 0) out[q] = t;
}

__device__ __forceinline__ int64_t nc_row(int q, int64_t m) {
  return (int64_t)(((uint64_t)(q + 1) * 2654435761ull) % (uint64_t)m);
}

// u = e_i - U w, w = row i of U without the columns still to be completed
// (this one included); written into column list[q], the block's share of its
// squared norm into part[blockIdx.x] (warps summed in a fixed order)
template <typename T>
__global__ void __launch_bounds__(256) nc_project_kernel(T* __restrict__ U, int64_t m, int n,
                                                         int64_t ldu, const int* __restrict__ list,
                                                         const int* __restrict__ count,
                                                         const double* __restrict__ sums, int q,
                                                         double* __restrict__ part) {
  if (q >= *count || !(sums[q] < 0.25)) return;
  extern __shared__ double ncw[];
  __shared__ double red[8];
  const int64_t i = nc_row(q, m);
  const int c = list[q];
  for (int j = threadIdx.x; j < n; j += blockDim.x) ncw[j] = (double)U[i * ldu + j];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int p = q; p < *count; ++p)
      if (sums[p] < 0.25) ncw[list[p]] = 0.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double mine = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * 8 + wib; r < m; r += (int64_t)gridDim.x * 8) {
    const T* row = U + r * ldu;
    double acc = 0.0;
    for (int j = lane; j < n; j += 32) acc = fma((double)row[j], ncw[j], acc);
    acc = warp_sum(acc);
    const double u = (r == i ? 1.0 : 0.0) - acc;
    if (lane == 0) {
      U[r * ldu + c] = (T)u;
      mine = fma(u, u, mine);
    }
  }
  if (lane == 0) red[wib] = mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// every block sums the gp partials of the projection in a fixed order, then
// scales its rows of the completed column to unit norm
template <typename T>
__global__ void __launch_bounds__(256) nc_scale_kernel(T* __restrict__ U, int64_t m, int64_t ldu,
                                                       const int* __restrict__ list,
                                                       const int* __restrict__ count,
                                                       const double* __restrict__ sums, int q,
                                                       const double* __restrict__ part, int gp) {
  if (q >= *count || !(sums[q] < 0.25)) return;
  __shared__ double red[8];
  double t = 0.0;
  for (int k = threadIdx.x; k < gp; k += blockDim.x) t += part[k];
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  double nrm2 = 0.0;
  for (int w = 0; w < 8; ++w) nrm2 += red[w];
  if (!(nrm2 > 0.0)) return;
  const int c = list[q];
  const double f = 1.0 / sqrt(nrm2);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x)
    U[r * ldu + c] = (T)((double)U[r * ldu + c] * f);
}

template <typename T>
int complete_null_columns(const double* S, int n, T* U, int64_t m, int64_t ldu, const double* G,
                          const double* Mf, Arena& ws, cudaStream_t st) {
  const unsigned gn = (unsigned)std::max<int64_t>(1, cdiv(n, 32));
  const unsigned gp = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(m, 8), (int64_t)num_sms() * 8));
  int* list = ws.take<int>(NC_MAX);
  int* count = ws.take<int>(1);
  double* sums = ws.take<double>(NC_MAX);
  double* npart = ws.take<double>((size_t)NC_MAX * gn);
  double* ppart = ws.take<double>(gp);
  if (ws.measuring() || n < 1 || m < 1) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "null-column completion: workspace too small");
  PLOM_REQUIRE(S && U && G && Mf && n <= 8192, PLOM_ERR_ARG,
               "null-column completion: bad arguments");
  ProfScope prof("null_cols", st, 0.0, (double)sizeof(T) * m, 3 + 2 * NC_MAX);
  nc_candidates_kernel<<<1, 32, 0, st>>>(S, n, list, count);
  PLOM_CHECK_LAUNCH();
  const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(m, 256), (int64_t)num_sms() * 4));
  nc_norms_kernel<<<dim3(gn, NC_MAX), 256, 0, st>>>(G, Mf, n, list, count, npart);
  PLOM_CHECK_LAUNCH();
  nc_sum_kernel<<<1, 32 * NC_MAX, 0, st>>>(npart, (int)gn, sums);
  PLOM_CHECK_LAUNCH();
  for (int q = 0; q < NC_MAX; ++q) {
    nc_project_kernel<T><<<gp, 256, sizeof(double) * n, st>>>(U, m, n, ldu, list, count, sums, q,
                                                              ppart);
    PLOM_CHECK_LAUNCH();
    nc_scale_kernel<T><<<gx, 256, 0, st>>>(U, m, ldu, list, count, sums, q, ppart, (int)gp);
    PLOM_CHECK_LAUNCH();
  }
  return PLOM_OK;
}
template int complete_null_columns<float>(const double*, int, float*, int64_t, int64_t,
                                          const double*, const double*, Arena&, cudaStream_t);
template int complete_null_columns<double>(const double*, int, double*, int64_t, int64_t,
                                           const double*, const double*, Arena&, cudaStream_t);

// ---------------------------------------------------------------------------
// Householder QR's column signs for CholeskyQR factors.  CholeskyQR gives R a
// positive diagonal; LAPACK's geqrf (the reference's qr, numpy.linalg.qr)
// chooses each reflection to avoid cancellation, so its factors are
// Q diag(s), diag(s) R for signs s that depend on the data.  s_k is minus the
// sign of the k-th pivot of the LU factorization of Q's top n x n block
// shifted by diag(s) as it is built (the sign rule of Householder
// reconstruction: Ballard, Demmel, Grigori, Jacquelin, Knight, Nguyen,
// J. Parallel Distrib. Comput. 85 (2015)); every shifted pivot is at least 1
// in magnitude, so the elimination needs no pivoting and FP32 arithmetic
// decides the signs.  For a square matrix LAPACK's last reflector is the
// identity (dlarfg of a 1-vector), so the last sign is the pivot's own.
// Right-looking, panels of HH_BW columns: one CTA eliminates a panel, a grid
// updates the trailing block with it.
// ---------------------------------------------------------------------------
constexpr int HH_BW = 32;

template <typename T>
__global__ void hh_load_kernel(const T* __restrict__ Q, int64_t ldq, int n, float* __restrict__ A) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    A[e] = (float)Q[(e / n) * ldq + e % n];
}

// columns k0 .. k0+kb-1, rows k0 .. n-1 of A (n x n, ld n): pivot signs into
// s, multipliers stored below the diagonal
__global__ void __launch_bounds__(1024) hh_panel_kernel(float* __restrict__ A, int n, int k0,
                                                        int kb, int square,
                                                        double* __restrict__ s) {
  for (int k = k0; k < k0 + kb; ++k) {
    if (threadIdx.x == 0) {
      const float p = A[(int64_t)k * n + k];
      const bool last_sq = square && k == n - 1;
      const float sk = (p >= 0.f) != last_sq ? -1.f : 1.f;
      A[(int64_t)k * n + k] = p - sk;
      s[k] = (double)sk;
    }
    __syncthreads();
    const float piv = A[(int64_t)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) {
      float* Ai = A + (int64_t)i * n;
      const float l = Ai[k] / piv;
      Ai[k] = l;
      for (int j = k + 1; j < k0 + kb; ++j) Ai[j] = fmaf(-l, A[(int64_t)k * n + j], Ai[j]);
    }
    __syncthreads();
  }
}

// trailing update after panel k0 (kb columns): for a tile of 32 columns J and
// 64 rows I past the panel, U12 = L11^-1 A[k0:k0+kb, J] (unit lower L11) and
// A[I, J] -= L21[I, :] U12.  U12 is not written back: later panels never read
// rows above them.
__global__ void __launch_bounds__(256) hh_update_kernel(float* __restrict__ A, int n, int k0,
                                                        int kb) {
  __shared__ float L11[HH_BW][HH_BW + 1];
  __shared__ float U12[HH_BW][33];
  __shared__ float L21[64][HH_BW + 1];
  const int c0 = k0 + kb + blockIdx.x * 32;
  const int r0 = k0 + kb + blockIdx.y * 64;
  const int tid = threadIdx.x;
  for (int e = tid; e < HH_BW * HH_BW; e += blockDim.x) {
    const int t = e / HH_BW, u = e % HH_BW;
    L11[t][u] = (t < kb && u < kb) ? A[(int64_t)(k0 + t) * n + k0 + u] : 0.f;
  }
  for (int e = tid; e < HH_BW * 32; e += blockDim.x) {
    const int t = e / 32, j = e % 32;
    U12[t][j] = (t < kb && c0 + j < n) ? A[(int64_t)(k0 + t) * n + c0 + j] : 0.f;
  }
  for (int e = tid; e < 64 * HH_BW; e += blockDim.x) {
    const int i = e / HH_BW, t = e % HH_BW;
    L21[i][t] = (t < kb && r0 + i < n) ? A[(int64_t)(r0 + i) * n + k0 + t] : 0.f;
  }
  __syncthreads();
  if (tid < 32) {
    for (int t = 1; t < kb; ++t) {
      float v = U12[t][tid];
      for (int u = 0; u < t; ++u) v = fmaf(-L11[t][u], U12[u][tid], v);
      U12[t][tid] = v;
    }
  }
  __syncthreads();
  const int j = tid & 31;
  if (c0 + j >= n) return;
  for (int i = tid >> 5; i < 64; i += 8) {
    if (r0 + i >= n) break;
    float acc = 0.f;
    for (int t = 0; t < kb; ++t) acc = fmaf(L21[i][t], U12[t][j], acc);
    float* a = A + (int64_t)(r0 + i) * n + c0 + j;
    *a -= acc;
  }
}

// W (n x n, ld n) <- W diag(s), R (n x n, ld n) <- diag(s) R
__global__ void sign_fold_kernel(double* __restrict__ W, double* __restrict__ R,
                                 const double* __restrict__ s, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e % n;
    if (W) W[e] *= s[j];
    if (R) R[e] *= s[i];
  }
}

template <typename T>
int householder_signs(const T* Qtop, int64_t ldq, int n, bool square, double* s, Arena& ws,
                      cudaStream_t st) {
  float* A = ws.take<float>((size_t)n * n);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "householder signs: workspace too small");
  PLOM_REQUIRE(Qtop && s && n >= 1 && ldq >= n, PLOM_ERR_ARG, "householder signs: bad arguments");
  ProfScope prof("hh_signs", st, 2.0 * n * (double)n * n / 3.0, 8.0 * n * (double)n,
                 1 + 2 * (int)cdiv(n, HH_BW));
  hh_load_kernel<T><<<grid1d((int64_t)n * n), 256, 0, st>>>(Qtop, ldq, n, A);
  PLOM_CHECK_LAUNCH();
  for (int k0 = 0; k0 < n; k0 += HH_BW) {
    const int kb = std::min(HH_BW, n - k0);
    hh_panel_kernel<<<1, 1024, 0, st>>>(A, n, k0, kb, square ? 1 : 0, s);
    PLOM_CHECK_LAUNCH();
    const int rest = n - k0 - kb;
    if (rest > 0) {
      hh_update_kernel<<<dim3((unsigned)cdiv(rest, 32), (unsigned)cdiv(rest, 64)), 256, 0, st>>>(
          A, n, k0, kb);
      PLOM_CHECK_LAUNCH();
    }
  }
  return PLOM_OK;
}
template int householder_signs<float>(const float*, int64_t, int, bool, double*, Arena&,
                                      cudaStream_t);
template int householder_signs<double>(const double*, int64_t, int, bool, double*, Arena&,
                                       cudaStream_t);

int sign_fold(double* W, double* R, const double* s, int n, cudaStream_t st) {
  if (n < 1) return PLOM_OK;
  sign_fold_kernel<<<grid1d((int64_t)n * n), 256, 0, st>>>(W, R, s, n);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

}  // namespace plom

extern "C" int plom_fill_uniform(int dtype, void* out, int64_t count, uint64_t seed,
                                 void* stream) {
  PLOM_REQUIRE(out || count == 0, PLOM_ERR_ARG, "null pointer");
  PLOM_REQUIRE(count >= 0, PLOM_ERR_ARG, "negative count");
  return plom::fill_uniform_dispatch(dtype, out, count, seed, (cudaStream_t)stream);
}
