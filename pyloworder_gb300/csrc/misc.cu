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

// sums[q] += m_c^T G m_c over the 32 rows k of this block (c = list[q])
__global__ void __launch_bounds__(256) nc_norms_kernel(const double* __restrict__ G,
                                                       const double* __restrict__ Mf, int N,
                                                       const int* __restrict__ list,
                                                       const int* __restrict__ count,
                                                       double* __restrict__ sums) {
  const int q = blockIdx.y;
  if (q >= *count) return;
  const int c = list[q];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double part = 0.0;
  for (int k = blockIdx.x * 32 + wib; k < min(N, (int)blockIdx.x * 32 + 32); k += 8) {
    double acc = 0.0;
    for (int l = lane; l < N; l += 32) acc = fma(G[(int64_t)k * N + l], Mf[(int64_t)l * N + c], acc);
    acc = warp_sum(acc);
    part = fma(Mf[(int64_t)k * N + c], acc, part);
  }
  if (lane == 0) atomicAdd(&sums[q], part);
}

__device__ __forceinline__ int64_t nc_row(int q, int64_t m) {
  return (int64_t)(((uint64_t)(q + 1) * 2654435761ull) % (uint64_t)m);
}

// u = e_i - U w, w = row i of U without the columns still to be completed
// (this one included); written into column list[q], its squared norm summed
template <typename T>
__global__ void __launch_bounds__(256) nc_project_kernel(T* __restrict__ U, int64_t m, int n,
                                                         int64_t ldu, const int* __restrict__ list,
                                                         const int* __restrict__ count,
                                                         const double* __restrict__ sums, int q,
                                                         double* __restrict__ nrm2) {
  if (q >= *count || !(sums[q] < 0.25)) return;
  extern __shared__ double ncw[];
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
  double part = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * 8 + wib; r < m; r += (int64_t)gridDim.x * 8) {
    const T* row = U + r * ldu;
    double acc = 0.0;
    for (int j = lane; j < n; j += 32) acc = fma((double)row[j], ncw[j], acc);
    acc = warp_sum(acc);
    const double u = (r == i ? 1.0 : 0.0) - acc;
    if (lane == 0) {
      U[r * ldu + c] = (T)u;
      part = fma(u, u, part);
    }
  }
  __syncwarp();
  if (lane == 0) atomicAdd(&nrm2[q], part);
}

template <typename T>
__global__ void __launch_bounds__(256) nc_scale_kernel(T* __restrict__ U, int64_t m, int64_t ldu,
                                                       const int* __restrict__ list,
                                                       const int* __restrict__ count,
                                                       const double* __restrict__ sums, int q,
                                                       const double* __restrict__ nrm2) {
  if (q >= *count || !(sums[q] < 0.25) || !(nrm2[q] > 0.0)) return;
  const int c = list[q];
  const double f = 1.0 / sqrt(nrm2[q]);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x)
    U[r * ldu + c] = (T)((double)U[r * ldu + c] * f);
}

template <typename T>
int complete_null_columns(const double* S, int n, T* U, int64_t m, int64_t ldu, const double* G,
                          const double* Mf, Arena& ws, cudaStream_t st) {
  int* list = ws.take<int>(NC_MAX);
  int* count = ws.take<int>(1);
  double* sums = ws.take<double>(NC_MAX);
  double* nrm2 = ws.take<double>(NC_MAX);
  if (ws.measuring() || n < 1 || m < 1) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "null-column completion: workspace too small");
  PLOM_REQUIRE(S && U && G && Mf && n <= 8192, PLOM_ERR_ARG,
               "null-column completion: bad arguments");
  ProfScope prof("null_cols", st, 0.0, (double)sizeof(T) * m, 2 + 2 * NC_MAX);
  PLOM_CHECK_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * NC_MAX, st));
  PLOM_CHECK_CUDA(cudaMemsetAsync(nrm2, 0, sizeof(double) * NC_MAX, st));
  nc_candidates_kernel<<<1, 32, 0, st>>>(S, n, list, count);
  PLOM_CHECK_LAUNCH();
  const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(m, 256), (int64_t)num_sms() * 4));
  nc_norms_kernel<<<dim3((unsigned)cdiv(n, 32), NC_MAX), 256, 0, st>>>(G, Mf, n, list, count,
                                                                      sums);
  PLOM_CHECK_LAUNCH();
  const unsigned gp = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(m, 8), (int64_t)num_sms() * 8));
  for (int q = 0; q < NC_MAX; ++q) {
    nc_project_kernel<T><<<gp, 256, sizeof(double) * n, st>>>(U, m, n, ldu, list, count, sums, q,
                                                              nrm2);
    PLOM_CHECK_LAUNCH();
    nc_scale_kernel<T><<<gx, 256, 0, st>>>(U, m, ldu, list, count, sums, q, nrm2);
    PLOM_CHECK_LAUNCH();
  }
  return PLOM_OK;
}
template int complete_null_columns<float>(const double*, int, float*, int64_t, int64_t,
                                          const double*, const double*, Arena&, cudaStream_t);
template int complete_null_columns<double>(const double*, int, double*, int64_t, int64_t,
                                           const double*, const double*, Arena&, cudaStream_t);

}  // namespace plom

extern "C" int plom_fill_uniform(int dtype, void* out, int64_t count, uint64_t seed,
                                 void* stream) {
  PLOM_REQUIRE(out || count == 0, PLOM_ERR_ARG, "null pointer");
  PLOM_REQUIRE(count >= 0, PLOM_ERR_ARG, "negative count");
  return plom::fill_uniform_dispatch(dtype, out, count, seed, (cudaStream_t)stream);
}
