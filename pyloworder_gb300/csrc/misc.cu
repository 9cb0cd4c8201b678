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

}  // namespace plom

extern "C" int plom_fill_uniform(int dtype, void* out, int64_t count, uint64_t seed,
                                 void* stream) {
  PLOM_REQUIRE(out || count == 0, PLOM_ERR_ARG, "null pointer");
  PLOM_REQUIRE(count >= 0, PLOM_ERR_ARG, "negative count");
  return plom::fill_uniform_dispatch(dtype, out, count, seed, (cudaStream_t)stream);
}
