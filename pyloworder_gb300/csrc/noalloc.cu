// plom_matmulp_static: the reduction product C = A^T B of plom_matmul
// (transA = 1, FP64 accumulation) for callers that cannot allocate device
// memory -- e.g. a host integration whose device memory belongs to another
// framework's pool, or a latency-critical loop in which a cudaMalloc/cudaFree
// (which synchronise the device) is not acceptable.  Instead of a caller
// workspace, its split-K partial sums live in a fixed static device array.
//
// The array is file-scope device memory of PLOM_STATIC_SCRATCH_BYTES; every
// GPU that loads the library holds it until the process exits.  Host code
// cannot use the array's name as a device address, so the device address is
// looked up with cudaGetSymbolAddress on the first call made with a device
// current, and cached per device together with the unique ID of the context
// it belongs to (cuCtxGetId).  A device reset (cudaDeviceReset, or a reset of
// the primary context) ends that context; the library's module is loaded
// again in the next one, so a call that finds a different context ID looks
// the address up again instead of using the old one.  All calls share the
// array: calls that overlap on the GPU (other streams, other host threads)
// race on it.
#include <cuda.h>

#include <mutex>

#include "plom_common.cuh"
#include "plom_kernels.cuh"

static __device__ __align__(256) unsigned char g_plom_static_scratch[PLOM_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 128;
std::mutex g_scratch_mutex;
struct ScratchAddr {
  void* ptr = nullptr;
  unsigned long long ctx_id = 0;
};
ScratchAddr g_scratch_addr[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// unique ID of the current context (0 when it cannot be read)
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx &&
      get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// device address of the static scratch for the current device and context
// (set-up on the first call per device, again after a device reset)
int static_scratch(void** out) {
  int dev = 0;
  PLOM_CHECK_CUDA(cudaGetDevice(&dev));
  PLOM_REQUIRE(dev >= 0 && dev < kMaxDevices, PLOM_ERR_UNSUPPORTED, "device id %d out of range",
               dev);
  // no context current on this thread yet reads as ID 0: the lookup below
  // binds the device's primary context, whose ID is then recorded
  const unsigned long long id = current_ctx_id();
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  ScratchAddr& a = g_scratch_addr[dev];
  if (!a.ptr || id == 0 || a.ctx_id != id) {
    void* p = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&p, g_plom_static_scratch);
    if (rc != cudaSuccess || p == nullptr) {
      plom::set_error("plom_matmulp_static: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(rc));
      return PLOM_ERR_CUDA;
    }
    a.ptr = p;
    a.ctx_id = current_ctx_id();
  }
  *out = a.ptr;
  return PLOM_OK;
}
}  // namespace

extern "C" int plom_matmulp_static(int dtype, const void* A, int64_t lda, const void* B,
                                   int64_t ldb, void* C, int64_t ldc, int64_t m, int64_t n,
                                   int64_t k, void* stream) {
  PLOM_REQUIRE(m >= 0 && n >= 0 && k >= 0, PLOM_ERR_ARG, "plom_matmulp_static: negative size");
  PLOM_REQUIRE(lda >= m && ldb >= n && ldc >= n, PLOM_ERR_ARG,
               "plom_matmulp_static: leading dimension too small");
  PLOM_REQUIRE((A && B && C) || m * n == 0, PLOM_ERR_ARG, "plom_matmulp_static: null pointer");
  PLOM_REQUIRE(dtype == PLOM_F32 || dtype == PLOM_F64, PLOM_ERR_UNSUPPORTED,
               "plom_matmulp_static: dtype must be F32 or F64");
  if (m == 0 || n == 0) return PLOM_OK;
  void* scratch = nullptr;
  PLOM_TRY(static_scratch(&scratch));
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == PLOM_F32)
    return plom::gemm_tn_in_scratch<float, float, float>(
        (const float*)A, lda, (const float*)B, ldb, (float*)C, ldc, m, n, k, scratch,
        PLOM_STATIC_SCRATCH_BYTES, st);
  return plom::gemm_tn_in_scratch<double, double, double>(
      (const double*)A, lda, (const double*)B, ldb, (double*)C, ldc, m, n, k, scratch,
      PLOM_STATIC_SCRATCH_BYTES, st);
}
