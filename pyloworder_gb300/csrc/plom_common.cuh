// Common definitions for libplom: error state, workspace carving, launch
// helpers and small device utilities shared by every translation unit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include <stdarg.h>
#include <string.h>

#include "../../include/plom.h"

namespace plom {

// ---------------------------------------------------------------------------
// error handling: every C-ABI entry returns an int status; the message of the
// last failure on the calling host thread is kept for plom_last_error_string.
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

#define PLOM_CHECK_CUDA(expr)                                                        \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess) {                                                         \
      ::plom::set_error("%s:%d: %s -> %s", __FILE__, __LINE__, #expr,                \
                        cudaGetErrorString(_e));                                     \
      return PLOM_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)

#define PLOM_CHECK_LAUNCH() PLOM_CHECK_CUDA(cudaGetLastError())

#define PLOM_TRY(expr)                                                               \
  do {                                                                               \
    int _s = (expr);                                                                 \
    if (_s != PLOM_OK) return _s;                                                    \
  } while (0)

#define PLOM_REQUIRE(cond, code, ...)                                                \
  do {                                                                               \
    if (!(cond)) {                                                                   \
      ::plom::set_error(__VA_ARGS__);                                                \
      return (code);                                                                 \
    }                                                                                \
  } while (0)

// ---------------------------------------------------------------------------
// workspace: a caller-owned device buffer carved into aligned sub-buffers.
// Running with base == nullptr only measures (workspace queries).
// ---------------------------------------------------------------------------
struct Arena {
  char* base;
  size_t cap;
  size_t off;
  Arena(void* b, size_t c) : base(static_cast<char*>(b)), cap(c), off(0) {}
  template <typename T>
  T* take(size_t count, size_t align = 256) {
    size_t o = (off + align - 1) / align * align;
    off = o + count * sizeof(T);
    if (base == nullptr) return nullptr;
    return reinterpret_cast<T*>(base + o);
  }
  bool measuring() const { return base == nullptr; }
  bool overflow() const { return base != nullptr && off > cap; }
};

// Run-time schedule and tile parameters of the tall kernels, set through
// plom_set_tuning (the package loads them from its tuning file, written by
// pyloworder_gb300.autotune on the target GPU).  Defaults: the values tuned
// on GB300.
struct Tuning {
  int gram_wave_mult = 4;        // Gram work items per SM per wave (row-chunk granularity)
  int gram_wide_wave_mult = 32;  // the same for Grams wider than 128 columns (128 x 256 tiles)
  int reduce_blocks_per_sm = 3;  // resident blocks of the Gram slab reduction
  int apply_dense_tn = 256;      // output tile width of dense products wider than 128 (128 or 256)
  int apply_dense_by_rows = 0;   // dense products: whole row blocks per CTA (1) or single tiles (0)
  int apply_tri_by_rows = 1;     // the same for triangular W
  int pass1_chunks = 8;          // large FP32 inputs: row chunks packed beside the first Gram (1: off)
  int apply_pair = 1;            // products on SM pairs (2-SM UMMA): 0 off, 1 dense, 2 dense + triangular
};
Tuning& tuning();

inline int num_sms() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---------------------------------------------------------------------------
// per-kernel device timing (host-thread local; off unless plom_profile_begin
// was called on this thread).  A ProfScope around a launch records CUDA events
// on the launch stream and the launch's algorithmic flops and bytes.
// ---------------------------------------------------------------------------
struct ProfEntry {
  const char* name;
  cudaEvent_t a, b;
  double flops, bytes;
  int launches = 1;  // kernel launches inside the scope
};
bool prof_on();
void prof_push(const ProfEntry& e);
struct ProfScope {
  ProfEntry e;
  cudaStream_t st;
  bool on;
  ProfScope(const char* name, cudaStream_t s, double flops, double bytes, int launches = 1)
      : st(s), on(prof_on()) {
    if (!on) return;
    e.name = name;
    e.flops = flops;
    e.bytes = bytes;
    e.launches = launches;
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
    cudaEventRecord(e.a, st);
  }
  ~ProfScope() {
    if (!on) return;
    cudaEventRecord(e.b, st);
    prof_push(e);
  }
};

// status words written by kernels (device side) and read back by the host.
// Index 0: numerical failure code (0 = ok), 1: count of Cholesky shift
// escalations, 2: Jacobi sweeps of the last small SVD, 3: non-finite input seen,
// 4: FP32 Jacobi sweeps, 5: refinement steps after them, 6: Cholesky
// factorisations of a Gram next to the identity written in closed form.
enum { ST_FAIL = 0, ST_SHIFTS = 1, ST_SWEEPS = 2, ST_NONFINITE = 3, ST_SWEEPS32 = 4, ST_REFINE = 5,
       ST_NEAR = 6, ST_WORDS = 8 };

}  // namespace plom
