// Tensor-core (tcgen05, sm_103a) tall products of the mixed form on
// "fp16 pairs".
//
// A tall FP32 operand Y (m x N) is packed once into two fp16 planes,
//     hi = fp16(y s_j),  lo = fp16(y s_j - hi),
// with a power-of-two scale s_j per column (max |y s_j| in [2^13, 2^14)), so
// hi + lo carries 22 significant bits of y s_j.  Products run on the f16
// tensor pipe (kind::f16, FP32 accumulation in TMEM) as hi*hi + hi*lo + lo*hi
// (the dropped lo*lo term is below 2^-22 |x y|), at twice the rate of TF32
// and with half the operand bytes.  Both planes are row-major m x ldp
// (ldp = N rounded up to 64; padding columns are zero), which serves both
// products without a transpose:
//
//  gram_packed  G (N x N, FP64) = Y^T Y over the m rows.  Upper 128 x 128
//               tiles x row chunks; operands are MN-major 128-byte-swizzled
//               tiles straight from TMA (the row-major planes are MN-major for
//               Y^T Y).  Every 4096 rows the FP32 TMEM accumulators (hi*hi and
//               the correction terms kept apart) are drained into an FP64
//               partial, and the diagonal of a diagonal tile (sums of squares,
//               where the FP32 accumulation bias does not cancel) is summed
//               on the CUDA cores with compensated FP32 sums folded into FP64.
//               Partials are summed in FP64 in a fixed order.
//  apply_packed C (m x k) = Y W for a small FP64 W: the row-major planes are
//               the K-major A operand; W is scaled per column and split into
//               K-major fp16 hi/lo copies once.  The epilogue writes FP32 C or
//               the packed planes of C (scale 2^14), ready for the next
//               product.  Persistent CTAs; two TMEM accumulator buffers so the
//               epilogue of one tile overlaps the products of the next.
//
// Every mbarrier wait is bounded (%globaltimer, 2 s); on expiry the CTA
// records PLOM_NUM_TIMEOUT in the caller's info word, stops issuing work,
// frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>

#include "plom_common.cuh"
#include "plom_kernels.cuh"
#include "plom_tc.cuh"

namespace plom {
namespace hp {

constexpr uint64_t WAIT_NS = 2000000000ull;
constexpr int PK_LOG2 = 14;  // packed values: max |y s| in [2^13, 2^14)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait.  False (and the CTA abort flag raised) on expiry, or when
// another role of the CTA or another CTA of the launch already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  uint32_t spins = 0;
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if ((++spins & 1023u) == 0 && err && *(volatile int*)err == PLOM_NUM_TIMEOUT) {
      *abort_flag = 1;
      return false;
    }
    if (gtimer() - t0 > WAIT_NS) {
      *abort_flag = 1;
      if (err) atomicMax(err, PLOM_NUM_TIMEOUT);
      return false;
    }
  }
}
__device__ __forceinline__ bool launch_aborted(const int* err) {
  return err && *(volatile const int*)err == PLOM_NUM_TIMEOUT;
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
// 32 lanes x 32 consecutive 32-bit columns; thread i of the warp gets lane
// (32 * (warp % 4) + i) of the addressed quarter.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
// 32 lanes x 16 consecutive 32-bit columns
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// 3-D tiled TMA load (plane z of the packed planes).  x is a multiple of 64
// fp16 (128 bytes) at every call site.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Shared-memory matrix descriptor, 128-byte swizzle, sm_100 version 1.
//  K-major tiles: 8-row core groups 1024 bytes apart (SBO), LBO unused.
//  MN-major tiles: 64-element swizzle atoms LBO bytes apart along M/N, 8-row
//  K groups 1024 bytes apart (SBO).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// K-major tile of rows of `bk` fp16 (bk = 64: 128-byte rows, 128-byte swizzle;
// bk = 32: 64-byte rows, 64-byte swizzle), 8-row core groups 8 * 2 bk bytes
// apart (SBO); layout type 2 = SWIZZLE_128B, 4 = SWIZZLE_64B
template <int BK>
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr) {
  static_assert(BK == 64 || BK == 32, "stage depth");
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;  // LBO (unused for swizzled K-major tiles)
  d |= (uint64_t)(((16u * BK) >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)(BK == 64 ? 2 : 4) << 61;
  return d;
}
// Instruction descriptor: kind::f16, D = F32, A = B = F16; a_mn/b_mn select
// MN-major operands.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, int a_mn, int b_mn) {
  return (1u << 4) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint16_t ld_shared_u16(uint32_t addr) {
  uint16_t v;
  asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ float2 ld_shared_h2f(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
  __half2 h;
  memcpy(&h, &v, sizeof(h));
  return __half22float2(h);
}

// ---------------------------------------------------------------------------
// packing
// ---------------------------------------------------------------------------
// column maxima of |Y| (bits of non-negative floats order like unsigned ints);
// each block takes a contiguous range of rows, threads take 4-column groups
// (16-byte loads when rows are aligned)
__global__ void __launch_bounds__(256) colmax_kernel(const float* __restrict__ Y, int64_t ld,
                                                     int64_t m, int N, int vec, int64_t bstride,
                                                     unsigned* __restrict__ cmax) {
  // problem blockIdx.y of a batch (matrices bstride elements apart)
  Y += (int64_t)blockIdx.y * bstride;
  cmax += (int64_t)blockIdx.y * N;
  const int64_t rows = (m + gridDim.x - 1) / gridDim.x;
  const int64_t r0b = (int64_t)blockIdx.x * rows;
  const int64_t r1 = (r0b + rows < m) ? r0b + rows : m;
  // narrow matrices: the block's threads split into (row lane, column group)
  // so that all of them read; rows r0b + tr, r0b + tr + TR, ...
  const int groups = vec ? N / 4 : N;
  const int TR = groups >= (int)blockDim.x ? 1 : (int)blockDim.x / groups;
  const int tr = (int)threadIdx.x / (groups >= (int)blockDim.x ? (int)blockDim.x : groups);
  const int tc = (int)threadIdx.x - tr * (groups >= (int)blockDim.x ? (int)blockDim.x : groups);
  if (tr >= TR) return;
  const int cstep = groups >= (int)blockDim.x ? (int)blockDim.x : groups;
  const int64_t r0 = r0b + tr;
  if (vec) {
    for (int c = tc * 4; c < N; c += cstep * 4) {
      float4 mx = make_float4(0.f, 0.f, 0.f, 0.f);
      const float* p = Y + r0 * ld + c;
#pragma unroll 8
      for (int64_t r = r0; r < r1; r += TR, p += TR * ld) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(p));
        mx.x = fmaxf(mx.x, fabsf(v.x));
        mx.y = fmaxf(mx.y, fabsf(v.y));
        mx.z = fmaxf(mx.z, fabsf(v.z));
        mx.w = fmaxf(mx.w, fabsf(v.w));
      }
      if (mx.x > 0.f) atomicMax(&cmax[c], __float_as_uint(mx.x));
      if (mx.y > 0.f) atomicMax(&cmax[c + 1], __float_as_uint(mx.y));
      if (mx.z > 0.f) atomicMax(&cmax[c + 2], __float_as_uint(mx.z));
      if (mx.w > 0.f) atomicMax(&cmax[c + 3], __float_as_uint(mx.w));
    }
  } else {
    for (int c = tc; c < N; c += cstep) {
      float mx = 0.f;
      const float* p = Y + r0 * ld + c;
#pragma unroll 8
      for (int64_t r = r0; r < r1; r += TR, p += TR * ld) mx = fmaxf(mx, fabsf(__ldg(p)));
      if (mx > 0.f) atomicMax(&cmax[c], __float_as_uint(mx));
    }
  }
}

// s_j = 2^(14 - e_j) with max_j = f 2^e_j, f in [0.5, 1); 1 for zero or
// padding columns (clamped so that s_j stays a finite float)
__global__ void colscale_kernel(const unsigned* __restrict__ cmax, int N, int ldp, int batch,
                                float* __restrict__ s) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)batch * ldp;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pb = e / ldp;
    const int j = (int)(e - pb * ldp);
    const float v = (j < N) ? __uint_as_float(cmax[pb * N + j]) : 0.f;
    int ex = 0;
    frexpf(v, &ex);
    ex = ex < -100 ? -100 : ex;
    s[e] = (v > 0.f) ? ldexpf(1.f, PK_LOG2 - ex) : 1.f;
  }
}

__global__ void fill_scale_kernel(float* __restrict__ s, int64_t count, float v) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count;
       j += (int64_t)gridDim.x * blockDim.x)
    s[j] = v;
}

__device__ __forceinline__ void split8(const float (&v)[8], uint4& h, uint4& l) {
  uint32_t hw[4], lw[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const __half h0 = __float2half_rn(v[2 * q]), h1 = __float2half_rn(v[2 * q + 1]);
    const __half l0 = __float2half_rn(v[2 * q] - __half2float(h0));
    const __half l1 = __float2half_rn(v[2 * q + 1] - __half2float(h1));
    hw[q] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
    lw[q] = (uint32_t)__half_as_ushort(l0) | ((uint32_t)__half_as_ushort(l1) << 16);
  }
  h = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  l = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// hi/lo planes (mp x ldp per problem) of Y diag(s); columns N..ldp-1 and
// rows m..mp-1 are zero.  Blocks take tiles of `rt` rows of one problem;
// threads take 8-column groups of a tile.
__global__ void __launch_bounds__(256) pack_kernel(const float* __restrict__ Y, int64_t ld,
                                                   int64_t m, int N, int ldp, int rt,
                                                   const float* __restrict__ s,
                                                   __half* __restrict__ hi,
                                                   __half* __restrict__ lo, int vec,
                                                   int64_t bstride, int64_t mp, int batch) {
  const int groups = ldp / 8;
  const int64_t tpp = (mp + rt - 1) / rt;  // tiles per problem
  for (int64_t tile = blockIdx.x; tile < tpp * batch; tile += gridDim.x) {
    const int64_t pb = tile / tpp;
    const int64_t r0 = (tile - pb * tpp) * rt;
    const int nr = (int)((mp - r0 < rt) ? mp - r0 : rt);
    const int items = nr * groups;
    const float* Yp = Y + pb * bstride;
    const float* sp = s + pb * ldp;
#pragma unroll 2
    for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
      const int rr = idx / groups;
      const int c0 = (idx - rr * groups) * 8;
      const int64_t r = r0 + rr;
      const float* src = Yp + r * ld + c0;
      float v[8];
      if (r >= m) {
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = 0.f;
      } else if (vec && c0 + 8 <= N) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(src));
        const float4 b = __ldg(reinterpret_cast<const float4*>(src + 4));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = (c0 + q < N) ? src[q] : 0.f;
      }
      const float4 s0 = __ldg(reinterpret_cast<const float4*>(sp + c0));
      const float4 s1 = __ldg(reinterpret_cast<const float4*>(sp + c0 + 4));
      v[0] *= s0.x; v[1] *= s0.y; v[2] *= s0.z; v[3] *= s0.w;
      v[4] *= s1.x; v[5] *= s1.y; v[6] *= s1.z; v[7] *= s1.w;
      uint4 h, l;
      split8(v, h, l);
      const int64_t ro = pb * mp + r;
      *reinterpret_cast<uint4*>(hi + ro * ldp + c0) = h;
      *reinterpret_cast<uint4*>(lo + ro * ldp + c0) = l;
    }
  }
}

// W (nin x k, FP64, ldw) -> Bt hi/lo (k rows x ldk, K-major fp16) of
// diag(1/s_in) W diag(t) with t_j a power of two (max |.| in [2^13, 2^14)),
// and the epilogue factor f_j = out_scale / t_j.  One block per column j of
// W; blocks j >= k write f_j = 0 (their Bt rows are never read).
__global__ void __launch_bounds__(256) split_w16_kernel(const double* __restrict__ W,
                                                        int64_t ldw, int nin, int k, int ldk,
                                                        const float* __restrict__ s_in,
                                                        float out_scale, __half* __restrict__ bhi,
                                                        __half* __restrict__ blo,
                                                        float* __restrict__ f, int64_t wstride,
                                                        int fstride) {
  __shared__ double red[8];
  // problem blockIdx.y of a batch: W_p, its input scales, its rows of Bt, its factors
  {
    const int64_t pb = blockIdx.y;
    W += pb * wstride;
    s_in += pb * ldk;
    bhi += pb * k * (int64_t)ldk;
    blo += pb * k * (int64_t)ldk;
    f += pb * fstride;
  }
  const int j = blockIdx.x;
  if (j >= k) {
    if (threadIdx.x == 0) f[j] = 0.f;
    return;
  }
  // 1 / s_in is exact (powers of two)
  double mx = 0.0;
  for (int i = threadIdx.x; i < nin; i += blockDim.x)
    mx = fmax(mx, fabs(W[(int64_t)i * ldw + j] * (double)(1.0f / s_in[i])));
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  mx = 0.0;
  for (int w = 0; w < 8; ++w) mx = fmax(mx, red[w]);
  int e = 0;
  frexp(mx, &e);
  e = e < -900 ? -900 : (e > 900 ? 900 : e);
  const double t = (mx > 0.0) ? ldexp(1.0, PK_LOG2 - e) : 1.0;
  for (int i = threadIdx.x; i < ldk; i += blockDim.x) {
    const float x = (i < nin) ? (float)(W[(int64_t)i * ldw + j] * (double)(1.0f / s_in[i]) * t) : 0.f;
    const __half h = __float2half_rn(x);
    const __half l = __float2half_rn(x - __half2float(h));
    bhi[(int64_t)j * ldk + i] = h;
    blo[(int64_t)j * ldk + i] = l;
  }
  if (threadIdx.x == 0) f[j] = (float)((double)out_scale / t);
}

// ---------------------------------------------------------------------------
// gram: upper 128 x 128 tiles x row chunks, MN-major operands from TMA
// ---------------------------------------------------------------------------
#ifndef PLOM_GRAM_BK
#define PLOM_GRAM_BK 64
#endif
#ifndef PLOM_GRAM_KSUB
#define PLOM_GRAM_KSUB 4096
#endif
// row chunks of the Gram: the fewest whole waves of CTAs that split evenly
// into tiles, times this factor (shorter chunks keep the tiles that share a
// row panel closer together in time, so more of the panel re-reads hit L2)

constexpr int G_BK = PLOM_GRAM_BK;             // rows per stage (a multiple of 16)
constexpr uint32_t G_BOX = G_BK * 128;         // G_BK rows x 64 fp16
constexpr uint32_t G_TILE = 2 * G_BOX;         // G_BK rows x 128 columns of one plane
constexpr uint32_t G_STAGE = 4 * G_TILE;       // A hi, A lo, B hi, B lo
constexpr int G_STAGES = (3 * 64) / G_BK;      // 192 KiB of stages
static_assert(G_BK % 16 == 0 && G_BK >= 16 && G_BK <= 64, "stage rows");
// Rows accumulated in TMEM (FP32) before the FP64 drain (4,096 rows: 256 UMMA
// of K = 16 per accumulator).
constexpr int G_KSUB = PLOM_GRAM_KSUB;
static_assert(G_KSUB % G_BK == 0, "drain on stage boundaries");
constexpr size_t G_SMEM = (size_t)G_STAGES * G_STAGE + 1024;
constexpr uint32_t G_TMEM = 512;               // 2 buffers x (main 128 + correction 128)

// Double-float (unevaluated sum of two FP32 numbers, ~48 bits) for the Gram's
// partial sums: GB300 runs FP64 at 1/64 of its FP32 rate, and the drains of
// the TMEM accumulators and the reduction of the partials would otherwise be
// FP64-bound.  TwoSum / Fast2Sum (Knuth, Dekker) and the accurate
// double-word addition of Joldes, Muller and Popescu (ACM TOMS 44, 2017,
// Algorithm 6; relative error below 3 u^2).
__device__ __forceinline__ float2 dw_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 dw_fast_two_sum(float a, float b) {
  const float s = a + b;
  return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 dw_add(float2 x, float2 y) {
  const float2 s = dw_two_sum(x.x, y.x);
  const float2 t = dw_two_sum(x.y, y.y);
  const float2 v = dw_fast_two_sum(s.x, s.y + t.x);
  return dw_fast_two_sum(v.x, t.y + v.y);
}
// x + y for a double-float x and an FP32 y
__device__ __forceinline__ float2 dw_add_f(float2 x, float y) {
  const float2 s = dw_two_sum(x.x, y);
  return dw_fast_two_sum(s.x, s.y + x.y);
}
__device__ __forceinline__ float2 dw_from_double(double d) {
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}
__device__ __forceinline__ double dw_value(float2 v) { return (double)v.x + (double)v.y; }

// SYM: upper tiles of A^T A (tmB unused) with the exact diagonal on diagonal
// tiles; otherwise every tile of A^T B (tna x tnb tiles, B from tmB).  The
// partial of a work item is 128 x 128 double-float values (8 bytes each).
template <bool SYM>
__global__ void __launch_bounds__(320, 1)
    gram16_kernel(const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmB,
                  int64_t m, int tn, int tnb, int64_t rows_per_chunk, int chunks,
                  double* __restrict__ part, int* err, int64_t mp) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[G_STAGES], empty_bar[G_STAGES];
  __shared__ uint64_t tfull[2], tempty[2], dfull[2];
  __shared__ double diag_sh[2][2][128];  // [buffer][row half][column]
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // consecutive CTAs take different tiles of the same row chunk, so the CTAs
  // resident together read the same rows and share them through L2
  // work item -> (problem of the batch, row chunk, tile); the problems' rows
  // are mp apart in the planes
  const int ntiles = SYM ? tn * (tn + 1) / 2 : tn * tnb;
  const int per_problem = ntiles * chunks;
  const int pb = (int)(blockIdx.x / per_problem);
  const int rem_item = (int)(blockIdx.x % per_problem);
  const int chunk = rem_item / ntiles, tile = rem_item % ntiles;
  const int item = (pb * ntiles + tile) * chunks + chunk;  // partial slab index (tile-major)
  int ti = 0, tj = 0;
  if (SYM) {
    int rem = tile;
    while (rem >= tn - ti) {
      rem -= tn - ti;
      ++ti;
    }
    tj = ti + rem;
  } else {
    ti = tile / tnb;
    tj = tile % tnb;
  }
  const bool diag = SYM && (ti == tj);
  const int I0 = ti * 128, J0 = tj * 128;
  const int64_t r_beg = (int64_t)chunk * rows_per_chunk;
  const int64_t r_end = (r_beg + rows_per_chunk < m) ? r_beg + rows_per_chunk : m;
  const int64_t nrows = (r_end > r_beg) ? r_end - r_beg : 0;
  const int KB = (int)((nrows + G_BK - 1) / G_BK);
  constexpr int KB_PER_SUB = G_KSUB / G_BK;
  const int nsub = (KB + KB_PER_SUB - 1) / KB_PER_SUB;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < G_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], diag ? 1 + 128 : 1);  // MMA commit (+ diagonal warps)
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 128);
      mbar_init(&dfull[b], 128);
    }
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == 8) {
    tmem_alloc(&tmem_sh, G_TMEM);
    tmem_relinquish();
  }
  if (warp == 9 && lane == 0) {
    tma_prefetch_map(&tmP);
    if (!SYM) tma_prefetch_map(&tmB);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;
  float2* P = reinterpret_cast<float2*>(part) + (int64_t)item * 128 * 128;

  if (warp == 9) {
    // ---- TMA producer: 64 rows x (I block [+ J block]) of both planes
    if (lane == 0) {
      const uint32_t bytes = (diag ? 2u : 4u) * G_TILE;
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % G_STAGES;
        const uint32_t ph = (uint32_t)(kb / G_STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) break;
        const uint32_t st = base + s * G_STAGE;
        const int y = (int)((int64_t)pb * mp + r_beg + (int64_t)kb * G_BK);
        mbar_expect_tx(&full_bar[s], bytes);
#pragma unroll
        for (int z = 0; z < 2; ++z) {
          tma_load_3d(st + z * G_TILE, &tmP, I0, y, z, &full_bar[s]);
          tma_load_3d(st + z * G_TILE + G_BOX, &tmP, I0 + 64, y, z, &full_bar[s]);
          if (!diag) {
            const CUtensorMap* mb = SYM ? &tmP : &tmB;
            tma_load_3d(st + (2 + z) * G_TILE, mb, J0, y, z, &full_bar[s]);
            tma_load_3d(st + (2 + z) * G_TILE + G_BOX, mb, J0 + 64, y, z, &full_bar[s]);
          }
        }
      }
    }
  } else if (warp >= 4 && warp < 8) {
    // ---- diagonal tiles: compensated sums of (hi + lo)^2 per column.  A
    // thread takes two adjacent columns (one 32-bit shared load per plane and
    // row) over one half of each stage's rows, even and odd rows in separate
    // chains: four independent compensated chains per thread, so the
    // diagonal keeps pace with the MMA
    if (diag) {
      const int t = threadIdx.x - 128;
      const int c = 2 * (t & 63);                // first of the two columns
      const int h = t >> 6;                      // row half of each stage
      const uint32_t cb = (uint32_t)(c >> 6) * G_BOX;
      const uint32_t w = (uint32_t)(c & 63);
      const uint32_t ch = w >> 3, within = (w & 7u) * 2u;
      const uint32_t k0 = (uint32_t)h * (G_BK / 2), k1 = k0 + G_BK / 2;
      // chains: [column][row parity]
      float sm[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, cp[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % G_STAGES;
        const uint32_t ph = (uint32_t)(kb / G_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) break;
        const uint32_t st = base + s * G_STAGE + cb;
#pragma unroll 4
        for (uint32_t k = k0; k < k1; k += 2) {
#pragma unroll
          for (uint32_t u = 0; u < 2; ++u) {
            const uint32_t kk = k + u;
            const uint32_t off = (kk >> 3) * 1024u + (kk & 7u) * 128u + (((ch ^ (kk & 7u)) << 4) | within);
            const float2 hv = ld_shared_h2f(st + off);
            const float2 lv = ld_shared_h2f(st + G_TILE + off);
            const float v[2] = {hv.x + lv.x, hv.y + lv.y};  // exact: 22 bits
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const float y = fmaf(v[q], v[q], -cp[q][u]);
              const float tt = sm[q][u] + y;
              cp[q][u] = (tt - sm[q][u]) - y;
              sm[q][u] = tt;
            }
          }
        }
        mbar_arrive(&empty_bar[s]);
        if ((kb % KB_PER_SUB) == KB_PER_SUB - 1 || kb == KB - 1) {
          const int b = (kb / KB_PER_SUB) & 1;
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            diag_sh[b][h][c + q] = ((double)sm[q][0] - (double)cp[q][0]) +
                                   ((double)sm[q][1] - (double)cp[q][1]);
            sm[q][0] = sm[q][1] = cp[q][0] = cp[q][1] = 0.f;
          }
          mbar_arrive(&dfull[b]);
        }
      }
    }
  } else if (warp == 8 && lane == 0) {
    // ---- UMMA issuer: main += hi*hi, correction += hi*lo + lo*hi
    constexpr uint32_t idesc = idesc_f16(128, 128, 1, 1);
    bool ok = true;
    int kb = 0;
    for (int sub = 0; sub < nsub && ok; ++sub) {
      const int b = sub & 1;
      if (!mbar_wait(&tempty[b], (((uint32_t)sub >> 1) & 1u) ^ 1u, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t dmain = tmem + (uint32_t)(b * 256);
      const uint32_t dcorr = dmain + 128u;
      const int kb_end = (kb + KB_PER_SUB < KB) ? kb + KB_PER_SUB : KB;
      for (int kl = 0; kb < kb_end; ++kb, ++kl) {
        const int s = kb % G_STAGES;
        const uint32_t ph = (uint32_t)(kb / G_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t st = base + s * G_STAGE;
        const uint32_t aH = st, aL = st + G_TILE;
        const uint32_t bH = diag ? aH : st + 2 * G_TILE, bL = diag ? aL : st + 3 * G_TILE;
#pragma unroll
        for (int kk = 0; kk < G_BK / 16; ++kk) {
          const uint32_t adv = (uint32_t)kk * 2048u;  // 16 rows of 128 bytes
          const uint64_t dAH = desc_sw128(aH + adv, G_BOX, 1024), dAL = desc_sw128(aL + adv, G_BOX, 1024);
          const uint64_t dBH = desc_sw128(bH + adv, G_BOX, 1024), dBL = desc_sw128(bL + adv, G_BOX, 1024);
          const uint32_t first = (kl > 0 || kk > 0) ? 1u : 0u;
          mma_f16(dmain, dAH, dBH, idesc, first);
          mma_f16(dcorr, dAH, dBL, idesc, first);
          mma_f16(dcorr, dAL, dBH, idesc, 1u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (ok) mma_commit(&tfull[b]);
    }
  } else if (warp < 4) {
    // ---- epilogue: drain each finished sub-chunk into the double-float partial
    const int rloc = warp * 32 + lane;
    for (int sub = 0; sub < nsub; ++sub) {
      const int b = sub & 1;
      const uint32_t par = ((uint32_t)sub >> 1) & 1u;
      bool ready = mbar_wait(&tfull[b], par, &abort_sh, err);
      if (diag) ready = ready && mbar_wait(&dfull[b], par, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      const float2 dval =
          diag ? dw_from_double(diag_sh[b][0][rloc] + diag_sh[b][1][rloc]) : make_float2(0.f, 0.f);
      float2* prow = P + (int64_t)rloc * 128;
#pragma unroll 1
      for (int cc = 0; cc < 4; ++cc) {
        uint32_t rm[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * 256 + cc * 32);
        tmem_ld32(ta, rm);
        tmem_ld32(ta + 128, rc);
        tmem_wait_ld();
        float2* d = prow + cc * 32;
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          // main + correction exactly, as a double-float pair
          float2 v0 = dw_two_sum(__uint_as_float(rm[j]), __uint_as_float(rc[j]));
          float2 v1 = dw_two_sum(__uint_as_float(rm[j + 1]), __uint_as_float(rc[j + 1]));
          if (diag && cc * 32 + j == rloc) v0 = dval;
          if (diag && cc * 32 + j + 1 == rloc) v1 = dval;
          float4* q = reinterpret_cast<float4*>(d + j);
          if (sub == 0) {
            *q = make_float4(v0.x, v0.y, v1.x, v1.y);
          } else {
            const float4 o = *q;
            const float2 a0 = dw_add(make_float2(o.x, o.y), v0);
            const float2 a1 = dw_add(make_float2(o.z, o.w), v1);
            *q = make_float4(a0.x, a0.y, a1.x, a1.y);
          }
        }
      }
      fence_before();
      mbar_arrive(&tempty[b]);
    }
    if (nsub == 0) {  // empty chunk: the partial is zero
      float2* prow = P + (int64_t)rloc * 128;
      for (int j = 0; j < 128; ++j) prow[j] = make_float2(0.f, 0.f);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 8) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, G_TMEM);
  }
}

// C[i][j] (Na x Nb, ldc) = sum over chunks of the tile partials / (sA_i sB_j)
__global__ void tn16_reduce_kernel(const double* __restrict__ part, int Na, int Nb, int tnb,
                                   int chunks, const float* __restrict__ sa,
                                   const float* __restrict__ sb, double* __restrict__ C,
                                   int64_t ldc) {
  const int64_t total = (int64_t)Na * Nb;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / Nb), j = (int)(e % Nb);
    const int ti = i / 128, tj = j / 128;
    const int tile = ti * tnb + tj;
    const float2* p = reinterpret_cast<const float2*>(part) + ((int64_t)tile * chunks) * 128 * 128 +
                      (int64_t)(i - ti * 128) * 128 + (j - tj * 128);
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < chunks; ++c) acc = dw_add(acc, p[(int64_t)c * 128 * 128]);
    C[(int64_t)i * ldc + j] = dw_value(acc) / ((double)sa[i] * (double)sb[j]);
  }
}

// G[i][j] = sum over chunks of the tile partials (fixed order) / (s_i s_j), mirrored
__global__ void gram16_reduce_kernel(const double* __restrict__ part, int N, int tn, int chunks,
                                     const float* __restrict__ s, double* __restrict__ G,
                                     int batch, int ld, int accumulate) {
  const int64_t total = (int64_t)N * N * batch;
  const int ntiles = tn * (tn + 1) / 2;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pb = e / ((int64_t)N * N);
    const int64_t r = e - pb * N * N;
    const int i = (int)(r / N), j = (int)(r % N);
    int a = i, b = j;
    if (a / 128 > b / 128) {
      a = j;
      b = i;
    }
    const int ti = a / 128, tj = b / 128;
    const int tile = ti * tn - ti * (ti - 1) / 2 + (tj - ti);
    const float2* p = reinterpret_cast<const float2*>(part) +
                      ((pb * ntiles + tile) * chunks) * 128 * 128 + (int64_t)(a - ti * 128) * 128 +
                      (b - tj * 128);
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < chunks; ++c) acc = dw_add(acc, p[(int64_t)c * 128 * 128]);
    const float* sp = s + pb * ld;
    const double v = dw_value(acc) / ((double)sp[i] * (double)sp[j]);
    G[e] = accumulate ? G[e] + v : v;
  }
}

// ---------------------------------------------------------------------------
// wide gram: 128 x 256 tiles (one 128 x 256 x 16 UMMA per product), for
// operands wider than 128 columns.  The 256-wide UMMA keeps the tensor pipe
// busy through the stage ring (see ApplyCfg) and the A panel is received once
// per 256 output columns instead of once per 128.  Stages of 32 rows (48 KiB,
// four of them); the two accumulators (main 256 + correction 256 columns) fill
// TMEM, so a sub-chunk's drain holds the next sub-chunk's products: the drain
// only reads TMEM and writes (no read-modify-write of a running partial).
// SYM tiles: for each 128-column block I of A and 256-column block J of B with
// J + 256 > I (the tiles that meet the upper triangle); where I lies inside J
// (the band tiles) A is the middle or first half of B and is not loaded, and
// the Gram diagonal is summed on the CUDA cores as in gram16_kernel.
// ---------------------------------------------------------------------------
constexpr int GW_BK = 32;                      // rows per stage
constexpr uint32_t GW_BOX = GW_BK * 128;       // GW_BK rows x 64 fp16
constexpr uint32_t GW_STAGE = 12 * GW_BOX;     // A hi/lo (2 boxes each), B hi/lo (4 each)
constexpr int GW_STAGES = 4;
constexpr size_t GW_SMEM = (size_t)GW_STAGES * GW_STAGE + 1024;
static_assert(G_KSUB % GW_BK == 0, "drain on stage boundaries");

// SYM tile index -> (ti, tj): ti-major, tj from ti / 2 to tn2 - 1
__host__ __device__ inline void gw_tile_sym(int tile, int tn2, int& ti, int& tj) {
  int rem = tile, t = 0;
  while (rem >= tn2 - (t >> 1)) {
    rem -= tn2 - (t >> 1);
    ++t;
  }
  ti = t;
  tj = (t >> 1) + rem;
}
__host__ __device__ inline int gw_tiles_sym(int tn, int tn2) {
  int c = 0;
  for (int t = 0; t < tn; ++t) c += tn2 - (t >> 1);
  return c;
}

template <bool SYM>
__global__ void __launch_bounds__(320, 1)
    gram16w_kernel(const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmB,
                   int64_t m, int tn, int tn2, int64_t rows_per_chunk, int chunks,
                   int subs_per_chunk, int nsubs, float* __restrict__ part,
                   double* __restrict__ diagp, int* err, int64_t mp, int64_t slab_off) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[GW_STAGES], empty_bar[GW_STAGES];
  __shared__ uint64_t tfull, tempty, dfull[2];
  __shared__ double diag_sh[2][2][128];  // [buffer][row half][column]
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // work item -> (problem, row chunk, tile): consecutive CTAs take different
  // tiles of the same row chunk (L2 sharing of the panels)
  const int ntiles = SYM ? gw_tiles_sym(tn, tn2) : tn * tn2;
  const int per_problem = ntiles * chunks;
  const int pb = (int)(blockIdx.x / per_problem);
  const int rem_item = (int)(blockIdx.x % per_problem);
  const int chunk = rem_item / ntiles, tile = rem_item % ntiles;
  // sub-chunk slabs of this item: (problem, tile) major, then the sub-chunks of all rows
  const int64_t slab0 =
      (int64_t)(pb * ntiles + tile) * nsubs + (int64_t)chunk * subs_per_chunk + slab_off;
  int ti = 0, tj = 0;
  if (SYM)
    gw_tile_sym(tile, tn2, ti, tj);
  else {
    ti = tile / tn2;
    tj = tile % tn2;
  }
  const int I0 = ti * 128, J0 = tj * 256;
  const bool band = SYM && I0 >= J0 && I0 < J0 + 256;   // A = columns I0.. of the B tile
  // the second band tile of a column block (I0 = J0 + 128): its left 128
  // columns lie below the diagonal, so only the 128 x 128 diagonal block is
  // formed (128-wide products on the B panel's right half, which is A)
  const bool half = band && I0 == J0 + 128;
  const uint32_t a_off = band ? (uint32_t)((I0 - J0) / 64) * GW_BOX : 0u;
  const int dcol = I0 - J0;  // tile column of the Gram diagonal (band tiles)
  const int64_t r_beg = (int64_t)chunk * rows_per_chunk;
  const int64_t r_end = (r_beg + rows_per_chunk < m) ? r_beg + rows_per_chunk : m;
  const int64_t nrows = (r_end > r_beg) ? r_end - r_beg : 0;
  const int KB = (int)((nrows + GW_BK - 1) / GW_BK);
  constexpr int KB_PER_SUB = G_KSUB / GW_BK;
  const int nsub = (KB + KB_PER_SUB - 1) / KB_PER_SUB;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GW_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], band ? 1 + 128 : 1);  // MMA commit (+ diagonal warps)
    }
    mbar_init(&tfull, 1);
    mbar_init(&tempty, band ? 128 : 256);  // drain warps: 0-3 on band tiles, 0-7 elsewhere
    for (int b = 0; b < 2; ++b) mbar_init(&dfull[b], 128);
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == 8) {
    tmem_alloc(&tmem_sh, G_TMEM);
    tmem_relinquish();
  }
  if (warp == 9 && lane == 0) {
    tma_prefetch_map(&tmP);
    if (!SYM) tma_prefetch_map(&tmB);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;
  // stage layout: A hi (2 boxes), A lo (2), B hi (4), B lo (4)
  constexpr uint32_t OFF_AL = 2 * GW_BOX, OFF_BH = 4 * GW_BOX, OFF_BL = 8 * GW_BOX;

  if (warp == 9) {
    // ---- TMA producer: GW_BK rows x (I block unless band, J block) of both planes
    if (lane == 0) {
      const uint32_t bytes = (half ? 4u : band ? 8u : 12u) * GW_BOX;
      const CUtensorMap* mb = SYM ? &tmP : &tmB;
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % GW_STAGES;
        const uint32_t ph = (uint32_t)(kb / GW_STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) break;
        const uint32_t st = base + s * GW_STAGE;
        const int y = (int)((int64_t)pb * mp + r_beg + (int64_t)kb * GW_BK);
        mbar_expect_tx(&full_bar[s], bytes);
#pragma unroll
        for (int z = 0; z < 2; ++z) {
          if (!band) {
            tma_load_3d(st + z * OFF_AL, &tmP, I0, y, z, &full_bar[s]);
            tma_load_3d(st + z * OFF_AL + GW_BOX, &tmP, I0 + 64, y, z, &full_bar[s]);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (half && q < 2) continue;
            tma_load_3d(st + OFF_BH + z * 4 * GW_BOX + q * GW_BOX, mb, J0 + 64 * q, y, z,
                        &full_bar[s]);
          }
        }
      }
    }
  } else if (warp >= 4 && warp < 8 && band) {
    // ---- band tiles: compensated sums of (hi + lo)^2 of A's columns on the
    // CUDA cores, the Gram diagonal (as in gram16_kernel: two adjacent columns
    // per thread, half of each stage's rows, four compensated chains)
    const int t = threadIdx.x - 128;
    const int c = 2 * (t & 63);                // first of the two columns of A
    const int h = t >> 6;                      // row half of each stage
    const uint32_t cbo = OFF_BH + a_off + (uint32_t)(c >> 6) * GW_BOX;
    const uint32_t cw = (uint32_t)(c & 63);
    const uint32_t ch = cw >> 3, within = (cw & 7u) * 2u;
    const uint32_t k0 = (uint32_t)h * (GW_BK / 2), k1 = k0 + GW_BK / 2;
    float sm[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, cp[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % GW_STAGES;
      const uint32_t ph = (uint32_t)(kb / GW_STAGES) & 1u;
      if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) break;
      const uint32_t st = base + s * GW_STAGE + cbo;
#pragma unroll 4
      for (uint32_t k = k0; k < k1; k += 2) {
#pragma unroll
        for (uint32_t u = 0; u < 2; ++u) {
          const uint32_t kk = k + u;
          const uint32_t off = (kk >> 3) * 1024u + (kk & 7u) * 128u + (((ch ^ (kk & 7u)) << 4) | within);
          const float2 hv = ld_shared_h2f(st + off);
          const float2 lv = ld_shared_h2f(st + 4 * GW_BOX + off);  // B lo = B hi + 4 boxes
          const float v[2] = {hv.x + lv.x, hv.y + lv.y};  // exact: 22 bits
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const float y = fmaf(v[q], v[q], -cp[q][u]);
            const float tt = sm[q][u] + y;
            cp[q][u] = (tt - sm[q][u]) - y;
            sm[q][u] = tt;
          }
        }
      }
      mbar_arrive(&empty_bar[s]);
      if ((kb % KB_PER_SUB) == KB_PER_SUB - 1 || kb == KB - 1) {
        const int b = (kb / KB_PER_SUB) & 1;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          diag_sh[b][h][c + q] = ((double)sm[q][0] - (double)cp[q][0]) +
                                 ((double)sm[q][1] - (double)cp[q][1]);
          sm[q][0] = sm[q][1] = cp[q][0] = cp[q][1] = 0.f;
        }
        mbar_arrive(&dfull[b]);
      }
    }
  } else if (warp == 8 && lane == 0) {
    // ---- UMMA issuer: main += hi*hi, correction += hi*lo + lo*hi
    constexpr uint32_t idesc = idesc_f16(128, 256, 1, 1);
    bool ok = true;
    int kb = 0;
    for (int sub = 0; sub < nsub && ok; ++sub) {
      if (!mbar_wait(&tempty, ((uint32_t)sub & 1u) ^ 1u, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t dmain = tmem, dcorr = tmem + 256u;
      const int kb_end = (kb + KB_PER_SUB < KB) ? kb + KB_PER_SUB : KB;
      for (int kl = 0; kb < kb_end; ++kb, ++kl) {
        const int s = kb % GW_STAGES;
        const uint32_t ph = (uint32_t)(kb / GW_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t st = base + s * GW_STAGE;
        const uint32_t bH = st + OFF_BH, bL = st + OFF_BL;
        const uint32_t aH = band ? bH + a_off : st, aL = band ? bL + a_off : st + OFF_AL;
        if (half) {
          // accumulators at column 128: the slab keeps its column layout
          constexpr uint32_t idesc_h = idesc_f16(128, 128, 1, 1);
#pragma unroll
          for (int kk = 0; kk < GW_BK / 16; ++kk) {
            const uint32_t adv = (uint32_t)kk * 2048u;
            const uint64_t dAH = desc_sw128(aH + adv, GW_BOX, 1024), dAL = desc_sw128(aL + adv, GW_BOX, 1024);
            const uint32_t first = (kl > 0 || kk > 0) ? 1u : 0u;
            mma_f16(dmain + 128u, dAH, dAH, idesc_h, first);
            mma_f16(dcorr + 128u, dAH, dAL, idesc_h, first);
            mma_f16(dcorr + 128u, dAL, dAH, idesc_h, 1u);
          }
          mma_commit(&empty_bar[s]);
          continue;
        }
#pragma unroll
        for (int kk = 0; kk < GW_BK / 16; ++kk) {
          const uint32_t adv = (uint32_t)kk * 2048u;  // 16 rows of 128 bytes
          const uint64_t dAH = desc_sw128(aH + adv, GW_BOX, 1024), dAL = desc_sw128(aL + adv, GW_BOX, 1024);
          const uint64_t dBH = desc_sw128(bH + adv, GW_BOX, 1024), dBL = desc_sw128(bL + adv, GW_BOX, 1024);
          const uint32_t first = (kl > 0 || kk > 0) ? 1u : 0u;
          mma_f16(dmain, dAH, dBH, idesc, first);
          mma_f16(dcorr, dAH, dBL, idesc, first);
          mma_f16(dcorr, dAL, dBH, idesc, 1u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (ok) mma_commit(&tfull);
    }
  } else if (warp < 8) {
    // ---- drain warps (TMEM lane quarter w % 4): 0-3 take all 256 columns on
    // band tiles, 0-7 take 128 columns each (half w / 4) elsewhere.  Each
    // finished sub-chunk is written once, main + correction rounded to FP32
    // (half an ulp of a 4,096-row partial), into its own slab; no slab is
    // read back here, so the drain is a TMEM read and a stream of stores, and
    // the reduction kernel sums the slabs in a fixed order.  Band tiles also
    // write their rows' diagonal (the CUDA-core sums, FP64) per sub-chunk.
    const int rloc = (warp & 3) * 32 + lane;
    const int cbeg = half ? 128 : band ? 0 : (warp >> 2) * 128, ncc = (band && !half) ? 8 : 4;
    for (int sub = 0; sub < nsub; ++sub) {
      const int b = sub & 1;
      bool ready = mbar_wait(&tfull, (uint32_t)sub & 1u, &abort_sh, err);
      if (band) ready = ready && mbar_wait(&dfull[b], ((uint32_t)sub >> 1) & 1u, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      float* prow = part + ((slab0 + sub) * 128 + rloc) * 256 + cbeg;
#pragma unroll 1
      for (int c8 = 0; c8 < ncc; ++c8) {
        uint32_t rm[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(cbeg + 32 * c8);
        tmem_ld32(ta, rm);
        tmem_ld32(ta + 256, rc);
        tmem_wait_ld();
        if (c8 == ncc - 1) {
          fence_before();
          mbar_arrive(&tempty);
        }
        float4* d = reinterpret_cast<float4*>(prow + 32 * c8);
#pragma unroll
        for (int j = 0; j < 32; j += 4)
          d[j / 4] = make_float4(__uint_as_float(rm[j]) + __uint_as_float(rc[j]),
                                 __uint_as_float(rm[j + 1]) + __uint_as_float(rc[j + 1]),
                                 __uint_as_float(rm[j + 2]) + __uint_as_float(rc[j + 2]),
                                 __uint_as_float(rm[j + 3]) + __uint_as_float(rc[j + 3]));
      }
      if (band) diagp[(slab0 + sub) * 128 + rloc] = diag_sh[b][0][rloc] + diag_sh[b][1][rloc];
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 8) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, G_TMEM);
  }
}

// G[i][j] = sum over the 4,096-row sub-chunk slabs (fixed order, double-float)
// / (s_i s_j), taken from the upper triangle (i <= j) and mirrored; the
// diagonal from the band tiles' FP64 slabs.  One thread per 4 consecutive
// columns of a tile row: 16-byte loads down the slabs, sixteen in flight;
// each batch of 16 slabs is summed in FP32 and added to a double-float sum,
// in sub-chunk order (the same order for every call; the slabs' own FP32
// sums over 4,096 rows carry the larger error).
constexpr int GWR_UNROLL = 16;
// subs_per_scale > 0: the slabs come from row chunks packed with their own
// column scales (scale vector q = sub-chunk / subs_per_scale, a multiple of
// GWR_UNROLL sub-chunks each): every batch is unscaled (exactly: powers of
// two) before it is added
__global__ void __launch_bounds__(256, 3) gram16w_reduce_kernel(const float* __restrict__ part,
                                                             const double* __restrict__ diagp,
                                                             int N, int tn, int tn2, int nsubs,
                                                             const float* __restrict__ s,
                                                             double* __restrict__ G, int batch,
                                                             int ld, int accumulate,
                                                             int subs_per_scale) {
  const int ntiles = gw_tiles_sym(tn, tn2);
  const int64_t units = (int64_t)batch * ntiles * 128 * 64;
  const int64_t slab_elems = 128 * 256;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(u & 63);
    const int row = (int)((u >> 6) & 127);
    const int64_t tb = u >> 13;
    const int tile = (int)(tb % ntiles);
    const int64_t pb = tb / ntiles;
    // tile -> (ti, tj): row block ti holds tn2 - ti / 2 tiles, from tj = ti / 2
    int ti = 0, rest = tile;
    while (rest >= tn2 - (ti >> 1)) {
      rest -= tn2 - (ti >> 1);
      ++ti;
    }
    const int tj = (ti >> 1) + rest;
    const int a = ti * 128 + row, b0 = tj * 256 + 4 * q;
    if (a >= N || b0 >= N || b0 + 3 < a) continue;
    const int64_t slab = (pb * ntiles + tile) * (int64_t)nsubs;
    const float4* p = reinterpret_cast<const float4*>(part + slab * slab_elems + (int64_t)row * 256 +
                                                      4 * q);
    float2 acc[4];
    double vsum[4] = {0.0, 0.0, 0.0, 0.0};  // per-chunk-scale mode: the unscaled chunk sums
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[e] = make_float2(0.f, 0.f);
    // whole batches: sixteen independent loads in flight, then the batch's
    // slabs in FP32 (in order) and into the double-float sums; the last
    // partial batch the same way, one slab at a time
    const int nfull = nsubs - nsubs % GWR_UNROLL;
    for (int c0 = 0; c0 < nsubs; c0 += GWR_UNROLL) {
      float4 v[GWR_UNROLL];
      const int cnt = c0 < nfull ? GWR_UNROLL : nsubs - c0;
      if (cnt == GWR_UNROLL) {
#pragma unroll
        for (int k = 0; k < GWR_UNROLL; ++k) v[k] = __ldcs(p + (int64_t)(c0 + k) * (slab_elems / 4));
      } else {
#pragma unroll
        for (int k = 0; k < GWR_UNROLL; ++k)
          v[k] = k < cnt ? __ldcs(p + (int64_t)(c0 + k) * (slab_elems / 4))
                         : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float4 bs = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int k = 0; k < GWR_UNROLL; ++k) {
        bs.x += v[k].x;
        bs.y += v[k].y;
        bs.z += v[k].z;
        bs.w += v[k].w;
      }
      acc[0] = dw_add_f(acc[0], bs.x);
      acc[1] = dw_add_f(acc[1], bs.y);
      acc[2] = dw_add_f(acc[2], bs.z);
      acc[3] = dw_add_f(acc[3], bs.w);
      if (subs_per_scale > 0 &&
          ((c0 + GWR_UNROLL) % subs_per_scale == 0 || c0 + GWR_UNROLL >= nsubs)) {
        // end of a row chunk: its sums unscaled in FP64 (any scale range)
        const float* sq = s + (int64_t)(c0 / subs_per_scale) * ld;
        const double sa_q = (double)sq[a];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          vsum[e] += dw_value(acc[e]) / (sa_q * (double)sq[min(b0 + e, N - 1)]);
          acc[e] = make_float2(0.f, 0.f);
        }
      }
    }
    const float* sp = s + pb * ld;
    const double sa = (double)sp[a];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int b = b0 + e;
      if (b >= N || b < a) continue;
      double v;
      if (b == a) {
        // the diagonal's FP64 slabs, in the same order, loads batched
        const double* dp = diagp + slab * 128 + row;
        float2 d = make_float2(0.f, 0.f);
        double dsum = 0.0;
        for (int c0 = 0; c0 < nsubs; c0 += GWR_UNROLL) {
          double dv[GWR_UNROLL];
#pragma unroll
          for (int k = 0; k < GWR_UNROLL; ++k)
            dv[k] = (c0 + k < nsubs) ? dp[(int64_t)(c0 + k) * 128] : 0.0;
#pragma unroll
          for (int k = 0; k < GWR_UNROLL; ++k) {
            if (c0 + k >= nsubs) break;
            d = dw_add(d, dw_from_double(dv[k]));
          }
          if (subs_per_scale > 0 &&
              ((c0 + GWR_UNROLL) % subs_per_scale == 0 || c0 + GWR_UNROLL >= nsubs)) {
            const double sa_q = (double)s[(int64_t)(c0 / subs_per_scale) * ld + a];
            dsum += dw_value(d) / (sa_q * sa_q);
            d = make_float2(0.f, 0.f);
          }
        }
        v = subs_per_scale > 0 ? dsum : dw_value(d);
      } else {
        v = subs_per_scale > 0 ? vsum[e] : dw_value(acc[e]);
      }
      if (subs_per_scale == 0) v /= sa * (double)sp[b];
      const int64_t e1 = pb * N * N + (int64_t)a * N + b;
      const int64_t e2 = pb * N * N + (int64_t)b * N + a;
      G[e1] = accumulate ? G[e1] + v : v;
      if (e2 != e1) G[e2] = accumulate ? G[e2] + v : v;
    }
  }
}

// C[i][j] (Na x Nb, ldc) = sum over the sub-chunk slabs / (sA_i sB_j)
__global__ void tn16w_reduce_kernel(const float* __restrict__ part, int Na, int Nb, int tn2,
                                    int nsubs, const float* __restrict__ sa,
                                    const float* __restrict__ sb, double* __restrict__ C,
                                    int64_t ldc) {
  const int64_t total = (int64_t)Na * Nb;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / Nb), j = (int)(e % Nb);
    const int ti = i / 128, tj = j / 256;
    const int tile = ti * tn2 + tj;
    const float* p = part + ((int64_t)tile * nsubs) * 128 * 256 + (int64_t)(i - ti * 128) * 256 +
                     (j - tj * 256);
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < nsubs; ++c) acc = dw_add(acc, make_float2(p[(int64_t)c * 128 * 256], 0.f));
    C[(int64_t)i * ldc + j] = dw_value(acc) / ((double)sa[i] * (double)sb[j]);
  }
}

// ---------------------------------------------------------------------------
// apply: C (m x k) = Y W, persistent CTAs over 128 x TN output tiles.
// TN = 256 (k > 128): one 128 x 256 x 16 UMMA per product.  A UMMA of N = 128
// takes 64 cycles, too short for the per-stage barrier round trip of the
// stage ring to hide (measured: a three-stage ring of 128 x 128 products runs
// the tensor pipe at 0.80 of its rate, the same ring of 128 x 256 products at
// 1.00), and a 256-wide tile also halves the A operand's share of the bytes
// each SM must receive per product.  Its two accumulators fill TMEM (256 + 256
// columns), so the epilogue of a tile does not overlap the next tile's
// products; two 96 KiB stages.  TN = 128 (narrow k): three 64 KiB stages and
// two accumulator buffers.
// ---------------------------------------------------------------------------
// K per stage: 64 (128-byte rows, 128-byte swizzle) for TN = 128; 32 (64-byte
// rows, 64-byte swizzle) for TN = 256, so that four stages fit in 192 KiB
// (32-deep stages for TN = 128, six of 32 KiB, measured 15 % slower on the
// triangular products than three of 64 KiB)
template <int TN, int BKV = (TN == 256 ? 32 : 64)>
struct ApplyCfg {
  static_assert(BKV == 32 || BKV == 64, "stage depth");
  static constexpr int BK = BKV;
  static constexpr uint32_t A_TILE = 128u * BK * 2;           // 128 rows x BK fp16
  static constexpr uint32_t B_TILE = (uint32_t)TN * BK * 2;   // TN rows x BK fp16
  static constexpr uint32_t STAGE = 2 * A_TILE + 2 * B_TILE;  // A hi, A lo, B hi, B lo
  static constexpr int STAGES = (int)(196608u / STAGE);
  static constexpr int NBUF = TN == 256 ? 1 : 2;   // TMEM accumulator buffers
};
// Warps: 0-7 epilogue (warp w drains TMEM lanes 32 (w % 4).. for the column
// half w / 4 of the tile), 8 UMMA issuer (and TMEM owner), 9 TMA producer.
// Eight epilogue warps keep short-K tiles (narrow problems, the first column
// blocks of a triangular W) from being paced by the TMEM drain and stores.
// Eight epilogue warps (two per TMEM lane quarter); with TN = 256 each reads
// its 128 columns out of TMEM into registers, releases the single accumulator
// buffer and then stores them through its staging rows, so the stores overlap
// the next tile's products.
// TN = 256 epilogue: 1 = read the tile into registers and release TMEM before
// the stores (the next tile's products overlap them), 0 = drain and store
// 32 columns at a time, releasing TMEM at the end
#ifndef PLOM_APPLY_HOLD
#define PLOM_APPLY_HOLD 1
#endif
template <int TN>
struct ApplyWarps {
  static constexpr int EPI = 8;
  static constexpr int THREADS = 32 * (EPI + 2);
  static constexpr uint32_t STG = EPI * 4096u;  // staging: 32 rows x 128 bytes a warp
};
constexpr int A_EPI_WARPS = 8;                 // TN = 128
constexpr int A_THREADS = 32 * (A_EPI_WARPS + 2);
template <int TN, int BKV = ApplyCfg<TN>::BK>
constexpr size_t apply_smem() {
  return (size_t)ApplyCfg<TN, BKV>::STAGES * ApplyCfg<TN, BKV>::STAGE + ApplyWarps<TN>::STG + 1024;
}

struct ApplyOut {
  float* C;        // FP32 output (m x k, ldc) or nullptr
  int64_t ldc;
  int64_t cstride; // elements between the problems' C (batch)
  __half* ohi;     // packed output planes (m x ldo) or nullptr
  __half* olo;
  int ldo;
};

// one 32-column group of an apply tile (FP32 or packed output) through the
// warp's staging rows: row r holds 8 chunks of 16 bytes, chunk q in slot
// q ^ (r & 7); each row leaves as 128 contiguous bytes (fewer at the last
// columns).  FP32 rows < m and columns < k; packed rows < mp (padding rows
// get the zeros their zero input rows produce)
__device__ __forceinline__ void apply_store_chunk(const float (&v)[32], int col0, uint4* stg,
                                            int lane, const ApplyOut& out, int k, int64_t m,
                                            int64_t mp, int64_t pb, int64_t row0,
                                            bool c_vec) {

  const bool staged = out.C ? (col0 < k) : (col0 < out.ldo);
  if (!staged) return;
  __syncwarp();
  if (out.C) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      stg[lane * 8 + (q ^ (lane & 7))] =
          make_uint4(__float_as_uint(v[4 * q]), __float_as_uint(v[4 * q + 1]),
                     __float_as_uint(v[4 * q + 2]), __float_as_uint(v[4 * q + 3]));
  } else {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      float w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) w[q] = v[8 * g + q];
      uint4 h, l;
      split8(w, h, l);
      stg[lane * 8 + (g ^ (lane & 7))] = h;
      stg[lane * 8 + ((4 + g) ^ (lane & 7))] = l;
    }
  }
  __syncwarp();
  const int q = lane & 7;
#pragma unroll
  for (int s8 = 0; s8 < 8; ++s8) {
    const int rr = 4 * s8 + (lane >> 3);
    const uint4 val = stg[rr * 8 + (q ^ (rr & 7))];
    const int64_t r = row0 + rr;
    if (out.C) {
      const int c = col0 + 4 * q;
      if (r < m && c < k) {
        float* dst = out.C + pb * out.cstride + r * out.ldc + c;
        if (c_vec && c + 4 <= k) {
          *reinterpret_cast<uint4*>(dst) = val;
        } else {
          const float w4[4] = {__uint_as_float(val.x), __uint_as_float(val.y),
                               __uint_as_float(val.z), __uint_as_float(val.w)};
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (c + e < k) dst[e] = w4[e];
        }
      }
    } else if (r < mp) {
      __half* plane = q < 4 ? out.ohi : out.olo;
      *reinterpret_cast<uint4*>(plane + (pb * mp + r) * out.ldo + col0 + 8 * (q & 3)) = val;
    }
  }
}

template <int TN, int BKV = ApplyCfg<TN>::BK>
__global__ void __launch_bounds__(ApplyWarps<TN>::THREADS, 1)
    apply16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   int64_t m, int kblocks, int k, int64_t col_tiles, int64_t tiles,
                   const float* __restrict__ f, ApplyOut out, int* err, int64_t mp,
                   int64_t row_tiles, int fstride, int upper, int by_rows) {
  // tile t -> (problem pb, row block rb, column block cb); a problem's rows are
  // mp apart in the packed planes (input and packed output alike).  With an
  // upper-triangular W (upper != 0) column block cb needs only the first
  // (cb + 1) TN rows of W: the K blocks below (cb + 1) TN / 64.
  // by_rows: CTA x takes whole row blocks (every column tile of row blocks x,
  // x + G, ...), so the column tiles that re-read a row block's input follow
  // each other on one SM (L2 hits) and every CTA gets the same work per row
  // block.  Otherwise it takes single tiles, tile r G + x in even rounds r and
  // r G + (G - 1 - x) in odd ones.
  using Cfg = ApplyCfg<TN, BKV>;
  constexpr int A_STAGES = Cfg::STAGES, NBUF = Cfg::NBUF, A_BK = Cfg::BK;
  constexpr uint32_t A_STAGE = Cfg::STAGE, B_TILE = Cfg::B_TILE;
  constexpr uint32_t A_TILE = Cfg::A_TILE;
  constexpr int A_EPI_WARPS = ApplyWarps<TN>::EPI;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[A_STAGES], empty_bar[A_STAGES], tfull[NBUF], tempty[NBUF];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t G = gridDim.x;
  const int64_t units = tiles / col_tiles;  // row blocks over the batch
  // tiles of this CTA (by rows), or rounds of G tiles (a round's tile past the
  // end is skipped)
  const int64_t my_tiles =
      by_rows ? (blockIdx.x < units ? ((units - 1 - blockIdx.x) / G + 1) * col_tiles : 0)
              : (tiles + G - 1) / G;
  // it-th tile of this CTA (it < my_tiles)
  auto apply_tile = [&](int64_t it) -> int64_t {
    if (by_rows) return (blockIdx.x + (it / col_tiles) * G) * col_tiles + it % col_tiles;
    return it * G + ((it & 1) ? G - 1 - blockIdx.x : (int64_t)blockIdx.x);
  };
  auto apply_kend = [&](int cb) -> int {
    return upper ? min(kblocks, (cb + 1) * (TN / A_BK)) : kblocks;
  };
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < A_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < NBUF; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 32 * A_EPI_WARPS);
    }
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == A_EPI_WARPS) {
    tmem_alloc(&tmem_sh, 512);  // NBUF buffers x (main TN + correction TN)
    tmem_relinquish();
  }
  if (warp == A_EPI_WARPS + 1 && lane == 0) {
    tma_prefetch_map(&tmA);
    tma_prefetch_map(&tmB);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;

  if (warp == A_EPI_WARPS + 1) {
    // ---- TMA producer, running ahead across tiles
    if (lane == 0) {
      int64_t g = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int64_t t = apply_tile(it);
        if (t >= tiles) continue;
        const int64_t pb = t / (row_tiles * col_tiles);
        const int64_t rt = t - pb * row_tiles * col_tiles;
        const int rb = (int)(rt / col_tiles), cb = (int)(rt % col_tiles);
        const int ya = (int)(pb * mp + (int64_t)rb * 128), yb = (int)(pb * k + (int64_t)cb * TN);
        const int kend = apply_kend(cb);
        for (int kb = 0; kb < kend; ++kb, ++g) {
          const int s = (int)(g % A_STAGES);
          const uint32_t ph = (uint32_t)(g / A_STAGES) & 1u;
          if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) {
            ok = false;
            break;
          }
          const uint32_t st = base + s * A_STAGE;
          mbar_expect_tx(&full_bar[s], A_STAGE);
          tma_load_3d(st, &tmA, kb * A_BK, ya, 0, &full_bar[s]);
          tma_load_3d(st + A_TILE, &tmA, kb * A_BK, ya, 1, &full_bar[s]);
          // B: TN rows of the W copy in boxes of 128 rows (the K-major swizzled
          // layout of a 256-row tile is two 128-row tiles back to back)
#pragma unroll
          for (int h = 0; h < TN / 128; ++h) {
            tma_load_3d(st + 2 * A_TILE + h * A_TILE, &tmB, kb * A_BK, yb + 128 * h, 0, &full_bar[s]);
            tma_load_3d(st + 2 * A_TILE + B_TILE + h * A_TILE, &tmB, kb * A_BK, yb + 128 * h, 1,
                        &full_bar[s]);
          }
        }
      }
    }
  } else if (warp == A_EPI_WARPS) {
    // ---- UMMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(128, TN, 0, 0);
      int64_t g = 0;
      int i = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int64_t t = apply_tile(it);
        if (t >= tiles) continue;
        const int b = i % NBUF;
        if (!mbar_wait(&tempty[b], (((uint32_t)(i / NBUF)) & 1u) ^ 1u, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t dmain = tmem + (uint32_t)(b * 2 * TN);
        const uint32_t dcorr = dmain + (uint32_t)TN;
        const int kend = apply_kend((int)(t % col_tiles));
        for (int kb = 0; kb < kend; ++kb, ++g) {
          const int s = (int)(g % A_STAGES);
          const uint32_t ph = (uint32_t)(g / A_STAGES) & 1u;
          if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t st = base + s * A_STAGE;
#pragma unroll
          for (int kk = 0; kk < A_BK / 16; ++kk) {
            const uint32_t adv = (uint32_t)kk * 32u;  // 16 fp16 along K
            const uint64_t dAH = desc_kmajor<A_BK>(st + adv);
            const uint64_t dAL = desc_kmajor<A_BK>(st + A_TILE + adv);
            const uint64_t dBH = desc_kmajor<A_BK>(st + 2 * A_TILE + adv);
            const uint64_t dBL = desc_kmajor<A_BK>(st + 2 * A_TILE + B_TILE + adv);
            const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
            mma_f16(dmain, dAH, dBH, idesc, acc);
            mma_f16(dcorr, dAH, dBL, idesc, acc);
            mma_f16(dcorr, dAL, dBH, idesc, 1u);
          }
          mma_commit(&empty_bar[s]);
        }
        if (ok) mma_commit(&tfull[b]);
        ++i;
      }
    }
  } else {
    // ---- epilogue (warps 0-7): TMEM -> scale -> FP32 or packed store
    uint4* stg = reinterpret_cast<uint4*>(smem_raw + (base - smem_u32(smem_raw)) +
                                          A_STAGES * A_STAGE + warp * 4096);
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lane quarter, column half
    int i = 0;
    for (int64_t it = 0; it < my_tiles; ++it) {
      const int64_t t = apply_tile(it);
      if (t >= tiles) continue;
      const int b = i % NBUF;
      const bool ready = mbar_wait(&tfull[b], ((uint32_t)(i / NBUF)) & 1u, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      const int64_t pb = t / (row_tiles * col_tiles);
      const int64_t rt = t - pb * row_tiles * col_tiles;
      const int64_t rb = rt / col_tiles, cb = rt % col_tiles;
      const int64_t row0 = rb * 128 + quarter * 32;  // first row of this warp (within the problem)
      const float* fp = f + pb * fstride;
      const bool c_vec = out.C && ((out.ldc & 3) == 0) && ((out.cstride & 3) == 0) &&
                         ((reinterpret_cast<uintptr_t>(out.C) & 15) == 0);
      if constexpr (TN == 256 && PLOM_APPLY_HOLD) {
        // one accumulator buffer: the warp's 128 columns are read out of TMEM
        // into registers first and the buffer is released before the stores,
        // so the next tile's products overlap them
        float vv[4][32];
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4) {
          const int col0 = (int)(cb * TN) + (4 * half + c4) * 32;
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            uint32_t rm[16], rc[16];
            const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) +
                                (uint32_t)((4 * half + c4) * 32 + hh * 16);
            tmem_ld16(ta, rm);
            tmem_ld16(ta + TN, rc);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; ++j)
              vv[c4][hh * 16 + j] = (__uint_as_float(rm[j]) + __uint_as_float(rc[j])) *
                                    __ldg(fp + col0 + hh * 16 + j);
          }
        }
        fence_before();
        mbar_arrive(&tempty[b]);
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4)
          apply_store_chunk(vv[c4], (int)(cb * TN) + (4 * half + c4) * 32, stg, lane, out, k, m, mp,
                            pb, row0, c_vec);
        ++i;
        continue;
      }
#pragma unroll 1
      for (int cc = (TN / 64) * half; cc < (TN / 64) * (half + 1); ++cc) {
        uint32_t rm[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * 2 * TN + cc * 32);
        tmem_ld32(ta, rm);
        tmem_ld32(ta + TN, rc);
        tmem_wait_ld();
        const int col0 = (int)(cb * TN) + cc * 32;
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; ++j)
          v[j] = (__uint_as_float(rm[j]) + __uint_as_float(rc[j])) * __ldg(fp + col0 + j);
        apply_store_chunk(v, col0, stg, lane, out, k, m, mp, pb, row0, c_vec);
      }
      fence_before();
      mbar_arrive(&tempty[b]);
      ++i;
    }
  }
  fence_before();
  __syncthreads();
  if (warp == A_EPI_WARPS) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// apply on SM pairs: C (m x k) = Y W with 2-SM products (tcgen05 cta_group::2).
// A cluster of two CTAs takes 256 x TN output tiles: CTA r of the pair holds
// rows 128 r .. 128 r + 127 of the tile's 256 Y rows (A) and W columns
// TN r / 2 .. TN (r + 1) / 2 - 1 of its TN (B) in its own shared memory, and
// the leader (r = 0) issues one 256 x TN x 16 UMMA per product that reads both
// halves of B; each CTA's TMEM receives its 128 rows x TN columns.  Per SM and
// per product this moves half the B bytes of the single-SM 128 x TN tile
// through shared memory (TMA writes and tensor-core reads).
//  TN = 256 (dense W wider than 128 columns): K = 32 per stage (64-byte
//    swizzle), 32 KiB stages x 6; the two accumulators fill TMEM, so the
//    epilogue reads the tile into registers and releases TMEM before its stores.
//  TN = 128 (upper-triangular W: column block cb takes exactly the K blocks
//    below (cb + 1) 128): K = 64 per stage (128-byte swizzle), 48 KiB stages x
//    4, two accumulator buffers, so the epilogue of one tile overlaps the
//    products of the next.  Per SM it has the bytes-per-product ratio of the
//    single-SM 128 x 256 tile instead of the 128 x 128 one.
// Barriers: the stage-full barrier of the leader counts both CTAs' TMA bytes
// (the peer's loads signal it across the pair); stage-empty and tile-full
// barriers live in both CTAs and are signalled by the leader's multicast
// commits; the tile-empty barriers of the leader collect one arrival per
// epilogue warp of both CTAs.  Every wait is bounded as in the other kernels;
// both CTAs always reach the TMEM allocation and the closing cluster barrier.
// ---------------------------------------------------------------------------
template <int TN>
struct PairCfg {
  static constexpr int BK = TN == 256 ? 32 : 64;               // K per stage
  static constexpr uint32_t A_TILE = 128u * BK * 2;            // 128 rows x BK fp16
  static constexpr uint32_t B_HALF = (uint32_t)(TN / 2) * BK * 2;
  static constexpr uint32_t STAGE = 2 * A_TILE + 2 * B_HALF;   // A hi, A lo, B-half hi, B-half lo
  static constexpr int STAGES = TN == 256 ? 6 : 4;
  static constexpr int NBUF = TN == 256 ? 1 : 2;               // TMEM accumulator buffers
  static constexpr int EPI = 8;                                // epilogue warps
  static constexpr int THREADS = 32 * (EPI + 2);               // + UMMA issuer, TMA producer
  static constexpr uint32_t STG = EPI * 4096u;
};
template <int TN>
constexpr size_t pair_smem() {
  return (size_t)PairCfg<TN>::STAGES * PairCfg<TN>::STAGE + PairCfg<TN>::STG + 1024;
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared::cluster address of this CTA's variable at `saddr` in CTA `rank`
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
  uint32_t d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(saddr), "r"(rank));
  return d;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t caddr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cl(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait with cluster-scope acquire (arrivals from the other CTA)
__device__ __forceinline__ bool mbar_wait_cl(uint64_t* bar, uint32_t parity,
                                             volatile int* abort_flag, int* err) {
  if (mbar_try_wait_cl(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  uint32_t spins = 0;
  while (true) {
    if (mbar_try_wait_cl(bar, parity)) return true;
    if (*abort_flag) return false;
    if ((++spins & 1023u) == 0 && err && *(volatile int*)err == PLOM_NUM_TIMEOUT) {
      *abort_flag = 1;
      return false;
    }
    if (gtimer() - t0 > WAIT_NS) {
      *abort_flag = 1;
      if (err) atomicMax(err, PLOM_NUM_TIMEOUT);
      return false;
    }
  }
}
// TMEM of both CTAs of the pair: one warp of each CTA takes part
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish_pair() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void mma_f16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                             uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}
// arrive on the barrier at the same offset in both CTAs of the pair once the
// issuing thread's earlier products are done
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(smem_u32(bar)),
      "h"((uint16_t)3)
      : "memory");
}
// TMA load into this CTA's shared memory whose completion is counted on a
// barrier of either CTA of the pair (`bar`: shared::cluster address)
__device__ __forceinline__ void tma_load_3d_pair(uint32_t dst, const CUtensorMap* map, int x, int y,
                                                 int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Tiles: 256-row pair blocks q x TN-column blocks cb (tiles = row_pairs x
// col_tiles); one problem (no batch).  upper: W upper triangular, column block
// cb takes the K blocks below (cb + 1) TN.  by_rows as in apply16_kernel, over
// pairs.
template <int TN>
__global__ void __launch_bounds__(PairCfg<TN>::THREADS, 1)
    apply16p_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    int64_t m, int kblocks, int k, int64_t col_tiles, int64_t tiles,
                    const float* __restrict__ f, ApplyOut out, int* err, int64_t mp, int upper,
                    int by_rows) {
  using C = PairCfg<TN>;
  constexpr int S = C::STAGES, BK = C::BK, EPI = C::EPI, NBUF = C::NBUF;
  constexpr uint32_t A_TILE = C::A_TILE, B_HALF = C::B_HALF, STAGE = C::STAGE;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[S], empty_bar[S], tfull[NBUF], tempty[NBUF];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();  // 0: the pair's leader (issues the products)
  const int64_t G = gridDim.x >> 1, pid = blockIdx.x >> 1;
  const int64_t units = tiles / col_tiles;  // 256-row pair blocks
  const int64_t my_tiles =
      by_rows ? (pid < units ? ((units - 1 - pid) / G + 1) * col_tiles : 0) : (tiles + G - 1) / G;
  auto pair_tile = [&](int64_t it) -> int64_t {
    if (by_rows) return (pid + (it / col_tiles) * G) * col_tiles + it % col_tiles;
    return it * G + ((it & 1) ? G - 1 - pid : pid);
  };
  auto pair_kend = [&](int cb) -> int {
    return upper ? min(kblocks, (cb + 1) * (TN / BK)) : kblocks;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < NBUF; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 2 * EPI);
    }
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == EPI) {
    tmem_alloc_pair(&tmem_sh, 512);  // NBUF x (main TN + correction TN) columns
    tmem_relinquish_pair();
  }
  if (warp == EPI + 1 && lane == 0) {
    tma_prefetch_map(&tmA);
    tma_prefetch_map(&tmB);
  }
  fence_before();
  __syncthreads();
  cluster_sync_all();  // both CTAs' barriers initialised and TMEM allocated
  fence_after();
  const uint32_t tmem = tmem_sh;

  if (warp == EPI + 1) {
    // ---- TMA producer of this CTA's halves; the bytes land on the leader's barrier
    if (lane == 0) {
      const uint32_t full0 = map_to_rank(smem_u32(&full_bar[0]), 0);
      int64_t g = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int64_t t = pair_tile(it);
        if (t >= tiles) continue;
        const int64_t q = t / col_tiles;
        const int cb = (int)(t - q * col_tiles);
        const int ya = (int)(q * 256 + 128 * (int64_t)rank), yb = cb * TN + (TN / 2) * (int)rank;
        const int kend = pair_kend(cb);
        for (int kb = 0; kb < kend; ++kb, ++g) {
          const int s = (int)(g % S);
          const uint32_t ph = (uint32_t)(g / S) & 1u;
          if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) {
            ok = false;
            break;
          }
          if (rank == 0) mbar_expect_tx(&full_bar[s], 2 * STAGE);
          const uint32_t st = base + s * STAGE, fb = full0 + 8u * (uint32_t)s;
          tma_load_3d_pair(st, &tmA, kb * BK, ya, 0, fb);
          tma_load_3d_pair(st + A_TILE, &tmA, kb * BK, ya, 1, fb);
          tma_load_3d_pair(st + 2 * A_TILE, &tmB, kb * BK, yb, 0, fb);
          tma_load_3d_pair(st + 2 * A_TILE + B_HALF, &tmB, kb * BK, yb, 1, fb);
        }
      }
      // the last commits on this CTA's stage barriers land before it may exit
      for (int64_t u = (g > S ? g - S : 0); ok && u < g; ++u)
        ok = mbar_wait(&empty_bar[u % S], (uint32_t)(u / S) & 1u, &abort_sh, err);
    }
  } else if (warp == EPI) {
    // ---- UMMA issuer (leader only)
    if (lane == 0 && rank == 0) {
      constexpr uint32_t idesc = idesc_f16(256, TN, 0, 0);
      int64_t g = 0;
      int i = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int64_t t = pair_tile(it);
        if (t >= tiles) continue;
        const int b = i % NBUF;
        if (!mbar_wait_cl(&tempty[b], (((uint32_t)(i / NBUF)) & 1u) ^ 1u, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t dmain = tmem + (uint32_t)(b * 2 * TN), dcorr = dmain + (uint32_t)TN;
        const int kend = pair_kend((int)(t % col_tiles));
        for (int kb = 0; kb < kend; ++kb, ++g) {
          const int s = (int)(g % S);
          const uint32_t ph = (uint32_t)(g / S) & 1u;
          if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t st = base + s * STAGE;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t adv = (uint32_t)kk * 32u;  // 16 fp16 along K
            const uint64_t dAH = desc_kmajor<BK>(st + adv);
            const uint64_t dAL = desc_kmajor<BK>(st + A_TILE + adv);
            const uint64_t dBH = desc_kmajor<BK>(st + 2 * A_TILE + adv);
            const uint64_t dBL = desc_kmajor<BK>(st + 2 * A_TILE + B_HALF + adv);
            const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
            mma_f16_pair(dmain, dAH, dBH, idesc, acc);
            mma_f16_pair(dcorr, dAH, dBL, idesc, acc);
            mma_f16_pair(dcorr, dAL, dBH, idesc, 1u);
          }
          mma_commit_pair(&empty_bar[s]);
        }
        if (ok) mma_commit_pair(&tfull[b]);
        ++i;
      }
    }
  } else {
    // ---- epilogue (warps 0-7) of this CTA's 128 rows: warp w drains TMEM
    // lanes 32 (w % 4).. for the column half w / 4 of the tile
    uint4* stg = reinterpret_cast<uint4*>(smem_raw + (base - smem_u32(smem_raw)) + S * STAGE +
                                          warp * 4096);
    const uint32_t tempty0 = map_to_rank(smem_u32(&tempty[0]), 0);
    const int quarter = warp & 3, half = warp >> 2;
    const bool c_vec = out.C && ((out.ldc & 3) == 0) &&
                       ((reinterpret_cast<uintptr_t>(out.C) & 15) == 0);
    int i = 0;
    for (int64_t it = 0; it < my_tiles; ++it) {
      const int64_t t = pair_tile(it);
      if (t >= tiles) continue;
      const int b = i % NBUF;
      const bool ready = mbar_wait(&tfull[b], ((uint32_t)(i / NBUF)) & 1u, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      const int64_t q = t / col_tiles, cb = t - q * col_tiles;
      const int64_t row0 = q * 256 + 128 * (int64_t)rank + quarter * 32;
      // release of accumulator buffer b to the leader: one arrival per warp
      auto release = [&]() {
        fence_before();
        __syncwarp();
        if (lane == 0) {
          if (rank == 0)
            mbar_arrive(&tempty[b]);
          else
            mbar_arrive_remote(tempty0 + 8u * (uint32_t)b);
        }
      };
      if constexpr (TN == 256) {
        // one accumulator buffer: read the warp's 128 columns into registers,
        // release TMEM, then store (the next tile's products overlap the stores)
        float vv[4][32];
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4) {
          const int col0 = (int)(cb * TN) + (4 * half + c4) * 32;
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            uint32_t rm[16], rc[16];
            const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) +
                                (uint32_t)((4 * half + c4) * 32 + hh * 16);
            tmem_ld16(ta, rm);
            tmem_ld16(ta + (uint32_t)TN, rc);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; ++j)
              vv[c4][hh * 16 + j] = (__uint_as_float(rm[j]) + __uint_as_float(rc[j])) *
                                    __ldg(f + col0 + hh * 16 + j);
          }
        }
        release();
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4)
          apply_store_chunk(vv[c4], (int)(cb * TN) + (4 * half + c4) * 32, stg, lane, out, k, m,
                            mp, 0, row0, c_vec);
      } else {
        // two buffers: drain and store 32 columns at a time, release at the end
#pragma unroll 1
        for (int cc = 2 * half; cc < 2 * half + 2; ++cc) {
          uint32_t rm[32], rc[32];
          const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) +
                              (uint32_t)(b * 2 * TN + cc * 32);
          tmem_ld32(ta, rm);
          tmem_ld32(ta + (uint32_t)TN, rc);
          tmem_wait_ld();
          const int col0 = (int)(cb * TN) + cc * 32;
          float v[32];
#pragma unroll
          for (int j = 0; j < 32; ++j)
            v[j] = (__uint_as_float(rm[j]) + __uint_as_float(rc[j])) * __ldg(f + col0 + j);
          apply_store_chunk(v, col0, stg, lane, out, k, m, mp, 0, row0, c_vec);
        }
        release();
      }
      ++i;
    }
  }
  fence_before();
  __syncthreads();
  cluster_sync_all();  // no arrival or load of the other CTA is still headed here
  if (warp == EPI) {
    __syncwarp();
    fence_after();
    tmem_dealloc_pair(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// renormalisation of long-factor columns of U = Q2 M (see renorm_long_columns).
// Deterministic: the columns are chosen by an ordered scan (the RN_MAX longest
// factor columns above the threshold, ties to the lower index, listed in index
// order) and every sum is taken in a fixed order (per-block partials, summed
// in block order by the consumer), so repeated calls on the same input give
// bitwise-identical U.
// ---------------------------------------------------------------------------
constexpr int RN_MAX = 32;      // columns per problem
constexpr int RN_THREADS = 256;

// nrm2[b n + j] = ||M e_(cw j)||^2: blocks of 32 columns x 8 row groups per
// problem, the row groups summed in a fixed order
__global__ void __launch_bounds__(256) rn_norms_kernel(const double* __restrict__ M, int N, int n,
                                                       int cw, int64_t mstride,
                                                       double* __restrict__ nrm2) {
  const int b = blockIdx.y;
  const double* Mb = M + (int64_t)b * mstride;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + tx;
  __shared__ double part[8][33];
  double s = 0.0;
  if (j < n)
    for (int i = ty; i < N; i += 8) {
      const double v = Mb[(int64_t)i * N + (int64_t)cw * j];
      s = fma(v, v, s);
    }
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && j < n) {
    double t = 0.0;
    for (int r = 0; r < 8; ++r) t += part[r][tx];
    nrm2[(int64_t)b * n + j] = t;
  }
}

// one warp per problem: the columns with nrm2 > thr2, at most RN_MAX of them
// (the longest, ties to the lower index), listed in increasing column order
__global__ void __launch_bounds__(32) rn_select_kernel(const double* __restrict__ nrm2, int n,
                                                       double thr2, int* __restrict__ list,
                                                       int* __restrict__ count) {
  const int b = blockIdx.x;
  const int lane = threadIdx.x;
  const double* v = nrm2 + (int64_t)b * n;
  int total = 0;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    total += __popc(__ballot_sync(0xffffffffu, j < n && v[j] > thr2));
  }
  int* out = list + b * RN_MAX;
  if (total <= RN_MAX) {
    int c = 0;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      const bool f = j < n && v[j] > thr2;
      const unsigned bal = __ballot_sync(0xffffffffu, f);
      if (f) out[c + __popc(bal & ((1u << lane) - 1u))] = j;
      c += __popc(bal);
    }
    if (lane == 0) count[b] = total;
    return;
  }
  // more candidates than slots: RN_MAX rounds of a warp arg-max over the
  // columns not yet taken (value above the previous pick's, or equal with a
  // larger index), then the picks are sorted by index
  double pv = INFINITY;
  int pj = -1;
  __shared__ int picks[RN_MAX];
  for (int r = 0; r < RN_MAX; ++r) {
    double bv = -1.0;
    int bj = n;
    for (int j = lane; j < n; j += 32) {
      const double x = v[j];
      const bool avail = x > thr2 && (x < pv || (x == pv && j > pj));
      if (avail && (x > bv || (x == bv && j < bj))) {
        bv = x;
        bj = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
      if (ov > bv || (ov == bv && oj < bj)) {
        bv = ov;
        bj = oj;
      }
    }
    pv = bv;
    pj = bj;
    if (lane == 0) picks[r] = bj;
  }
  __syncwarp();
  if (lane < RN_MAX) {
    const int mine = picks[lane];
    int rank = 0;
    for (int r = 0; r < RN_MAX; ++r) rank += picks[r] < mine;
    out[rank] = mine;
  }
  if (lane == 0) count[b] = RN_MAX;
}

// per-block partial sums of squares of the listed columns (FP32 per thread
// over a few hundred rows, FP64 across the block in a fixed order):
// part[((b RN_MAX) + c) gx + blockIdx.x]
__global__ void __launch_bounds__(RN_THREADS) rn_sumsq_kernel(const float* __restrict__ U,
                                                              int64_t m, int64_t ldu, int cw,
                                                              int64_t ustride,
                                                              const int* __restrict__ list,
                                                              const int* __restrict__ count,
                                                              double* __restrict__ part) {
  const int b = blockIdx.y;
  const int d = min(count[b], RN_MAX);
  if (d == 0) return;
  const float* Ub = U + (int64_t)b * ustride;
  __shared__ double red[RN_THREADS / 32];
  for (int c = 0; c < d; ++c) {
    const int64_t col = (int64_t)cw * list[b * RN_MAX + c];
    float acc = 0.f;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
      const float x = Ub[r * ldu + col];
      acc = fmaf(x, x, acc);
      if (cw == 2) {
        const float y = Ub[r * ldu + col + 1];
        acc = fmaf(y, y, acc);
      }
    }
    double s = warp_sum((double)acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < RN_THREADS / 32; ++w) t += red[w];
      part[((int64_t)b * RN_MAX + c) * gridDim.x + blockIdx.x] = t;
    }
    __syncthreads();
  }
}

// every block sums the partials of each listed column in block order (the
// same fixed order in every block), then scales its rows of that column
__global__ void __launch_bounds__(RN_THREADS) rn_scale_kernel(float* __restrict__ U, int64_t m,
                                                              int64_t ldu, int cw, int64_t ustride,
                                                              const int* __restrict__ list,
                                                              const int* __restrict__ count,
                                                              const double* __restrict__ part) {
  const int b = blockIdx.y;
  const int d = min(count[b], RN_MAX);
  if (d == 0) return;
  float* Ub = U + (int64_t)b * ustride;
  __shared__ double red[RN_THREADS / 32];
  for (int c = 0; c < d; ++c) {
    const double* pc = part + ((int64_t)b * RN_MAX + c) * gridDim.x;
    double t = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) t += pc[k];
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    double s2 = 0.0;
    for (int w = 0; w < RN_THREADS / 32; ++w) s2 += red[w];
    __syncthreads();
    if (!(s2 > 0.0)) continue;
    const float f = (float)(1.0 / sqrt(s2));
    const int64_t col = (int64_t)cw * list[b * RN_MAX + c];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m;
         r += (int64_t)gridDim.x * blockDim.x) {
      Ub[r * ldu + col] *= f;
      if (cw == 2) Ub[r * ldu + col + 1] *= f;
    }
  }
}

}  // namespace hp

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn16() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 3-D fp16 map over two planes of `rows` x `inner` (row pitch ld elements),
// 128-byte swizzle, zero fill out of bounds
// planes as a 3-D tensor {inner, rows, 2}; pstride: elements from the hi to the
// lo plane (0: rows * ld, planes back to back)
static bool make_map_planes(CUtensorMap* map, const __half* base, uint64_t inner, uint64_t rows,
                            uint64_t ld, uint32_t box_inner, uint32_t box_rows,
                            uint64_t pstride = 0, bool sw64 = false) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn16();
  if (!fn) return false;
  if (pstride == 0) pstride = ld * rows;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * 2) & 15) || ((pstride * 2) & 15)) return false;
  cuuint64_t dims[3] = {inner, rows, 2};
  cuuint64_t strides[2] = {ld * 2, pstride * 2};
  cuuint32_t box[3] = {box_inner, box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<__half*>(base), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  sw64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int64_t packed_ld(int64_t N) { return cdiv(N, 64) * 64; }

static void pair_launch_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* at, unsigned grid,
                               unsigned threads, size_t smem, cudaStream_t st) {
  cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
}

// two-CTA clusters of apply16p_kernel<TN> resident at once (0: not available)
template <int TN>
static int pair_clusters() {
  static int n = -1;
  if (n < 0) {
    n = 0;
    if (cudaFuncSetAttribute(hp::apply16p_kernel<TN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hp::pair_smem<TN>()) == cudaSuccess) {
      cudaLaunchConfig_t cfg;
      cudaLaunchAttribute at[1];
      pair_launch_config(cfg, at, 2 * (unsigned)num_sms(), hp::PairCfg<TN>::THREADS,
                         hp::pair_smem<TN>(), 0);
      int c = 0;
      if (cudaOccupancyMaxActiveClusters(&c, hp::apply16p_kernel<TN>, &cfg) == cudaSuccess) n = c;
    }
    cudaGetLastError();
  }
  return n;
}

// rows per problem in the planes: m for one problem; for a batch, m rounded
// up to 128 so that no stage or output tile of one problem reaches the next
int64_t packed_rows(int64_t m, int64_t batch) { return batch > 1 ? cdiv(m, 128) * 128 : m; }

void packed_carve(Arena& ws, Packed& p, int64_t m, int64_t N, int64_t batch) {
  p.m = m;
  p.N = N;
  p.ld = packed_ld(N);
  p.batch = batch;
  p.mp = packed_rows(m, batch);
  p.hi = ws.take<__half>((size_t)(2 * batch * p.mp * p.ld));
  p.lo = p.hi ? p.hi + batch * p.mp * p.ld : nullptr;
  p.scale = ws.take<float>((size_t)(batch * p.ld));
}

Packed packed_rows_view(const Packed& p, int64_t r0, int64_t rows, int64_t mp, float* scale) {
  Packed v = p;
  v.pstride = p.pstride ? p.pstride : p.batch * p.mp * p.ld;
  v.hi = p.hi ? p.hi + r0 * p.ld : nullptr;
  v.lo = p.lo ? p.lo + r0 * p.ld : nullptr;
  v.scale = scale;
  v.m = rows;
  v.mp = mp;
  v.batch = 1;
  return v;
}

void packed_view(Packed& p, void* storage, int64_t m, int64_t N, float* scale, int64_t batch) {
  p.m = m;
  p.N = N;
  p.ld = packed_ld(N);
  p.batch = batch;
  p.mp = packed_rows(m, batch);
  p.hi = static_cast<__half*>(storage);
  p.lo = p.hi ? p.hi + batch * p.mp * p.ld : nullptr;
  p.scale = scale;
}

int pack_f32(const float* Y, int64_t ld, int64_t m, int64_t N, Packed& p, Arena& ws,
             cudaStream_t st, int64_t bstride) {
  const int64_t batch = p.batch;
  unsigned* cmax = ws.take<unsigned>((size_t)(N * batch));
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "pack: workspace too small");
  PLOM_REQUIRE(Y && p.hi && p.scale && cmax && m >= 1 && N >= 1 && ld >= N, PLOM_ERR_ARG,
               "pack: bad arguments");
  PLOM_REQUIRE(batch == 1 || bstride >= m * ld, PLOM_ERR_ARG, "pack: batch stride < m * ld");
  PLOM_CHECK_CUDA(cudaMemsetAsync(cmax, 0, (size_t)(N * batch) * sizeof(unsigned), st));
  const int threads = 256;
  {
    ProfScope prof("colmax", st, 0.0, 4.0 * (double)m * N);
    const int rblocks = (int)std::max<int64_t>(
        1, std::min<int64_t>(m, cdiv((int64_t)num_sms() * 8, batch)));
    const int cvec = ((ld & 3) == 0) && ((N & 3) == 0) && ((bstride & 3) == 0) &&
                     ((reinterpret_cast<uintptr_t>(Y) & 15) == 0);
    hp::colmax_kernel<<<dim3(rblocks, (unsigned)batch), threads, 0, st>>>(Y, ld, m, (int)N, cvec,
                                                                         bstride, cmax);
    PLOM_CHECK_LAUNCH();
    hp::colscale_kernel<<<(int)std::min<int64_t>(cdiv(p.ld * batch, 256), 4096), 256, 0, st>>>(
        cmax, (int)N, (int)p.ld, (int)batch, p.scale);
    PLOM_CHECK_LAUNCH();
  }
  ProfScope prof("pack_f16x2", st, 0.0, 4.0 * (double)m * N * batch + 4.0 * (double)p.mp * p.ld * batch);
  const int vec = ((ld & 3) == 0) && ((reinterpret_cast<uintptr_t>(Y) & 15) == 0);
  const int groups = (int)(p.ld / 8);
  const int rt = std::max(1, 2048 / groups);  // rows per tile: >= 2048 groups when rows are short
  const int64_t tiles = cdiv(p.mp, rt) * batch;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)num_sms() * 8));
  hp::pack_kernel<<<blocks, 256, 0, st>>>(Y, ld, m, (int)N, (int)p.ld, rt, p.scale, p.hi, p.lo,
                                          vec && ((bstride & 3) == 0), bstride, p.mp, (int)batch);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// work items of the Gram: tiles x chunks, the fewest whole waves of the GPU
// (one CTA per SM) that the tile count divides, with chunks of at least four
// stages; fewer chunks keep the partial slabs (and their reduction) small
static int gram16_chunks(int64_t m, int tiles, int bk = hp::G_BK, int wave_mult = 0) {
  const int64_t sms = num_sms();
  const int64_t maxc = std::max<int64_t>(1, cdiv(m, 4 * (int64_t)bk));
  if (wave_mult <= 0) wave_mult = tuning().gram_wave_mult;
  for (int64_t waves = 1; waves <= 64; ++waves) {
    const int64_t items = waves * sms * wave_mult;
    if (items % tiles) continue;
    return (int)std::max<int64_t>(1, std::min(maxc, items / tiles));
  }
  return (int)std::max<int64_t>(1, std::min<int64_t>(maxc, cdiv(2 * sms, tiles)));
}

// Gram of operands wider than 128 columns: 128 x 256 tiles (gram16w_kernel);
// row chunks are whole 4,096-row sub-chunks, each with its own FP32 slab.
// Short chunks keep the tiles of one chunk that run at the same time close
// together in the rows, so that they share its panels in L2 (the slabs do
// not depend on the chunking)
static void wide_chunks(int64_t m, int items_per_chunk, int& chunks_eff, int64_t& rpc,
                        int& subs_per_chunk, int& nsubs) {
  const int chunks =
      gram16_chunks(m, items_per_chunk, hp::G_KSUB / 4, tuning().gram_wide_wave_mult);
  rpc = cdiv(cdiv(m, chunks), hp::G_KSUB) * hp::G_KSUB;
  chunks_eff = (int)std::max<int64_t>(1, cdiv(m, rpc));
  subs_per_chunk = (int)(rpc / hp::G_KSUB);
  nsubs = (int)std::max<int64_t>(1, cdiv(m, hp::G_KSUB));
}

static int gram_packed_wide(const Packed& p, double* G, int* err, Arena& ws, cudaStream_t st,
                            bool accumulate) {
  const int64_t m = p.m, N = p.N, batch = p.batch;
  const int tn = (int)cdiv(p.ld, 128), tn2 = (int)cdiv(p.ld, 256);
  const int tiles = hp::gw_tiles_sym(tn, tn2);
  int chunks_eff, subs_per_chunk, nsubs;
  int64_t rpc;
  wide_chunks(m, (int)std::min<int64_t>(tiles * batch, 1 << 20), chunks_eff, rpc, subs_per_chunk,
              nsubs);
  const int64_t slabs = batch * tiles * (int64_t)nsubs;
  float* part = ws.take<float>((size_t)slabs * 128 * 256);
  double* diagp = ws.take<double>((size_t)slabs * 128);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gram16w: workspace too small");
  PLOM_REQUIRE(p.hi && G && part && m >= 1 && batch * p.mp < (1ll << 31) &&
                   batch * tiles * chunks_eff < (1ll << 31),
               PLOM_ERR_ARG, "gram16w: bad arguments");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16w_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::GW_SMEM));
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16w_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::GW_SMEM));
    attr = true;
  }
  CUtensorMap tm;
  PLOM_REQUIRE(make_map_planes(&tm, p.hi, (uint64_t)p.ld, (uint64_t)(batch * p.mp),
                               (uint64_t)p.ld, 64, hp::GW_BK, (uint64_t)p.pstride),
               PLOM_ERR_CUDA, "gram16w: tensor map encoding failed");
  ProfScope prof_g("tc_gram_f16x3", st, (double)m * N * N * batch, 4.0 * (double)m * p.ld * batch);
  hp::gram16w_kernel<true><<<(unsigned)(batch * tiles * chunks_eff), 320, hp::GW_SMEM, st>>>(
      tm, tm, m, tn, tn2, rpc, chunks_eff, subs_per_chunk, nsubs, part, diagp, err, p.mp, 0);
  PLOM_CHECK_LAUNCH();
  const int64_t units = (int64_t)batch * hp::gw_tiles_sym(tn, tn2) * 128 * 64;
  // a few resident blocks per SM (80 registers a thread), a grid-stride loop
  const int blocks = (int)std::min<int64_t>(
      cdiv(units, 256), (int64_t)num_sms() * tuning().reduce_blocks_per_sm);
  ProfScope prof_r("gram_reduce", st, 0.0, 4.0 * (double)slabs * 128 * 256);
  hp::gram16w_reduce_kernel<<<blocks, 256, 0, st>>>(part, diagp, (int)N, tn, tn2, nsubs, p.scale,
                                                    G, (int)batch, (int)p.ld, accumulate ? 1 : 0, 0);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// Gram of a matrix packed in C row chunks of mc rows (mc a multiple of
// 16 x 4,096), chunk c with its own column scales (scales + c ld): one wide
// Gram launch per chunk, each writing its sub-chunk slabs into one array,
// and one reduction over all of them.  Before chunk c's products the stream
// waits for ready[c] (when given), so that chunks packed on another stream
// are taken as they come.
int gram_packed_chunks(const Packed& p, int C, int64_t mc, const float* scales, double* G,
                       const cudaEvent_t* ready, int* err, Arena& ws, cudaStream_t st) {
  const int64_t N = p.N;
  const int tn = (int)cdiv(p.ld, 128), tn2 = (int)cdiv(p.ld, 256);
  const int tiles = hp::gw_tiles_sym(tn, tn2);
  int chunks_eff, subs_per_chunk, nsubs_c;
  int64_t rpc;
  wide_chunks(mc, tiles, chunks_eff, rpc, subs_per_chunk, nsubs_c);
  const int64_t nsubs = (int64_t)C * nsubs_c;
  const int64_t slabs = tiles * nsubs;
  float* part = ws.take<float>((size_t)slabs * 128 * 256);
  double* diagp = ws.take<double>((size_t)slabs * 128);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gram16w chunks: workspace too small");
  PLOM_REQUIRE(p.hi && G && scales && p.batch == 1 && p.ld > 128 && C >= 1 &&
                   mc % ((int64_t)hp::G_KSUB * hp::GWR_UNROLL) == 0 && p.mp >= (int64_t)C * mc &&
                   nsubs < (1ll << 31),
               PLOM_ERR_ARG, "gram16w chunks: bad arguments");
  PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16w_kernel<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)hp::GW_SMEM));
  for (int c = 0; c < C; ++c) {
    if (ready) PLOM_CHECK_CUDA(cudaStreamWaitEvent(st, ready[c], 0));
    const Packed v = packed_rows_view(p, (int64_t)c * mc, mc, mc, nullptr);
    CUtensorMap tm;
    PLOM_REQUIRE(make_map_planes(&tm, v.hi, (uint64_t)v.ld, (uint64_t)mc, (uint64_t)v.ld, 64,
                                 hp::GW_BK, (uint64_t)v.pstride),
                 PLOM_ERR_CUDA, "gram16w chunks: tensor map encoding failed");
    ProfScope prof_g("tc_gram_f16x3", st, (double)mc * N * N, 4.0 * (double)mc * p.ld);
    hp::gram16w_kernel<true><<<(unsigned)(tiles * chunks_eff), 320, hp::GW_SMEM, st>>>(
        tm, tm, mc, tn, tn2, rpc, chunks_eff, subs_per_chunk, (int)nsubs, part, diagp, err, mc,
        (int64_t)c * nsubs_c);
    PLOM_CHECK_LAUNCH();
  }
  const int64_t units = (int64_t)tiles * 128 * 64;
  const int blocks = (int)std::min<int64_t>(
      cdiv(units, 256), (int64_t)num_sms() * tuning().reduce_blocks_per_sm);
  ProfScope prof_r("gram_reduce", st, 0.0, 4.0 * (double)slabs * 128 * 256);
  hp::gram16w_reduce_kernel<<<blocks, 256, 0, st>>>(part, diagp, (int)N, tn, tn2, (int)nsubs, scales,
                                                    G, 1, (int)p.ld, 0, nsubs_c);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

int gram_packed(const Packed& p, double* G, int* err, Arena& ws, cudaStream_t st,
                bool accumulate) {
  if (p.ld > 128) return gram_packed_wide(p, G, err, ws, st, accumulate);
  const int64_t m = p.m, N = p.N, batch = p.batch;
  const int tn = (int)cdiv(p.ld, 128);
  const int tiles = tn * (tn + 1) / 2;
  const int chunks = gram16_chunks(m, (int)std::min<int64_t>(tiles * batch, 1 << 20));
  int64_t rpc = cdiv(m, chunks);
  rpc = cdiv(rpc, hp::G_BK) * hp::G_BK;  // chunk boundaries on stage boundaries
  const int chunks_eff = (int)std::max<int64_t>(1, cdiv(m, rpc));
  double* part = ws.take<double>((size_t)(batch * tiles * chunks_eff) * 128 * 128);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "gram16: workspace too small");
  PLOM_REQUIRE(p.hi && G && part && m >= 1 && batch * p.mp < (1ll << 31) &&
                   batch * tiles * chunks_eff < (1ll << 31),
               PLOM_ERR_ARG, "gram16: bad arguments");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::G_SMEM));
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::G_SMEM));
    attr = true;
  }
  CUtensorMap tm;
  PLOM_REQUIRE(make_map_planes(&tm, p.hi, (uint64_t)p.ld, (uint64_t)(batch * p.mp),
                               (uint64_t)p.ld, 64, hp::G_BK, (uint64_t)p.pstride),
               PLOM_ERR_CUDA, "gram16: tensor map encoding failed");
  ProfScope prof_g("tc_gram_f16x3", st, (double)m * N * N * batch, 4.0 * (double)m * p.ld * batch);
  hp::gram16_kernel<true><<<(unsigned)(batch * tiles * chunks_eff), 320, hp::G_SMEM, st>>>(
      tm, tm, m, tn, tn, rpc, chunks_eff, part, err, p.mp);
  PLOM_CHECK_LAUNCH();
  const int64_t total = N * N * batch;
  const int blocks = (int)std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16);
  ProfScope prof_r("gram_reduce", st, 0.0, 8.0 * (double)batch * tiles * chunks_eff * 128 * 128);
  hp::gram16_reduce_kernel<<<blocks, 256, 0, st>>>(part, (int)N, tn, chunks_eff, p.scale, G,
                                                   (int)batch, (int)p.ld, accumulate ? 1 : 0);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

// A^T B with B wider than 128 columns: 128 x 256 tiles (gram16w_kernel<false>)
static int tn_packed_wide(const Packed& a, const Packed& b, double* C, int64_t ldc, int* err,
                          Arena& ws, cudaStream_t st) {
  const int64_t m = a.m;
  const int tna = (int)cdiv(a.ld, 128), tn2 = (int)cdiv(b.ld, 256);
  const int tiles = tna * tn2;
  int chunks_eff, subs_per_chunk, nsubs;
  int64_t rpc;
  wide_chunks(m, tiles, chunks_eff, rpc, subs_per_chunk, nsubs);
  const int64_t slabs = tiles * (int64_t)nsubs;
  float* part = ws.take<float>((size_t)slabs * 128 * 256);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tn16w: workspace too small");
  PLOM_REQUIRE(a.hi && b.hi && C && part && m >= 1 && m < (1ll << 31) && b.m == m &&
                   ldc >= b.N && a.batch == 1 && b.batch == 1,
               PLOM_ERR_ARG, "tn16w: bad arguments");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16w_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::GW_SMEM));
    attr = true;
  }
  CUtensorMap ta, tb;
  PLOM_REQUIRE(make_map_planes(&ta, a.hi, (uint64_t)a.ld, (uint64_t)m, (uint64_t)a.ld, 64,
                               hp::GW_BK, (uint64_t)a.pstride) &&
                   make_map_planes(&tb, b.hi, (uint64_t)b.ld, (uint64_t)m, (uint64_t)b.ld, 64,
                                   hp::GW_BK, (uint64_t)b.pstride),
               PLOM_ERR_CUDA, "tn16w: tensor map encoding failed");
  {
    ProfScope prof("tc_tn_f16x3", st, 2.0 * (double)m * a.N * b.N,
                   4.0 * (double)m * (a.ld + b.ld));
    hp::gram16w_kernel<false><<<tiles * chunks_eff, 320, hp::GW_SMEM, st>>>(
        ta, tb, m, tna, tn2, rpc, chunks_eff, subs_per_chunk, nsubs, part, nullptr, err, m, 0);
    PLOM_CHECK_LAUNCH();
  }
  const int64_t total = a.N * b.N;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16));
  hp::tn16w_reduce_kernel<<<blocks, 256, 0, st>>>(part, (int)a.N, (int)b.N, tn2, nsubs, a.scale,
                                                  b.scale, C, ldc);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

int tn_packed(const Packed& a, const Packed& b, double* C, int64_t ldc, int* err, Arena& ws,
              cudaStream_t st) {
  if (b.ld > 128) return tn_packed_wide(a, b, C, ldc, err, ws, st);
  const int64_t m = a.m;
  const int tna = (int)cdiv(a.ld, 128), tnb = (int)cdiv(b.ld, 128);
  const int tiles = tna * tnb;
  const int chunks = gram16_chunks(m, tiles);
  int64_t rpc = cdiv(m, chunks);
  rpc = cdiv(rpc, hp::G_BK) * hp::G_BK;
  const int chunks_eff = (int)std::max<int64_t>(1, cdiv(m, rpc));
  double* part = ws.take<double>((size_t)tiles * chunks_eff * 128 * 128);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tn16: workspace too small");
  PLOM_REQUIRE(a.hi && b.hi && C && part && m >= 1 && m < (1ll << 31) && b.m == m &&
                   ldc >= b.N && a.batch == 1 && b.batch == 1,
               PLOM_ERR_ARG, "tn16: bad arguments");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::gram16_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::G_SMEM));
    attr = true;
  }
  CUtensorMap ta, tb;
  PLOM_REQUIRE(make_map_planes(&ta, a.hi, (uint64_t)a.ld, (uint64_t)m, (uint64_t)a.ld, 64, hp::G_BK,
                               (uint64_t)a.pstride) &&
                   make_map_planes(&tb, b.hi, (uint64_t)b.ld, (uint64_t)m, (uint64_t)b.ld, 64, hp::G_BK,
                                   (uint64_t)b.pstride),
               PLOM_ERR_CUDA, "tn16: tensor map encoding failed");
  {
    ProfScope prof("tc_tn_f16x3", st, 2.0 * (double)m * a.N * b.N,
                   4.0 * (double)m * (a.ld + b.ld));
    hp::gram16_kernel<false><<<tiles * chunks_eff, 320, hp::G_SMEM, st>>>(
        ta, tb, m, tna, tnb, rpc, chunks_eff, part, err, m);
    PLOM_CHECK_LAUNCH();
  }
  const int64_t total = a.N * b.N;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16));
  hp::tn16_reduce_kernel<<<blocks, 256, 0, st>>>(part, (int)a.N, (int)b.N, tnb, chunks_eff, a.scale,
                                                 b.scale, C, ldc);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

int apply_packed(const Packed& p, const double* W, int64_t ldw, int64_t k, float* C, int64_t ldc,
                 Packed* out, int* err, Arena& ws, cudaStream_t st, int64_t wstride,
                 int64_t cstride, bool upper) {
  const int64_t m = p.m, batch = p.batch;
  const int64_t ldk = p.ld;  // K extent of the W copies (= packed pitch of the input)
  // output tile width (see ApplyCfg): 256 for dense W wider than 128 columns.
  // An upper-triangular W keeps 128-wide tiles: its short column tiles (the
  // first K blocks only) finish their products faster than the single
  // 256-wide accumulator is drained, while the 128-wide kernel's two
  // accumulator buffers overlap them (measured: 0.70 of the dense product's
  // time for 0.56 of its products, against 0.75 with 256-wide tiles and
  // 128-wide products on the diagonal band)
  const bool tri_w = upper && k == p.N;
  // SM pairs (apply16p_kernel) for one problem wider than 128 columns, when
  // enabled for its kind of W and the device runs two-CTA clusters of it:
  // 256 x 256 tiles for a dense W, 256 x 128 tiles for a triangular one
  const int pair_tn = (batch != 1 || k <= 128) ? 0
                      : (!tri_w && tuning().apply_pair >= 1 && pair_clusters<256>() > 0) ? 256
                      : (tri_w && tuning().apply_pair == 2 && pair_clusters<128>() > 0) ? 128
                                                                                      : 0;
  const bool pair = pair_tn != 0;
  const int TN = pair ? pair_tn : (k > 128 && !tri_w) ? tuning().apply_dense_tn : 128;
  const int64_t col_tiles = cdiv(k, TN);
  const int fstride = (int)(col_tiles * TN);
  __half* bhi = ws.take<__half>((size_t)(2 * batch * k * ldk));
  __half* blo = bhi ? bhi + batch * k * ldk : nullptr;
  float* f = ws.take<float>((size_t)(batch * fstride));
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "apply16: workspace too small");
  PLOM_REQUIRE(p.hi && W && (C || out) && m >= 1 && batch * p.mp < (1ll << 31) && k >= 1 &&
                   batch * k < (1ll << 31),
               PLOM_ERR_ARG, "apply16: bad arguments");
  PLOM_REQUIRE(batch == 1 || ((wstride == 0 || wstride >= p.N * ldw) && (out || cstride >= m * ldc)),
               PLOM_ERR_ARG, "apply16: batch strides too small");
  if (out) PLOM_REQUIRE(out->hi && out->scale && out->m == m && out->N == k && out->batch == batch &&
                            out->mp == p.mp,
                        PLOM_ERR_ARG, "apply16: bad packed output");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::apply16_kernel<128>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::apply_smem<128>()));
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(hp::apply16_kernel<256>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)hp::apply_smem<256>()));
    attr = true;
  }
  const float out_scale = out ? (float)(1 << hp::PK_LOG2) : 1.0f;
  hp::split_w16_kernel<<<dim3((unsigned)fstride, (unsigned)batch), 256, 0, st>>>(
      W, ldw, (int)p.N, (int)k, (int)ldk, p.scale, out_scale, bhi, blo, f, wstride, fstride);
  PLOM_CHECK_LAUNCH();
  if (out) {
    // packed output columns carry the fixed scale 2^14
    hp::fill_scale_kernel<<<(int)std::min<int64_t>(cdiv(out->ld * batch, 256), 4096), 256, 0, st>>>(
        out->scale, out->ld * batch, out_scale);
    PLOM_CHECK_LAUNCH();
  }
  CUtensorMap tmA, tmB;
  const uint32_t bk = TN == 256 ? (uint32_t)hp::ApplyCfg<256>::BK : (uint32_t)hp::ApplyCfg<128>::BK;
  static_assert(hp::ApplyCfg<256>::BK == hp::PairCfg<256>::BK &&
                    hp::ApplyCfg<128>::BK == hp::PairCfg<128>::BK,
                "pair tiles use the single-SM kernels' K depth");
  // B boxes: TN rows of W (single SM, in boxes of 128) or the CTA's half (pair)
  const uint32_t b_rows = pair ? (uint32_t)(TN / 2) : 128u;
  PLOM_REQUIRE(make_map_planes(&tmA, p.hi, (uint64_t)p.ld, (uint64_t)(batch * p.mp),
                               (uint64_t)p.ld, bk, 128, (uint64_t)p.pstride, bk == 32) &&
                   make_map_planes(&tmB, bhi, (uint64_t)ldk, (uint64_t)(batch * k), (uint64_t)ldk,
                                   bk, b_rows, 0, bk == 32),
               PLOM_ERR_CUDA, "apply16: tensor map encoding failed");
  const int64_t row_tiles = cdiv(p.mp, 128);
  const int64_t tiles = batch * row_tiles * col_tiles;
  // whole row blocks per CTA pay for the triangular case (column tiles of very
  // different lengths; interleaved single tiles measured 10 % slower there);
  // the dense case keeps concurrent tiles of one row block on different SMs
  // (fewer DRAM re-reads)
  const int by_rows = ((tri_w ? tuning().apply_tri_by_rows : tuning().apply_dense_by_rows) &&
                       batch * row_tiles >= 2 * num_sms())
                          ? 1
                          : 0;
  const int grid = (int)std::min<int64_t>(by_rows ? batch * row_tiles : tiles, num_sms());
  hp::ApplyOut o;
  o.C = out ? nullptr : C;
  o.ldc = ldc;
  o.cstride = cstride;
  o.ohi = out ? out->hi : nullptr;
  o.olo = out ? out->lo : nullptr;
  o.ldo = out ? (int)out->ld : 0;
  // an upper-triangular W (k = N) needs m N (N + 1) flops: row i of W meets
  // columns j >= i only
  const bool tri = tri_w;
  const double flops = tri ? (double)m * p.N * (p.N + 1) * batch : 2.0 * m * p.N * k * batch;
  ProfScope prof(pair ? "tc_apply_f16x3_pair" : "tc_apply_f16x3", st, flops,
                 4.0 * ((double)m * p.ld + (double)m * k) * batch);
  if (pair) {
    const int clusters_max = TN == 256 ? pair_clusters<256>() : pair_clusters<128>();
    const int64_t pairs = cdiv(p.mp, 256), ptiles = pairs * col_tiles;
    const int pby_rows =
        ((tri ? tuning().apply_tri_by_rows : tuning().apply_dense_by_rows) &&
         pairs >= 2 * (int64_t)clusters_max)
            ? 1
            : 0;
    const int64_t clusters = std::min<int64_t>(pby_rows ? pairs : ptiles, clusters_max);
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at[1];
    if (TN == 256) {
      pair_launch_config(cfg, at, (unsigned)(2 * clusters), hp::PairCfg<256>::THREADS,
                         hp::pair_smem<256>(), st);
      PLOM_CHECK_CUDA(cudaLaunchKernelEx(&cfg, hp::apply16p_kernel<256>, tmA, tmB, m,
                                         (int)(ldk / hp::PairCfg<256>::BK), (int)k, col_tiles,
                                         ptiles, (const float*)f, o, err, p.mp, tri ? 1 : 0,
                                         pby_rows));
    } else {
      pair_launch_config(cfg, at, (unsigned)(2 * clusters), hp::PairCfg<128>::THREADS,
                         hp::pair_smem<128>(), st);
      PLOM_CHECK_CUDA(cudaLaunchKernelEx(&cfg, hp::apply16p_kernel<128>, tmA, tmB, m,
                                         (int)(ldk / hp::PairCfg<128>::BK), (int)k, col_tiles,
                                         ptiles, (const float*)f, o, err, p.mp, tri ? 1 : 0,
                                         pby_rows));
    }
    PLOM_CHECK_LAUNCH();
    return PLOM_OK;
  }
  if (TN == 256)
    hp::apply16_kernel<256><<<grid, hp::ApplyWarps<256>::THREADS, hp::apply_smem<256>(), st>>>(
        tmA, tmB, m, (int)(ldk / hp::ApplyCfg<256>::BK), (int)k, col_tiles, tiles, f, o, err, p.mp,
        row_tiles, fstride, tri ? 1 : 0, by_rows);
  else
    hp::apply16_kernel<128><<<grid, hp::ApplyWarps<128>::THREADS, hp::apply_smem<128>(), st>>>(
        tmA, tmB, m, (int)(ldk / 64), (int)k, col_tiles, tiles, f, o, err, p.mp, row_tiles,
        fstride, tri ? 1 : 0, by_rows);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

}  // namespace plom

namespace plom {

// U = Q2 M in the mixed form: a column of M much longer than 1 means R3^-1
// is large in a direction that Q2 barely spans -- X is numerically
// rank-deficient below the 22-bit operand precision (e.g. the null vector of
// mean-removed snapshots) -- and the FP32 product loses that column's unit
// norm (its orthogonality to the other columns stays at the operand level).
// Such columns (||M e_j|| > 4; the RN_MAX = 32 longest per problem) are
// renormalised in the tall space: two strided passes over each column.  The
// choice of columns and every sum are deterministic (see the kernels).
int renorm_long_columns(const double* M, int N, int n, int cw, float* U, int64_t m, int64_t ldu,
                        int batch, int64_t mstride, int64_t ustride, Arena& ws, cudaStream_t st) {
  const unsigned gx = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(cdiv(m, hp::RN_THREADS), (int64_t)num_sms() * 4));
  int* list = ws.take<int>((size_t)batch * hp::RN_MAX);
  int* count = ws.take<int>((size_t)batch);
  double* nrm2 = ws.take<double>((size_t)batch * n);
  double* part = ws.take<double>((size_t)batch * hp::RN_MAX * gx);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "renorm: workspace too small");
  PLOM_REQUIRE(M && U && batch >= 1 && batch <= 65535, PLOM_ERR_ARG, "renorm: bad arguments");
  ProfScope prof("renorm_cols", st, 0.0, 8.0 * (double)m * batch, 4);
  hp::rn_norms_kernel<<<dim3((unsigned)cdiv(n, 32), (unsigned)batch), 256, 0, st>>>(M, N, n, cw,
                                                                                   mstride, nrm2);
  PLOM_CHECK_LAUNCH();
  hp::rn_select_kernel<<<(unsigned)batch, 32, 0, st>>>(nrm2, n, 16.0, list, count);
  PLOM_CHECK_LAUNCH();
  hp::rn_sumsq_kernel<<<dim3(gx, (unsigned)batch), hp::RN_THREADS, 0, st>>>(U, m, ldu, cw, ustride,
                                                                           list, count, part);
  PLOM_CHECK_LAUNCH();
  hp::rn_scale_kernel<<<dim3(gx, (unsigned)batch), hp::RN_THREADS, 0, st>>>(U, m, ldu, cw, ustride,
                                                                           list, count, part);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

}  // namespace plom

// ---------------------------------------------------------------------------
// C ABI: packed tall operands kept by the caller.  A buffer holds the two
// fp16 planes (m x ld each), the ld column scales and the column-maxima
// scratch of the packing; products read it as often as the caller needs (the
// streaming range finder packs a batch of snapshots once for all its
// products).
// ---------------------------------------------------------------------------
using namespace plom;

namespace {
struct PackedBuf {
  Packed p;
  char* scratch;
  size_t scratch_bytes;
};
size_t packed_buf_layout(int64_t m, int64_t N, void* base, PackedBuf* out) {
  Arena a(base, ~size_t(0) >> 1);
  Packed p;
  packed_carve(a, p, m, N);
  const size_t scr0 = (a.off + 255) / 256 * 256;
  a.off = scr0 + sizeof(unsigned) * (size_t)N + 256;
  if (out) {
    out->p = p;
    out->scratch = base ? static_cast<char*>(base) + scr0 : nullptr;
    out->scratch_bytes = sizeof(unsigned) * (size_t)N + 256;
  }
  return a.off;
}
}  // namespace

extern "C" size_t plom_packed_bytes(int64_t m, int64_t N) {
  if (m < 1 || N < 1) return 0;
  return packed_buf_layout(m, N, nullptr, nullptr);
}

extern "C" int plom_pack(const void* X, int64_t m, int64_t N, int64_t ldx, void* packed,
                         size_t bytes, void* stream) {
  PLOM_REQUIRE(X && packed && m >= 1 && N >= 1 && ldx >= N, PLOM_ERR_ARG, "pack: bad arguments");
  PLOM_REQUIRE(m < (1ll << 31), PLOM_ERR_UNSUPPORTED, "pack: m >= 2^31");
  PLOM_REQUIRE(bytes >= plom_packed_bytes(m, N), PLOM_ERR_WORKSPACE, "pack: buffer too small");
  PackedBuf b;
  packed_buf_layout(m, N, packed, &b);
  Arena scr(b.scratch, b.scratch_bytes);
  return pack_f32(static_cast<const float*>(X), ldx, m, N, b.p, scr, (cudaStream_t)stream);
}

extern "C" size_t plom_packed_apply_workspace(int64_t m, int64_t N, int64_t k) {
  if (m < 1 || N < 1 || k < 1) return 0;
  Packed p;
  Arena a(nullptr, 0);
  packed_carve(a, p, m, N);  // only to size the product's own workspace below
  Arena w(nullptr, 0);
  apply_packed(p, nullptr, k, k, nullptr, k, nullptr, nullptr, w, 0);
  return w.off + 1024;
}

extern "C" int plom_packed_apply(const void* packed, int64_t m, int64_t N, const double* W,
                                 int64_t ldw, int64_t k, void* C, int64_t ldc, void* ws,
                                 size_t ws_bytes, int* info, void* stream) {
  PLOM_REQUIRE(packed && W && C && ws && info && m >= 1 && N >= 1 && k >= 1 && ldw >= k &&
                   ldc >= k,
               PLOM_ERR_ARG, "packed_apply: bad arguments");
  PLOM_REQUIRE(ws_bytes >= plom_packed_apply_workspace(m, N, k), PLOM_ERR_WORKSPACE,
               "packed_apply: workspace too small");
  PackedBuf b;
  packed_buf_layout(m, N, const_cast<void*>(packed), &b);
  Arena a(ws, ws_bytes);
  return apply_packed(b.p, W, ldw, k, static_cast<float*>(C), ldc, nullptr, info, a,
                      (cudaStream_t)stream);
}

extern "C" size_t plom_packed_tn_workspace(int64_t m, int64_t Na, int64_t Nb) {
  if (m < 1 || Na < 1 || Nb < 1) return 0;
  Packed pa, pb;
  Arena a(nullptr, 0);
  packed_carve(a, pa, m, Na);
  packed_carve(a, pb, m, Nb);
  Arena w(nullptr, 0);
  tn_packed(pa, pb, nullptr, Nb, nullptr, w, 0);
  return w.off + 1024;
}

extern "C" int plom_packed_tn(const void* pa, int64_t Na, const void* pb, int64_t Nb, int64_t m,
                              double* C, int64_t ldc, void* ws, size_t ws_bytes, int* info,
                              void* stream) {
  PLOM_REQUIRE(pa && pb && C && ws && info && m >= 1 && Na >= 1 && Nb >= 1 && ldc >= Nb,
               PLOM_ERR_ARG, "packed_tn: bad arguments");
  PLOM_REQUIRE(ws_bytes >= plom_packed_tn_workspace(m, Na, Nb), PLOM_ERR_WORKSPACE,
               "packed_tn: workspace too small");
  PackedBuf a, b;
  packed_buf_layout(m, Na, const_cast<void*>(pa), &a);
  packed_buf_layout(m, Nb, const_cast<void*>(pb), &b);
  Arena w(ws, ws_bytes);
  return tn_packed(a.p, b.p, C, ldc, info, w, (cudaStream_t)stream);
}
