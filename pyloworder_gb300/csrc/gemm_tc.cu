// Tensor-core (tcgen05, sm_103a) kernels of the mixed precision form.
//
// Both kernels compute FP32-accurate products of FP32 data on the TF32
// tensor pipe by splitting every operand x into hi = rna_tf32(x) and
// lo = rna_tf32(x - hi) and accumulating hi*hi + hi*lo + lo*hi (three UMMA
// per k-step; the dropped lo*lo term is below 2^-22 |x y|).  Operands live in
// shared memory in the K-major, 128-byte-swizzled canonical layout; the
// accumulator lives in TMEM and is read back with tcgen05.ld.
//
//  tc_apply  C(m x k) = A(m x N) W(N x k): the tall-times-small products of
//            the TSQR (Q = X R^-1, U = Q M).  W is split once on the device
//            into K-major hi/lo copies (k x N).
//  tc_gram   G(N x N) = A^T A over the m rows: the Gram/R-merge of the TSQR.
//            Upper 128 x 128 tiles x row chunks; every 4096 rows the FP32
//            TMEM accumulator is drained into a per-work-item FP64 partial,
//            so FP32 accumulation never spans more than 4096 terms; the
//            partials are summed in FP64 in a fixed order.
//
// Warp roles (one CTA per SM; ~193 KB shared memory):
//  apply: warps 0-3 load + split operands and later run the epilogue,
//         warp 4 allocates TMEM and one lane issues the UMMA.
//  gram:  warps 0-3 drain TMEM (epilogue), warps 4-7 load + transpose + split,
//         warp 8 issues the UMMA.
// Every mbarrier wait is bounded (%globaltimer, ~2 s); on expiry the CTA
// records PLOM_NUM_TIMEOUT in the caller's info word, stops issuing work,
// frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "plom_common.cuh"
#include "plom_kernels.cuh"
#include "plom_tc.cuh"

namespace plom {
namespace tc {

constexpr int BM = 128;             // UMMA M (rows of the accumulator)
constexpr int BK = 32;              // K per stage: one 128-byte swizzle row of fp32
constexpr uint32_t ROWB = 128;      // bytes per operand row per stage
constexpr uint64_t WAIT_NS = 2000000000ull;

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
// Bounded wait.  Returns false (and raises the CTA abort flag) on expiry or
// when another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  uint32_t spins = 0;
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if ((++spins & 1023u) == 0 && err && *(volatile int*)err == PLOM_NUM_TIMEOUT) {
      *abort_flag = 1;  // another CTA of this launch gave up: stop too
      return false;
    }
    if (gtimer() - t0 > WAIT_NS) {
      *abort_flag = 1;
      if (err) atomicMax(err, PLOM_NUM_TIMEOUT);
      return false;
    }
  }
}

// A CTA that starts after another CTA of the same launch timed out skips its
// work (the launch's result is already invalid and reported).
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
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
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
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row core
// groups 1024 bytes apart (SBO), sm_100 descriptor version 1.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;             // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;  // SBO
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}
// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float rna_tf32(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return __uint_as_float(u);
}

// byte offset of (row, 16-byte chunk) inside a K-major SW128 operand tile
__device__ __forceinline__ uint32_t sw128(uint32_t row, uint32_t chunk) {
  return row * ROWB + ((chunk ^ (row & 7u)) << 4);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float4 v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}
__device__ __forceinline__ void st_shared_f32(uint32_t addr, float v) {
  asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// 2-D tiled TMA load (box defined by the tensor map) into shared memory,
// completion signalled on `bar` as transaction bytes.  x = innermost
// coordinate (a multiple of 4 fp32 = 16 bytes at every call site).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}
__device__ __forceinline__ float4 ld_shared_v4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}

// four consecutive elements of row `row`, columns [col, col+4), zero outside
// (rows >= nrows or columns >= ncols); vector load when fully inside and aligned
__device__ __forceinline__ float4 load4(const float* __restrict__ P, int64_t ld, int64_t row,
                                        int64_t nrows, int64_t col, int64_t ncols, bool vec_ok) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (row >= nrows) return v;
  const float* p = P + row * ld + col;
  if (vec_ok && col + 4 <= ncols) return __ldg(reinterpret_cast<const float4*>(p));
  if (col + 0 < ncols) v.x = p[0];
  if (col + 1 < ncols) v.y = p[1];
  if (col + 2 < ncols) v.z = p[2];
  if (col + 3 < ncols) v.w = p[3];
  return v;
}

__device__ __forceinline__ void split4(float4 v, float4& hi, float4& lo) {
  hi.x = rna_tf32(v.x);
  hi.y = rna_tf32(v.y);
  hi.z = rna_tf32(v.z);
  hi.w = rna_tf32(v.w);
  lo.x = rna_tf32(v.x - hi.x);
  lo.y = rna_tf32(v.y - hi.y);
  lo.z = rna_tf32(v.z - hi.z);
  lo.w = rna_tf32(v.w - hi.w);
}

// ---------------------------------------------------------------------------
// W (N x k, FP64) -> WhiT, WloT (k x N, K-major fp32)
// ---------------------------------------------------------------------------
template <typename TW>
__global__ void split_w_kernel(const TW* __restrict__ W, int64_t N, int64_t k, int64_t ldw,
                               float* __restrict__ Whi, float* __restrict__ Wlo, int64_t ldo) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ldo * k;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = e / ldo, i = e % ldo;
    double w = (i < N) ? (double)W[i * ldw + j] : 0.0;  // pad columns N..ldo-1 with zeros
    float hi = rna_tf32((float)w);
    float lo = rna_tf32((float)(w - (double)hi));
    Whi[e] = hi;
    Wlo[e] = lo;
  }
}

// ---------------------------------------------------------------------------
// apply: C(m x k) = A(m x K) W(K x k)
// ---------------------------------------------------------------------------
constexpr int AP_BN = 128;
constexpr int AP_STAGES = 3;
constexpr uint32_t AP_A_BYTES = BM * ROWB;
constexpr uint32_t AP_B_BYTES = AP_BN * ROWB;
constexpr uint32_t AP_STAGE_BYTES = 2 * AP_A_BYTES + 2 * AP_B_BYTES;
constexpr size_t AP_SMEM = (size_t)AP_STAGES * AP_STAGE_BYTES + 1024;

__global__ void __launch_bounds__(160, 1)
    tc_apply_kernel(const float* __restrict__ A, int64_t lda, int64_t m, int K,
                    const float* __restrict__ Bhi, const float* __restrict__ Blo, int ldb,
                    int ncols, int64_t col_tiles, float* __restrict__ C, int64_t ldc, int a_vec,
                    int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[AP_STAGES], empty_bar[AP_STAGES], acc_bar;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = blockIdx.x;
  const int64_t m0 = (tile / col_tiles) * BM;
  const int n0 = (int)(tile % col_tiles) * AP_BN;
  const int KB = (K + BK - 1) / BK;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < AP_STAGES; ++s) {
      mbar_init(&full_bar[s], 128);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == 4) {
    tmem_alloc(&tmem_sh, 2 * AP_BN);  // main hi*hi + correction hi*lo + lo*hi
    tmem_relinquish();
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;

  if (warp < 4) {
    // ---- producers: load + split A and copy pre-split B into SW128 tiles
    const int t = threadIdx.x;
    const int c = t & 7;
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % AP_STAGES;
      const uint32_t ph = (uint32_t)(kb / AP_STAGES) & 1u;
      if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) break;
      const uint32_t st = base + s * AP_STAGE_BYTES;
      const uint32_t sAhi = st, sAlo = st + AP_A_BYTES;
      const uint32_t sBhi = st + 2 * AP_A_BYTES, sBlo = sBhi + AP_B_BYTES;
      const int64_t col = (int64_t)kb * BK + 4 * c;
#pragma unroll 4
      for (int i = 0; i < BM / 16; ++i) {
        const int r = (t >> 3) + 16 * i;
        float4 v = load4(A, lda, m0 + r, m, col, K, a_vec != 0);
        float4 hi, lo;
        split4(v, hi, lo);
        const uint32_t off = sw128(r, c);
        st_shared_v4(sAhi + off, hi);
        st_shared_v4(sAlo + off, lo);
      }
#pragma unroll 4
      for (int i = 0; i < AP_BN / 16; ++i) {
        const int r = (t >> 3) + 16 * i;
        const uint32_t off = sw128(r, c);
        st_shared_v4(sBhi + off, load4(Bhi, ldb, (int64_t)n0 + r, ncols, col, K, true));
        st_shared_v4(sBlo + off, load4(Blo, ldb, (int64_t)n0 + r, ncols, col, K, true));
      }
      fence_proxy_async();
      mbar_arrive(&full_bar[s]);
    }
  } else if (lane == 0) {
    // ---- UMMA issuer
    constexpr uint32_t idesc = idesc_tf32(BM, AP_BN);
    bool ok = true;
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % AP_STAGES;
      const uint32_t ph = (uint32_t)(kb / AP_STAGES) & 1u;
      if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t st = base + s * AP_STAGE_BYTES;
      const uint64_t dAhi = desc_sw128(st), dAlo = desc_sw128(st + AP_A_BYTES);
      const uint64_t dBhi = desc_sw128(st + 2 * AP_A_BYTES);
      const uint64_t dBlo = desc_sw128(st + 2 * AP_A_BYTES + AP_B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 8; ++kk) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;  // 8 tf32 = 32 bytes along K
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        mma_tf32(tmem, dAhi + adv, dBhi + adv, idesc, acc);
        mma_tf32(tmem + AP_BN, dAhi + adv, dBlo + adv, idesc, acc);
        mma_tf32(tmem + AP_BN, dAlo + adv, dBhi + adv, idesc, 1u);
      }
      mma_commit(&empty_bar[s]);
    }
    if (ok) mma_commit(&acc_bar);
  }

  if (warp < 4) {
    // ---- epilogue: TMEM -> registers -> C
    const bool ready = mbar_wait(&acc_bar, 0, &abort_sh, err);
    __syncwarp();
    if (__all_sync(0xffffffffu, ready)) {
      fence_after();
      const int64_t row = m0 + warp * 32 + lane;
      const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
      for (int cc = 0; cc < AP_BN / 32; ++cc) {
        uint32_t r[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32);
        tmem_ld32(ta, r);
        tmem_ld32(ta + AP_BN, rc);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j)
          r[j] = __float_as_uint(__uint_as_float(r[j]) + __uint_as_float(rc[j]));
        const int col0 = n0 + cc * 32;
        if (row < m && col0 < ncols) {
          float* dst = C + row * ldc + col0;
          if (vec && col0 + 32 <= ncols) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(dst + j) =
                  make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                              __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (col0 + j < ncols) dst[j] = __uint_as_float(r[j]);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 4) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, 2 * AP_BN);
  }
}

// ---------------------------------------------------------------------------
// gram: upper 128x128 tiles of A^T A, split over row chunks
// ---------------------------------------------------------------------------
constexpr int GR_BN = 128;
constexpr int GR_STAGES = 3;
// Rows accumulated in TMEM (FP32) before the FP64 drain.  The tensor core's
// FP32 accumulation truncates on every UMMA, so the bias grows with the number
// of UMMA per drain; 2048 rows = 256 UMMA per accumulator keeps it near
// 7e-6 relative on off-diagonal entries, and the diagonal (sums of squares,
// where the bias does not cancel) is computed separately on the CUDA cores
// with compensated FP32 sums (Kahan) folded into FP64 at every drain.
constexpr int GR_KSUB = 2048;
constexpr uint32_t GR_T_BYTES = BM * ROWB;  // one 128 x 32 fp32 operand tile
constexpr uint32_t GR_STAGE_BYTES = 4 * GR_T_BYTES;
constexpr size_t GR_SMEM = (size_t)GR_STAGES * GR_STAGE_BYTES + 1024;
constexpr uint32_t GR_TMEM_COLS = 512;  // 2 buffers x (main 128 + correction 128)

__global__ void __launch_bounds__(288, 1)
    tc_gram_kernel(const float* __restrict__ A, int64_t lda, int64_t m, int N, int tn,
                   int64_t rows_per_chunk, int chunks, double* __restrict__ part, int a_vec,
                   int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full_bar[GR_STAGES], empty_bar[GR_STAGES], tfull[2], tempty[2], dfull[2];
  __shared__ double diag_sh[2][BM];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // work item -> (upper tile ti <= tj, chunk)
  // consecutive CTAs take different tiles of the same row chunk, so the CTAs
  // resident together read the same rows and share them through L2
  const int ntiles_all = tn * (tn + 1) / 2;
  const int chunk = (int)(blockIdx.x / ntiles_all), tile = (int)(blockIdx.x % ntiles_all);
  const int item = tile * chunks + chunk;  // partial slab index (tile-major)
  int ti = 0, rem = tile;
  while (rem >= tn - ti) {
    rem -= tn - ti;
    ++ti;
  }
  const int tj = ti + rem;
  const bool diag = (ti == tj);
  const int I0 = ti * BM, J0 = tj * GR_BN;
  const int64_t r_beg = (int64_t)chunk * rows_per_chunk;
  const int64_t r_end = (r_beg + rows_per_chunk < m) ? r_beg + rows_per_chunk : m;
  const int64_t nrows = (r_end > r_beg) ? r_end - r_beg : 0;
  const int KB = (int)((nrows + BK - 1) / BK);
  const int nsub = (int)((nrows + GR_KSUB - 1) / GR_KSUB);
  constexpr int KB_PER_SUB = GR_KSUB / BK;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GR_STAGES; ++s) {
      mbar_init(&full_bar[s], 128);
      mbar_init(&empty_bar[s], 1);
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
    tmem_alloc(&tmem_sh, GR_TMEM_COLS);
    tmem_relinquish();
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;
  double* P = part + (int64_t)item * BM * GR_BN;

  if (warp >= 4 && warp < 8) {
    // ---- producers: rows r0..r0+31 of A, columns of the I and J blocks,
    // transposed into K-major tiles (lane = K index) and split hi/lo.  On a
    // diagonal tile they also keep Kahan sums of x^2 for their 32 columns.
    const int w = warp - 4;
    float dsum[32], dcmp[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) dsum[q] = dcmp[q] = 0.f;
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % GR_STAGES;
      const uint32_t ph = (uint32_t)(kb / GR_STAGES) & 1u;
      if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) break;
      const uint32_t st = base + s * GR_STAGE_BYTES;
      const int64_t row = r_beg + (int64_t)kb * BK + lane;
      const uint32_t kchunk = (uint32_t)lane >> 2, kin = ((uint32_t)lane & 3u) << 2;
#pragma unroll 1
      for (int blk = 0; blk < (diag ? 1 : 2); ++blk) {
        const int C0 = blk ? J0 : I0;
        const uint32_t shi = st + (blk ? 2 * GR_T_BYTES : 0), slo = shi + GR_T_BYTES;
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const int mr0 = 32 * w + 4 * j4;
          float4 v = load4(A, lda, row, r_end, (int64_t)C0 + mr0, N, a_vec != 0);
          float4 hi, lo;
          split4(v, hi, lo);
          const float xv[4] = {v.x, v.y, v.z, v.w};
          const float hv[4] = {hi.x, hi.y, hi.z, hi.w}, lv[4] = {lo.x, lo.y, lo.z, lo.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint32_t mr = (uint32_t)(mr0 + q);
            const uint32_t off = mr * ROWB + ((kchunk ^ (mr & 7u)) << 4) + kin;
            st_shared_f32(shi + off, hv[q]);
            st_shared_f32(slo + off, lv[q]);
            if (diag) {  // Kahan: dsum += x^2
              const float y = xv[q] * xv[q] - dcmp[4 * j4 + q];
              const float t = dsum[4 * j4 + q] + y;
              dcmp[4 * j4 + q] = (t - dsum[4 * j4 + q]) - y;
              dsum[4 * j4 + q] = t;
            }
          }
        }
      }
      fence_proxy_async();
      mbar_arrive(&full_bar[s]);
      if ((kb % KB_PER_SUB) == KB_PER_SUB - 1 || kb == KB - 1) {
        // end of a sub-chunk: column sums over the 32 lanes in FP64
        const int b = (kb / KB_PER_SUB) & 1;
        double mine = 0.0;
        if (diag) {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const double v = warp_sum((double)dsum[q] - (double)dcmp[q]);
            if (lane == q) mine = v;
            dsum[q] = dcmp[q] = 0.f;
          }
        }
        diag_sh[b][32 * w + lane] = mine;
        mbar_arrive(&dfull[b]);
      }
    }
  } else if (warp == 8 && lane == 0) {
    // ---- UMMA issuer: main += hi*hi, correction += hi*lo + lo*hi
    constexpr uint32_t idesc = idesc_tf32(BM, GR_BN);
    bool ok = true;
    int kb = 0;
    for (int sub = 0; sub < nsub && ok; ++sub) {
      const int b = sub & 1;
      if (!mbar_wait(&tempty[b], (((uint32_t)sub >> 1) & 1u) ^ 1u, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t dmain = tmem + (uint32_t)(b * 2 * GR_BN);
      const uint32_t dcorr = dmain + (uint32_t)GR_BN;
      const int kb_end = (kb + KB_PER_SUB < KB) ? kb + KB_PER_SUB : KB;
      for (int kl = 0; kb < kb_end; ++kb, ++kl) {
        const int s = kb % GR_STAGES;
        const uint32_t ph = (uint32_t)(kb / GR_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t st = base + s * GR_STAGE_BYTES;
        const uint64_t dAhi = desc_sw128(st), dAlo = desc_sw128(st + GR_T_BYTES);
        const uint64_t dBhi = diag ? dAhi : desc_sw128(st + 2 * GR_T_BYTES);
        const uint64_t dBlo = diag ? dAlo : desc_sw128(st + 3 * GR_T_BYTES);
#pragma unroll
        for (int kk = 0; kk < BK / 8; ++kk) {
          const uint64_t adv = (uint64_t)(kk * 32) >> 4;
          const uint32_t first = (kl > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(dmain, dAhi + adv, dBhi + adv, idesc, first);
          mma_tf32(dcorr, dAhi + adv, dBlo + adv, idesc, first);
          mma_tf32(dcorr, dAlo + adv, dBhi + adv, idesc, 1u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (ok) mma_commit(&tfull[b]);
    }
  } else if (warp < 4) {
    // ---- epilogue: drain each finished sub-chunk into the FP64 partial
    const int rloc = warp * 32 + lane;
    for (int sub = 0; sub < nsub; ++sub) {
      const int b = sub & 1;
      const uint32_t par = ((uint32_t)sub >> 1) & 1u;
      bool ready = mbar_wait(&tfull[b], par, &abort_sh, err);
      ready = ready && mbar_wait(&dfull[b], par, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      const double dval = diag_sh[b][rloc];
      double* prow = P + (int64_t)rloc * GR_BN;
#pragma unroll 1
      for (int cc = 0; cc < GR_BN / 32; ++cc) {
        uint32_t rm[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * 2 * GR_BN + cc * 32);
        tmem_ld32(ta, rm);
        tmem_ld32(ta + GR_BN, rc);
        tmem_wait_ld();
        double* d = prow + cc * 32;
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          double v0 = (double)__uint_as_float(rm[j]) + (double)__uint_as_float(rc[j]);
          double v1 = (double)__uint_as_float(rm[j + 1]) + (double)__uint_as_float(rc[j + 1]);
          if (diag && cc * 32 + j == rloc) v0 = dval;
          if (diag && cc * 32 + j + 1 == rloc) v1 = dval;
          if (sub == 0) {
            *reinterpret_cast<double2*>(d + j) = make_double2(v0, v1);
          } else {
            double2 o = *reinterpret_cast<double2*>(d + j);
            o.x += v0;
            o.y += v1;
            *reinterpret_cast<double2*>(d + j) = o;
          }
        }
      }
      fence_before();
      mbar_arrive(&tempty[b]);
    }
    if (nsub == 0) {  // empty chunk: the partial is zero
      double* prow = P + (int64_t)rloc * GR_BN;
      for (int j = 0; j < GR_BN; ++j) prow[j] = 0.0;
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 8) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, GR_TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// TMA-fed variants (A with 16-byte-aligned rows).  A TMA producer warp fills
// the stages; the split/transform warps only touch shared memory.
// ---------------------------------------------------------------------------

// apply: stage = [A raw -> hi (in place)][A lo][B hi][B lo]; A and B tiles
// arrive by TMA in the K-major SW128 layout the UMMA reads.  Warps 0-3 split
// and later drain TMEM, warp 4 issues UMMA, warp 5 issues TMA.
__global__ void __launch_bounds__(192, 1)
    tc_apply_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                        const __grid_constant__ CUtensorMap tmBhi,
                        const __grid_constant__ CUtensorMap tmBlo, int64_t m, int K, int ncols,
                        int64_t col_tiles, float* __restrict__ C, int64_t ldc, int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t tma_bar[AP_STAGES], split_bar[AP_STAGES], empty_bar[AP_STAGES], acc_bar;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = blockIdx.x;
  const int64_t m0 = (tile / col_tiles) * BM;
  const int n0 = (int)(tile % col_tiles) * AP_BN;
  const int KB = (K + BK - 1) / BK;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < AP_STAGES; ++s) {
      mbar_init(&tma_bar[s], 1);
      mbar_init(&split_bar[s], 128);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    abort_sh = 0;
    mbar_fence_init();
  }
  if (warp == 4) {
    tmem_alloc(&tmem_sh, 2 * AP_BN);
    tmem_relinquish();
  }
  if (warp == 5 && lane == 0) {
    tma_prefetch_map(&tmA);
    tma_prefetch_map(&tmBhi);
    tma_prefetch_map(&tmBlo);
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;

  if (warp == 5) {
    if (lane == 0) {
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % AP_STAGES;
        const uint32_t ph = (uint32_t)(kb / AP_STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_sh, err)) break;
        const uint32_t st = base + s * AP_STAGE_BYTES;
        mbar_expect_tx(&tma_bar[s], AP_A_BYTES + 2 * AP_B_BYTES);
        tma_load_2d(st, &tmA, kb * BK, (int)m0, &tma_bar[s]);
        tma_load_2d(st + 2 * AP_A_BYTES, &tmBhi, kb * BK, n0, &tma_bar[s]);
        tma_load_2d(st + 2 * AP_A_BYTES + AP_B_BYTES, &tmBlo, kb * BK, n0, &tma_bar[s]);
      }
    }
  } else if (warp < 4) {
    // ---- split A in place: raw -> hi, lo into the next tile (same offsets)
    const int t = threadIdx.x;
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % AP_STAGES;
      const uint32_t ph = (uint32_t)(kb / AP_STAGES) & 1u;
      if (!mbar_wait(&tma_bar[s], ph, &abort_sh, err)) break;
      const uint32_t sA = base + s * AP_STAGE_BYTES;
#pragma unroll
      for (int i = 0; i < (int)(AP_A_BYTES / 16 / 128); ++i) {
        const uint32_t off = (uint32_t)(t + 128 * i) * 16u;
        float4 v = ld_shared_v4(sA + off), hi, lo;
        split4(v, hi, lo);
        st_shared_v4(sA + off, hi);
        st_shared_v4(sA + AP_A_BYTES + off, lo);
      }
      fence_proxy_async();
      mbar_arrive(&split_bar[s]);
    }
  } else if (lane == 0) {
    // ---- UMMA issuer (warp 4)
    constexpr uint32_t idesc = idesc_tf32(BM, AP_BN);
    bool ok = true;
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % AP_STAGES;
      const uint32_t ph = (uint32_t)(kb / AP_STAGES) & 1u;
      if (!mbar_wait(&tma_bar[s], ph, &abort_sh, err) ||
          !mbar_wait(&split_bar[s], ph, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t st = base + s * AP_STAGE_BYTES;
      const uint64_t dAhi = desc_sw128(st), dAlo = desc_sw128(st + AP_A_BYTES);
      const uint64_t dBhi = desc_sw128(st + 2 * AP_A_BYTES);
      const uint64_t dBlo = desc_sw128(st + 2 * AP_A_BYTES + AP_B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 8; ++kk) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        mma_tf32(tmem, dAhi + adv, dBhi + adv, idesc, acc);
        mma_tf32(tmem + AP_BN, dAhi + adv, dBlo + adv, idesc, acc);
        mma_tf32(tmem + AP_BN, dAlo + adv, dBhi + adv, idesc, 1u);
      }
      mma_commit(&empty_bar[s]);
    }
    if (ok) mma_commit(&acc_bar);
  }

  if (warp < 4) {
    const bool ready = mbar_wait(&acc_bar, 0, &abort_sh, err);
    __syncwarp();
    if (__all_sync(0xffffffffu, ready)) {
      fence_after();
      const int64_t row = m0 + warp * 32 + lane;
      const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
      for (int cc = 0; cc < AP_BN / 32; ++cc) {
        uint32_t r[32], rc[32];
        const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32);
        tmem_ld32(ta, r);
        tmem_ld32(ta + AP_BN, rc);
        tmem_wait_ld();
        const int col0 = n0 + cc * 32;
        if (row < m && col0 < ncols) {
          float* dst = C + row * ldc + col0;
          if (vec && col0 + 32 <= ncols) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(dst + j) = make_float4(
                  __uint_as_float(r[j]) + __uint_as_float(rc[j]),
                  __uint_as_float(r[j + 1]) + __uint_as_float(rc[j + 1]),
                  __uint_as_float(r[j + 2]) + __uint_as_float(rc[j + 2]),
                  __uint_as_float(r[j + 3]) + __uint_as_float(rc[j + 3]));
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (col0 + j < ncols) dst[j] = __uint_as_float(r[j]) + __uint_as_float(rc[j]);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 4) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, 2 * AP_BN);
  }
}

// gram: raw rows arrive by TMA as 32 x 32 fp32 boxes (SW128) in a raw ring;
// warps 4-7 transpose + split them into the operand ring; warps 0-3 drain
// TMEM, warp 8 issues UMMA, warp 9 issues TMA.
constexpr int GT_RAW_STAGES = 2;
constexpr int GT_OP_STAGES = 2;
constexpr uint32_t GT_BOX_BYTES = 32 * 32 * 4;            // one 32 x 32 fp32 box
constexpr uint32_t GT_RAW_BYTES = 8 * GT_BOX_BYTES;        // I block + J block
constexpr uint32_t GT_OP_BYTES = 4 * GR_T_BYTES;           // Ahi Alo Bhi Blo
constexpr size_t GT_SMEM = (size_t)GT_RAW_STAGES * GT_RAW_BYTES +
                           (size_t)GT_OP_STAGES * GT_OP_BYTES + 1024;

__global__ void __launch_bounds__(320, 1)
    tc_gram_tma_kernel(const __grid_constant__ CUtensorMap tmA, int64_t m, int N, int tn,
                       int64_t rows_per_chunk, int chunks, double* __restrict__ part, int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t raw_full[GT_RAW_STAGES], raw_empty[GT_RAW_STAGES];
  __shared__ uint64_t op_full[GT_OP_STAGES], op_empty[GT_OP_STAGES];
  __shared__ uint64_t tfull[2], tempty[2], dfull[2];
  __shared__ double diag_sh[2][BM];
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t raw_base = base, op_base = base + GT_RAW_STAGES * GT_RAW_BYTES;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // consecutive CTAs take different tiles of the same row chunk, so the CTAs
  // resident together read the same rows and share them through L2
  const int ntiles_all = tn * (tn + 1) / 2;
  const int chunk = (int)(blockIdx.x / ntiles_all), tile = (int)(blockIdx.x % ntiles_all);
  const int item = tile * chunks + chunk;  // partial slab index (tile-major)
  int ti = 0, rem = tile;
  while (rem >= tn - ti) {
    rem -= tn - ti;
    ++ti;
  }
  const int tj = ti + rem;
  const bool diag = (ti == tj);
  const int I0 = ti * BM, J0 = tj * GR_BN;
  const int64_t r_beg = (int64_t)chunk * rows_per_chunk;
  const int64_t r_end = (r_beg + rows_per_chunk < m) ? r_beg + rows_per_chunk : m;
  const int64_t nrows = (r_end > r_beg) ? r_end - r_beg : 0;
  const int KB = (int)((nrows + BK - 1) / BK);
  const int nsub = (int)((nrows + GR_KSUB - 1) / GR_KSUB);
  constexpr int KB_PER_SUB = GR_KSUB / BK;
  if (launch_aborted(err)) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GT_RAW_STAGES; ++s) {
      mbar_init(&raw_full[s], 1);
      mbar_init(&raw_empty[s], 128);
    }
    for (int s = 0; s < GT_OP_STAGES; ++s) {
      mbar_init(&op_full[s], 128);
      mbar_init(&op_empty[s], 1);
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
    tmem_alloc(&tmem_sh, GR_TMEM_COLS);
    tmem_relinquish();
  }
  if (warp == 9 && lane == 0) tma_prefetch_map(&tmA);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_sh;
  double* P = part + (int64_t)item * BM * GR_BN;

  if (warp == 9) {
    // ---- TMA producer: 4 boxes of the I block (+ 4 of the J block)
    if (lane == 0) {
      const uint32_t bytes = (diag ? 4u : 8u) * GT_BOX_BYTES;
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % GT_RAW_STAGES;
        const uint32_t ph = (uint32_t)(kb / GT_RAW_STAGES) & 1u;
        if (!mbar_wait(&raw_empty[s], ph ^ 1u, &abort_sh, err)) break;
        const uint32_t st = raw_base + s * GT_RAW_BYTES;
        const int y = (int)(r_beg + (int64_t)kb * BK);
        mbar_expect_tx(&raw_full[s], bytes);
#pragma unroll
        for (int q = 0; q < 4; ++q) tma_load_2d(st + q * GT_BOX_BYTES, &tmA, I0 + 32 * q, y, &raw_full[s]);
        if (!diag) {
#pragma unroll
          for (int q = 0; q < 4; ++q)
            tma_load_2d(st + (4 + q) * GT_BOX_BYTES, &tmA, J0 + 32 * q, y, &raw_full[s]);
        }
      }
    }
  } else if (warp >= 4 && warp < 8) {
    // ---- transpose + split: warp w owns operand rows 32w..32w+31 (= box w);
    // lane = K index (row of the raw box)
    const int w = warp - 4;
    float dsum[32], dcmp[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) dsum[q] = dcmp[q] = 0.f;
    const uint32_t kchunk = (uint32_t)lane >> 2, kin = ((uint32_t)lane & 3u) << 2;
    for (int kb = 0; kb < KB; ++kb) {
      const int rs = kb % GT_RAW_STAGES, os = kb % GT_OP_STAGES;
      const uint32_t rph = (uint32_t)(kb / GT_RAW_STAGES) & 1u;
      const uint32_t oph = (uint32_t)(kb / GT_OP_STAGES) & 1u;
      if (!mbar_wait(&raw_full[rs], rph, &abort_sh, err)) break;
      if (!mbar_wait(&op_empty[os], oph ^ 1u, &abort_sh, err)) break;
      const uint32_t rst = raw_base + rs * GT_RAW_BYTES;
      const uint32_t ost = op_base + os * GT_OP_BYTES;
      // rows past the end of this chunk (next chunk's rows) must not count
      const bool live = (r_beg + (int64_t)kb * BK + lane) < r_end;
#pragma unroll 1
      for (int blk = 0; blk < (diag ? 1 : 2); ++blk) {
        const uint32_t box = rst + (uint32_t)(4 * blk + w) * GT_BOX_BYTES + (uint32_t)lane * ROWB;
        const uint32_t shi = ost + (blk ? 2 * GR_T_BYTES : 0), slo = shi + GR_T_BYTES;
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          float4 v = ld_shared_v4(box + (((uint32_t)j4 ^ ((uint32_t)lane & 7u)) << 4));
          if (!live) v = make_float4(0.f, 0.f, 0.f, 0.f);
          float4 hi, lo;
          split4(v, hi, lo);
          const float xv[4] = {v.x, v.y, v.z, v.w};
          const float hv[4] = {hi.x, hi.y, hi.z, hi.w}, lv[4] = {lo.x, lo.y, lo.z, lo.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint32_t mr = (uint32_t)(32 * w + 4 * j4 + q);
            const uint32_t off = mr * ROWB + ((kchunk ^ (mr & 7u)) << 4) + kin;
            st_shared_f32(shi + off, hv[q]);
            st_shared_f32(slo + off, lv[q]);
            if (diag) {
              const float y = xv[q] * xv[q] - dcmp[4 * j4 + q];
              const float tt = dsum[4 * j4 + q] + y;
              dcmp[4 * j4 + q] = (tt - dsum[4 * j4 + q]) - y;
              dsum[4 * j4 + q] = tt;
            }
          }
        }
      }
      fence_proxy_async();
      mbar_arrive(&raw_empty[rs]);
      mbar_arrive(&op_full[os]);
      if ((kb % KB_PER_SUB) == KB_PER_SUB - 1 || kb == KB - 1) {
        const int b = (kb / KB_PER_SUB) & 1;
        double mine = 0.0;
        if (diag) {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const double v = warp_sum((double)dsum[q] - (double)dcmp[q]);
            if (lane == q) mine = v;
            dsum[q] = dcmp[q] = 0.f;
          }
        }
        diag_sh[b][32 * w + lane] = mine;
        mbar_arrive(&dfull[b]);
      }
    }
  } else if (warp == 8 && lane == 0) {
    // ---- UMMA issuer
    constexpr uint32_t idesc = idesc_tf32(BM, GR_BN);
    bool ok = true;
    int kb = 0;
    for (int sub = 0; sub < nsub && ok; ++sub) {
      const int b = sub & 1;
      if (!mbar_wait(&tempty[b], (((uint32_t)sub >> 1) & 1u) ^ 1u, &abort_sh, err)) {
        ok = false;
        break;
      }
      fence_after();
      const uint32_t dmain = tmem + (uint32_t)(b * 2 * GR_BN);
      const uint32_t dcorr = dmain + (uint32_t)GR_BN;
      const int kb_end = (kb + KB_PER_SUB < KB) ? kb + KB_PER_SUB : KB;
      for (int kl = 0; kb < kb_end; ++kb, ++kl) {
        const int os = kb % GT_OP_STAGES;
        const uint32_t oph = (uint32_t)(kb / GT_OP_STAGES) & 1u;
        if (!mbar_wait(&op_full[os], oph, &abort_sh, err)) {
          ok = false;
          break;
        }
        fence_after();
        const uint32_t st = op_base + os * GT_OP_BYTES;
        const uint64_t dAhi = desc_sw128(st), dAlo = desc_sw128(st + GR_T_BYTES);
        const uint64_t dBhi = diag ? dAhi : desc_sw128(st + 2 * GR_T_BYTES);
        const uint64_t dBlo = diag ? dAlo : desc_sw128(st + 3 * GR_T_BYTES);
#pragma unroll
        for (int kk = 0; kk < BK / 8; ++kk) {
          const uint64_t adv = (uint64_t)(kk * 32) >> 4;
          const uint32_t first = (kl > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(dmain, dAhi + adv, dBhi + adv, idesc, first);
          mma_tf32(dcorr, dAhi + adv, dBlo + adv, idesc, first);
          mma_tf32(dcorr, dAlo + adv, dBhi + adv, idesc, 1u);
        }
        mma_commit(&op_empty[os]);
      }
      if (ok) mma_commit(&tfull[b]);
    }
  } else if (warp < 4) {
    // ---- epilogue: drain each finished sub-chunk into the FP64 partial
    const int rloc = warp * 32 + lane;
    for (int sub = 0; sub < nsub; ++sub) {
      const int b = sub & 1;
      const uint32_t par = ((uint32_t)sub >> 1) & 1u;
      bool ready = mbar_wait(&tfull[b], par, &abort_sh, err);
      ready = ready && mbar_wait(&dfull[b], par, &abort_sh, err);
      __syncwarp();
      if (!__all_sync(0xffffffffu, ready)) break;
      fence_after();
      const double dval = diag_sh[b][rloc];
      double* prow = P + (int64_t)rloc * GR_BN;
#pragma unroll 1
      for (int cc = 0; cc < GR_BN / 32; ++cc) {
        uint32_t rm[32], rc[32];
        const uint32_t ta =
            tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * 2 * GR_BN + cc * 32);
        tmem_ld32(ta, rm);
        tmem_ld32(ta + GR_BN, rc);
        tmem_wait_ld();
        double* d = prow + cc * 32;
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
          double v0 = (double)__uint_as_float(rm[j]) + (double)__uint_as_float(rc[j]);
          double v1 = (double)__uint_as_float(rm[j + 1]) + (double)__uint_as_float(rc[j + 1]);
          if (diag && cc * 32 + j == rloc) v0 = dval;
          if (diag && cc * 32 + j + 1 == rloc) v1 = dval;
          if (sub == 0) {
            *reinterpret_cast<double2*>(d + j) = make_double2(v0, v1);
          } else {
            double2 o = *reinterpret_cast<double2*>(d + j);
            o.x += v0;
            o.y += v1;
            *reinterpret_cast<double2*>(d + j) = o;
          }
        }
      }
      fence_before();
      mbar_arrive(&tempty[b]);
    }
    if (nsub == 0) {
      double* prow = P + (int64_t)rloc * GR_BN;
      for (int j = 0; j < GR_BN; ++j) prow[j] = 0.0;
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 8) {
    __syncwarp();
    fence_after();
    tmem_dealloc(tmem, GR_TMEM_COLS);
  }
}

// G[i][j] = sum over chunks of the tile partials (fixed order), mirrored
__global__ void gram_reduce_kernel(const double* __restrict__ part, int N, int tn, int chunks,
                                   double* __restrict__ G) {
  const int64_t total = (int64_t)N * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / N), j = (int)(e % N);
    int a = i, b = j;
    if (a / BM > b / GR_BN) {
      a = j;
      b = i;
    }
    const int ti = a / BM, tj = b / GR_BN;
    const int tile = ti * tn - ti * (ti - 1) / 2 + (tj - ti);
    const double* p = part + ((int64_t)tile * chunks) * BM * GR_BN + (int64_t)(a - ti * BM) * GR_BN +
                      (b - tj * GR_BN);
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += p[(int64_t)c * BM * GR_BN];
    G[e] = s;
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

// 2-D fp32 tensor map, 128-byte swizzle, zero fill out of bounds
static bool make_map_2d(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer,
                        uint64_t row_bytes, uint32_t box_inner, uint32_t box_outer) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (row_bytes & 15)) return false;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}
bool tc_gram_supported(int64_t m, int64_t N, int64_t lda) {
  return m >= 1 && N >= 1 && N <= 8192 && lda >= N;
}

static int gram_chunks(int64_t m, int tiles) {
  int64_t target = (int64_t)num_sms() * 2;
  int64_t c = cdiv(target, tiles);
  int64_t maxc = std::max<int64_t>(1, cdiv(m, tc::GR_KSUB));
  return (int)std::max<int64_t>(1, std::min(c, maxc));
}

int tc_gram_tf32x3(const float* A, int64_t lda, int64_t m, int64_t N, double* G, int* err,
                   Arena& ws, cudaStream_t st) {
  const int tn = (int)cdiv(N, tc::BM);
  const int tiles = tn * (tn + 1) / 2;
  const int chunks = gram_chunks(m, tiles);
  int64_t rpc = cdiv(m, chunks);
  rpc = cdiv(rpc, tc::GR_KSUB) * tc::GR_KSUB;
  const int chunks_eff = (int)std::max<int64_t>(1, cdiv(m, rpc));
  double* part = ws.take<double>((size_t)tiles * chunks_eff * tc::BM * tc::GR_BN);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tc_gram: workspace too small");
  PLOM_REQUIRE(A && G && part, PLOM_ERR_ARG, "tc_gram: null pointer");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(tc::tc_gram_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::GR_SMEM));
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(tc::tc_gram_tma_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::GT_SMEM));
    attr = true;
  }
  const int a_vec = ((lda & 3) == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  CUtensorMap tmA;
  const bool tma = a_vec && m < (1ll << 31) &&
                   make_map_2d(&tmA, A, (uint64_t)N, (uint64_t)m, (uint64_t)lda * 4, 32, 32);
  ProfScope prof_g("tc_gram_tf32x3", st, (double)m * N * N, 4.0 * m * N);
  if (tma)
    tc::tc_gram_tma_kernel<<<tiles * chunks_eff, 320, tc::GT_SMEM, st>>>(tmA, m, (int)N, tn, rpc,
                                                                         chunks_eff, part, err);
  else
    tc::tc_gram_kernel<<<tiles * chunks_eff, 288, tc::GR_SMEM, st>>>(A, lda, m, (int)N, tn, rpc,
                                                                     chunks_eff, part, a_vec, err);
  PLOM_CHECK_LAUNCH();
  const int64_t total = N * N;
  int blocks = (int)std::min<int64_t>(cdiv(total, 256), (int64_t)num_sms() * 16);
  ProfScope prof_r("gram_reduce", st, 0.0, 8.0 * (double)tiles * chunks_eff * tc::BM * tc::GR_BN);
  tc::gram_reduce_kernel<<<blocks, 256, 0, st>>>(part, (int)N, tn, chunks_eff, G);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

bool tc_apply_supported(int64_t m, int64_t N, int64_t k, int64_t lda, int64_t ldc) {
  return m >= 1 && N >= 1 && k >= 1 && N <= (1 << 20) && lda >= N && ldc >= k;
}

template <typename TW>
int tc_apply_tf32x3(const float* A, int64_t lda, int64_t m, int64_t N, const TW* W, int64_t ldw,
                    int64_t k, float* C, int64_t ldc, int* err, Arena& ws, cudaStream_t st) {
  const int64_t ldo = cdiv(N, 4) * 4;  // 16-byte rows for the tensor map
  float* Whi = ws.take<float>((size_t)ldo * k);
  float* Wlo = ws.take<float>((size_t)ldo * k);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tc_apply: workspace too small");
  PLOM_REQUIRE(A && W && C, PLOM_ERR_ARG, "tc_apply: null pointer");
  static bool attr = false;
  if (!attr) {
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(tc::tc_apply_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::AP_SMEM));
    PLOM_CHECK_CUDA(cudaFuncSetAttribute(tc::tc_apply_tma_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tc::AP_SMEM));
    attr = true;
  }
  {
    int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(cdiv(ldo * k, 256), num_sms() * 8));
    tc::split_w_kernel<TW><<<blocks, 256, 0, st>>>(W, N, k, ldw, Whi, Wlo, ldo);
    PLOM_CHECK_LAUNCH();
  }
  const int64_t col_tiles = cdiv(k, tc::AP_BN);
  const int64_t tiles = cdiv(m, tc::BM) * col_tiles;
  PLOM_REQUIRE(tiles < (1ll << 31), PLOM_ERR_ARG, "tc_apply: too many tiles");
  const int a_vec = ((lda & 3) == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  CUtensorMap tmA, tmBhi, tmBlo;
  const bool tma = a_vec && m < (1ll << 31) &&
                   make_map_2d(&tmA, A, (uint64_t)N, (uint64_t)m, (uint64_t)lda * 4, 32, tc::BM) &&
                   make_map_2d(&tmBhi, Whi, (uint64_t)N, (uint64_t)k, (uint64_t)ldo * 4, 32,
                               tc::AP_BN) &&
                   make_map_2d(&tmBlo, Wlo, (uint64_t)N, (uint64_t)k, (uint64_t)ldo * 4, 32,
                               tc::AP_BN);
  ProfScope prof_a("tc_apply_tf32x3", st, 2.0 * m * N * k, 4.0 * ((double)m * N + (double)m * k));
  if (tma)
    tc::tc_apply_tma_kernel<<<(unsigned)tiles, 192, tc::AP_SMEM, st>>>(
        tmA, tmBhi, tmBlo, m, (int)N, (int)k, col_tiles, C, ldc, err);
  else
    tc::tc_apply_kernel<<<(unsigned)tiles, 160, tc::AP_SMEM, st>>>(A, lda, m, (int)N, Whi, Wlo,
                                                                   (int)ldo, (int)k, col_tiles, C,
                                                                   ldc, a_vec, err);
  PLOM_CHECK_LAUNCH();
  return PLOM_OK;
}

template int tc_apply_tf32x3<double>(const float*, int64_t, int64_t, int64_t, const double*,
                                      int64_t, int64_t, float*, int64_t, int*, Arena&,
                                      cudaStream_t);
template int tc_apply_tf32x3<float>(const float*, int64_t, int64_t, int64_t, const float*, int64_t,
                                     int64_t, float*, int64_t, int*, Arena&, cudaStream_t);

}  // namespace plom
