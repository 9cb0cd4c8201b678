// Host-side orchestration of the tall-skinny QR and SVD (all kernels launched
// on the caller's stream; nothing allocated, nothing synchronised).
//
// Algorithm (GB300 restatement of pyLOM's TSQR-SVD, pyLOM/vmmath/svd.py:
// 50-118 and 228-252, pyLOM/vmmath/src/svd.c:565-712):
//   The MPI butterfly that merges per-rank R factors becomes an in-GPU
//   reduction over row tiles.  Each tile contributes its Gram block
//   A_t^T A_t (the R-merge in Gram form: R_ab^T R_ab = R_a^T R_a + R_b^T R_b),
//   the partial Grams are summed in FP64, and the n x n factor comes from a
//   shifted Cholesky.  Three passes (shifted CholeskyQR3, Fukaya et al.,
//   SIAM J. Sci. Comput. 42 (2020)) give a backward-stable Q with orthonormal
//   columns:
//       G1 = X^T X,   R1 = chol(G1 + s I),  Q1 = X R1^-1
//       G2 = Q1^T Q1, R2 = chol(G2),        Q2 = Q1 R2^-1
//       G3 = Q2^T Q2, R3 = chol(G3),        R = R3 R2 R1
//   then svd(R) = Ur S V^T (FP64 one-sided Jacobi) and U = Q2 (R3^-1 Ur).
//   The identity GEMM pyLOM runs on one rank (svd.py:117, svd.c:673) is not
//   performed.
//
// Precision forms: PLOM_PREC_FP64 runs every product in FP64 (Q1, Q2 stored
// in FP64); PLOM_PREC_MIXED packs the FP32 operand once as fp16 hi/lo pairs
// and runs every tall product on the tensor cores (gemm_f16.cu), each apply
// writing the next Q already packed; every n x n step stays in FP64.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <type_traits>

#include "plom_common.cuh"
#include "plom_kernels.cuh"
#include "plom_tc.cuh"

namespace plom {

static const double U64 = 1.1102230246251565e-16;  // 2^-53
static const double U32 = 5.9604644775390625e-08;  // 2^-24 (the fp16-pair products are FP32-accurate)
// n x n products of the mixed form in double-float sums from this size on
static const int DF_PRODUCT_MIN_N = 256;

// ---------------------------------------------------------------------------
// tall operations, dispatched on precision
// ---------------------------------------------------------------------------
// the packed tensor-core kernels address rows with 32-bit TMA coordinates
static bool packed_ok(int64_t m) { return m >= 1 && m < (1ll << 31); }

template <typename TA>
static int tall_gram(int prec, const TA* A, int64_t lda, int64_t m, int64_t N, double* G,
                     int* err, Arena& ws, cudaStream_t st) {
  if (prec == PLOM_PREC_FP64)
    return gemm_tn<TA, TA, double, double>(A, lda, A, lda, G, N, N, N, m, true, ws, st);
  if constexpr (sizeof(TA) == 4) {
    if (packed_ok(m)) {
      Packed p;
      packed_carve(ws, p, m, N);
      PLOM_TRY(pack_f32(A, lda, m, N, p, ws, st));
      return gram_packed(p, G, err, ws, st);
    }
    return gemm_tn<TA, TA, float, double>(A, lda, A, lda, G, N, N, N, m, true, ws, st);
  } else {
    return gemm_tn<TA, TA, double, double>(A, lda, A, lda, G, N, N, N, m, true, ws, st);
  }
}

// C(m x k) = A(m x N) W(N x k), W in FP64 (converted for the mixed form)
template <typename TA, typename TO>
static int tall_apply(int prec, const TA* A, int64_t lda, int64_t m, int64_t N, const double* W,
                      int64_t k, TO* C, int64_t ldc, int* err, Arena& ws, cudaStream_t st,
                      bool upper = false) {
  if (prec == PLOM_PREC_FP64 || sizeof(TA) == 8) {
    if (ws.measuring()) return PLOM_OK;  // workspace query: launch nothing
    return gemm_nn<TA, double, TO, double>(A, lda, W, k, C, ldc, m, k, N, st, upper);
  }
  if constexpr (sizeof(TA) == 4 && sizeof(TO) == 4) {
    if (packed_ok(m)) {
      Packed p;
      packed_carve(ws, p, m, N);
      PLOM_TRY(pack_f32(A, lda, m, N, p, ws, st));
      return apply_packed(p, W, k, k, C, ldc, nullptr, err, ws, st, 0, 0, upper);
    }
  }
  float* Wf = ws.take<float>((size_t)N * k);
  if (ws.measuring()) return PLOM_OK;
  PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tall_apply: workspace too small");
  PLOM_TRY((convert<double, float>(W, Wf, N * k, st)));
  return gemm_nn<TA, float, TO, float>(A, lda, Wf, k, C, ldc, m, k, N, st, upper);
}

// Shifts are passed to the Cholesky relative to trace(G)/N; the absolute
// shift is s = c u trace(G) (trace(G) = ||X||_F^2 >= ||X||_2^2).
#ifndef PLOM_MIXED_SHIFT
#define PLOM_MIXED_SHIFT 16
#endif
static void shifts_for(int prec, int64_t m, int64_t N, double& rel1, double& relfail) {
  const double u = (prec == PLOM_PREC_FP64) ? U64 : U32;
  const double n = (double)N;
  // FP64: the sCholeskyQR3 bound 11 (mn + n(n+1)) u; mixed: a fixed 16 u,
  // escalated on breakdown (the bound grows with m far past what the FP64
  // partial-Gram summation needs).
  const double c1 = (prec == PLOM_PREC_FP64) ? std::max(11.0 * ((double)m * n + n * (n + 1.0)), 4.0)
                                             : (double)PLOM_MIXED_SHIFT;
  rel1 = c1 * u * n;
  relfail = 16.0 * u * n;
}

// ---------------------------------------------------------------------------
// CholeskyQR3 core.  X: m x N real (complex data as its interleaved real view
// with N = 2n).  Produces Q2 (m x N, TC), W3e = R3^-1, Re = R3 R2 R1 (N x N,
// FP64; for complex data these are real embeddings of the complex factors).
// ---------------------------------------------------------------------------
template <typename TI, typename TC>
struct CoreBufs {
  TC* Q1;
  TC* Q2;
  double *G, *H, *R1, *R2, *R3, *W1, *W2, *W3, *Rp, *Re, *F;
};

template <typename TI, typename TC>
static int chol_pass(int prec, bool cplx, int n, int64_t m, const TC* Q, int64_t ldq,
                     const TI* Xin, int64_t ldx, bool first, CoreBufs<TI, TC>& b, double* R,
                     double* W, double rel0, double relfail, int* info, Arena& ws,
                     cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  double* Gtarget = cplx ? b.H : b.G;
  const size_t mark = ws.off;
  size_t need = mark;
  if (first)
    PLOM_TRY(tall_gram<TI>(prec, Xin, ldx, m, N, Gtarget, info, ws, st));
  else
    PLOM_TRY(tall_gram<TC>(prec, Q, ldq, m, N, Gtarget, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  if (cplx && !ws.measuring()) PLOM_TRY(complexify_gram(b.H, b.G, n, 1, st));
  PLOM_TRY(chol_shifted(b.G, R, N, 1, rel0, relfail, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  PLOM_TRY(trtri_upper(R, W, N, 1, ws, st));
  need = std::max(need, ws.off);
  ws.off = need;
  return PLOM_OK;
}

// right operand of a real GEMM on interleaved complex data: real_embed(conj(W))
static const double* rowform(bool cplx, const double* We, double* F, int n, cudaStream_t st,
                             int& status) {
  status = PLOM_OK;
  if (!cplx) return We;
  status = embed_to_rowform(We, F, n, 1, st);
  return F;
}

template <typename TI, typename TC>
static int cholqr3(int prec, bool cplx, const TI* X, int64_t m, int n, int64_t ldx, TC* q1_store,
                   int64_t ldq1, CoreBufs<TI, TC>& b, int* info, Arena& ws, cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  double rel1, relfail;
  shifts_for(prec, m, N, rel1, relfail);
  const size_t mark = ws.off;
  size_t need = mark;
  int s;
  // pass 1
  PLOM_TRY((chol_pass<TI, TC>(prec, cplx, n, m, nullptr, 0, X, ldx, true, b, b.R1, b.W1, rel1,
                              relfail, info, ws, st)));
  const double* F1 = ws.measuring() ? b.W1 : rowform(cplx, b.W1, b.F, n, st, s);
  if (!ws.measuring()) PLOM_TRY(s);
  need = std::max(need, ws.off);
  ws.off = mark;
  TC* Q1 = q1_store ? q1_store : b.Q1;
  int64_t ld1 = q1_store ? ldq1 : N;
  PLOM_TRY((tall_apply<TI, TC>(prec, X, ldx, m, N, F1, N, Q1, ld1, info, ws, st, true)));
  need = std::max(need, ws.off);
  ws.off = mark;
  // pass 2
  PLOM_TRY((chol_pass<TI, TC>(prec, cplx, n, m, Q1, ld1, nullptr, 0, false, b, b.R2, b.W2, 0.0,
                              relfail, info, ws, st)));
  need = std::max(need, ws.off);
  ws.off = mark;
  const double* F2 = ws.measuring() ? b.W2 : rowform(cplx, b.W2, b.F, n, st, s);
  if (!ws.measuring()) PLOM_TRY(s);
  PLOM_TRY((tall_apply<TC, TC>(prec, Q1, ld1, m, N, F2, N, b.Q2, N, info, ws, st, true)));
  need = std::max(need, ws.off);
  ws.off = mark;
  // pass 3
  PLOM_TRY((chol_pass<TI, TC>(prec, cplx, n, m, b.Q2, N, nullptr, 0, false, b, b.R3, b.W3, 0.0,
                              relfail, info, ws, st)));
  need = std::max(need, ws.off);
  ws.off = need;
  // Re = R3 R2 R1
  if (!ws.measuring()) {
    PLOM_TRY((gemm_sq_nn(b.R3, b.R2, b.Rp, N, 1, 3, st)));
    PLOM_TRY((gemm_sq_nn(b.Rp, b.R1, b.Re, N, 1, 3, st)));
  }
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// mixed form on FP32 data: CholeskyQR3 on packed fp16-pair operands.  X is
// packed once (P0); every apply writes the next Q already packed (P1, P2),
// so each tall operand is read by the tensor cores without conversion.
// P2 reuses P0's storage; P1 lives in the caller's output buffer when that
// is large enough (`p1_store`, 4 m packed_ld(N) bytes), else in the workspace.
// ---------------------------------------------------------------------------
struct PackedCore {
  Packed P0, P1, P2;
  double *G, *H, *R1, *R2, *R3, *W1, *W2, *W3, *Rp, *Re, *F;
};

static void carve_packed_core(Arena& ws, PackedCore& b, int64_t m, int N, bool p1_external,
                              void* p1_store) {
  const size_t nn = (size_t)N * N;
  b.G = ws.take<double>(nn);
  b.H = ws.take<double>(nn);
  b.R1 = ws.take<double>(nn);
  b.R2 = ws.take<double>(nn);
  b.R3 = ws.take<double>(nn);
  b.W1 = ws.take<double>(nn);
  b.W2 = ws.take<double>(nn);
  b.W3 = ws.take<double>(nn);
  b.Rp = ws.take<double>(nn);
  b.Re = ws.take<double>(nn);
  b.F = ws.take<double>(nn);
  packed_carve(ws, b.P0, m, N);
  b.P2 = b.P0;
  b.P2.scale = ws.take<float>((size_t)b.P0.ld);
  if (p1_external) {
    float* sc = ws.take<float>((size_t)b.P0.ld);
    packed_view(b.P1, p1_store, m, N, sc);
  } else {
    packed_carve(ws, b.P1, m, N);
  }
}

static int chol_pass_packed(bool cplx, int n, const Packed& P, PackedCore& b, double* R,
                            double* W, double rel0, double relfail, int* info, Arena& ws,
                            cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  double* Gtarget = cplx ? b.H : b.G;
  const size_t mark = ws.off;
  size_t need = mark;
  PLOM_TRY(gram_packed(P, Gtarget, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  if (cplx && !ws.measuring()) PLOM_TRY(complexify_gram(b.H, b.G, n, 1, st));
  // the Gram of a factor next to orthonormal is factored in closed form when
  // the implied perturbation of G is below 1e-10 (the operands carry 22 bits)
  PLOM_TRY(chol_shifted(b.G, R, N, 1, rel0, relfail, info, ws, st, rel0 == 0.0 ? 1e-10 : 0.0));
  need = std::max(need, ws.off);
  ws.off = mark;
  PLOM_TRY(trtri_upper(R, W, N, 1, ws, st));
  need = std::max(need, ws.off);
  ws.off = need;
  return PLOM_OK;
}

// passes 2 and 3 from Q1 (packed in b.P1; R1 in b.R1) and Re = R3 R2 R1
static int cholqr3_packed_passes23(bool cplx, int n, PackedCore& b, double relfail, int* info,
                                   Arena& ws, cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  int s = PLOM_OK;
  // pass 2
  PLOM_TRY(sub([&] { return chol_pass_packed(cplx, n, b.P1, b, b.R2, b.W2, 0.0, relfail, info, ws, st); }));
  const double* F2 = ws.measuring() ? b.W2 : rowform(cplx, b.W2, b.F, n, st, s);
  PLOM_TRY(s);
  PLOM_TRY(sub([&] { return apply_packed(b.P1, F2, N, N, nullptr, 0, &b.P2, info, ws, st, 0, 0, true); }));
  // pass 3
  PLOM_TRY(sub([&] { return chol_pass_packed(cplx, n, b.P2, b, b.R3, b.W3, 0.0, relfail, info, ws, st); }));
  // Re = R3 R2 R1: double-float products from n = 256 on (the factors carry
  // the 22-bit operands' information; FP64 runs at 1/64 of the FP32 rate)
  if (N >= DF_PRODUCT_MIN_N) {
    PLOM_TRY(sub([&] { return gemm_nn_df(b.R3, b.R2, b.Rp, N, ws, st); }));
    PLOM_TRY(sub([&] { return gemm_nn_df(b.Rp, b.R1, b.Re, N, ws, st); }));
  } else if (!ws.measuring()) {
    PLOM_TRY((gemm_sq_nn(b.R3, b.R2, b.Rp, N, 1, 3, st)));
    PLOM_TRY((gemm_sq_nn(b.Rp, b.R1, b.Re, N, 1, 3, st)));
  }
  ws.off = need;
  return PLOM_OK;
}

// Large real FP32 inputs: pass 1 in row chunks, each packed with its own
// column scales on a second stream while the previous chunk's Gram runs, so
// that the packing (HBM-bound, ~15 ms at 8,388,608 x 1,024) overlaps the
// tensor-core Gram; Q1 = X R1^-1 then treats the chunks as a batch (one W,
// each chunk's input scales), as the host entry does.  The chunks must tile
// the rows exactly (Q1 lives in the caller's U).
constexpr int OVERLAP_CHUNKS = 8;
constexpr int64_t OVERLAP_MIN_CHUNK_ROWS = 262144;
static int overlap_chunks(bool cplx, int64_t m, int N) {
  if (cplx || N <= 128) return 1;  // the chunked Gram is the wide (128 x 256 tile) kernel
  const int64_t C = std::min(OVERLAP_CHUNKS, tuning().pass1_chunks);
  if (C <= 1) return 1;
  // whole chunks of 16 x 4,096-row sub-chunks (the slab reduction's batches)
  if (m % (C * 65536) != 0 || m / C < OVERLAP_MIN_CHUNK_ROWS) return 1;
  return (int)C;
}

// one non-blocking auxiliary stream per device (host copies, chunk packing),
// created on first use
static cudaStream_t host_copy_stream() {
  static std::mutex mu;
  static std::map<int, cudaStream_t> streams;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  streams[dev] = s;
  return s;
}


struct ChunkEvents {
  cudaEvent_t start = nullptr, packed[OVERLAP_CHUNKS] = {};
  bool ok = false;
  ChunkEvents() {
    ok = cudaEventCreateWithFlags(&start, cudaEventDisableTiming) == cudaSuccess;
    for (auto& e : packed) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  }
  ~ChunkEvents() {  // released once their pending work completes
    if (start) cudaEventDestroy(start);
    for (auto& e : packed)
      if (e) cudaEventDestroy(e);
  }
};

static int cholqr3_packed_chunked(const float* X, int64_t m, int n, int64_t ldx, int C,
                                  PackedCore& b, int* info, Arena& ws, cudaStream_t st) {
  const int N = n;
  const int64_t mc = m / C, ldp = b.P0.ld;
  const bool meas = ws.measuring();
  float* xscale = ws.take<float>((size_t)C * ldp);
  float* qscale = ws.take<float>((size_t)C * ldp);
  const size_t pack_bytes = sizeof(unsigned) * (size_t)N + 1024;  // pack_f32's column maxima
  uint8_t* pbuf = ws.take<uint8_t>(pack_bytes);
  if (!meas) PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd: workspace too small");
  b.P1.scale = qscale;
  double rel1, relfail;
  shifts_for(PLOM_PREC_MIXED, m, N, rel1, relfail);
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  ChunkEvents ev;
  cudaStream_t cs = nullptr;
  if (!meas) {
    cs = host_copy_stream();
    PLOM_REQUIRE(cs && ev.ok, PLOM_ERR_CUDA, "tsqr_svd: packing stream or events unavailable");
    PLOM_CHECK_CUDA(cudaEventRecord(ev.start, st));  // X and the planes are ready from here
    PLOM_CHECK_CUDA(cudaStreamWaitEvent(cs, ev.start, 0));
  }
  for (int c = 0; c < C; ++c) {
    const int64_t r0 = (int64_t)c * mc;
    Packed v = packed_rows_view(b.P0, r0, mc, mc, xscale ? xscale + (int64_t)c * ldp : nullptr);
    // the packing stream's own workspace (its launches run beside the Grams')
    Arena pa(pbuf, meas ? 0 : pack_bytes);
    PLOM_TRY(pack_f32(X + r0 * ldx, ldx, mc, N, v, pa, meas ? st : cs));
    if (!meas) PLOM_CHECK_CUDA(cudaEventRecord(ev.packed[c], cs));
  }
  // the chunks' Grams as they are packed, one reduction over all of them
  PLOM_TRY(sub([&] {
    return gram_packed_chunks(b.P0, C, mc, xscale, b.G, meas ? nullptr : ev.packed, info, ws, st);
  }));
  PLOM_TRY(sub([&] { return chol_shifted(b.G, b.R1, N, 1, rel1, relfail, info, ws, st); }));
  PLOM_TRY(sub([&] { return trtri_upper(b.R1, b.W1, N, 1, ws, st); }));
  Packed P0b = b.P0, P1b = b.P1;
  P0b.batch = P1b.batch = C;
  P0b.m = P1b.m = mc;
  P0b.mp = P1b.mp = mc;
  P0b.scale = xscale;
  P1b.scale = qscale;
  PLOM_TRY(sub([&] { return apply_packed(P0b, b.W1, N, N, nullptr, 0, &P1b, info, ws, st, 0, 0, true); }));
  PLOM_TRY(sub([&] { return cholqr3_packed_passes23(false, n, b, relfail, info, ws, st); }));
  ws.off = need;
  return PLOM_OK;
}

static int cholqr3_packed(bool cplx, const float* X, int64_t m, int n, int64_t ldx,
                          PackedCore& b, int* info, Arena& ws, cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  const int C = overlap_chunks(cplx, m, N);
  if (C > 1 && b.P0.mp == m && b.P1.mp == m)
    return cholqr3_packed_chunked(X, m, n, ldx, C, b, info, ws, st);
  double rel1, relfail;
  shifts_for(PLOM_PREC_MIXED, m, N, rel1, relfail);
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  int s = PLOM_OK;
  PLOM_TRY(sub([&] { return pack_f32(X, ldx, m, N, b.P0, ws, st); }));
  // pass 1
  PLOM_TRY(sub([&] { return chol_pass_packed(cplx, n, b.P0, b, b.R1, b.W1, rel1, relfail, info, ws, st); }));
  const double* F1 = ws.measuring() ? b.W1 : rowform(cplx, b.W1, b.F, n, st, s);
  PLOM_TRY(s);
  PLOM_TRY(sub([&] { return apply_packed(b.P0, F1, N, N, nullptr, 0, &b.P1, info, ws, st, 0, 0, true); }));
  PLOM_TRY(sub([&] { return cholqr3_packed_passes23(cplx, n, b, relfail, info, ws, st); }));
  ws.off = need;
  return PLOM_OK;
}

// P1 may live in a float output buffer of m rows x ld floats when ld covers
// the packed pitch (4 m packed_ld(N) bytes)
static bool p1_fits(int64_t ld_floats, int N) { return ld_floats >= packed_ld(N); }

// svd(Re) = Ur S V^T and U = Q2 (R3^-1 Ur) into the first m rows of U (ldu),
// S, VT, after the CholeskyQR3 passes (b.P2, b.W3, b.Re)
static int svd_tail_packed(bool cplx, int n, PackedCore& b, int64_t m, float* U, int64_t ldu,
                           float* S, float* VT, int* info, Arena& ws, cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  const int cw = cplx ? 2 : 1;
  double* Rc = ws.take<double>((size_t)n * n * cw);
  double* Ur = ws.take<double>((size_t)n * n * cw);
  double* VH = ws.take<double>((size_t)n * n * cw);
  double* S64 = ws.take<double>(n);
  double* Me = ws.take<double>((size_t)N * N);
  double* Ue = ws.take<double>((size_t)N * N);
  if (!ws.measuring())
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd: workspace too small (%zu > %zu)",
                 ws.off, ws.cap);
  const size_t mark = ws.off;
  size_t need = mark;
  const double* Rin = b.Re;
  if (cplx && !ws.measuring()) {
    PLOM_TRY(embed_to_complex(b.Re, Rc, n, 1, st));
    Rin = Rc;
  }
  // the mixed form's R carries FP32-level information: columns orthogonal to
  // 1e-8 are final there
  PLOM_TRY(jacobi_svd(Rin, n, 1, cplx ? 1 : 0, 1e-8, S64, Ur, VH, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = mark;
  const double* Mop = b.F;
  if (!cplx && N >= DF_PRODUCT_MIN_N) {
    // M = R3^-1 Ur, the right operand of Q2 x M (double-float products)
    PLOM_TRY(gemm_nn_df(b.W3, Ur, Me, N, ws, st));
    need = std::max(need, ws.off);
    ws.off = mark;
    Mop = Me;
  } else if (!ws.measuring()) {
    // M = R3^-1 Ur (embedded for complex), the right operand of Q2 x M
    if (cplx) {
      PLOM_TRY(complex_to_embed(Ur, Ue, n, 1, st));
      PLOM_TRY((gemm_sq_nn(b.W3, Ue, Me, N, 1, 1, st)));
      PLOM_TRY(embed_to_rowform(Me, b.F, n, 1, st));
    } else {
      PLOM_TRY((gemm_sq_nn(b.W3, Ur, Me, N, 1, 1, st)));
      Mop = Me;
    }
  }
  Packed P2 = b.P2;
  P2.m = m;  // output rows (the planes may carry zero padding rows past m)
  PLOM_TRY(apply_packed(P2, Mop, N, N, U, ldu, nullptr, info, ws, st));
  PLOM_TRY(renorm_long_columns(Me, N, n, cw, U, m, ldu, 1, 0, 0, ws, st));
  if (!cplx) PLOM_TRY(complete_null_columns<float>(S64, n, U, m, ldu, b.G, Me, ws, st));
  if (!ws.measuring()) {
    PLOM_TRY((convert<double, float>(S64, S, n, st)));
    PLOM_TRY((convert<double, float>(VH, VT, (int64_t)n * n * cw, st)));
  }
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

static int tsqr_svd_packed(bool cplx, const float* X, int64_t m, int n, int64_t ldx, float* U,
                           int64_t ldu, float* S, float* VT, int* info, Arena& ws,
                           cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  PackedCore b;
  carve_packed_core(ws, b, m, N, p1_fits(ldu, N), U);
  if (!ws.measuring())
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd: workspace too small (%zu > %zu)",
                 ws.off, ws.cap);
  const size_t mark = ws.off;
  PLOM_TRY(cholqr3_packed(cplx, X, m, n, ldx, b, info, ws, st));
  const size_t need = ws.off;
  ws.off = mark;
  PLOM_TRY(svd_tail_packed(cplx, n, b, m, U, ldu, S, VT, info, ws, st));
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// Batched mixed-form TSQR-SVD: `batch` FP32 problems of the same shape (real,
// or complex as interleaved real views), e.g. SPOD's per-frequency matrices.
// Every stage is one launch over the whole batch: packed Grams and applies
// with a problem index on the work items, batched Cholesky / inverse /
// Jacobi, batched small GEMMs.
// ---------------------------------------------------------------------------
static int tsqr_svd_batched_packed(bool cplx, const float* X, int64_t batch, int64_t m, int n,
                                   int64_t ldx, int64_t xstride, float* U, int64_t ldu,
                                   int64_t ustride, float* S, float* VT, int* info, Arena& ws,
                                   cudaStream_t st) {
  const int N = cplx ? 2 * n : n;
  const int cw = cplx ? 2 : 1;
  const int bi = (int)batch;
  const int64_t NN = (int64_t)N * N;
  const size_t nnb = (size_t)(NN * batch);
  double* G = ws.take<double>(nnb);
  double* H = ws.take<double>(nnb);
  double* R1 = ws.take<double>(nnb);
  double* R2 = ws.take<double>(nnb);
  double* R3 = ws.take<double>(nnb);
  double* W1 = ws.take<double>(nnb);
  double* W2 = ws.take<double>(nnb);
  double* W3 = ws.take<double>(nnb);
  double* Rp = ws.take<double>(nnb);
  double* Re = ws.take<double>(nnb);
  double* F = ws.take<double>(nnb);
  double* Me = ws.take<double>(nnb);
  double* Ue = ws.take<double>(nnb);
  const size_t cnb = (size_t)n * n * cw * batch;
  double* Rc = ws.take<double>(cnb);
  double* Ur = ws.take<double>(cnb);
  double* VH = ws.take<double>(cnb);
  double* S64 = ws.take<double>((size_t)n * batch);
  Packed P0, P1, P2;
  packed_carve(ws, P0, m, N, batch);
  packed_carve(ws, P1, m, N, batch);
  P2 = P0;
  P2.scale = ws.take<float>((size_t)(P0.ld * batch));
  if (!ws.measuring())
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd_batched: workspace too small");
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  const bool meas = ws.measuring();
  double rel1, relfail;
  shifts_for(PLOM_PREC_MIXED, m, N, rel1, relfail);
  auto pass = [&](const Packed& P, double* R, double* W, double rel0) -> int {
    PLOM_TRY(sub([&] { return gram_packed(P, cplx ? H : G, info, ws, st); }));
    if (cplx && !meas) PLOM_TRY(complexify_gram(H, G, n, bi, st));
    PLOM_TRY(sub([&] { return chol_shifted(G, R, N, bi, rel0, relfail, info, ws, st); }));
    return sub([&] { return trtri_upper(R, W, N, bi, ws, st); });
  };
  auto rowform_b = [&](const double* W) -> const double* {
    if (!cplx || meas) return W;
    return embed_to_rowform(W, F, n, bi, st) == PLOM_OK ? F : nullptr;
  };
  PLOM_TRY(sub([&] { return pack_f32(X, ldx, m, N, P0, ws, st, xstride); }));
  PLOM_TRY(pass(P0, R1, W1, rel1));
  const double* F1 = rowform_b(W1);
  PLOM_REQUIRE(meas || F1, PLOM_ERR_CUDA, "tsqr_svd_batched: embedding failed");
  PLOM_TRY(sub([&] { return apply_packed(P0, F1, N, N, nullptr, 0, &P1, info, ws, st, NN, 0, true); }));
  PLOM_TRY(pass(P1, R2, W2, 0.0));
  const double* F2 = rowform_b(W2);
  PLOM_REQUIRE(meas || F2, PLOM_ERR_CUDA, "tsqr_svd_batched: embedding failed");
  PLOM_TRY(sub([&] { return apply_packed(P1, F2, N, N, nullptr, 0, &P2, info, ws, st, NN, 0, true); }));
  PLOM_TRY(pass(P2, R3, W3, 0.0));
  const double* Rin = Re;
  if (!meas) {
    PLOM_TRY((gemm_sq_nn(R3, R2, Rp, N, bi, 3, st)));
    PLOM_TRY((gemm_sq_nn(Rp, R1, Re, N, bi, 3, st)));
    if (cplx) {
      PLOM_TRY(embed_to_complex(Re, Rc, n, bi, st));
      Rin = Rc;
    }
  }
  PLOM_TRY(sub([&] { return jacobi_svd(Rin, n, bi, cplx ? 1 : 0, 1e-8, S64, Ur, VH, info, ws, st); }));
  const double* Mop = F;
  if (!meas) {
    // M = R3^-1 Ur (embedded for complex), the right operand of Q2 x M
    if (cplx) {
      PLOM_TRY(complex_to_embed(Ur, Ue, n, bi, st));
      PLOM_TRY((gemm_sq_nn(W3, Ue, Me, N, bi, 1, st)));
      PLOM_TRY(embed_to_rowform(Me, F, n, bi, st));
    } else {
      PLOM_TRY((gemm_sq_nn(W3, Ur, Me, N, bi, 1, st)));
      Mop = Me;
    }
  }
  PLOM_TRY(sub([&] {
    PLOM_TRY(apply_packed(P2, Mop, N, N, U, ldu, nullptr, info, ws, st, NN, ustride));
    return renorm_long_columns(Me, N, n, cw, U, m, ldu, bi, NN, ustride, ws, st);
  }));
  if (!meas) {
    PLOM_TRY((convert<double, float>(S64, S, (int64_t)n * batch, st)));
    PLOM_TRY((convert<double, float>(VH, VT, (int64_t)n * n * cw * batch, st)));
  }
  ws.off = need;
  return PLOM_OK;
}

// Q = Q2 R3^-1 and R = R3 R2 R1.  hh: with Householder QR's column signs
// (LAPACK geqrf's factors, which the reference's qr/tsqr return): the signs
// come from the top n rows of Q, computed first, and are folded into R3^-1
// and R before the full product, so Q is written once.  Needs m >= n.
static int tsqr_packed(const float* X, int64_t m, int n, int64_t ldx, float* Q, int64_t ldq,
                       float* R, int* info, Arena& ws, cudaStream_t st, bool hh = false) {
  PackedCore b;
  carve_packed_core(ws, b, m, n, p1_fits(ldq, n), Q);
  if (!ws.measuring()) PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr: workspace too small");
  const size_t mark = ws.off;
  PLOM_TRY(cholqr3_packed(false, X, m, n, ldx, b, info, ws, st));
  size_t need = ws.off;
  ws.off = mark;
  if (hh) {
    float* T = ws.take<float>((size_t)n * n);
    double* sg = ws.take<double>(n);
    Packed top = packed_rows_view(b.P2, 0, n, n, b.P2.scale);
    PLOM_TRY(apply_packed(top, b.W3, n, n, T, n, nullptr, info, ws, st, 0, 0, true));
    PLOM_TRY(householder_signs<float>(T, n, n, m == n, sg, ws, st));
    if (!ws.measuring()) PLOM_TRY(sign_fold(b.W3, b.Re, sg, n, st));
    need = std::max(need, ws.off);
    ws.off = mark;
  }
  PLOM_TRY(apply_packed(b.P2, b.W3, n, n, Q, ldq, nullptr, info, ws, st, 0, 0, true));
  if (!ws.measuring()) PLOM_TRY((convert<double, float>(b.Re, R, (int64_t)n * n, st)));
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

template <typename TI, typename TC>
static void carve_core(Arena& ws, CoreBufs<TI, TC>& b, int64_t m, int N, bool need_q1) {
  const size_t nn = (size_t)N * N;
  b.G = ws.take<double>(nn);
  b.H = ws.take<double>(nn);
  b.R1 = ws.take<double>(nn);
  b.R2 = ws.take<double>(nn);
  b.R3 = ws.take<double>(nn);
  b.W1 = ws.take<double>(nn);
  b.W2 = ws.take<double>(nn);
  b.W3 = ws.take<double>(nn);
  b.Rp = ws.take<double>(nn);
  b.Re = ws.take<double>(nn);
  b.F = ws.take<double>(nn);
  b.Q1 = need_q1 ? ws.take<TC>((size_t)m * N) : nullptr;
  b.Q2 = ws.take<TC>((size_t)m * N);
}

// ---------------------------------------------------------------------------
// tsqr_svd driver
// ---------------------------------------------------------------------------
template <typename TI, typename TC>
static int tsqr_svd_impl(int prec, bool cplx, const TI* X, int64_t m, int n, int64_t ldx, TI* U,
                         int64_t ldu, TI* S, TI* VT, int* info, Arena& ws, cudaStream_t st) {
  if constexpr (std::is_same<TI, float>::value && std::is_same<TC, float>::value) {
    if (prec == PLOM_PREC_MIXED && packed_ok(m))
      return tsqr_svd_packed(cplx, X, m, n, ldx, U, ldu, S, VT, info, ws, st);
  }
  const int N = cplx ? 2 * n : n;
  // Q1 can live in U when U has the compute type and is densely packed
  const bool q1_in_u = std::is_same<TI, TC>::value && ldu == N;
  CoreBufs<TI, TC> b;
  carve_core<TI, TC>(ws, b, m, N, !q1_in_u);
  const int cw = cplx ? 2 : 1;
  double* Rc = ws.take<double>((size_t)n * n * cw);
  double* Ur = ws.take<double>((size_t)n * n * cw);
  double* VH = ws.take<double>((size_t)n * n * cw);
  double* S64 = ws.take<double>(n);
  double* Me = ws.take<double>((size_t)N * N);
  double* Ue = ws.take<double>((size_t)N * N);
  if (!ws.measuring())
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd: workspace too small (%zu > %zu)",
                 ws.off, ws.cap);
  size_t scratch_mark = ws.off;
  PLOM_TRY((cholqr3<TI, TC>(prec, cplx, X, m, n, ldx, q1_in_u ? (TC*)(void*)U : nullptr, N, b,
                            info, ws, st)));
  size_t need = ws.off;
  ws.off = scratch_mark;
  // small SVD of R (FP64)
  const double* Rin = b.Re;
  if (cplx && !ws.measuring()) {
    PLOM_TRY(embed_to_complex(b.Re, Rc, n, 1, st));
    Rin = Rc;
  }
  // the mixed form's R carries FP32-level information: columns orthogonal to
  // 1e-8 are final there; the FP64 form iterates to n * DBL_EPSILON
  const double jtol = (prec == PLOM_PREC_MIXED) ? 1e-8 : 0.0;
  PLOM_TRY(jacobi_svd(Rin, n, 1, cplx ? 1 : 0, jtol, S64, Ur, VH, info, ws, st));
  need = std::max(need, ws.off);
  ws.off = scratch_mark;
  if (!ws.measuring()) {
    // M = R3^-1 Ur (embedded for complex), as the right operand of Q2 x M
    const double* Mop;
    if (cplx) {
      PLOM_TRY(complex_to_embed(Ur, Ue, n, 1, st));
      PLOM_TRY((gemm_sq_nn(b.W3, Ue, Me, N, 1, 1, st)));
      PLOM_TRY(embed_to_rowform(Me, b.F, n, 1, st));
      Mop = b.F;
    } else {
      PLOM_TRY((gemm_sq_nn(b.W3, Ur, Me, N, 1, 1, st)));
      Mop = Me;
    }
    PLOM_TRY((tall_apply<TC, TI>(prec, b.Q2, N, m, N, Mop, N, U, ldu, info, ws, st)));
    PLOM_TRY((convert<double, TI>(S64, S, n, st)));
    PLOM_TRY((convert<double, TI>(VH, VT, (int64_t)n * n * cw, st)));
  } else {
    PLOM_TRY((tall_apply<TC, TI>(prec, b.Q2, N, m, N, b.F, N, U, ldu, info, ws, st)));
  }
  if (!cplx) PLOM_TRY(complete_null_columns<TI>(S64, n, U, m, ldu, b.G, Me, ws, st));
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

template <typename TI, typename TC>
static int tsqr_impl(int prec, const TI* X, int64_t m, int n, int64_t ldx, TI* Q, int64_t ldq,
                     TI* R, int* info, Arena& ws, cudaStream_t st, bool hh = false) {
  if constexpr (std::is_same<TI, float>::value && std::is_same<TC, float>::value) {
    if (prec == PLOM_PREC_MIXED && packed_ok(m))
      return tsqr_packed(X, m, n, ldx, Q, ldq, R, info, ws, st, hh);
  }
  CoreBufs<TI, TC> b;
  const bool q1_in_q = std::is_same<TI, TC>::value && ldq == n;
  carve_core<TI, TC>(ws, b, m, n, !q1_in_q);
  TI* T = hh ? ws.take<TI>((size_t)n * n) : nullptr;
  double* sg = hh ? ws.take<double>(n) : nullptr;
  if (!ws.measuring()) PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr: workspace too small");
  PLOM_TRY((cholqr3<TI, TC>(prec, false, X, m, n, ldx, q1_in_q ? (TC*)(void*)Q : nullptr, n, b,
                            info, ws, st)));
  size_t need = ws.off;
  if (hh) {
    // signs from the top n rows of Q (see tsqr_packed), folded into R3^-1 and R
    PLOM_TRY((tall_apply<TC, TI>(prec, b.Q2, n, n, n, b.W3, n, T, n, info, ws, st, true)));
    PLOM_TRY(householder_signs<TI>(T, n, n, m == n, sg, ws, st));
    if (!ws.measuring()) PLOM_TRY(sign_fold(b.W3, b.Re, sg, n, st));
    need = std::max(need, ws.off);
  }
  PLOM_TRY((tall_apply<TC, TI>(prec, b.Q2, n, m, n, b.W3, n, Q, ldq, info, ws, st, true)));
  if (!ws.measuring()) PLOM_TRY((convert<double, TI>(b.Re, R, (int64_t)n * n, st)));
  ws.off = std::max(need, ws.off);
  return PLOM_OK;
}

// ---------------------------------------------------------------------------
// randomized SVD (pyLOM/vmmath/svd.py:121-144, 255-273; svd.c:1267-1519)
// ---------------------------------------------------------------------------
// Mixed form on FP32 data: A is packed once; the passes over it (A Omega,
// A^T Q, A Q2, Q^T A) run on the tensor cores from the packed planes.
// Two modes: randomized_svd (U, S, VT) and, with `qr`, randomized_qr (Q m x r
// with Householder QR's column signs into Qout (ldq), B = Q^T A r x n into
// Bout).  omega_in (n x r, or null): the test matrix instead of Philox(seed).
static int rsvd_packed(const float* A, int64_t m, int64_t n, int64_t lda, int r, int q,
                       uint64_t seed, const float* omega_in, bool qr, float* U, int64_t ldu,
                       float* S, float* VT, float* Qout, int64_t ldq, float* Bout, int* info,
                       Arena& ws, cudaStream_t st) {
  Packed Ap, Qp;
  packed_carve(ws, Ap, m, n);
  packed_carve(ws, Qp, m, r);
  float* omega = ws.take<float>((size_t)n * r);
  double* om64 = ws.take<double>((size_t)n * r);
  float* Y = ws.take<float>((size_t)m * r);
  float* Qm = qr ? Qout : ws.take<float>((size_t)m * r);
  const int64_t ldqm = qr ? ldq : r;
  float* Rq = ws.take<float>((size_t)r * r);
  double* Q2 = ws.take<double>((size_t)n * r);  // A^T Q (n x r); the last one is B^T
  double* Ub = qr ? nullptr : ws.take<double>((size_t)n * r);
  double* Sb = qr ? nullptr : ws.take<double>(r);
  double* VbH = qr ? nullptr : ws.take<double>((size_t)r * r);
  double* Ur = qr ? nullptr : ws.take<double>((size_t)r * r);
  double* Vo = ws.take<double>((size_t)r * n);
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  const bool meas = ws.measuring();
  if (!meas) {
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "randomized_svd: workspace too small");
    if (omega_in)
      PLOM_TRY((convert<float, double>(omega_in, om64, n * r, st)));
    else {
      PLOM_TRY(fill_uniform_dispatch(PLOM_F32, omega, n * r, seed, st));
      PLOM_TRY((convert<float, double>(omega, om64, n * r, st)));
    }
  }
  PLOM_TRY(sub([&] { return pack_f32(A, lda, m, n, Ap, ws, st); }));
  // Y = A Omega
  PLOM_TRY(sub([&] { return apply_packed(Ap, om64, r, r, Y, r, nullptr, info, ws, st); }));
  for (int j = 0; j <= q; ++j) {
    // only the final range basis needs Householder QR's signs
    const bool hh = qr && j == q;
    PLOM_TRY(sub([&] { return tsqr_packed(Y, m, r, r, Qm, ldqm, Rq, info, ws, st, hh); }));
    PLOM_TRY(sub([&] { return pack_f32(Qm, ldqm, m, r, Qp, ws, st); }));
    // Q2 = A^T Q (n x r); after the last iteration this is B^T = (Q^T A)^T
    PLOM_TRY(sub([&] { return tn_packed(Ap, Qp, Q2, r, info, ws, st); }));
    if (j == q) break;
    PLOM_TRY(sub([&] { return apply_packed(Ap, Q2, r, r, Y, r, nullptr, info, ws, st); }));
  }
  if (qr) {
    if (!meas) {
      PLOM_TRY(transpose_f64(Q2, Vo, n, r, 1, st));  // B (r x n) = (B^T)^T
      PLOM_TRY((convert<double, float>(Vo, Bout, (int64_t)r * n, st)));
    }
    ws.off = need;
    return PLOM_OK;
  }
  // svd(B) through the tall n x r matrix B^T: B^T = Ub Sb VbH -> B = Vb Sb Ub^T
  PLOM_TRY(sub([&]() {
    return tsqr_svd_impl<double, double>(PLOM_PREC_FP64, false, Q2, n, r, r, Ub, r, Sb, VbH, info,
                                         ws, st);
  }));
  if (!meas) {
    PLOM_TRY(transpose_f64(VbH, Ur, r, r, 1, st));  // Ur = Vb = VbH^T (real)
    PLOM_TRY(transpose_f64(Ub, Vo, n, r, 1, st));   // V (r x n) = Ub^T
    PLOM_TRY((convert<double, float>(Sb, S, r, st)));
    PLOM_TRY((convert<double, float>(Vo, VT, (int64_t)r * n, st)));
  }
  // U = Q Ur
  PLOM_TRY(sub([&] { return tall_apply<float, float>(PLOM_PREC_MIXED, Qm, r, m, r, Ur, r, U, ldu, info, ws, st); }));
  ws.off = need;
  return PLOM_OK;
}

template <typename TI, typename TC>
static int rsvd_impl(int prec, const TI* A, int64_t m, int64_t n, int64_t lda, int r, int q,
                     uint64_t seed, const TI* omega_in, bool qr, TI* U, int64_t ldu, TI* S,
                     TI* VT, TI* Qout, int64_t ldq, TI* Bout, int* info, Arena& ws,
                     cudaStream_t st) {
  if constexpr (std::is_same<TI, float>::value && std::is_same<TC, float>::value) {
    if (prec == PLOM_PREC_MIXED && packed_ok(m))
      return rsvd_packed(A, m, n, lda, r, q, seed, omega_in, qr, U, ldu, S, VT, Qout, ldq, Bout,
                         info, ws, st);
  }
  TI* omega = ws.take<TI>((size_t)n * r);
  TC* omc = ws.take<TC>((size_t)n * r);
  TC* Y = ws.take<TC>((size_t)m * r);
  TC* Qm = ws.take<TC>((size_t)m * r);
  double* Rr = ws.take<double>((size_t)r * r);
  TC* Q2 = ws.take<TC>((size_t)n * r);
  double* B = ws.take<double>((size_t)r * n);
  double* Bt = ws.take<double>((size_t)n * r);
  double* Ub = ws.take<double>((size_t)n * r);
  double* Sb = ws.take<double>(r);
  double* VbH = ws.take<double>((size_t)r * r);
  double* Ur = ws.take<double>((size_t)r * r);
  double* Vo = ws.take<double>((size_t)r * n);
  TC* Rq = ws.take<TC>((size_t)r * r);
  (void)Rr;
  size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  const bool meas = ws.measuring();
  if (!meas) {
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "randomized_svd: workspace too small");
    if (omega_in)
      PLOM_TRY((convert<TI, TC>(omega_in, omc, n * r, st)));
    else {
      PLOM_TRY(fill_uniform_dispatch(sizeof(TI) == 8 ? PLOM_F64 : PLOM_F32, omega, n * r, seed, st));
      PLOM_TRY((convert<TI, TC>(omega, omc, n * r, st)));
    }
  }
  // Y = A Omega
  auto apply_small = [&](const TC* Bm, TC* C) -> int {  // C(m x r) = A(m x n) Bm(n x r)
    if (prec == PLOM_PREC_FP64 || sizeof(TC) == 8)
      return gemm_nn<TI, TC, TC, double>(A, lda, Bm, r, C, r, m, r, n, st);
    return gemm_nn<TI, TC, TC, float>(A, lda, Bm, r, C, r, m, r, n, st);
  };
  if (!meas) PLOM_TRY(apply_small(omc, Y));
  for (int j = 0; j <= q; ++j) {
    // only the final range basis needs Householder QR's signs
    const bool hh = qr && j == q;
    PLOM_TRY(sub([&]() { return tsqr_impl<TC, TC>(prec, Y, m, r, r, Qm, r, Rq, info, ws, st, hh); }));
    if (j == q) break;
    // Q2 = A^T Q  (n x r), then Y = A Q2
    PLOM_TRY(sub([&]() {
      if (prec == PLOM_PREC_FP64 || sizeof(TC) == 8)
        return gemm_tn<TI, TC, double, TC>(A, lda, Qm, r, Q2, r, n, r, m, false, ws, st);
      return gemm_tn<TI, TC, float, TC>(A, lda, Qm, r, Q2, r, n, r, m, false, ws, st);
    }));
    if (!meas) PLOM_TRY(apply_small(Q2, Y));
  }
  // B = Q^T A  (r x n, FP64)
  PLOM_TRY(sub([&]() {
    if (prec == PLOM_PREC_FP64 || sizeof(TC) == 8)
      return gemm_tn<TC, TI, double, double>(Qm, r, A, lda, B, n, r, n, m, false, ws, st);
    return gemm_tn<TC, TI, float, double>(Qm, r, A, lda, B, n, r, n, m, false, ws, st);
  }));
  if (qr) {
    if (!meas) {
      PLOM_TRY((copy2d<TC, TI>(Qm, r, Qout, ldq, m, r, st)));
      PLOM_TRY((convert<double, TI>(B, Bout, (int64_t)r * n, st)));
    }
    ws.off = need;
    return PLOM_OK;
  }
  // svd(B) through the tall n x r matrix B^T: B^T = Ub Sb VbH -> B = Vb Sb Ub^T
  if (!meas) PLOM_TRY(transpose_f64(B, Bt, r, n, 1, st));
  PLOM_TRY(sub([&]() {
    return tsqr_svd_impl<double, double>(PLOM_PREC_FP64, false, Bt, n, r, r, Ub, r, Sb, VbH,
                                         info, ws, st);
  }));
  if (!meas) {
    PLOM_TRY(transpose_f64(VbH, Ur, r, r, 1, st));  // Ur = Vb = VbH^T (real)
    PLOM_TRY(transpose_f64(Ub, Vo, n, r, 1, st));   // V (r x n) = Ub^T
    PLOM_TRY((convert<double, TI>(Sb, S, r, st)));
    PLOM_TRY((convert<double, TI>(Vo, VT, (int64_t)r * n, st)));
  }
  // U = Q Ur
  PLOM_TRY(sub([&]() { return tall_apply<TC, TI>(prec, Qm, r, m, r, Ur, r, U, ldu, info, ws, st); }));
  ws.off = need;
  return PLOM_OK;
}

}  // namespace plom

using namespace plom;

static bool prec_ok(int p) { return p == PLOM_PREC_FP64 || p == PLOM_PREC_MIXED; }

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// Workspace queries run the driver with a null arena: nothing may launch.
// A failing dry run (a launch attempted, an unsupported shape) reports 0.
template <typename Fn>
static int run_measured(size_t* bytes, Fn&& fn) {
  Arena a(nullptr, 0);
  int s = fn(a);
  *bytes = (s == PLOM_OK) ? a.off + 1024 : 0;
  return s;
}

static int tsqr_svd_dispatch(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                             void* U, int64_t ldu, void* S, void* VT, int* info, Arena& ws,
                             cudaStream_t st) {
  const int ni = (int)n;
  switch (dtype) {
    case PLOM_F32:
      if (prec == PLOM_PREC_FP64)
        return tsqr_svd_impl<float, double>(prec, false, (const float*)X, m, ni, ldx, (float*)U,
                                            ldu, (float*)S, (float*)VT, info, ws, st);
      return tsqr_svd_impl<float, float>(prec, false, (const float*)X, m, ni, ldx, (float*)U, ldu,
                                         (float*)S, (float*)VT, info, ws, st);
    case PLOM_F64:
      return tsqr_svd_impl<double, double>(PLOM_PREC_FP64, false, (const double*)X, m, ni, ldx,
                                           (double*)U, ldu, (double*)S, (double*)VT, info, ws, st);
    case PLOM_C64:
      if (prec == PLOM_PREC_FP64)
        return tsqr_svd_impl<float, double>(prec, true, (const float*)X, m, ni, 2 * ldx,
                                            (float*)U, 2 * ldu, (float*)S, (float*)VT, info, ws,
                                            st);
      return tsqr_svd_impl<float, float>(prec, true, (const float*)X, m, ni, 2 * ldx, (float*)U,
                                         2 * ldu, (float*)S, (float*)VT, info, ws, st);
    case PLOM_C128:
      return tsqr_svd_impl<double, double>(PLOM_PREC_FP64, true, (const double*)X, m, ni, 2 * ldx,
                                           (double*)U, 2 * ldu, (double*)S, (double*)VT, info, ws,
                                           st);
  }
  set_error("tsqr_svd: unknown dtype %d", dtype);
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" size_t plom_tsqr_svd_workspace(int dtype, int prec, int64_t m, int64_t n) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return tsqr_svd_dispatch(dtype, prec, nullptr, m, n, n, nullptr, n, nullptr, nullptr, dummy, a,
                             0);
  });
  return bytes;
}

extern "C" int plom_tsqr_svd(int dtype, int prec, const void* X, int64_t m, int64_t n,
                             int64_t ldx, void* U, int64_t ldu, void* S, void* VT, void* ws,
                             size_t ws_bytes, int* info, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(m >= 1 && n >= 1 && n <= 4096, PLOM_ERR_ARG,
               "tsqr_svd: need m >= 1 and 1 <= n <= 4096 (m=%lld n=%lld)", (long long)m,
               (long long)n);
  PLOM_REQUIRE(ldx >= n && ldu >= n, PLOM_ERR_ARG, "tsqr_svd: leading dimension < n");
  PLOM_REQUIRE(X && U && S && VT && info && ws, PLOM_ERR_ARG, "tsqr_svd: null pointer");
  size_t need = plom_tsqr_svd_workspace(dtype, prec, m, n);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "tsqr_svd: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "tsqr_svd: workspace %zu < required %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return tsqr_svd_dispatch(dtype, prec, X, m, n, ldx, U, ldu, S, VT, info, a, (cudaStream_t)stream);
}

// batch of problems: the mixed form on FP32 / complex64 data runs batched;
// every other form runs the single-problem driver per problem, reusing one
// workspace.  Strides in elements of the data type.
static int tsqr_svd_batched_dispatch(int dtype, int prec, const void* X, int64_t batch, int64_t m,
                                     int64_t n, int64_t ldx, int64_t xstride, void* U, int64_t ldu,
                                     int64_t ustride, void* S, void* VT, int* info, Arena& ws,
                                     cudaStream_t st) {
  const bool mixed32 = prec == PLOM_PREC_MIXED && (dtype == PLOM_F32 || dtype == PLOM_C64) &&
                       m >= n && packed_ok(cdiv(m, 128) * 128 * batch);
  if (mixed32) {
    const int c = dtype == PLOM_C64 ? 2 : 1;
    return tsqr_svd_batched_packed(c == 2, (const float*)X, batch, m, (int)n, c * ldx, c * xstride,
                                   (float*)U, c * ldu, c * ustride, (float*)S, (float*)VT, info, ws,
                                   st);
  }
  const size_t es = (dtype == PLOM_F32) ? 4 : (dtype == PLOM_F64 || dtype == PLOM_C64) ? 8 : 16;
  const size_t rs = (dtype == PLOM_F32 || dtype == PLOM_C64) ? 4 : 8;
  const size_t mark = ws.off;
  size_t need = mark;
  for (int64_t p = 0; p < (ws.measuring() ? 1 : batch); ++p) {
    ws.off = mark;
    const char* xp = X ? (const char*)X + (size_t)p * xstride * es : nullptr;
    char* up = U ? (char*)U + (size_t)p * ustride * es : nullptr;
    char* sp = S ? (char*)S + (size_t)p * n * rs : nullptr;
    char* vp = VT ? (char*)VT + (size_t)p * n * n * es : nullptr;
    PLOM_TRY(tsqr_svd_dispatch(dtype, prec, xp, m, n, ldx, up, ldu, sp, vp, info, ws, st));
    need = std::max(need, ws.off);
  }
  ws.off = need;
  return PLOM_OK;
}

extern "C" size_t plom_tsqr_svd_batched_workspace(int dtype, int prec, int64_t batch, int64_t m,
                                                  int64_t n) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return tsqr_svd_batched_dispatch(dtype, prec, nullptr, batch, m, n, n, m * n, nullptr, n,
                                     m * n, nullptr, nullptr, dummy, a, 0);
  });
  return bytes;
}

extern "C" int plom_tsqr_svd_batched(int dtype, int prec, const void* X, int64_t batch, int64_t m,
                                     int64_t n, int64_t ldx, int64_t xstride, void* U, int64_t ldu,
                                     int64_t ustride, void* S, void* VT, void* ws, size_t ws_bytes,
                                     int* info, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(batch >= 1 && m >= 1 && n >= 1 && n <= 4096 && m >= n, PLOM_ERR_ARG,
               "tsqr_svd_batched: need batch >= 1 and 1 <= n <= min(m, 4096)");
  PLOM_REQUIRE(ldx >= n && ldu >= n && xstride >= m * ldx && ustride >= m * ldu, PLOM_ERR_ARG,
               "tsqr_svd_batched: leading dimension or stride too small");
  PLOM_REQUIRE(X && U && S && VT && info && ws, PLOM_ERR_ARG, "tsqr_svd_batched: null pointer");
  size_t need = plom_tsqr_svd_batched_workspace(dtype, prec, batch, m, n);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "tsqr_svd_batched: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "tsqr_svd_batched: workspace %zu < %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return tsqr_svd_batched_dispatch(dtype, prec, X, batch, m, n, ldx, xstride, U, ldu, ustride, S,
                                   VT, info, a, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Host-buffer entry: X, U, S, VT in host memory (page-locked memory lets the
// copies overlap the GPU work).  The mixed form on real FP32 data streams X
// in row chunks: the copy engine moves chunk c + 1 while the GPU packs chunk
// c with its own power-of-two column scales and adds its Gram into G1; the
// pass-1 product then runs over the chunks as a batch (one W = R1^-1, the
// chunks' own input scales, one packed Q1 of all rows), and the remaining
// passes, the small SVD and U = Q2 (R3^-1 Ur) are the device pipeline.  The
// last chunk is padded with zero rows (they stay zero through every pass).
// Other forms copy X in whole, run the device driver and copy back.
// ---------------------------------------------------------------------------
constexpr int HOST_CHUNKS = 16;

struct HostPlan {
  int64_t mc;  // rows per chunk (a multiple of 128)
  int C;       // chunks
  int64_t M;   // C * mc >= m
};

static HostPlan host_plan(int64_t m) {
  HostPlan h;
  const int64_t want = std::min<int64_t>(HOST_CHUNKS, std::max<int64_t>(1, m / 65536));
  h.mc = cdiv(cdiv(m, want), 128) * 128;
  h.C = (int)cdiv(m, h.mc);
  h.M = h.mc * h.C;
  return h;
}

struct HostEvents {
  cudaEvent_t start = nullptr, copied[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr};
  bool ok = false;
  HostEvents() {
    ok = cudaEventCreateWithFlags(&start, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < 2; ++i) {
      ok = ok && cudaEventCreateWithFlags(&copied[i], cudaEventDisableTiming) == cudaSuccess;
      ok = ok && cudaEventCreateWithFlags(&freed[i], cudaEventDisableTiming) == cudaSuccess;
    }
  }
  ~HostEvents() {  // released once their pending work completes
    if (start) cudaEventDestroy(start);
    for (int i = 0; i < 2; ++i) {
      if (copied[i]) cudaEventDestroy(copied[i]);
      if (freed[i]) cudaEventDestroy(freed[i]);
    }
  }
};

static int tsqr_svd_host_mixed(const float* Xh, int64_t m, int n, int64_t ldx, float* Uh,
                               int64_t ldu, float* Sh, float* VTh, int* info, Arena& ws,
                               cudaStream_t st) {
  const int N = n;
  const HostPlan pl = host_plan(m);
  const int64_t ldp = packed_ld(N);
  const int64_t M = pl.M;
  const bool meas = ws.measuring();
  float* Ud = ws.take<float>((size_t)M * std::max<int64_t>(n, ldp));  // U, and Q1's planes before it
  float* stage = ws.take<float>((size_t)2 * pl.mc * n);
  float* Sd = ws.take<float>((size_t)n);
  float* VTd = ws.take<float>((size_t)n * n);
  float* xscale = ws.take<float>((size_t)pl.C * ldp);
  float* qscale = ws.take<float>((size_t)pl.C * ldp);
  PackedCore b;
  carve_packed_core(ws, b, M, N, true, Ud);
  b.P1.scale = qscale;
  if (!meas) {
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd_host: workspace too small");
    PLOM_REQUIRE(Xh && Uh && Sh && VTh, PLOM_ERR_ARG, "tsqr_svd_host: null host pointer");
  }
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  double rel1, relfail;
  shifts_for(PLOM_PREC_MIXED, M, N, rel1, relfail);
  HostEvents ev;
  cudaStream_t cs = nullptr;
  if (!meas) {
    cs = host_copy_stream();
    PLOM_REQUIRE(cs && ev.ok, PLOM_ERR_CUDA, "tsqr_svd_host: copy stream or events unavailable");
    PLOM_CHECK_CUDA(cudaEventRecord(ev.start, st));  // the staging buffers are free from here
    PLOM_CHECK_CUDA(cudaStreamWaitEvent(cs, ev.start, 0));
  }
  // pass 1, chunk by chunk: copy, pack with the chunk's scales, add its Gram
  for (int c = 0; c < pl.C; ++c) {
    const int slot = c & 1;
    const int64_t r0 = (int64_t)c * pl.mc;
    const int64_t rows = std::min<int64_t>(pl.mc, m - r0);
    float* sb = stage ? stage + (int64_t)slot * pl.mc * n : nullptr;
    if (!meas) {
      if (c >= 2) PLOM_CHECK_CUDA(cudaStreamWaitEvent(cs, ev.freed[slot], 0));
      PLOM_CHECK_CUDA(cudaMemcpy2DAsync(sb, sizeof(float) * n, Xh + r0 * ldx, sizeof(float) * ldx,
                                        sizeof(float) * n, rows, cudaMemcpyHostToDevice, cs));
      PLOM_CHECK_CUDA(cudaEventRecord(ev.copied[slot], cs));
      PLOM_CHECK_CUDA(cudaStreamWaitEvent(st, ev.copied[slot], 0));
    }
    Packed v = packed_rows_view(b.P0, r0, rows, pl.mc, xscale ? xscale + (int64_t)c * ldp : nullptr);
    PLOM_TRY(sub([&] { return pack_f32(sb, n, rows, N, v, ws, st); }));
    if (!meas) PLOM_CHECK_CUDA(cudaEventRecord(ev.freed[slot], st));
    PLOM_TRY(sub([&] { return gram_packed(v, b.G, info, ws, st, c > 0); }));
  }
  PLOM_TRY(sub([&] { return chol_shifted(b.G, b.R1, N, 1, rel1, relfail, info, ws, st); }));
  PLOM_TRY(sub([&] { return trtri_upper(b.R1, b.W1, N, 1, ws, st); }));
  // Q1 = X R1^-1 with the chunks as a batch: one W, each chunk's input scales
  Packed P0b = b.P0, P1b = b.P1;
  P0b.batch = P1b.batch = pl.C;
  P0b.m = P1b.m = pl.mc;
  P0b.mp = P1b.mp = pl.mc;
  P0b.scale = xscale;
  P1b.scale = qscale;
  PLOM_TRY(sub([&] { return apply_packed(P0b, b.W1, N, N, nullptr, 0, &P1b, info, ws, st, 0, 0, true); }));
  PLOM_TRY(sub([&] { return cholqr3_packed_passes23(false, n, b, relfail, info, ws, st); }));
  // U straight into page-locked host memory when the caller's U is mapped
  // (the final product's stores cross the host link while it computes);
  // otherwise into the device buffer and copied back
  float* Umapped = nullptr;
  if (!meas) {
    void* dp = nullptr;
    if (cudaHostGetDevicePointer(&dp, Uh, 0) == cudaSuccess) Umapped = static_cast<float*>(dp);
    else cudaGetLastError();  // pageable U: clear the error and copy
  }
  PLOM_TRY(sub([&] {
    return svd_tail_packed(false, n, b, m, Umapped ? Umapped : Ud, Umapped ? ldu : n, Sd, VTd, info,
                           ws, st);
  }));
  ws.off = need;
  if (!meas) {
    if (!Umapped)
      PLOM_CHECK_CUDA(cudaMemcpy2DAsync(Uh, sizeof(float) * ldu, Ud, sizeof(float) * n,
                                        sizeof(float) * n, m, cudaMemcpyDeviceToHost, st));
    PLOM_CHECK_CUDA(cudaMemcpyAsync(Sh, Sd, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    PLOM_CHECK_CUDA(cudaMemcpyAsync(VTh, VTd, sizeof(float) * n * n, cudaMemcpyDeviceToHost, st));
  }
  return PLOM_OK;
}

static size_t dtype_bytes(int dtype) {
  return dtype == PLOM_F32 ? 4 : (dtype == PLOM_F64 || dtype == PLOM_C64) ? 8 : 16;
}
static size_t real_bytes(int dtype) { return (dtype == PLOM_F32 || dtype == PLOM_C64) ? 4 : 8; }

static int tsqr_svd_host_dispatch(int dtype, int prec, const void* X, int64_t m, int64_t n,
                                  int64_t ldx, void* U, int64_t ldu, void* S, void* VT, int* info,
                                  Arena& ws, cudaStream_t st) {
  if (prec == PLOM_PREC_MIXED && dtype == PLOM_F32 && packed_ok(host_plan(m).M))
    return tsqr_svd_host_mixed((const float*)X, m, (int)n, ldx, (float*)U, ldu, (float*)S,
                               (float*)VT, info, ws, st);
  // whole copies around the device driver
  const size_t es = dtype_bytes(dtype), rs = real_bytes(dtype);
  char* Xd = ws.take<char>((size_t)m * n * es);
  char* Ud = ws.take<char>((size_t)m * n * es);
  char* Sd = ws.take<char>((size_t)n * rs);
  char* VTd = ws.take<char>((size_t)n * n * es);
  if (!ws.measuring()) {
    PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "tsqr_svd_host: workspace too small");
    PLOM_REQUIRE(X && U && S && VT, PLOM_ERR_ARG, "tsqr_svd_host: null host pointer");
    PLOM_CHECK_CUDA(cudaMemcpy2DAsync(Xd, es * n, X, es * ldx, es * n, m, cudaMemcpyHostToDevice, st));
  }
  PLOM_TRY(tsqr_svd_dispatch(dtype, prec, Xd, m, n, n, Ud, n, Sd, VTd, info, ws, st));
  if (!ws.measuring()) {
    PLOM_CHECK_CUDA(cudaMemcpy2DAsync(U, es * ldu, Ud, es * n, es * n, m, cudaMemcpyDeviceToHost, st));
    PLOM_CHECK_CUDA(cudaMemcpyAsync(S, Sd, rs * n, cudaMemcpyDeviceToHost, st));
    PLOM_CHECK_CUDA(cudaMemcpyAsync(VT, VTd, es * n * n, cudaMemcpyDeviceToHost, st));
  }
  return PLOM_OK;
}

extern "C" size_t plom_tsqr_svd_host_workspace(int dtype, int prec, int64_t m, int64_t n) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return tsqr_svd_host_dispatch(dtype, prec, nullptr, m, n, n, nullptr, n, nullptr, nullptr,
                                  dummy, a, 0);
  });
  return bytes;
}

extern "C" int plom_tsqr_svd_host(int dtype, int prec, const void* X, int64_t m, int64_t n,
                                  int64_t ldx, void* U, int64_t ldu, void* S, void* VT, void* ws,
                                  size_t ws_bytes, int* info, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(m >= 1 && n >= 1 && n <= 4096 && m >= n, PLOM_ERR_ARG,
               "tsqr_svd_host: need 1 <= n <= min(m, 4096) (m=%lld n=%lld)", (long long)m,
               (long long)n);
  PLOM_REQUIRE(ldx >= n && ldu >= n, PLOM_ERR_ARG, "tsqr_svd_host: leading dimension < n");
  PLOM_REQUIRE(X && U && S && VT && info && ws, PLOM_ERR_ARG, "tsqr_svd_host: null pointer");
  size_t need = plom_tsqr_svd_host_workspace(dtype, prec, m, n);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "tsqr_svd_host: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "tsqr_svd_host: workspace %zu < required %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return tsqr_svd_host_dispatch(dtype, prec, X, m, n, ldx, U, ldu, S, VT, info, a,
                                (cudaStream_t)stream);
}

static int tsqr_dispatch(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                         void* Q, int64_t ldq, void* R, int* info, Arena& ws, cudaStream_t st) {
  if (dtype == PLOM_F32) {
    if (prec == PLOM_PREC_FP64)
      return tsqr_impl<float, double>(prec, (const float*)X, m, (int)n, ldx, (float*)Q, ldq,
                                      (float*)R, info, ws, st, true);
    return tsqr_impl<float, float>(prec, (const float*)X, m, (int)n, ldx, (float*)Q, ldq,
                                   (float*)R, info, ws, st, true);
  }
  if (dtype == PLOM_F64)
    return tsqr_impl<double, double>(PLOM_PREC_FP64, (const double*)X, m, (int)n, ldx, (double*)Q,
                                     ldq, (double*)R, info, ws, st, true);
  set_error("tsqr: dtype must be F32 or F64");
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" size_t plom_tsqr_workspace(int dtype, int prec, int64_t m, int64_t n) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return tsqr_dispatch(dtype, prec, nullptr, m, n, n, nullptr, n, nullptr, dummy, a, 0);
  });
  return bytes;
}

extern "C" int plom_tsqr(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                         void* Q, int64_t ldq, void* R, void* ws, size_t ws_bytes, int* info,
                         void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(n >= 1 && m >= n && n <= 4096, PLOM_ERR_ARG, "tsqr: need 1 <= n <= min(m, 4096)");
  PLOM_REQUIRE(ldx >= n && ldq >= n, PLOM_ERR_ARG, "tsqr: leading dimension < n");
  PLOM_REQUIRE(X && Q && R && info && ws, PLOM_ERR_ARG, "tsqr: null pointer");
  size_t need = plom_tsqr_workspace(dtype, prec, m, n);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "tsqr: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "tsqr: workspace %zu < required %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return tsqr_dispatch(dtype, prec, X, m, n, ldx, Q, ldq, R, info, a, (cudaStream_t)stream);
}

static int rsvd_dispatch(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                         int64_t r, int q, uint64_t seed, const void* omega, bool qr, void* U,
                         int64_t ldu, void* S, void* VT, void* Q, int64_t ldq, void* B, int* info,
                         Arena& ws, cudaStream_t st) {
  if (dtype == PLOM_F32) {
    if (prec == PLOM_PREC_FP64)
      return rsvd_impl<float, double>(prec, (const float*)X, m, n, ldx, (int)r, q, seed,
                                      (const float*)omega, qr, (float*)U, ldu, (float*)S,
                                      (float*)VT, (float*)Q, ldq, (float*)B, info, ws, st);
    return rsvd_impl<float, float>(prec, (const float*)X, m, n, ldx, (int)r, q, seed,
                                   (const float*)omega, qr, (float*)U, ldu, (float*)S, (float*)VT,
                                   (float*)Q, ldq, (float*)B, info, ws, st);
  }
  if (dtype == PLOM_F64)
    return rsvd_impl<double, double>(PLOM_PREC_FP64, (const double*)X, m, n, ldx, (int)r, q, seed,
                                     (const double*)omega, qr, (double*)U, ldu, (double*)S,
                                     (double*)VT, (double*)Q, ldq, (double*)B, info, ws, st);
  set_error("randomized_svd: dtype must be F32 or F64");
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" size_t plom_randomized_svd_workspace(int dtype, int prec, int64_t m, int64_t n,
                                                int64_t r) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return rsvd_dispatch(dtype, prec, nullptr, m, n, n, r, 1, 0, nullptr, false, nullptr, r,
                         nullptr, nullptr, nullptr, r, nullptr, dummy, a, 0);
  });
  return bytes;
}

extern "C" int plom_randomized_svd(int dtype, int prec, const void* X, int64_t m, int64_t n,
                                   int64_t ldx, int64_t r, int q, uint64_t seed, void* U,
                                   int64_t ldu, void* S, void* VT, void* ws, size_t ws_bytes,
                                   int* info, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(m >= 1 && n >= 1 && r >= 1 && r <= n && r <= m && r <= 4096 && q >= 0,
               PLOM_ERR_ARG, "randomized_svd: need 1 <= r <= min(m, n, 4096), q >= 0");
  PLOM_REQUIRE(ldx >= n && ldu >= r, PLOM_ERR_ARG, "randomized_svd: leading dimension too small");
  PLOM_REQUIRE(X && U && S && VT && info && ws, PLOM_ERR_ARG, "randomized_svd: null pointer");
  size_t need = plom_randomized_svd_workspace(dtype, prec, m, n, r);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "randomized_svd: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "randomized_svd: workspace %zu < %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return rsvd_dispatch(dtype, prec, X, m, n, ldx, r, q, seed, nullptr, false, U, ldu, S, VT,
                       nullptr, r, nullptr, info, a, (cudaStream_t)stream);
}

extern "C" size_t plom_randomized_qr_workspace(int dtype, int prec, int64_t m, int64_t n,
                                               int64_t r) {
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return rsvd_dispatch(dtype, prec, nullptr, m, n, n, r, 1, 0, nullptr, true, nullptr, r,
                         nullptr, nullptr, nullptr, r, nullptr, dummy, a, 0);
  });
  return bytes;
}

extern "C" int plom_randomized_qr(int dtype, int prec, const void* X, int64_t m, int64_t n,
                                  int64_t ldx, int64_t r, int q, uint64_t seed, const void* omega,
                                  void* Q, int64_t ldq, void* B, void* ws, size_t ws_bytes,
                                  int* info, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(m >= 1 && n >= 1 && r >= 1 && r <= n && r <= m && r <= 4096 && q >= 0,
               PLOM_ERR_ARG, "randomized_qr: need 1 <= r <= min(m, n, 4096), q >= 0");
  PLOM_REQUIRE(ldx >= n && ldq >= r, PLOM_ERR_ARG, "randomized_qr: leading dimension too small");
  PLOM_REQUIRE(X && Q && B && info && ws, PLOM_ERR_ARG, "randomized_qr: null pointer");
  size_t need = plom_randomized_qr_workspace(dtype, prec, m, n, r);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "randomized_qr: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "randomized_qr: workspace %zu < %zu",
               ws_bytes, need);
  Arena a(ws, ws_bytes);
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, (cudaStream_t)stream));
  return rsvd_dispatch(dtype, prec, X, m, n, ldx, r, q, seed, omega, true, nullptr, r, nullptr,
                       nullptr, Q, ldq, B, info, a, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// matmul / matmulp
// ---------------------------------------------------------------------------
template <typename T>
static int matmul_impl(int prec, int transA, const T* A, int64_t lda, const T* B, int64_t ldb,
                       T* C, int64_t ldc, int64_t m, int64_t n, int64_t k, Arena& ws,
                       cudaStream_t st) {
  const bool fp64 = (prec == PLOM_PREC_FP64) || sizeof(T) == 8;
  if (transA == 0) {
    if constexpr (sizeof(T) == 4) {
      if (!fp64 && packed_ok(m) && m >= 1 && n >= 1 && k >= 1) {
        int* flag = ws.take<int>(PLOM_INFO_WORDS);  // launch-wide abort word
        double* B64 = ws.take<double>((size_t)k * n);
        Packed p;
        packed_carve(ws, p, m, k);
        if (!ws.measuring()) {
          PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "matmul: workspace too small");
          PLOM_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int) * PLOM_INFO_WORDS, st));
          PLOM_TRY((copy2d<float, double>(B, ldb, B64, n, k, n, st)));
        }
        PLOM_TRY(pack_f32(A, lda, m, k, p, ws, st));
        return apply_packed(p, B64, n, n, C, ldc, nullptr, flag, ws, st);
      }
    }
    if (ws.measuring()) return PLOM_OK;
    if (fp64) return gemm_nn<T, T, T, double>(A, lda, B, ldb, C, ldc, m, n, k, st);
    return gemm_nn<T, T, T, float>(A, lda, B, ldb, C, ldc, m, n, k, st);
  }
  if constexpr (sizeof(T) == 4) {
    // mixed form: both tall operands packed, the reduction over their k rows
    // on the tensor cores (A^T B, double-float partials), FP32 result
    if (!fp64 && packed_ok(k) && m >= 1 && n >= 1 && k >= 1) {
      int* flag = ws.take<int>(PLOM_INFO_WORDS);
      double* C64 = ws.take<double>((size_t)m * n);
      Packed pa, pb;
      packed_carve(ws, pa, k, m);
      packed_carve(ws, pb, k, n);
      if (!ws.measuring()) {
        PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "matmul: workspace too small");
        PLOM_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int) * PLOM_INFO_WORDS, st));
      }
      PLOM_TRY(pack_f32(A, lda, k, m, pa, ws, st));
      PLOM_TRY(pack_f32(B, ldb, k, n, pb, ws, st));
      PLOM_TRY(tn_packed(pa, pb, C64, n, flag, ws, st));
      if (ws.measuring()) return PLOM_OK;
      return copy2d<double, float>(C64, n, C, ldc, m, n, st);
    }
  }
  if (fp64) return gemm_tn<T, T, double, T>(A, lda, B, ldb, C, ldc, m, n, k, false, ws, st);
  return gemm_tn<T, T, float, T>(A, lda, B, ldb, C, ldc, m, n, k, false, ws, st);
}

static int matmul_dispatch(int dtype, int prec, int transA, const void* A, int64_t lda,
                           const void* B, int64_t ldb, void* C, int64_t ldc, int64_t m, int64_t n,
                           int64_t k, Arena& ws, cudaStream_t st) {
  if (dtype == PLOM_F32)
    return matmul_impl<float>(prec, transA, (const float*)A, lda, (const float*)B, ldb, (float*)C,
                              ldc, m, n, k, ws, st);
  if (dtype == PLOM_F64)
    return matmul_impl<double>(prec, transA, (const double*)A, lda, (const double*)B, ldb,
                               (double*)C, ldc, m, n, k, ws, st);
  set_error("matmul: dtype must be F32 or F64");
  return PLOM_ERR_UNSUPPORTED;
}

extern "C" size_t plom_matmul_workspace(int dtype, int prec, int transA, int64_t m, int64_t n,
                                        int64_t k) {
  size_t bytes = 0;
  run_measured(&bytes, [&](Arena& a) {
    return matmul_dispatch(dtype, prec, transA, nullptr, m, nullptr, n, nullptr, n, m, n, k, a, 0);
  });
  return bytes;
}

// ---------------------------------------------------------------------------
// DMD's reduced operator on span(U_r) (pyLOM/DMD/wrapper.py:78-84 computes
// U_r^T Y2 V_r S_r^-1 from the truncated SVD of Y1 = Y[:, :-1]).  With FP32
// factors (and the mixed form's ~1e-5 tensor-core accumulation error in U, S,
// V) that formula takes the factors' mutual inconsistency into the
// eigenvalues.  Here every quantity is recomputed from span(U_r) alone:
//   C = U_r^T U_r and B = U_r^T Y      (exact products, double-float sums),
//   R^T R = C,  Bt = R^-T B            (coordinates of Y in an orthonormal
//                                       basis Ut = U_r R^-1 of span(U_r)),
//   Bt[:, :nt] = Vb S' V'^T            (FP64 SVD, through its transpose),
//   aux1 = Vb^T Bt[:, 1:],  S',  V'^T  (for the reduced stage).
// In exact arithmetic Ut Vb = U_r, S' = S_r, V' = V_r and aux1 = U_r^T Y2.
// ---------------------------------------------------------------------------
static int dmd_project_impl(const float* U, int64_t ldu, const float* Y, int64_t ldy, int64_t m,
                            int n, int r, double* aux1, double* S, double* VT, int* info,
                            Arena& ws, cudaStream_t st) {
  const int nt = n - 1;
  double* C = ws.take<double>((size_t)r * r);
  double* B = ws.take<double>((size_t)r * n);
  double* R = ws.take<double>((size_t)r * r);
  double* W = ws.take<double>((size_t)r * r);
  double* Wt = ws.take<double>((size_t)r * r);
  double* Bt = ws.take<double>((size_t)r * n);
  double* BtT = ws.take<double>((size_t)n * r);
  double* Ub = ws.take<double>((size_t)nt * r);
  double* VbH = ws.take<double>((size_t)r * r);
  const size_t mark = ws.off;
  size_t need = mark;
  auto sub = [&](auto&& fn) -> int {
    ws.off = mark;
    const int s = fn();
    need = std::max(need, ws.off);
    ws.off = mark;
    return s;
  };
  const bool meas = ws.measuring();
  if (!meas) PLOM_REQUIRE(!ws.overflow(), PLOM_ERR_WORKSPACE, "dmd_project: workspace too small");
  PLOM_TRY(sub([&] { return gemm_tn_df(U, ldu, U, ldu, C, r, r, r, m, ws, st); }));
  PLOM_TRY(sub([&] { return gemm_tn_df(U, ldu, Y, ldy, B, n, r, n, m, ws, st); }));
  const double u = 2.220446049250313e-16;
  PLOM_TRY(sub([&] { return chol_shifted(C, R, r, 1, 0.0, 16.0 * u * r, info, ws, st); }));
  PLOM_TRY(sub([&] { return trtri_upper(R, W, r, 1, ws, st); }));
  if (!meas) {
    PLOM_TRY(transpose_f64(W, Wt, r, r, 1, st));
    PLOM_TRY((gemm_nn<double, double, double, double>(Wt, r, B, n, Bt, n, r, n, r, st)));
    PLOM_TRY(transpose_f64(Bt, BtT, r, n, 1, st));  // rows 0..nt-1: Bt[:, :nt]^T
  }
  // Bt[:, :nt]^T (nt x r) = Ub S' VbH  ->  Bt[:, :nt] = Vb S' Ub^T
  PLOM_TRY(sub([&] {
    return tsqr_svd_impl<double, double>(PLOM_PREC_FP64, false, BtT, nt, r, r, Ub, r, S, VbH,
                                         info, ws, st);
  }));
  if (!meas) {
    // aux1 = Vb^T Bt[:, 1:] = VbH Bt[:, 1:];  V'^T = Ub^T
    PLOM_TRY((gemm_nn<double, double, double, double>(VbH, r, Bt + 1, n, aux1, nt, r, nt, r, st)));
    PLOM_TRY(transpose_f64(Ub, VT, nt, r, 1, st));
  }
  ws.off = need;
  return PLOM_OK;
}

extern "C" size_t plom_dmd_project_workspace(int64_t m, int64_t n, int64_t r) {
  if (m < 1 || n < 2 || r < 1 || r > n - 1 || r > 1024 || n > INT32_MAX) return 0;
  size_t bytes = 0;
  int dummy[PLOM_INFO_WORDS];
  run_measured(&bytes, [&](Arena& a) {
    return dmd_project_impl(nullptr, r, nullptr, n, m, (int)n, (int)r, nullptr, nullptr, nullptr,
                            dummy, a, nullptr);
  });
  return bytes;
}

extern "C" int plom_dmd_project(const float* U, int64_t ldu, const float* Y, int64_t ldy,
                                int64_t m, int64_t n, int64_t r, double* aux1, double* S,
                                double* VT, void* ws, size_t ws_bytes, int* info, void* stream) {
  PLOM_REQUIRE(m >= 1 && n >= 2 && r >= 1 && r <= n - 1 && r <= 1024 && n <= INT32_MAX,
               PLOM_ERR_ARG, "dmd_project: need m >= 1, n >= 2 and 1 <= r <= min(n - 1, 1024)");
  PLOM_REQUIRE(ldu >= r && ldy >= n, PLOM_ERR_ARG, "dmd_project: leading dimension too small");
  PLOM_REQUIRE(U && Y && aux1 && S && VT && ws && info, PLOM_ERR_ARG,
               "dmd_project: null pointer");
  const size_t need = plom_dmd_project_workspace(m, n, r);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "dmd_project: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "dmd_project: workspace %zu < %zu", ws_bytes,
               need);
  cudaStream_t st = (cudaStream_t)stream;
  PLOM_CHECK_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * PLOM_INFO_WORDS, st));
  Arena a(ws, ws_bytes);
  return dmd_project_impl(U, ldu, Y, ldy, m, (int)n, (int)r, aux1, S, VT, info, a, st);
}

extern "C" int plom_matmul(int dtype, int prec, int transA, const void* A, int64_t lda,
                           const void* B, int64_t ldb, void* C, int64_t ldc, int64_t m, int64_t n,
                           int64_t k, void* ws, size_t ws_bytes, void* stream) {
  PLOM_REQUIRE(prec_ok(prec), PLOM_ERR_ARG, "bad precision %d", prec);
  PLOM_REQUIRE(transA == 0 || transA == 1, PLOM_ERR_ARG, "transA must be 0 or 1");
  PLOM_REQUIRE(m >= 0 && n >= 0 && k >= 0, PLOM_ERR_ARG, "negative size");
  PLOM_REQUIRE(ldb >= n && ldc >= n && lda >= (transA ? m : k), PLOM_ERR_ARG,
               "matmul: leading dimension too small");
  PLOM_REQUIRE((A && B && C) || m * n == 0, PLOM_ERR_ARG, "matmul: null pointer");
  size_t need = plom_matmul_workspace(dtype, prec, transA, m, n, k);
  PLOM_REQUIRE(need > 0, PLOM_ERR_ARG, "matmul: workspace query failed");
  PLOM_REQUIRE(ws_bytes >= need, PLOM_ERR_WORKSPACE, "matmul: workspace %zu < %zu", ws_bytes,
               need);
  Arena a(ws, ws_bytes);
  return matmul_dispatch(dtype, prec, transA, A, lda, B, ldb, C, ldc, m, n, k, a,
                         (cudaStream_t)stream);
}
