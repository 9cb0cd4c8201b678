/*
 * libplom -- C ABI of the GB300 (sm_103a) implementation of pyLOM's SVD hot
 * path.  Every entry point:
 *   - takes DEVICE pointers (row-major, C-contiguous matrices with an explicit
 *     leading dimension), int64 sizes and a cudaStream_t passed as void*;
 *   - allocates nothing: outputs and workspace are owned by the caller
 *     (workspace sizes come from the matching *_workspace query);
 *   - is stream-ordered and re-entrant per stream (no global mutable state);
 *   - returns an int status (PLOM_OK, or a negative PLOM_ERR_* for argument,
 *     workspace or CUDA-launch errors; the message is in
 *     plom_last_error_string(), kept per host thread).  Numerical failures
 *     detected on the device (Cholesky breakdown after all shift escalations,
 *     Jacobi non-convergence, non-finite input) are written to the caller's
 *     device array `info` (PLOM_INFO_WORDS int32 words), info[0] = PLOM_NUM_*.
 *     Diagnostics in the same array: info[1] Cholesky shift escalations,
 *     info[2] Jacobi sweeps (FP64 or double-float rows), info[4] FP32
 *     Jacobi pre-sweeps (mixed form, real, 512 <= n <= 1600; 0 otherwise).
 *
 * Each declaration names the pyLOM interface it replaces (paths inside the
 * pyLowOrder project): the C symbols pyLOM binds through Cython in
 * pyLOM/vmmath/cfuncs.pxd and the Python functions of pyLOM/vmmath/*.py.
 */
#ifndef PLOM_H
#define PLOM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (return values) */
#define PLOM_OK 0
#define PLOM_ERR_ARG (-1)
#define PLOM_ERR_WORKSPACE (-2)
#define PLOM_ERR_CUDA (-3)
#define PLOM_ERR_UNSUPPORTED (-4)

/* numerical failure codes (info[0], written on the device) */
#define PLOM_NUM_OK 0
#define PLOM_NUM_CHOLESKY 1
#define PLOM_NUM_JACOBI 2
#define PLOM_NUM_NONFINITE 3
#define PLOM_NUM_EIG 4
#define PLOM_NUM_TIMEOUT 5 /* a bounded device-side wait expired (the kernel stopped early) */
#define PLOM_INFO_WORDS 8

/* element types */
#define PLOM_F32 0
#define PLOM_F64 1
#define PLOM_C64 2
#define PLOM_C128 3

/* precision forms */
#define PLOM_PREC_FP64 0  /* every product and reduction in FP64 (plain FP64 GPU form) */
#define PLOM_PREC_MIXED 1 /* tall-skinny products on tensor cores (FP32 operands packed as
                             fp16 hi/lo pairs with per-column power-of-two scales, three f16
                             products, FP32 accumulate), small n x n factorizations in FP64 */

const char* plom_last_error_string(void);
int plom_version(void);

/* Run-time schedule and tile parameters of the tall tensor-core kernels (no
   counterpart in pyLOM, whose products are LAPACK/BLAS calls): the Gram's
   work items per SM per wave ("gram_wave_mult", 1-32; "gram_wide_wave_mult",
   1-256, for Grams wider than 128 columns), the resident blocks
   per SM of its slab reduction ("reduce_blocks_per_sm", 1-16), the output
   tile width of dense products wider than 128 columns ("apply_dense_tn",
   128 or 256), whether such products give each CTA whole row blocks
   ("apply_dense_by_rows", 0 or 1; "apply_tri_by_rows" for triangular W)
   and the row chunks of a large FP32 input
   packed on a second stream beside the first Gram ("pass1_chunks", 1, 2, 4
   or 8; 1 packs it whole first) and which products of one tall matrix wider
   than 128 columns run on SM pairs with 256 x 256 tiles (2-SM UMMA,
   "apply_pair": 0 none, 1 dense W, 2 dense and triangular W).  Process-wide; set them before the
   workspace queries of the calls they are to govern.  The Python package
   applies the values in its tuning file at load (pyloworder_gb300.autotune
   measures and writes them).  plom_set_tuning returns PLOM_ERR_ARG for an
   unknown key or a value outside the listed range; plom_get_tuning returns
   -1 for an unknown key. */
int plom_set_tuning(const char* key, double value);
double plom_get_tuning(const char* key);

/* Per-kernel device timing on the calling host thread, the device-side
   counterpart of pyLOM's named timing channels (pyLOM/utils/cr.py:199-246
   cr_start/cr_stop, cr_info).  plom_profile_begin starts recording CUDA
   events around every kernel launch; plom_profile_end waits for them and
   writes one line per timed region name: "name regions total_ms flops bytes
   launches" (algorithmic flops/bytes of the regions; a region is one kernel
   launch, or a routine's few launches timed together). */
int plom_profile_begin(void);
int plom_profile_end(char* buf, size_t cap);

/* ---- averaging --------------------------------------------------------- */
/* replaces stemporal_mean/dtemporal_mean (pyLOM/vmmath/src/averaging.c:10,29;
   Python pyLOM/vmmath/averaging.py:18).  mean has m entries. */
int plom_temporal_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx, void* mean,
                       void* stream);
/* replaces ssubtract_mean/dsubtract_mean (averaging.c:92,109; averaging.py:32) */
int plom_subtract_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                       const void* mean, void* Y, int64_t ldy, void* stream);
/* replaces stemporal_variance/dtemporal_variance (averaging.c:48,70; averaging.py:47) */
int plom_temporal_variance(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                           const void* mean, void* var, void* stream);
/* replaces snorm_variance/dnorm_variance (averaging.c:126,143; averaging.py:62):
   Y = (X - mean) / var */
int plom_norm_variance(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx,
                       const void* mean, const void* var, void* Y, int64_t ldy, void* stream);
/* fused mean (+variance) + subtract (+divide) in one pass over X: the
   POD/DMD/SPOD preamble (pyLOM/POD/wrapper.py:33-43).  var may be NULL when
   divide_variance == 0. */
int plom_remove_mean(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx, void* mean,
                     void* var, int divide_variance, void* Y, int64_t ldy, void* stream);

/* ---- products ---------------------------------------------------------- */
/* replaces smatmul/dmatmul (pyLOM/vmmath/src/vector_matrix.c:224,234; Python
   maths.py:77) for transA == 0:  C(m x n) = A(m x k) B(k x n);
   and smatmulp/dmatmulp (vector_matrix.c:330,344; maths.py:93, called as
   matmulp(A.T, B)) for transA == 1:  C(m x n) = A(k x m)^T B(k x n), the sum
   over the long k axis done as a split-K reduction on the device. */
size_t plom_matmul_workspace(int dtype, int prec, int transA, int64_t m, int64_t n, int64_t k);
int plom_matmul(int dtype, int prec, int transA, const void* A, int64_t lda, const void* B,
                int64_t ldb, void* C, int64_t ldc, int64_t m, int64_t n, int64_t k, void* ws,
                size_t ws_bytes, void* stream);

/* ---- SVD family -------------------------------------------------------- */
/* replaces stsqr/dtsqr (pyLOM/vmmath/src/svd.c:416,565; svd.py:50):
   Q (m x n, ldq) with orthonormal columns and upper-triangular R (n x n) with
   X = Q R, m >= n.  The factors carry the column signs of Householder QR
   (LAPACK geqrf + orgqr, which the reference's qr and one-rank tsqr return):
   R_kk = -sign(pivot_k) |R_kk| as Householder's reflections choose it, not
   CholeskyQR's positive diagonal.  dtype F32 or F64 (R has the same type). */
size_t plom_tsqr_workspace(int dtype, int prec, int64_t m, int64_t n);
int plom_tsqr(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx, void* Q,
              int64_t ldq, void* R, void* ws, size_t ws_bytes, int* info, void* stream);

/* replaces stsqr_svd/dtsqr_svd/ctsqr_svd/ztsqr_svd (svd.c:529,678,827,976;
   svd.pyx:446; svd.py:228):  X (m x n) = U diag(S) VT with U m x n (ldu),
   S n (real, descending), VT n x n (rows = right singular vectors).
   Complex dtypes take interleaved (re,im) storage; S is then real of the
   matching precision. */
size_t plom_tsqr_svd_workspace(int dtype, int prec, int64_t m, int64_t n);
int plom_tsqr_svd(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx, void* U,
                  int64_t ldu, void* S, void* VT, void* ws, size_t ws_bytes, int* info,
                  void* stream);

/* a batch of tsqr_svd problems of one shape (problem p at X + p xstride,
   U + p ustride, S + p n, VT + p n n; strides in elements of dtype): the
   per-frequency SVDs of SPOD (pyLOM/SPOD/wrapper.py:75-85 calls tsqr_svd once
   per frequency).  The mixed form on F32/C64 data runs every stage as one
   launch over the batch; the other forms run the problems one by one. */
/* plom_tsqr_svd with X, U, S, VT in HOST memory (page-locked memory lets
   the copies overlap the GPU work; pageable memory works too).  The same
   pyLOM interface (svd.py:228); the call streams X to the device in row
   chunks on an internal copy stream, overlapping the first pass, and copies
   U, S, VT back on `stream`.  m >= n. */
size_t plom_tsqr_svd_host_workspace(int dtype, int prec, int64_t m, int64_t n);
int plom_tsqr_svd_host(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                       void* U, int64_t ldu, void* S, void* VT, void* ws, size_t ws_bytes,
                       int* info, void* stream);

size_t plom_tsqr_svd_batched_workspace(int dtype, int prec, int64_t batch, int64_t m, int64_t n);
int plom_tsqr_svd_batched(int dtype, int prec, const void* X, int64_t batch, int64_t m, int64_t n,
                          int64_t ldx, int64_t xstride, void* U, int64_t ldu, int64_t ustride,
                          void* S, void* VT, void* ws, size_t ws_bytes, int* info, void* stream);

/* replaces srandomized_svd/drandomized_svd (svd.c:1198,1453; svd.py:255):
   U m x r, S r, VT r x n.  The test matrix Omega (n x r) is uniform [0,1)
   from a Philox4x32-10 counter stream keyed by seed (see plom_fill_uniform). */
size_t plom_randomized_svd_workspace(int dtype, int prec, int64_t m, int64_t n, int64_t r);
int plom_randomized_svd(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                        int64_t r, int q, uint64_t seed, void* U, int64_t ldu, void* S, void* VT,
                        void* ws, size_t ws_bytes, int* info, void* stream);

/* replaces srandomized_qr/drandomized_qr (svd.c:1012,1267; svd.py:121,
   randomized_qr2 at svd.py:147 computes the same factors): the randomized
   range finder Y = X Omega, q times (Q = tsqr(Y), Y = X (X^T Q)), Q =
   tsqr(Y) with Householder QR's column signs, B = Q^T X.  Outputs Q (m x r,
   ldq) and B (r x n, dense), both of dtype.  omega: the n x r test matrix
   (dtype, dense) when not NULL, else uniform [0,1) from Philox4x32-10 keyed by
   seed (see plom_fill_uniform). */
size_t plom_randomized_qr_workspace(int dtype, int prec, int64_t m, int64_t n, int64_t r);
int plom_randomized_qr(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                       int64_t r, int q, uint64_t seed, const void* omega, void* Q, int64_t ldq,
                       void* B, void* ws, size_t ws_bytes, int* info, void* stream);

/* replaces srandom_matrix/drandom_matrix (vector_matrix.c:950,964): out[i] =
   uniform [0,1) for flat index i, Philox4x32-10 with key = seed, counter = i. */
int plom_fill_uniform(int dtype, void* out, int64_t count, uint64_t seed, void* stream);

/* ---- DMD ------------------------------------------------------------- */
/* replaces the reduced-operator part of DMD.run (pyLOM/DMD/wrapper.py:84-117:
   Atilde, eigen -> maths.py:161 / vector_matrix.c:500 zeigen, vandermonde
   maths.py:203, cholesky maths.py:249, inv maths.py:277, _order_modes
   wrapper.py:18-45), all FP64 on the device.  Inputs: aux1 = U^T Y2 (r x nt),
   S (r), VT (r x nt) with nt = n_snapshots - 1.  Outputs (device, FP64):
   muReal, muImag (r), bJov (r complex, interleaved) in pyLOM's mode order,
   and Mphi (nt x r complex, interleaved) such that the DMD modes are
   Phi = Y2 Mphi (one tall product, plom_matmul with the real view). */
/* the inputs of plom_dmd_reduced for FP32 snapshots, from span(U_r) alone
   (replaces the U^T Y2 product of DMD/wrapper.py:78-84 and the use of the
   FP32 S and V there): U (m x r, ld ldu) = the retained left singular vectors
   of Y1 = Y[:, :-1], Y (m x n, ld ldy).  C = U^T U and B = U^T Y are formed
   with exact products and double-float sums; R^T R = C gives the coordinates
   Bt = R^-T B of Y in an orthonormal basis of span(U); the FP64 SVD
   Bt[:, :n-1] = Vb S V'^T gives S (r), VT = V'^T (r x (n-1)) and
   aux1 = Vb^T Bt[:, 1:] (r x (n-1)), all FP64 on the device.  In exact
   arithmetic these equal S_r, V_r^T and U_r^T Y2; the reduced operator then
   depends only on the subspace, not on the accuracy of U's norms, S or V.
   Needs n >= 2 and 1 <= r <= min(n - 1, 1024). */
size_t plom_dmd_project_workspace(int64_t m, int64_t n, int64_t r);
int plom_dmd_project(const float* U, int64_t ldu, const float* Y, int64_t ldy, int64_t m,
                     int64_t n, int64_t r, double* aux1, double* S, double* VT, void* ws,
                     size_t ws_bytes, int* info, void* stream);
size_t plom_dmd_reduced_workspace(int64_t r, int64_t nt);
int plom_dmd_reduced(const double* aux1, const double* S, const double* VT, int64_t r, int64_t nt,
                     double* muReal, double* muImag, double* bJov, double* Mphi, void* ws,
                     size_t ws_bytes, int* info, void* stream);

/* ---- SPOD ------------------------------------------------------------ */
/* replaces the Welch/FFT loop of SPOD.run (pyLOM/SPOD/wrapper.py:66-76 with
   _fft at :18-20, window from pyLOM/vmmath/fft.py:17 hammwin): for every block
   b (start b*step) and point i, the windowed FFT of Y[i, b*step : b*step+nDFT]
   is scaled by `scale` (pyLOM: winWeight/nDFT, here also /sqrt(nBlks)), bins
   1..nf-2 doubled, and bins 0..nf-1 written to Q[f][i][b] (complex,
   interleaved; Q_f is row-major M x nBlks).  twr/twi: cos/-sin(2 pi j/nDFT).
   mean (M values, or NULL): subtracted from each point's samples as they are
   loaded (SPOD.run's temporal-mean removal, wrapper.py:58-61, without a
   centred copy of Y). */
int plom_spod_fft(int dtype, const void* Y, int64_t M, int64_t N, int64_t ldy, const void* mean,
                  int64_t nDFT, int64_t step, int64_t nBlks, int64_t nf, const void* window,
                  const void* twr, const void* twi, double scale, void* Q, void* stream);

/* replaces the mode layout of SPOD.run (pyLOM/SPOD/wrapper.py:84,
   P[:, ifreq] = real(U).reshape(M*nBlks, order='F')) for the G frequencies
   f0 .. f0+G-1 of one batched SVD: P[(b*M + i)*nf + f0 + g] = Re U_g[i][b].
   U: G problems of M x nBlks complex values (interleaved, dtype = the real
   type), ustride complex elements apart; P: (M*nBlks) x nf, row-major. */
int plom_spod_modes(int dtype, const void* U, int64_t G, int64_t M, int64_t nBlks,
                    int64_t ustride, void* P, int64_t nf, int64_t f0, void* stream);
/* the final column order of P (SPOD/wrapper.py:86-95 sorts the frequencies
   by their leading energy): P[row][c] = T_k[row][g] for f = order[c] =
   k G + g, where the frequency groups' modes were written densely, group k
   as a rows x G_k block T_k = T + k gstride (G_k = min(G, nf - k G);
   plom_spod_modes with nf = G_k, f0 = 0).  rows = M nBlks; order is a device
   array of nf ints.  Every P row is written whole and contiguous.  SPOD.run
   puts T_k in the part of the Fourier coefficients its batch has consumed
   (gstride = 2 G rows). */
int plom_spod_assemble(int dtype, const void* T, int64_t rows, int64_t nf, int64_t G,
                       int64_t gstride, const int* order, void* P, void* stream);

/* ---- packed tall operands (mixed form) --------------------------------- */
/* No counterpart in the reference.  A caller that multiplies the same FP32
   matrix X (m x N, ldx) several times -- the streaming range finder uses one
   batch of snapshots in every product of a batch -- packs it once into a
   device buffer of plom_packed_bytes(m, N) bytes (two fp16 planes with
   per-column power-of-two scales, the mixed form's operand) and passes the
   buffer to the products:
     plom_packed_apply: C (m x k FP32, ldc) = X W, W N x k FP64 (ldw);
     plom_packed_tn:    C (Na x Nb FP64, ldc) = Xa^T Xb, both packed with
                        the same m rows.
   Buffers and workspaces are device memory; info as everywhere. */
size_t plom_packed_bytes(int64_t m, int64_t N);
int plom_pack(const void* X, int64_t m, int64_t N, int64_t ldx, void* packed, size_t bytes,
              void* stream);
size_t plom_packed_apply_workspace(int64_t m, int64_t N, int64_t k);
int plom_packed_apply(const void* packed, int64_t m, int64_t N, const double* W, int64_t ldw,
                      int64_t k, void* C, int64_t ldc, void* ws, size_t ws_bytes, int* info,
                      void* stream);
size_t plom_packed_tn_workspace(int64_t m, int64_t Na, int64_t Nb);
int plom_packed_tn(const void* pa, int64_t Na, const void* pb, int64_t Nb, int64_t m, double* C,
                   int64_t ldc, void* ws, size_t ws_bytes, int* info, void* stream);

/* ---- allocation-free reduction product ------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
   memory -- a host integration whose device memory is owned by another
   framework's pool, or a latency-critical loop where cudaMalloc/cudaFree
   (which synchronise the device) are not acceptable -- this computes the same
   product as plom_matmul(dtype, PLOM_PREC_FP64, transA = 1, ...):
   C(m x n) = A(k x m)^T B(k x n), FP64 accumulation, F32 or F64 data, with
   no workspace argument.  Its split-K partial sums (m * n * 8 bytes per
   chunk, at least one chunk) live in a static device array of
   PLOM_STATIC_SCRATCH_BYTES that every GPU loading the library holds until
   the process exits; larger results are rejected with PLOM_ERR_WORKSPACE
   before anything is launched.  The first call on each device looks up the
   array's device address (cudaGetSymbolAddress, with that device current):
   make that first call before any stream capture.  After a device reset
   (cudaDeviceReset, or a reset of the primary context) the array lives at a
   new address in the new context; the first call made in that context looks
   it up again (the address is cached per device with the context's unique
   ID), so that call, too, should come before any capture.  All calls share
   the array, so calls that overlap on the GPU race; serialise them (one
   stream, or events).  Allocates nothing and calls no allocating routine. */
#define PLOM_STATIC_SCRATCH_BYTES (32u << 20)
int plom_matmulp_static(int dtype, const void* A, int64_t lda, const void* B, int64_t ldb,
                        void* C, int64_t ldc, int64_t m, int64_t n, int64_t k, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLOM_H */
