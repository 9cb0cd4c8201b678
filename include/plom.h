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
#define PLOM_PREC_MIXED 1 /* tall-skinny products on tensor cores (TF32 split into three
                             terms, FP32 accumulate), small n x n factorizations in FP64 */

const char* plom_last_error_string(void);
int plom_version(void);

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
   X = Q R.  dtype F32 or F64 (R has the same type). */
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

/* replaces srandomized_svd/drandomized_svd (svd.c:1198,1453; svd.py:255):
   U m x r, S r, VT r x n.  The test matrix Omega (n x r) is uniform [0,1)
   from a Philox4x32-10 counter stream keyed by seed (see plom_fill_uniform). */
size_t plom_randomized_svd_workspace(int dtype, int prec, int64_t m, int64_t n, int64_t r);
int plom_randomized_svd(int dtype, int prec, const void* X, int64_t m, int64_t n, int64_t ldx,
                        int64_t r, int q, uint64_t seed, void* U, int64_t ldu, void* S, void* VT,
                        void* ws, size_t ws_bytes, int* info, void* stream);

/* replaces srandom_matrix/drandom_matrix (vector_matrix.c:950,964): out[i] =
   uniform [0,1) for flat index i, Philox4x32-10 with key = seed, counter = i. */
int plom_fill_uniform(int dtype, void* out, int64_t count, uint64_t seed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLOM_H */
