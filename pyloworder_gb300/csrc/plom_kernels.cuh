// Internal (C++) interfaces shared between libplom translation units.
#pragma once
#include "plom_common.cuh"

namespace plom {

// ---- averaging.cu ----
int rows_dispatch(int dtype, const void* X, int64_t m, int64_t n, int64_t ldx, const void* mean_in,
                  const void* var_in, void* mean_out, void* var_out, int want_var, int ymode,
                  void* Y, int64_t ldy, cudaStream_t st);

// ---- gemm_simt.cu ----
template <typename TA, typename TB, typename TC, typename Acc>
int gemm_nn(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc, int64_t M,
            int64_t N, int64_t K, cudaStream_t st, bool b_upper = false);
// b_upper: B is upper triangular (B[k][j] = 0 for k > j), its zero band is skipped
template <typename TA, typename TB, typename TC, typename Acc>
int gemm_nn_batched(const TA* A, int64_t lda, int64_t sA, const TB* B, int64_t ldb, int64_t sB,
                    TC* C, int64_t ldc, int64_t sC, int64_t M, int64_t N, int64_t K, int batch,
                    cudaStream_t st, bool b_upper = false);
template <typename TA, typename TB, typename Acc, typename TC>
int gemm_tn(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc, int64_t M,
            int64_t N, int64_t K, bool sym, Arena& ws, cudaStream_t st);
template <typename TA, typename TB, typename Acc, typename TC>
int gemm_tn_batched(const TA* A, int64_t lda, int64_t sA, const TB* B, int64_t ldb, int64_t sB,
                    TC* C, int64_t ldc, int64_t sC, int64_t M, int64_t N, int64_t K, bool sym,
                    int batch, Arena& ws, cudaStream_t st);
size_t gemm_tn_workspace(int64_t M, int64_t N, int64_t K, bool sym, size_t acc_bytes);
// C = alpha A B for small FP64 operands (n x n stage), 32 x 32 tiles; tri bit
// 0: A upper triangular, bit 1: B upper triangular (the zero bands are
// skipped).  Operands of problem b, sub-block t sit at b * s + t * tstride.
int gemm_sq(const double* A, int64_t lda, int64_t sA, int64_t tA, const double* B, int64_t ldb,
            int64_t sB, int64_t tB, double* C, int64_t ldc, int64_t sC, int64_t tC, int M, int N,
            int K, int batch, int nsub, double alpha, int tri, cudaStream_t st,
            const char* tag = "gemm_sq_fp64");
// square n x n products, batch of problems n*n apart
inline int gemm_sq_nn(const double* A, const double* B, double* C, int n, int batch, int tri,
                      cudaStream_t st) {
  const int64_t nn = (int64_t)n * n;
  return gemm_sq(A, n, nn, 0, B, n, nn, 0, C, n, nn, 0, n, n, n, batch, 1, 1.0, tri, st);
}
template <typename TA, typename TB, typename TC>
int gemm_tn_in_scratch(const TA* A, int64_t lda, const TB* B, int64_t ldb, TC* C, int64_t ldc,
                       int64_t M, int64_t N, int64_t K, void* scratch, size_t cap,
                       cudaStream_t st);
size_t gemm_tn_workspace_batched(int64_t M, int64_t N, int64_t K, bool sym, size_t acc_bytes,
                                 int batch);
// C (M x N, FP64, ld ldc) = A^T B for FP32 A (K x M), B (K x N): exact products,
// compensated double-float sums over row chunks, FP64 chunk reduction.
// ---- dense.cu ----
// C = A B for n x n FP64 operands as double-float sums of exact FP32 products
// (~1e-9 relative to sum |a_ik b_kj|; the mixed form's n x n products, whose
// factors carry FP32-level information), on the CUDA cores' FP32 pipe
int gemm_nn_df(const double* A, const double* B, double* C, int n, Arena& ws, cudaStream_t st);
int gemm_tn_df(const float* A, int64_t lda, const float* B, int64_t ldb, double* C, int64_t ldc,
               int64_t M, int64_t N, int64_t K, Arena& ws, cudaStream_t st);

// ---- dense.cu (FP64 small dense, batched, cooperative) ----
// Upper Cholesky R^T R = G + s I of `batch` n x n matrices (stride n*n, ld n).
// s starts at shift_rel0 * trace(G)/n; on a non-positive pivot the whole
// factorization restarts with s = max(s*100, shift_rel_fail*trace/n).  With
// shift_rel0 = 0 a non-positive pivot is instead floored alone at
// shift_rel_fail*trace/n (a null direction of a positive semidefinite G).
// info[ST_FAIL] = PLOM_NUM_CHOLESKY when all attempts fail.  near_tol > 0
// (one unshifted problem): a G within that bound of the identity (the largest
// squared column of triu(G - I, 1) + diag(G - I) / 2) is factored in closed
// form, R = I + that matrix, which is the exact factor of G perturbed by at
// most near_tol per element; info[ST_NEAR] counts such factorisations.
int chol_shifted(const double* G, double* R, int n, int batch, double shift_rel0,
                 double shift_rel_fail, int* info, Arena& ws, cudaStream_t st,
                 double near_tol = 0.0);
// W = R^{-1} for upper-triangular R (batch, stride n*n).
int trtri_upper(const double* R, double* W, int n, int batch, Arena& ws, cudaStream_t st);
// One-sided Jacobi SVD of `batch` square n x n matrices A (ld n, stride n*n),
// real (cplx=0) or complex interleaved (cplx=1, A holds n x 2n doubles).
// Outputs: S (batch x n, descending), U (n x n, row-major, A = U diag(S) V^H),
// VH (n x n rows = conj of right singular vectors, i.e. V^H).  Rotation
// stops when every column pair has |a_p^H a_q| <= tol ||a_p|| ||a_q||
// (tol <= 0: n * DBL_EPSILON).
int jacobi_svd(const double* A, int n, int batch, int cplx, double tol, double* S, double* U,
               double* VH, int* info, Arena& ws, cudaStream_t st);
size_t dense_workspace(int n, int batch, int cplx);

// complex <-> real-embedding helpers for n x n matrices (batched)
//  complexify_gram: H = Zr^T Zr (2n x 2n) of the interleaved real view of a
//  complex Z -> real_embed(Z^H Z)
int complexify_gram(const double* H, double* G, int n, int batch, cudaStream_t st);
//  real_embed(Mc) (column-vector form) -> real_embed(conj(Mc)) (row-vector
//  form used as the right operand of a real GEMM on interleaved data)
int embed_to_rowform(const double* E, double* F, int n, int batch, cudaStream_t st);
//  complex n x n (interleaved) -> real_embed (2n x 2n)
int complex_to_embed(const double* C, double* E, int n, int batch, cudaStream_t st);
//  real_embed (2n x 2n) -> complex n x n interleaved
int embed_to_complex(const double* E, double* C, int n, int batch, cudaStream_t st);

// ---- misc kernels (misc.cu) ----
template <typename TI, typename TO>
int convert(const TI* in, TO* out, int64_t count, cudaStream_t st);
template <typename TI, typename TO>
int copy2d(const TI* in, int64_t ldi, TO* out, int64_t ldo, int64_t rows, int64_t cols,
           cudaStream_t st);
int fill_uniform_dispatch(int dtype, void* out, int64_t count, uint64_t seed, cudaStream_t st);
int transpose_f64(const double* in, double* out, int64_t rows, int64_t cols, int batch,
                  cudaStream_t st);
// Orthonormal completion of the columns of U (m x n real, ld ldu) whose
// singular value is <= 1e-6 sigma_1 and whose norm is below 1/2 (the zero
// columns an exact zero column of the input leaves); S: n FP64 values,
// descending; U = F Mf with Mf (n x n, FP64) and G = F^T F (n x n, FP64),
// from which the candidates' norms are computed.
template <typename T>
int complete_null_columns(const double* S, int n, T* U, int64_t m, int64_t ldu, const double* G,
                          const double* Mf, Arena& ws, cudaStream_t st);

// Householder QR's column signs s (n values, +-1) for CholeskyQR factors Q, R
// (R with a positive diagonal), from Q's top n x n block (ld ldq; square:
// Q has exactly n rows): the factors LAPACK's geqrf returns are Q diag(s)
// and diag(s) R.
template <typename T>
int householder_signs(const T* Qtop, int64_t ldq, int n, bool square, double* s, Arena& ws,
                      cudaStream_t st);
// W <- W diag(s) and R <- diag(s) R (n x n FP64, ld n; either may be null)
int sign_fold(double* W, double* R, const double* s, int n, cudaStream_t st);

}  // namespace plom
