// Tensor-core (tcgen05) kernels of the mixed form: FP32 operands packed as
// fp16 hi/lo pairs, products as three terms (hi*hi + hi*lo + lo*hi) with FP32
// accumulation in TMEM.
#pragma once
#include <cuda_fp16.h>

#include "plom_common.cuh"

namespace plom {

// Tall FP32 operand packed as two fp16 planes (gemm_f16.cu):
//   hi + lo = Y diag(scale), hi and lo row-major (batch x mp) x ld (ld = N
//   rounded up to 64, padding columns zero; lo right after hi), scale[p][j]
//   a power of two per problem and column.  A batch holds `batch` problems
//   of m rows each, mp rows apart (mp = m for one problem, else m rounded up
//   to 128 with zero padding rows).
struct Packed {
  __half* hi;
  __half* lo;
  float* scale;  // [batch][ld]
  int64_t m, N, ld;
  int64_t batch = 1, mp = 0;
  int64_t pstride = 0;  // elements from hi to lo; 0: batch mp ld (planes back to back)
};
// a row range [r0, r0 + rows) of one packed problem as a problem of its own
// (planes and plane stride of the parent; scales as given)
Packed packed_rows_view(const Packed& p, int64_t r0, int64_t rows, int64_t mp, float* scale);
int64_t packed_ld(int64_t N);
int64_t packed_rows(int64_t m, int64_t batch);
// carve planes and scales from the workspace
void packed_carve(Arena& ws, Packed& p, int64_t m, int64_t N, int64_t batch = 1);
// planes in caller storage of 4 batch packed_rows(m) packed_ld(N) bytes, scales in `scale`
void packed_view(Packed& p, void* storage, int64_t m, int64_t N, float* scale, int64_t batch = 1);
// pack an FP32 matrix (a batch: matrices bstride elements apart) with
// per-column power-of-two scales
int pack_f32(const float* Y, int64_t ld, int64_t m, int64_t N, Packed& p, Arena& ws,
             cudaStream_t st, int64_t bstride = 0);
// G (N x N, FP64; a batch: batch x N x N) = Y^T Y
int gram_packed(const Packed& p, double* G, int* err, Arena& ws, cudaStream_t st,
                bool accumulate = false);
// G = Y^T Y for Y packed in C row chunks of mc rows with per-chunk column
// scales (scales: C x ld); chunk c's products start after ready[c] (if given)
int gram_packed_chunks(const Packed& p, int C, int64_t mc, const float* scales, double* G,
                       const cudaEvent_t* ready, int* err, Arena& ws, cudaStream_t st);
// C (A.N x B.N, FP64, ldc) = A^T B for two packed operands with the same rows
int tn_packed(const Packed& a, const Packed& b, double* C, int64_t ldc, int* err, Arena& ws,
              cudaStream_t st);
// Y W for W (N x k, FP64, ldw; a batch: W_p wstride apart): FP32 into C
// (ldc; C_p cstride apart) when out == nullptr, else packed into *out
// (planes like the input, scale 2^14).  upper: W (k = N) is upper triangular,
// and the zero blocks below its diagonal are skipped
int apply_packed(const Packed& p, const double* W, int64_t ldw, int64_t k, float* C, int64_t ldc,
                 Packed* out, int* err, Arena& ws, cudaStream_t st, int64_t wstride = 0,
                 int64_t cstride = 0, bool upper = false);

// U = Q2 M (m x cw*n FP32, ldu; a batch: U_p ustride, M_p mstride apart):
// renormalise the columns whose M column (N x N, real or embedded complex)
// is longer than 4
int renorm_long_columns(const double* M, int N, int n, int cw, float* U, int64_t m, int64_t ldu,
                        int batch, int64_t mstride, int64_t ustride, Arena& ws, cudaStream_t st);

}  // namespace plom
