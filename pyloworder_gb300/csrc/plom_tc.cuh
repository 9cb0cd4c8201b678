// Tensor-core (tcgen05) kernels of the mixed form: TF32 products split into
// three terms (hi*hi + hi*lo + lo*hi) with FP32 accumulation in TMEM.
#pragma once
#include "plom_common.cuh"

namespace plom {

// Gram G (N x N, FP64) = A^T A for a tall FP32 A (m x N, lda)
bool tc_gram_supported(int64_t m, int64_t N, int64_t lda);
int tc_gram_tf32x3(const float* A, int64_t lda, int64_t m, int64_t N, double* G, int* err,
                   Arena& ws, cudaStream_t st);
// C (m x k, FP32) = A (m x N, FP32) W (N x k, ldw; FP64 or FP32, split on the device)
bool tc_apply_supported(int64_t m, int64_t N, int64_t k, int64_t lda, int64_t ldc);
template <typename TW>
int tc_apply_tf32x3(const float* A, int64_t lda, int64_t m, int64_t N, const TW* W, int64_t ldw,
                    int64_t k, float* C, int64_t ldc, int* err, Arena& ws, cudaStream_t st);

}  // namespace plom
