// gemm_df.h -- FP64-accurate GEMM in double-FP32 arithmetic (gemm_df.cu).
#pragma once

#include <cuda_runtime.h>

namespace opsec {

// C[i + j ldc] = sum_k a(i, k) B[k + j ldb] for i < M, j < N, all FP64 column-major, computed in
// double-FP32 (~46 bits of sum_k |a(i, k) B_kj|): a(i, k) = A[k + i lda] when a_kmajor (C = A^T B,
// A is K x M), else A[i + k lda] (C = A B, A is M x K).  C may not overlap A or B.
void df_gemm(bool a_kmajor, int M, int N, int K, const double* A, long long lda, const double* B, long long ldb,
             double* C, long long ldc, cudaStream_t s, long long* launches);

}  // namespace opsec
