// gemm_df.h -- FP64-accurate GEMM in double-FP32 arithmetic (gemm_df.cu).
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace opsec {

// x (n FP64 values) -> out (n pairs of floats hi, lo with hi + lo = x to ~48 bits)
void df_split(size_t n, const double* x, float* out, cudaStream_t s, long long* launches);

// C[i + j ldc] = sum_k a(i, k) B[k + j ldb] for i < M, j < N (FP64 out, column-major), from
// operands already split by df_split (element indices below count pairs), in double-FP32 (~46 bits
// of sum_k |a(i, k) B_kj|): a(i, k) = A[k + i lda] when a_kmajor (C = A^T B, A is K x M), else
// A[i + k lda] (C = A B, A is M x K).  C may not overlap A or B.  `work` holds split-K partial
// sums when the output has few tiles (grown as needed).
void df_gemm(bool a_kmajor, int M, int N, int K, const float* A, long long lda, const float* B, long long ldb,
             double* C, long long ldc, DevBuf<double>& work, cudaStream_t s, long long* launches);

}  // namespace opsec
