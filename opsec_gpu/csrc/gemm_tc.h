// gemm_tc.h -- products of a dense symmetric matrix with blocks of vectors on the tensor cores
// (gemm_tc.cu), for the iterative eigensolver.
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace opsec {

// An operand of tc_gemm: `rows` rows of `k` values each (row r of a column-major block is its
// column r; row i of a symmetric matrix is its column i), split into FP16 hi + lo after an
// exact power-of-two scaling that puts its largest magnitude in [2^13, 2^14).  Rows are padded
// to 256 and k to 64 with zeros.  One device allocation: hi, lo, then the max |x| (float bits).
struct TcOperand {
    int rows = 0, k = 0, rows_pad = 0, kpad = 0;
    DevBuf<unsigned char> store;
    void shape(int rows, int k);  // (re)sizes the buffers for rows x k
    size_t elems() const { return (size_t)rows_pad * kpad; }
    void* hi() const { return store.p; }
    void* lo() const { return store.p + 2 * elems(); }
    unsigned* maxbits() const { return reinterpret_cast<unsigned*>(store.p + 4 * elems()); }
};

// x[r ld + c], r < op.rows, c < op.k  ->  op (rows of FP64 values are split from the FP64 value)
void tc_split(const double* x, long long ld, TcOperand& op, cudaStream_t s, long long* launches);
void tc_split(const float* x, long long ld, TcOperand& op, cudaStream_t s, long long* launches);

// C[i + j ldc] = alpha sum_k A[i][k] B[j][k] + beta C[i + j ldc] + gamma D[i + j ldd] for
// i < A.rows, j < B.rows (FP32; C and D may not overlap).  `chunk`: K slices of 64 per
// accumulator restart; `tile_cols`: output tiles of 128 x 128 or 128 x 256 (0: whichever fills
// the SMs' waves better).  A barrier wait that exceeds wait_cycles sets *err (device) and the
// kernel returns; the caller reads *err.
void tc_gemm(const TcOperand& A, const TcOperand& B, float alpha, float beta, float* C, long long ldc, float gamma,
             const float* D, long long ldd, int chunk, int tile_cols, int* err, long long wait_cycles,
             cudaStream_t s, long long* launches);

}  // namespace opsec
