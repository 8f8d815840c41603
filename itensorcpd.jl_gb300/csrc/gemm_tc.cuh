// Interface of the tcgen05 BF16 GEMM (k_gemm_tc.cu) that the warm-start network runs on.
//
// Operands live in "panels": a matrix P (rows x K, K the reduction index) stored as BF16
// tiles of 128 rows x 64 K values (16 KB), tile (row / 128, k / 64) at index
// (row / 128) * KT + k / 64 with KT = ceil(K / 64); inside a tile row r is one 128-byte line
// and its 16-byte chunk c sits at chunk c ^ (r % 8) -- the SWIZZLE_128B K-major arrangement
// the tensor core reads, so a stage is two plain bulk copies.  Entries outside the matrix
// are zero where they meet the reduction (k >= K); rows past the end only feed outputs that
// are never written.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace cpals {

constexpr int kPanelRows = 128;
constexpr int kPanelK = 64;

// BF16 elements of a panel holding a rows x K matrix.
inline int64_t panel_elems(int64_t rows, int64_t K) {
  return ((rows + kPanelRows - 1) / kPanelRows) * kPanelRows * ((K + kPanelK - 1) / kPanelK) * kPanelK;
}

// Sets the GEMM kernel's shared-memory limit on the current device (before any stream capture).
cudaError_t gemm_tc_prepare();

// Split-K slices the GEMM of an M x N output over K uses on `sms` SMs (partials are
// float [splits][M][N]).
int gemm_tc_splits(int M, int N, int K, int sms);

// part[s][M][N] = A[M x K] B[N x K]^T over slice s of the reduction, A and B panels; BF16
// products, FP32 accumulation in TMEM.  err: two device ints, err[0] set non-zero when a
// bounded wait expired.
cudaError_t gemm_tc_launch(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, int splits,
                           float* part, int* err, cudaStream_t st);

// out = sum_s part[s] (fixed order) + bias[n], then mode 1: ReLU; mode 2: zero where
// bf16(mask[m][n]) <= 0.  Writes any of: out32 (FP32 [M][N]), prm (panel of out, M rows,
// K = N), ptr (panel of out^T, N rows, K = M); the panels' reduction padding is zeroed.
// With splits = 1 and no bias this packs a row-major FP32 matrix into panels.
cudaError_t gemm_tc_epilogue(const float* part, int splits, int M, int N, const float* bias, int mode,
                             const float* mask, float* out32, __nv_bfloat16* prm, __nv_bfloat16* ptr, cudaStream_t st);

}  // namespace cpals
