// Host-side launchers of the contraction kernels (gemm.cu, gemm_tc.cu).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace cc {

// C[M,N] = A[M,K] * B[K,N] on the CUDA cores.  exact: each output is the
// sequential left fold over k of separately rounded products (the reference's
// broadcast+split+reduce order); otherwise fused multiply-adds.
cudaError_t launch_sgemm(const float *A, const float *B, float *C, int M, int N, int K, long long lda, long long ldb,
                         long long ldc, bool exact, cudaStream_t stream);

// Three bf16 planes (hi, mid, lo) of A[M,K] as Mp x Kp row-major, zero padded.
cudaError_t launch_split_a(const float *A, long long lda, int M, int K, __nv_bfloat16 *planes, int Mp, int Kp,
                           int sm_count, cudaStream_t stream);
// Three bf16 planes of B^T (Np x Kp row-major) from B[K,N], zero padded.
cudaError_t launch_split_bt(const float *B, long long ldb, int K, int N, __nv_bfloat16 *planes, int Np, int Kp,
                            cudaStream_t stream);

// Tile sizes of the tensor-core kernel: planes are padded to these multiples
// (kTcBN covers both tile widths).
constexpr int kTcBM = 128, kTcBN = 256, kTcBK = 32;
// Kernel variants: 0 = 128-column tiles, accumulators restarted every 4
// k-blocks and summed in registers (FP32-level error at any K); 1 = 256-column
// tiles, one accumulator pair per tile (fastest; error grows with K);
// 2 = 128-column tiles, one pair per tile; 3 / 4 = as 0 with accumulators restarted
// every 8 / 16 k-blocks; 5 = 256-column tiles, hi*hi restarted every 8 k-blocks and
// the small products over the whole K, a partial last round in column halves.
// gemm_tc_variant: the kernel a variant runs for K_padded (a kernel that sums K
// chunks in registers hands a K that fits one chunk to a one-pair-per-tile
// kernel); the tensor maps and the launch both take the resolved variant.
// gemm_tc_box_n: the tile width of a resolved variant.
int gemm_tc_variant(int variant, int K_padded);
int gemm_tc_box_n(int variant);
// maps: A planes 0..2 (box 32 x 128), B^T planes 0..2 (box 32 x gemm_tc_box_n), the B^T planes
// again with box 32 x gemm_tc_box_n / 2 (6..8: column halves of split tiles), 64-byte swizzle.
// group_m: output tiles are visited in groups of this many tile rows (1 = row-major);
// variant: as resolved by gemm_tc_variant (any other is rejected).
cudaError_t launch_gemm_bf16x6(const CUtensorMap *maps, float *C, int M, int N, int K_padded, long long ldc,
                               int sm_count, int *err, int variant, int group_m, cudaStream_t stream);

}  // namespace cc
