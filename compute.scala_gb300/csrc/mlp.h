// Host-side launchers of the cost model's kernels (mlp.cu).
#pragma once

#include <cuda_runtime.h>

namespace cc {

enum { kMlpNone = 0, kMlpBiasRelu = 1, kMlpBias = 2, kMlpReluMask = 3 };

// C = epilogue(op(A) op(B)); op transposes when ta / tb.  Epilogues: bias then
// ReLU, bias only, or zero where mask (same layout as C) is not positive.
cudaError_t launch_mlp_gemm(bool ta, bool tb, const float *A, const float *B, float *C, int M, int N, int K, int lda,
                            int ldb, int ldc, const float *bias, int epilogue, const float *mask, cudaStream_t s);
// Partial-sum rows the column sum of `rows` rows needs (partial holds chunks x cols floats).
int colsum_chunks(int rows);
cudaError_t launch_colsum(const float *X, int rows, int cols, float *partial, float *out, cudaStream_t s);
cudaError_t launch_mse(const float *y, const float *t, int n, float *d, float *loss, cudaStream_t s);
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                        float eps, float c1, float c2, int sm_count, cudaStream_t s);

}  // namespace cc
