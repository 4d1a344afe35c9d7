// The tuner's cost model: a multilayer perceptron trained and evaluated by
// these kernels (FP32, CUDA cores; the network is small, so its GEMMs are
// latency- rather than throughput-bound and stay off the tensor cores).
//
//   h_0 = x (batch x 64 features)
//   h_l = relu(h_{l-1} W_l + b_l)   for the hidden layers
//   y   = h_{L-1} W_L + b_L         (the predicted log-runtime)
//
// Training minimises the mean squared error with Adam.  Every sum runs in a
// fixed order (no atomics), so gradients are reproducible bit for bit.
#include <cuda_runtime.h>

#include "mlp.h"

namespace cc {
namespace {

constexpr int kT = 64;   // output tile (rows and columns)
constexpr int kTk = 16;  // k per stage

// C[m][n] = epilogue(sum_k a(m,k) * b(k,n)),
//   a(m,k) = TA ? A[k*lda + m] : A[m*lda + k],  b(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n].
// Each of the 256 threads owns a 4x4 block of the 64x64 tile; k runs in order.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) mlp_gemm(const float *__restrict__ A, const float *__restrict__ B,
                                                float *__restrict__ C, int M, int N, int K, int lda, int ldb, int ldc,
                                                const float *__restrict__ bias, int epilogue,
                                                const float *__restrict__ mask) {
  __shared__ float As[kTk][kT + 4];
  __shared__ float Bs[kTk][kT + 4];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTk) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int e = tid + i * 256;
      int ml, kl;
      if (TA) {
        ml = e & 63;
        kl = e >> 6;
      } else {
        ml = e >> 4;
        kl = e & 15;
      }
      const int m = m0 + ml, k = k0 + kl;
      As[kl][ml] = (m < M && k < K) ? (TA ? A[(long long)k * lda + m] : A[(long long)m * lda + k]) : 0.0f;
      int nl, kb;
      if (TB) {
        nl = e >> 4;
        kb = e & 15;
      } else {
        nl = e & 63;
        kb = e >> 6;
      }
      const int n = n0 + nl, kk = k0 + kb;
      Bs[kb][nl] = (n < N && kk < K) ? (TB ? B[(long long)n * ldb + kk] : B[(long long)kk * ldb + n]) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTk; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        a[r] = As[kk][ty * 4 + r];
        b[r] = Bs[kk][tx * 4 + r];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) acc[r][s] = fmaf(a[r], b[s], acc[r][s]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int m = m0 + ty * 4 + r;
    if (m >= M) continue;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int n = n0 + tx * 4 + s;
      if (n >= N) continue;
      float v = acc[r][s];
      if (epilogue == kMlpBiasRelu) {
        v += bias[n];
        v = v > 0.0f ? v : 0.0f;
      } else if (epilogue == kMlpBias) {
        v += bias[n];
      } else if (epilogue == kMlpReluMask) {
        v = mask[(long long)m * ldc + n] > 0.0f ? v : 0.0f;
      }
      C[(long long)m * ldc + n] = v;
    }
  }
}

// Column sums of a rows x cols matrix in two fixed-order passes.
constexpr int kColChunk = 256;
__global__ void __launch_bounds__(256) colsum_partial(const float *__restrict__ X, int rows, int cols,
                                                      float *__restrict__ partial) {
  const int r0 = blockIdx.x * kColChunk;
  const int r1 = r0 + kColChunk < rows ? r0 + kColChunk : rows;
  for (int c = threadIdx.x; c < cols; c += blockDim.x) {
    float s = 0.0f;
    for (int r = r0; r < r1; ++r) s += X[(long long)r * cols + c];
    partial[(long long)blockIdx.x * cols + c] = s;
  }
}

__global__ void __launch_bounds__(256) colsum_final(const float *__restrict__ partial, int chunks, int cols,
                                                    float *__restrict__ out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < chunks; ++k) s += partial[(long long)k * cols + c];
    out[c] = s;
  }
}

// d = 2 (y - t) / n and the mean squared error (one block, fixed-order tree).
__global__ void __launch_bounds__(1024) mse_kernel(const float *__restrict__ y, const float *__restrict__ t, int n,
                                                   float *__restrict__ d, float *__restrict__ loss) {
  __shared__ float red[1024];
  float s = 0.0f;
  const float scale = 2.0f / (float)n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float e = y[i] - t[i];
    d[i] = scale * e;
    s += e * e;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[0] = red[0] / (float)n;
}

// Adam (Kingma & Ba 2015): c1 = 1 - beta1^t, c2 = 1 - beta2^t.
__global__ void __launch_bounds__(256) adam_kernel(float *__restrict__ p, const float *__restrict__ g,
                                                   float *__restrict__ m, float *__restrict__ v, long long n, float lr,
                                                   float b1, float b2, float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace

cudaError_t launch_mlp_gemm(bool ta, bool tb, const float *A, const float *B, float *C, int M, int N, int K, int lda,
                            int ldb, int ldc, const float *bias, int epilogue, const float *mask, cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  dim3 grid((N + kT - 1) / kT, (M + kT - 1) / kT);
  if (!ta && !tb)
    mlp_gemm<false, false><<<grid, 256, 0, s>>>(A, B, C, M, N, K, lda, ldb, ldc, bias, epilogue, mask);
  else if (ta && !tb)
    mlp_gemm<true, false><<<grid, 256, 0, s>>>(A, B, C, M, N, K, lda, ldb, ldc, bias, epilogue, mask);
  else if (!ta && tb)
    mlp_gemm<false, true><<<grid, 256, 0, s>>>(A, B, C, M, N, K, lda, ldb, ldc, bias, epilogue, mask);
  else
    mlp_gemm<true, true><<<grid, 256, 0, s>>>(A, B, C, M, N, K, lda, ldb, ldc, bias, epilogue, mask);
  return cudaGetLastError();
}

int colsum_chunks(int rows) { return (rows + kColChunk - 1) / kColChunk; }

cudaError_t launch_colsum(const float *X, int rows, int cols, float *partial, float *out, cudaStream_t s) {
  const int chunks = colsum_chunks(rows);
  if (chunks > 0) colsum_partial<<<chunks, 256, 0, s>>>(X, rows, cols, partial);
  colsum_final<<<(cols + 255) / 256, 256, 0, s>>>(partial, chunks, cols, out);
  return cudaGetLastError();
}

cudaError_t launch_mse(const float *y, const float *t, int n, float *d, float *loss, cudaStream_t s) {
  mse_kernel<<<1, 1024, 0, s>>>(y, t, n, d, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                        float eps, float c1, float c2, int sm_count, cudaStream_t s) {
  long long grid = (n + 255) / 256;
  if (grid > (long long)sm_count * 8) grid = (long long)sm_count * 8;
  if (grid < 1) grid = 1;
  adam_kernel<<<(unsigned)grid, 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace cc
