// Contraction kernels on the CUDA cores, and the operand split for the tensor cores.
//
// The reference multiplies matrices as a broadcast product followed by a
// left-fold of `split(1)` views (Tensors/src/test/scala/com/thoughtworks/
// compute/TensorsSpec.scala:468-485, README.md:311-343):
//   C[i][k] = ((A[i][0]*B[0][k] + A[i][1]*B[1][k]) + A[i][2]*B[2][k]) + ...
// with every product and every sum rounded to float.
//
// sgemm_kernel<kExact=true> keeps exactly that order per output (the k loop is
// sequential in every thread, products and sums rounded separately), so it is
// bit-identical to the reference's result.  sgemm_kernel<false> is the plain
// FP32 CUDA-core GEMM with fused multiply-adds.  split_planes_kernel prepares
// the three-way BF16 split the tensor-core kernel (gemm_tc.cu) consumes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm.h"

namespace cc {
namespace {

constexpr int kTile = 128;  // block tile (rows and columns)
constexpr int kTk = 8;      // k per smem stage

// One 128x128 output tile per block of 256 threads; each thread owns an 8x8
// sub-tile made of rows {ty*4+r, 64+ty*4+r} and columns {tx*4+c, 64+tx*4+c}.
// The accumulators are pairs of adjacent columns.  The plain GEMM updates them
// with the packed FP32 fused multiply-add (fma.rn.f32x2: one instruction for
// two outputs, each lane the scalar fmaf); the exact fold keeps the scalar
// __fmul_rn / __fadd_rn, which no compiler stage fuses.
template <bool kExact>
__global__ void __launch_bounds__(256) sgemm_kernel(const float *__restrict__ A, const float *__restrict__ B,
                                                    float *__restrict__ C, int M, int N, int K, long long lda,
                                                    long long ldb, long long ldc) {
  __shared__ float As[2][kTk][kTile + 4];
  __shared__ float Bs[2][kTk][kTile + 4];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int bm = blockIdx.y * kTile, bn = blockIdx.x * kTile;
  float2 acc[8][4];  // acc[i][jp]: columns 2*jp and 2*jp + 1 of the thread's eight
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.0f, 0.0f);

  // global -> register staging: A: row tid/2, k (tid%2)*4..+3; B: k-row tid/32, cols (tid%32)*4..+3
  const int a_r = tid >> 1, a_c = (tid & 1) * 4;
  const int b_r = tid >> 5, b_c = (tid & 31) * 4;
  float ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gr = bm + a_r, gk = k0 + a_c + q;
      ra[q] = (gr < M && gk < K) ? __ldg(A + gr * lda + gk) : 0.0f;
      const int gk2 = k0 + b_r, gc = bn + b_c + q;
      rb[q] = (gk2 < K && gc < N) ? __ldg(B + gk2 * ldb + gc) : 0.0f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      As[buf][a_c + q][a_r] = ra[q];
      Bs[buf][b_r][b_c + q] = rb[q];
    }
  };
  const int ntiles = (K + kTk - 1) / kTk;
  load(0);
  store(0);
  __syncthreads();
  for (int t = 0; t < ntiles; ++t) {
    const int buf = t & 1;
    if (t + 1 < ntiles) load((t + 1) * kTk);
    const int kcount = (K - t * kTk) < kTk ? (K - t * kTk) : kTk;
#pragma unroll
    for (int kk = 0; kk < kTk; ++kk) {
      if (kk < kcount) {
        float a[8], b[8];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          a[r] = As[buf][kk][ty * 4 + r];
          a[4 + r] = As[buf][kk][64 + ty * 4 + r];
          b[r] = Bs[buf][kk][tx * 4 + r];
          b[4 + r] = Bs[buf][kk][64 + tx * 4 + r];
        }
        const bool first = (t == 0 && kk == 0);
        float2 b2[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) b2[j] = make_float2(b[2 * j], b[2 * j + 1]);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float2 a2 = make_float2(a[i], a[i]);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (kExact) {
              const float px = __fmul_rn(a[i], b2[j].x), py = __fmul_rn(a[i], b2[j].y);
              acc[i][j].x = first ? px : __fadd_rn(acc[i][j].x, px);
              acc[i][j].y = first ? py : __fadd_rn(acc[i][j].y, py);
            } else {
              acc[i][j] = __ffma2_rn(a2, b2[j], acc[i][j]);
            }
          }
        }
      }
    }
    if (t + 1 < ntiles) store(buf ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int gr = bm + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
    if (gr >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int gc = bn + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
      if (gc < N) C[gr * ldc + gc] = (j & 1) ? acc[i][j >> 1].y : acc[i][j >> 1].x;
    }
  }
}

// x = hi + mid + lo with each part a bfloat16 (round-to-nearest): three 8-bit
// significands cover float's 24, and each residual is exact in float.
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
  h = __float2bfloat16_rn(x);
  const float r1 = __fsub_rn(x, __bfloat162float(h));
  m = __float2bfloat16_rn(r1);
  const float r2 = __fsub_rn(r1, __bfloat162float(m));
  l = __float2bfloat16_rn(r2);
}

// Eight floats to three planes of eight bfloat16 each (one 16-byte word per plane).
__device__ __forceinline__ void split8(const float (&x)[8], uint4 &h, uint4 &m, uint4 &l) {
  __nv_bfloat16 hh[8], mm[8], ll[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) split3(x[e], hh[e], mm[e], ll[e]);
  h = *reinterpret_cast<const uint4 *>(hh);
  m = *reinterpret_cast<const uint4 *>(mm);
  l = *reinterpret_cast<const uint4 *>(ll);
}

// src: rows x cols floats, row-major with leading dimension ld.  dst: three
// planes of prows x pcols bf16, row-major, zero outside rows x cols (pcols a
// multiple of 32).  Each thread takes runs of eight columns: two 16-byte loads
// when the run lies inside the matrix and src is 16-byte aligned with ld a
// multiple of 4, and one 16-byte store per plane.
__global__ void __launch_bounds__(256) split_planes_kernel(const float *__restrict__ src, long long ld, int rows,
                                                           int cols, int vec, __nv_bfloat16 *__restrict__ dst,
                                                           int prows, int pcols) {
  const long long plane = (long long)prows * pcols;
  const unsigned runs = (unsigned)pcols >> 3;
  const long long total = (long long)prows * runs;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int r = (int)(i / runs), c0 = (int)(i - (long long)r * runs) * 8;
    float x[8];
    const float *row = src + (long long)r * ld;
    if (vec && r < rows && c0 + 8 <= cols) {
      const float4 a = __ldg(reinterpret_cast<const float4 *>(row + c0));
      const float4 b = __ldg(reinterpret_cast<const float4 *>(row + c0 + 4));
      x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
      x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) x[e] = (r < rows && c0 + e < cols) ? __ldg(row + c0 + e) : 0.0f;
    }
    uint4 h, m, l;
    split8(x, h, m, l);
    const long long o = (long long)r * pcols + c0;
    *reinterpret_cast<uint4 *>(dst + o) = h;
    *reinterpret_cast<uint4 *>(dst + plane + o) = m;
    *reinterpret_cast<uint4 *>(dst + 2 * plane + o) = l;
  }
}

// Transposing split through shared memory: a 64 (k) x 64 (n) tile of src
// (rows = K, cols = N, row-major) becomes a 64 x 64 tile of the planes (rows =
// N, cols = K).  Loads are 16-byte reads along n (when src allows); in the
// store phase eight threads share one n, each splitting eight consecutive k
// into one 16-byte word per plane, so a warp writes four whole 128-byte plane
// rows per store.  The odd row pitch keeps the column reads at most two-way
// bank conflicted.
__global__ void __launch_bounds__(256) split_planes_t_kernel(const float *__restrict__ src, long long ld, int krows,
                                                             int ncols, int vec, __nv_bfloat16 *__restrict__ dst,
                                                             int prows, int pcols) {
  __shared__ float tile[64][65];
  const long long plane = (long long)prows * pcols;
  const int k0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  const int t = threadIdx.x;
  const int lc = (t & 15) * 4;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int kr = (t >> 4) + 16 * q;
    const int k = k0 + kr, n = n0 + lc;
    float4 v;
    if (vec && k < krows && n + 4 <= ncols) {
      v = __ldg(reinterpret_cast<const float4 *>(src + (long long)k * ld + n));
    } else {
      const float *p = src + (long long)k * ld;
      v.x = (k < krows && n + 0 < ncols) ? __ldg(p + n + 0) : 0.0f;
      v.y = (k < krows && n + 1 < ncols) ? __ldg(p + n + 1) : 0.0f;
      v.z = (k < krows && n + 2 < ncols) ? __ldg(p + n + 2) : 0.0f;
      v.w = (k < krows && n + 3 < ncols) ? __ldg(p + n + 3) : 0.0f;
    }
    tile[kr][lc + 0] = v.x;
    tile[kr][lc + 1] = v.y;
    tile[kr][lc + 2] = v.z;
    tile[kr][lc + 3] = v.w;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int u = t + 256 * r;
    const int nl = u >> 3, kc = (u & 7) * 8;
    const int n = n0 + nl, k = k0 + kc;
    if (n >= prows || k >= pcols) continue;
    float x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) x[e] = tile[kc + e][nl];
    uint4 h, m, l;
    split8(x, h, m, l);
    const long long o = (long long)n * pcols + k;
    *reinterpret_cast<uint4 *>(dst + o) = h;
    *reinterpret_cast<uint4 *>(dst + plane + o) = m;
    *reinterpret_cast<uint4 *>(dst + 2 * plane + o) = l;
  }
}

}  // namespace

cudaError_t launch_sgemm(const float *A, const float *B, float *C, int M, int N, int K, long long lda, long long ldb,
                         long long ldc, bool exact, cudaStream_t stream) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (K <= 0) return cudaErrorInvalidValue;
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  if (exact)
    sgemm_kernel<true><<<grid, 256, 0, stream>>>(A, B, C, M, N, K, lda, ldb, ldc);
  else
    sgemm_kernel<false><<<grid, 256, 0, stream>>>(A, B, C, M, N, K, lda, ldb, ldc);
  return cudaGetLastError();
}

cudaError_t launch_split_a(const float *A, long long lda, int M, int K, __nv_bfloat16 *planes, int Mp, int Kp,
                           int sm_count, cudaStream_t stream) {
  if (Kp % 32 != 0) return cudaErrorInvalidValue;
  long long total = (long long)Mp * (Kp / 8);
  long long grid = (total + 255) / 256;
  if (grid > (long long)sm_count * 8) grid = (long long)sm_count * 8;
  const int vec = ((reinterpret_cast<uintptr_t>(A) & 15u) == 0 && lda % 4 == 0) ? 1 : 0;
  split_planes_kernel<<<(unsigned)grid, 256, 0, stream>>>(A, lda, M, K, vec, planes, Mp, Kp);
  return cudaGetLastError();
}

cudaError_t launch_split_bt(const float *B, long long ldb, int K, int N, __nv_bfloat16 *planes, int Np, int Kp,
                            cudaStream_t stream) {
  if (Kp % 32 != 0 || Np % 64 != 0) return cudaErrorInvalidValue;
  dim3 grid((Kp + 63) / 64, Np / 64);
  const int vec = ((reinterpret_cast<uintptr_t>(B) & 15u) == 0 && ldb % 4 == 0) ? 1 : 0;
  split_planes_t_kernel<<<grid, 256, 0, stream>>>(B, ldb, K, N, vec, planes, Np, Kp);
  return cudaGetLastError();
}

}  // namespace cc
