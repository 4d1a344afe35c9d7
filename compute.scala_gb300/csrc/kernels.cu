// Precompiled sm_103a kernels whose code does not depend on an expression tree:
// the random-number generators and the plain full sum of a float buffer.
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"
#include "kernels.h"

namespace cc {
namespace {

// Thomas Wang's 32-bit integer hash, the reference's default generator
// (Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:106-117).
__device__ __forceinline__ unsigned int wang_hash(unsigned int v) {
  v = (v ^ 61u) ^ (v >> 16);
  v *= 9u;
  v ^= v << 4;
  v *= 0x27d4eb2du;
  v ^= v >> 15;
  return v;
}

// Marsaglia xorshift32 step (Tensors.scala:402-406).
__device__ __forceinline__ unsigned int xorshift(unsigned int s) {
  const unsigned int t1 = s ^ (s << 13);
  const unsigned int t2 = t1 ^ (t1 >> 17);
  return t2 ^ (t2 << 5);
}

// hash / 2^32 as the reference writes it: the uint converts to float with
// round-to-nearest-even, and the division by a power of two is exact.
__device__ __forceinline__ float unit_float(unsigned int h) {
  return __fmul_rn(__uint2float_rn(h), 2.3283064365386963e-10f);
}

// Tensors.scala:431-443: buffer[i] = hash(i ^ seed) / 4294967296.0f
__global__ void __launch_bounds__(256) random_uniform_kernel(float *__restrict__ out, long long n,
                                                             unsigned int seed) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    out[i] = unit_float(wang_hash((unsigned int)i ^ seed));
  }
}

// Tensors.scala:397-429: one Box-Muller pair per work item.  Every float step
// rounds once, as the reference's statements are written; log, cos and sin are
// taken in double precision and rounded to float once, which gives the
// correctly rounded float in all but vanishingly rare cases, so the output
// matches the reference's golden values bit for bit.
__global__ void __launch_bounds__(256) random_normal_kernel(float2 *__restrict__ out, long long pairs,
                                                            unsigned int seed) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const float two_pi = 6.28318548202514648f;  // 2 * M_PI_F, exact in binary32
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < pairs; i += stride) {
    const unsigned int r1 = wang_hash((unsigned int)i ^ seed);
    const unsigned int r2 = xorshift(r1);
    const float u1 = unit_float(r1);
    const float u2 = unit_float(r2);
    const float lg = (float)log((double)u1);
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, lg));
    const float theta = __fmul_rn(two_pi, u2);
    double sn, cs;
    sincos((double)theta, &sn, &cs);
    out[i] = make_float2(__fmul_rn(r, (float)cs), __fmul_rn(r, (float)sn));
  }
}

// Plain compensated sum of a float buffer (the kind-1 program of a bare
// parameter, precompiled): float4 loads when the address allows.
__global__ void __launch_bounds__(256) sum_kernel(const float *__restrict__ in, long long n,
                                                  float2 *__restrict__ partials, unsigned int *__restrict__ counter,
                                                  float *__restrict__ out, int vec4) {
  float s = 0.0f, c = 0.0f;
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long start = 0;
  if (vec4) {
    const long long n4 = n >> 2;
    const float4 *in4 = reinterpret_cast<const float4 *>(in);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride) {
      const float4 v = __ldg(in4 + q);
      cc_acc(s, c, v.x);
      cc_acc(s, c, v.y);
      cc_acc(s, c, v.z);
      cc_acc(s, c, v.w);
    }
    start = n4 << 2;
  }
  for (long long i = start + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    cc_acc(s, c, __ldg(in + i));
  }
  cc_grid_finish(s, c, partials, counter, out);
}

// Bulk copy by the SMs, 16 bytes per access, four accesses in flight per
// thread.  Used between pinned host memory and device memory, where loads
// and stores issued by all SMs over the chip-to-chip link outrun one DMA
// engine.  src, dst and n16 * 16 bytes are 16-byte aligned.
__global__ void __launch_bounds__(256) copy16_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst,
                                                     long long n16) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

// One thread waits until *flag is nonzero, for at most limit_ns of
// %globaltimer time; when the limit passes it records `code` in *err (the first
// error stays) and returns.  The pattern of every spinning wait in this library.
__global__ void flag_wait_kernel(const volatile int *flag, unsigned long long limit_ns, int *err, int code) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    if (*flag != 0) return;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > limit_ns) {
      atomicCAS(err, 0, code);
      return;
    }
    __nanosleep(1000);
  }
}

}  // namespace

cudaError_t launch_flag_wait(const int *flag, unsigned long long limit_ns, int *err, int code, cudaStream_t stream) {
  flag_wait_kernel<<<1, 1, 0, stream>>>(flag, limit_ns, err, code);
  return cudaGetLastError();
}

// Many copies in one launch: the copies are cut into kCopyChunk-byte chunks,
// numbered in table order (entry e owns chunks [chunk_begin(e), chunk_begin(e+1))),
// and each block takes chunks grid-stride, finds the chunk's entry by binary
// search and copies it 16 bytes per thread-step (4 bytes when an end of the
// copy is not 16-byte aligned).
__global__ void __launch_bounds__(256) copy_table_kernel(const CopyEntry *__restrict__ table, int n,
                                                         long long chunks) {
  for (long long c = blockIdx.x; c < chunks; c += gridDim.x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (table[mid].chunk_begin <= c) lo = mid; else hi = mid - 1;
    }
    const CopyEntry e = table[lo];
    const unsigned long long off = (unsigned long long)(c - e.chunk_begin) * kCopyChunk;
    if (off >= e.bytes) continue;
    const unsigned long long len = e.bytes - off < kCopyChunk ? e.bytes - off : kCopyChunk;
    const char *src = reinterpret_cast<const char *>(e.src) + off;
    char *dst = reinterpret_cast<char *>(e.dst) + off;
    if (((e.src | e.dst) & 15ull) == 0) {
      const long long n16 = (long long)(len >> 4);
      const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
      uint4 *d4 = reinterpret_cast<uint4 *>(dst);
      long long i = threadIdx.x;
      for (; i + 3 * 256 < n16; i += 4 * 256) {
        const uint4 a = s4[i], b = s4[i + 256], cc = s4[i + 512], d = s4[i + 768];
        d4[i] = a;
        d4[i + 256] = b;
        d4[i + 512] = cc;
        d4[i + 768] = d;
      }
      for (; i < n16; i += 256) d4[i] = s4[i];
      for (long long j = (n16 << 4) + threadIdx.x; j < (long long)len; j += 256) dst[j] = src[j];
    } else {
      for (long long j = threadIdx.x; j < (long long)len; j += 256) dst[j] = src[j];
    }
  }
}

cudaError_t launch_copy_table(const CopyEntry *table, int n, long long chunks, int blocks, cudaStream_t stream) {
  if (n <= 0 || chunks <= 0) return cudaSuccess;
  const long long grid = chunks < blocks ? chunks : blocks;
  copy_table_kernel<<<(unsigned)grid, 256, 0, stream>>>(table, n, chunks);
  return cudaGetLastError();
}

cudaError_t launch_copy16(void *dst, const void *src, size_t bytes, int sm_count, cudaStream_t stream) {
  const long long n16 = (long long)(bytes / 16);
  if (n16 <= 0) return cudaSuccess;
  long long grid = (n16 + 255) / 256;
  const long long cap = (long long)sm_count * 8;
  if (grid > cap) grid = cap;
  copy16_kernel<<<(unsigned)grid, 256, 0, stream>>>(static_cast<const uint4 *>(src), static_cast<uint4 *>(dst), n16);
  return cudaGetLastError();
}

cudaError_t launch_random(float *out, long long n, unsigned int seed, int normal, int sm_count,
                          cudaStream_t stream) {
  const int block = 256;
  long long work = normal ? (n + 1) / 2 : n;
  if (work <= 0) return cudaSuccess;
  long long grid = (work + block - 1) / block;
  long long cap = (long long)sm_count * 16;
  if (grid > cap) grid = cap;
  if (normal) {
    random_normal_kernel<<<(unsigned)grid, block, 0, stream>>>(reinterpret_cast<float2 *>(out), work, seed);
  } else {
    random_uniform_kernel<<<(unsigned)grid, block, 0, stream>>>(out, work, seed);
  }
  return cudaGetLastError();
}

int sum_grid(long long work, int sm_count) {
  long long grid = (work + 255) / 256;
  long long cap = (long long)sm_count * 8;
  if (cap > kMaxSumBlocks) cap = kMaxSumBlocks;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return (int)grid;
}

int sum_grid_for(long long work, int block, int max_blocks) {
  long long grid = (work + block - 1) / block;
  long long cap = max_blocks < kMaxSumBlocks ? max_blocks : kMaxSumBlocks;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return (int)grid;
}

cudaError_t launch_sum(const float *in, long long n, float2 *partials, unsigned int *counter, float *out,
                       int sm_count, cudaStream_t stream) {
  const int vec4 = (reinterpret_cast<uintptr_t>(in) & 15u) == 0;
  const int grid = sum_grid(vec4 ? (n >> 2) : n, sm_count);
  sum_kernel<<<grid, 256, 0, stream>>>(in, n, partials, counter, out, vec4);
  return cudaGetLastError();
}

}  // namespace cc
