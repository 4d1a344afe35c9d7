// Host-side launchers of the precompiled kernels in kernels.cu.
#pragma once

#include <cuda_runtime.h>

namespace cc {

// Upper bound on the blocks of one grid sum; the scratch of a sum holds this
// many float2 partials plus one completion counter.
constexpr int kMaxSumBlocks = 4096;

cudaError_t launch_random(float *out, long long n, unsigned int seed, int normal, int sm_count,
                          cudaStream_t stream);
int sum_grid(long long work, int sm_count);
// Copies bytes / 16 sixteen-byte words with a kernel (both pointers 16-byte aligned,
// device-accessible: device memory or pinned host memory); the remainder is the caller's.
cudaError_t launch_copy16(void *dst, const void *src, size_t bytes, int sm_count, cudaStream_t stream);
// One copy of a copy table (device-accessible addresses: device memory or
// pinned host memory); chunk_begin = the copies before it, in kCopyChunk-byte chunks.
constexpr unsigned long long kCopyChunk = 65536;
struct CopyEntry {
  unsigned long long dst, src, bytes;
  long long chunk_begin;
};
// Every copy of a table of n entries (device memory), `chunks` chunks in all,
// with at most `blocks` blocks of 256 threads.
cudaError_t launch_copy_table(const CopyEntry *table, int n, long long chunks, int blocks, cudaStream_t stream);
// One thread waits until *flag is nonzero, at most limit_ns; on expiry *err = code
// (if it was 0).
cudaError_t launch_flag_wait(const int *flag, unsigned long long limit_ns, int *err, int code, cudaStream_t stream);
// Blocks of a grid sum: one element (or float4) per thread, capped at max_blocks.
int sum_grid_for(long long work, int block, int max_blocks);
cudaError_t launch_sum(const float *in, long long n, float2 *partials, unsigned int *counter, float *out,
                       int sm_count, cudaStream_t stream);

}  // namespace cc
