// cc_reduce_sum_f32_noalloc: the plain float sum with no device allocation.
//
// cc_reduce_sum_f32 takes its scratch (one compensated partial per block plus a
// completion counter) from the context's buffer pool, which means cc_init and
// cudaMalloc.  Some callers cannot allow either: a host framework that has
// already reserved the device's memory for its own allocator and forbids side
// allocations, or a latency-critical caller for whom cudaMalloc's device-wide
// synchronisation is unacceptable.  This variant keeps its scratch in a
// fixed-size array in device global memory that every GPU loading the library
// holds until the process exits, so it allocates nothing and needs no cc_init.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace cc {
namespace {

// Capacity of the scratch: one float2 partial per block, each block reducing a
// fixed chunk, so the largest input is kNoAllocMaxBlocks * kNoAllocChunk floats.
constexpr int kNoAllocMaxBlocks = 16384;
constexpr long long kNoAllocChunk = 8192;  // floats per block
constexpr long long kNoAllocMaxElements = (long long)kNoAllocMaxBlocks * kNoAllocChunk;  // 134,217,728
constexpr size_t kNoAllocPartialBytes = sizeof(float2) * kNoAllocMaxBlocks;               // 128 KiB
constexpr size_t kNoAllocScratchBytes = kNoAllocPartialBytes + 256;                      // + counter

// The scratch itself.  In host code `g_noalloc_scratch` names a host-side
// stand-in, not device memory: host code must use the address that
// cudaGetSymbolAddress returns in the current context (see scratch_address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Each block sums its own chunk [blockIdx.x * kNoAllocChunk, +kNoAllocChunk)
// with compensated accumulation, then the blocks combine through the partials
// and the completion counter exactly as the pooled sum does.
__global__ void __launch_bounds__(256) sum_noalloc_kernel(const float *__restrict__ in, long long n,
                                                          float2 *__restrict__ partials,
                                                          unsigned int *__restrict__ counter,
                                                          float *__restrict__ out, int vec4) {
  float s = 0.0f, c = 0.0f;
  const long long begin = (long long)blockIdx.x * kNoAllocChunk;
  const long long end = begin + kNoAllocChunk < n ? begin + kNoAllocChunk : n;
  long long tail = begin;
  if (vec4 && end > begin) {
    const long long count4 = (end - begin) >> 2;
    const float4 *in4 = reinterpret_cast<const float4 *>(in + begin);
    for (long long q = threadIdx.x; q < count4; q += blockDim.x) {
      const float4 v = __ldg(in4 + q);
      cc_acc(s, c, v.x);
      cc_acc(s, c, v.y);
      cc_acc(s, c, v.z);
      cc_acc(s, c, v.w);
    }
    tail = begin + (count4 << 2);
  }
  for (long long i = tail + threadIdx.x; i < end; i += blockDim.x) cc_acc(s, c, __ldg(in + i));
  cc_grid_finish(s, c, partials, counter, out);
}

// The scratch's device address belongs to the CUDA context that loaded this
// library's module on the device (the primary context, or a host framework's
// own driver-API context), not to the device number: after cudaDeviceReset, or
// under another context, the same array has another address.  Set-up therefore
// runs once per context, keyed by the context's unique ID (cuCtxGetId, which a
// re-created context never repeats), with that context current.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

struct ScratchSetup {
  std::mutex mu;
  bool resolved = false;
  CtxGetCurrentFn ctx_get_current = nullptr;
  CtxGetIdFn ctx_get_id = nullptr;
  std::vector<std::pair<unsigned long long, void *>> addr;  // context ID -> scratch address
};
ScratchSetup g_setup;

template <class F>
F driver_entry(const char *symbol) {
  cudaDriverEntryPointQueryResult q;
  void *p = nullptr;
  cudaError_t e = cudaGetDriverEntryPointByVersion(symbol, &p, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    cudaGetLastError();
    fail(CC_ERR_CUDA, std::string("driver entry point ") + symbol + " is unavailable");
  }
  return reinterpret_cast<F>(p);
}

void *symbol_address() {
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) {
    cudaGetLastError();
    fail(CC_ERR_CUDA, std::string("cudaGetSymbolAddress of the sum scratch failed: ") + cudaGetErrorString(e));
  }
  return ptr;
}

// The device address of the scratch in the calling thread's current context.
void *scratch_address() {
  std::lock_guard<std::mutex> g(g_setup.mu);
  if (!g_setup.resolved) {
    g_setup.ctx_get_current = driver_entry<CtxGetCurrentFn>("cuCtxGetCurrent");
    g_setup.ctx_get_id = driver_entry<CtxGetIdFn>("cuCtxGetId");
    g_setup.resolved = true;
  }
  CUcontext cur = nullptr;
  if (g_setup.ctx_get_current(&cur) != CUDA_SUCCESS) cur = nullptr;
  void *fresh = nullptr;
  if (!cur) {
    // No context is current yet: this runtime call makes the current device's
    // primary context current (it allocates nothing).
    fresh = symbol_address();
    if (g_setup.ctx_get_current(&cur) != CUDA_SUCCESS || !cur) fail(CC_ERR_CUDA, "no current CUDA context");
  }
  unsigned long long id = 0;
  if (g_setup.ctx_get_id(cur, &id) != CUDA_SUCCESS) fail(CC_ERR_CUDA, "cuCtxGetId failed");
  for (const auto &kv : g_setup.addr)
    if (kv.first == id) return kv.second;
  if (!fresh) fresh = symbol_address();
  g_setup.addr.emplace_back(id, fresh);
  return fresh;
}

}  // namespace
}  // namespace cc

extern "C" int cc_reduce_sum_f32_noalloc(uint64_t in_ptr, size_t n, uint64_t out_ptr, uint64_t stream) {
  using namespace cc;
  try {
    if (!out_ptr || (n && !in_ptr)) fail(CC_ERR_INVALID_VALUE, "null pointer");
    if (n > (size_t)kNoAllocMaxElements)
      fail(CC_ERR_INVALID_VALUE, "cc_reduce_sum_f32_noalloc: n = " + std::to_string(n) +
                                     " exceeds the fixed scratch capacity of " +
                                     std::to_string(kNoAllocMaxElements) + " floats");
    char *scratch = static_cast<char *>(scratch_address());
    // a generated kernel launched next must not start its loads before this sum ends
    g_foreign_enqueues.fetch_add(1, std::memory_order_acq_rel);
    auto *partials = reinterpret_cast<float2 *>(scratch);
    auto *counter = reinterpret_cast<unsigned int *>(scratch + kNoAllocPartialBytes);
    auto s = reinterpret_cast<cudaStream_t>(stream);
    // The array keeps the previous call's contents; the completion counter must start at zero.
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(CC_ERR_CUDA, std::string("cudaMemsetAsync of the sum counter: ") + cudaGetErrorString(e));
    }
    const long long nn = (long long)n;
    const int grid = nn == 0 ? 1 : (int)((nn + kNoAllocChunk - 1) / kNoAllocChunk);
    const int vec4 = (in_ptr & 15u) == 0;
    sum_noalloc_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const float *>(in_ptr), nn, partials, counter,
                                            reinterpret_cast<float *>(out_ptr), vec4);
    e = cudaGetLastError();
    if (e != cudaSuccess) fail(CC_ERR_CUDA, std::string("sum launch: ") + cudaGetErrorString(e));
  } catch (const Error &err) {
    record_error(err.message);
    return err.code;
  }
  return CC_OK;
}
