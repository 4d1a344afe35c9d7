// Device helpers shared by the precompiled kernels (kernels.cu) and every
// NVRTC-generated program (codegen.cpp embeds this file as its prelude).
#pragma once

typedef long long cc_i64;
typedef unsigned long long cc_u64;

// Error-free transformation of a + b (Knuth's TwoSum); the intrinsics are never
// contracted into FMAs, so the error term is exact under any compile flags.
__device__ __forceinline__ void cc_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void cc_acc(float &s, float &c, float v) {
  float t, e;
  cc_two_sum(s, v, t, e);
  s = t;
  c = __fadd_rn(c, e);
}
__device__ __forceinline__ void cc_merge(float &s, float &c, float s2, float c2) {
  float t, e;
  cc_two_sum(s, s2, t, e);
  s = t;
  c = __fadd_rn(__fadd_rn(c, c2), e);
}
__device__ __forceinline__ void cc_warp_merge(float &s, float &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float s2 = __shfl_down_sync(0xffffffffu, s, o);
    float c2 = __shfl_down_sync(0xffffffffu, c, o);
    cc_merge(s, c, s2, c2);
  }
}
// Block reduction of (s, c) pairs into thread 0, in a fixed order.
__device__ __forceinline__ void cc_block_merge(float &s, float &c, float2 *ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  cc_warp_merge(s, c);
  if (lane == 0) ws[wid] = make_float2(s, c);
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? ws[lane].x : 0.0f;
    c = lane < nw ? ws[lane].y : 0.0f;
    cc_warp_merge(s, c);
  }
  __syncthreads();
}
// Single-pass grid sum: each block publishes its compensated partial; the last
// block to finish (completion counter) combines all partials in block order, so
// the result does not depend on which block finishes last, and resets the
// counter for the next launch.
__device__ __forceinline__ void cc_grid_finish(float s, float c, float2 *__restrict__ partials,
                                               unsigned int *__restrict__ counter, float *__restrict__ out) {
  __shared__ float2 ws[32];
  __shared__ int last;
  cc_block_merge(s, c, ws);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = make_float2(s, c);
    __threadfence();
    unsigned int ticket = atomicAdd(counter, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  s = 0.0f;
  c = 0.0f;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    float2 p = __ldcg(&partials[i]);
    cc_merge(s, c, p.x, p.y);
  }
  cc_block_merge(s, c, ws);
  if (threadIdx.x == 0) {
    out[0] = isfinite(s) ? __fadd_rn(s, c) : s;
    *counter = 0u;
  }
}

// Predicated read-only load that stays where the code generator put it: the
// value keeps its initial contents (the padding) when `ok` is false, and no
// memory is touched then.
__device__ __forceinline__ void cc_ld(float &v, const float *p, int ok) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %2, 0;\n @q ld.global.nc.f32 %0, [%1];\n}\n"
      : "+f"(v)
      : "l"(p), "r"(ok));
}

// Four consecutive floats from a 16-byte aligned address, predicated like cc_ld.
__device__ __forceinline__ void cc_ld4(float4 &v, const float *p, int ok) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n @q ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%5];\n}\n"
      : "+f"(v.x), "+f"(v.y), "+f"(v.z), "+f"(v.w)
      : "r"(ok), "l"(p));
}

// Programmatic dependent launch (griddepcontrol).  A generated kernel waits
// until the kernels it depends on have completed and their writes are
// visible, and only then lets the next kernel in the stream be scheduled, so a
// dependent of this kernel never starts before this kernel's own inputs exist.
// Without the launch attribute both steps are no-ops.
__device__ __forceinline__ void cc_pdl_wait_then_release() {
  asm volatile("griddepcontrol.wait;\n griddepcontrol.launch_dependents;\n" ::: "memory");
}

// At entry.  early = 0: the kernel may read what the previous kernel wrote, so
// it waits before its first load.  early = 1 (the runtime checked that no input
// overlaps the previous kernel's output): the loads and arithmetic proceed
// while the previous kernel drains, and cc_pdl_gate waits before the first
// store, which keeps write-after-read and write-after-write order.
__device__ __forceinline__ void cc_pdl_begin(int early) {
  if (!early) cc_pdl_wait_then_release();
}

__device__ __forceinline__ void cc_pdl_gate(int &early) {
  if (early) {
    cc_pdl_wait_then_release();
    early = 0;
  }
}

// The grid sum's finish in generated kernels (launched with programmatic
// dependent launch): every block first waits for the previous kernel when it
// started early (cc_pdl_gate: the partials, the counter and `out` may still be
// the previous sum's), then publishes its partial.  Thread 0 orders its
// partial before its ticket with the atomic's release semantics, and the last
// block's thread 0 acquires every partial through its own ticket; the barrier
// passes that on to the block (no separate fences).  One block needs no
// partials at all.
__device__ __forceinline__ void cc_grid_finish_pdl(float s, float c, float2 *__restrict__ partials,
                                                   unsigned int *__restrict__ counter, float *__restrict__ out,
                                                   int early) {
  __shared__ float2 ws[32];
  __shared__ int last;
  cc_pdl_gate(early);
  cc_block_merge(s, c, ws);
  if (gridDim.x == 1) {
    if (threadIdx.x == 0) out[0] = isfinite(s) ? __fadd_rn(s, c) : s;
    return;
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = make_float2(s, c);
    unsigned int ticket;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], 1;" : "=r"(ticket) : "l"(counter) : "memory");
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  s = 0.0f;
  c = 0.0f;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    float2 p = __ldcg(&partials[i]);
    cc_merge(s, c, p.x, p.y);
  }
  cc_block_merge(s, c, ws);
  if (threadIdx.x == 0) {
    out[0] = isfinite(s) ? __fadd_rn(s, c) : s;
    *counter = 0u;
  }
}

// Asynchronous 4-byte copy from global memory into a shared-memory slot
// (cp.async): the load holds no register while it is in flight, so a thread
// can have as many loads outstanding as its slots allow.  Each copy is its own
// commit group.  ok = 0 copies no byte and the slot reads +0.0f (zero fill);
// the caller then passes an address inside the buffer.
__device__ __forceinline__ void cc_cp4(float *slot, const float *p, int ok) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(slot);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n cp.async.commit_group;\n" ::"r"(s), "l"(p),
               "r"(ok ? 4 : 0)
               : "memory");
}

// Waits until at most N of this thread's most recent copy groups are pending.
template <int N>
__device__ __forceinline__ void cc_cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// L2 prefetch of the line holding *p, skipped when `ok` is false (so no
// address outside a buffer is ever touched).  It needs no register, so a
// thread can have all of its future loads' lines requested at once.
__device__ __forceinline__ void cc_prefetch(const float *p, int ok) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %1, 0;\n @q prefetch.global.L2 [%0];\n}\n" ::"l"(p), "r"(ok));
}

// ---- shared-memory staging by the Tensor Memory Accelerator (generated
// inner-axis folds).  A tensor map is an opaque 128-byte, 64-byte aligned
// descriptor passed by value as a __grid_constant__ kernel parameter.
struct __align__(64) cc_tensor_map {
  unsigned long long words[16];
};

__device__ __forceinline__ unsigned cc_smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long cc_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void cc_mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the async proxy (the TMA unit).
__device__ __forceinline__ void cc_mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void cc_mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool cc_mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of a barrier for at most limit_ns of %globaltimer
// time; false when the limit ran out.
__device__ __forceinline__ bool cc_mbar_wait_bounded(unsigned bar, unsigned parity, unsigned long long limit_ns) {
  if (cc_mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = cc_globaltimer();
  for (;;) {
    if (cc_mbar_try_wait(bar, parity)) return true;
    if (cc_globaltimer() - t0 > limit_ns) return false;
    __nanosleep(32);
  }
}

// A 2-D tile of a tensor map into shared memory, completing on `bar`.  The
// innermost coordinate x must be a multiple of 16 bytes (here of 4 floats).
__device__ __forceinline__ void cc_tma_load_2d(unsigned dst, const cc_tensor_map *map, int x, int y, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
