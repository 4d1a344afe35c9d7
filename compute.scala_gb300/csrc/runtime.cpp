// The C ABI of include/compute_cuda.h: context, buffer pool, NVRTC program
// cache, launches, reductions, random numbers and events.
//
// It stands where the reference's OpenCL layer stands
// (OpenCL/src/main/scala/com/thoughtworks/compute/OpenCL.scala): one CUDA
// stream per context instead of a pool of command queues (:423-448), a
// size-binned pool instead of one clCreateBuffer per result (:1397-1431), NVRTC
// to cubin instead of clBuildProgram (:885-932, :1266-1294), and bounded event
// waits instead of driver callbacks (:1246-1263).
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gemm.h"
#include "internal.h"
#include "kernels.h"
#include "mlp.h"

namespace cc {

namespace {
thread_local std::string t_last_error;
}

void fail(int code, const std::string &message) { throw Error{code, message}; }

void record_error(const std::string &message) { t_last_error = message; }

// Driver API entry points, resolved through the CUDA runtime at cc_init so the
// library loads (and its GPU-free entry points work) on hosts without a driver.
Driver g_drv;

std::atomic<uint64_t> g_foreign_enqueues{0};

namespace {

void check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  int code = CC_ERR_CUDA;
  if (e == cudaErrorMemoryAllocation) code = CC_ERR_OUT_OF_MEMORY;
  fail(code, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

template <class F>
void resolve(F &fn, const char *symbol) {
  cudaDriverEntryPointQueryResult q;
  void *p = nullptr;
  cudaError_t e = cudaGetDriverEntryPointByVersion(symbol, &p, 12080, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    cudaGetLastError();
    fail(CC_ERR_CUDA, std::string("driver entry point ") + symbol + " is unavailable");
  }
  fn = reinterpret_cast<F>(p);
}

void load_driver() {
  if (g_drv.loaded) return;
  resolve(g_drv.ModuleLoadData, "cuModuleLoadData");
  resolve(g_drv.ModuleGetFunction, "cuModuleGetFunction");
  resolve(g_drv.ModuleUnload, "cuModuleUnload");
  resolve(g_drv.LaunchKernel, "cuLaunchKernel");
  resolve(g_drv.LaunchKernelEx, "cuLaunchKernelEx");
  resolve(g_drv.GetErrorName, "cuGetErrorName");
  resolve(g_drv.GetErrorString, "cuGetErrorString");
  resolve(g_drv.CtxGetCurrent, "cuCtxGetCurrent");
  resolve(g_drv.CtxSetCurrent, "cuCtxSetCurrent");
  resolve(g_drv.FuncSetAttribute, "cuFuncSetAttribute");
  resolve(g_drv.FuncGetAttribute, "cuFuncGetAttribute");
  resolve(g_drv.TensorMapEncodeTiled, "cuTensorMapEncodeTiled");
  resolve(g_drv.OccupancyMaxActiveBlocks, "cuOccupancyMaxActiveBlocksPerMultiprocessor");
  resolve(g_drv.LinkCreate, "cuLinkCreate");
  resolve(g_drv.LinkAddData, "cuLinkAddData");
  resolve(g_drv.LinkComplete, "cuLinkComplete");
  resolve(g_drv.LinkDestroy, "cuLinkDestroy");
  g_drv.loaded = true;
}

void check_cu(CUresult r, const char *what) {
  if (r == CUDA_SUCCESS) return;
  const char *name = nullptr, *str = nullptr;
  if (g_drv.GetErrorName) g_drv.GetErrorName(r, &name);
  if (g_drv.GetErrorString) g_drv.GetErrorString(r, &str);
  int code = r == CUDA_ERROR_OUT_OF_MEMORY ? CC_ERR_OUT_OF_MEMORY : CC_ERR_CUDA;
  fail(code, std::string(what) + ": " + (name ? name : "?") + " (" + (str ? str : "?") + ")");
}

// ---------------------------------------------------------------- fences
//
// A point recorded in a stream (a CUDA event without timing), shared by every
// holder: an event handle returned by an *_ev entry point, or a block of the
// pool released while work on several streams may still use it.  Its CUDA
// event returns to a free list when the last holder drops it.
struct Fence {
  cudaEvent_t ev = nullptr;
  cudaStream_t stream = nullptr;
};
using FencePtr = std::shared_ptr<Fence>;

bool fences_done(std::vector<FencePtr> &fences) {
  for (auto it = fences.begin(); it != fences.end();) {
    cudaError_t r = cudaEventQuery((*it)->ev);
    if (r == cudaSuccess) {
      it = fences.erase(it);
    } else {
      if (r != cudaErrorNotReady) cudaGetLastError();
      return false;
    }
  }
  return true;
}

// ---------------------------------------------------------------- buffer pool
//
// Blocks are binned by size class (eight classes per power of two above 4 KiB,
// so at most 12.5% slack).  While all work is ordered on the context stream, a
// released block goes back to its class's free list and a later allocation may
// reuse it at once.  Once the queue pool is in use (the *_ev entry points), a
// released block carries fences recorded on every stream that may still read
// or write it and waits on a deferred list until they have all completed.  A
// cap (cc_pool_set_limit) turns allocations past it into CC_ERR_OUT_OF_MEMORY,
// the reference's MemObjectAllocationFailure.
class Pool {
 public:
  static size_t size_class(size_t bytes) {
    if (bytes <= 4096) {
      size_t c = 256;
      while (c < bytes) c <<= 1;
      return c;
    }
    size_t p = 4096;
    while (p < bytes) p <<= 1;       // p/2 < bytes <= p
    size_t base = p >> 1, step = base >> 3;
    return base + ((bytes - base + step - 1) / step) * step;
  }

  void *alloc(size_t bytes, size_t *cls_out) {
    size_t cls = size_class(bytes == 0 ? 1 : bytes);
    *cls_out = cls;
    reclaim();
    auto it = free_.find(cls);
    if (it != free_.end() && !it->second.empty()) {
      void *p = it->second.back();
      it->second.pop_back();
      cached_ -= cls;
      in_use_ += cls;
      ++reuses_;
      return p;
    }
    if (limit_ && in_use_ + cls > limit_) {
      fail(CC_ERR_OUT_OF_MEMORY, "buffer pool limit reached: " + std::to_string(in_use_) + " bytes in use, " +
                                     std::to_string(cls) + " requested, limit " + std::to_string(limit_));
    }
    if (limit_ && in_use_ + cached_ + cls > limit_) trim();
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, cls);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      trim();
      e = cudaMalloc(&p, cls);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(CC_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(cls) + " bytes failed: " + cudaGetErrorString(e));
    }
    in_use_ += cls;
    ++allocs_;
    return p;
  }

  void release(void *p, size_t cls, std::vector<FencePtr> fences = {}) {
    in_use_ -= cls;
    cached_ += cls;
    if (fences.empty())
      free_[cls].push_back(p);
    else
      deferred_.push_back(Deferred{p, cls, std::move(fences)});
  }

  // Deferred blocks whose fences have all completed become free.
  void reclaim() {
    for (auto it = deferred_.begin(); it != deferred_.end();) {
      if (fences_done(it->fences)) {
        free_[it->cls].push_back(it->p);
        it = deferred_.erase(it);
      } else {
        ++it;
      }
    }
  }

  void trim() {
    reclaim();
    for (auto &kv : free_) {
      for (void *p : kv.second) {
        cudaFree(p);
        cached_ -= kv.first;
      }
      kv.second.clear();
    }
  }

  size_t in_use_ = 0, cached_ = 0, limit_ = 0;
  uint64_t allocs_ = 0, reuses_ = 0;

 private:
  struct Deferred {
    void *p;
    size_t cls;
    std::vector<FencePtr> fences;
  };
  std::map<size_t, std::vector<void *>> free_;
  std::vector<Deferred> deferred_;
};

struct Buffer {
  void *ptr = nullptr;
  size_t bytes = 0;
  size_t cls = 0;
  int refs = 1;
};

// A compiled module.  Programs whose inputs are all read contiguously share one
// module per structure whatever their shape (the length is a launch argument);
// other programs have their own.
struct Module {
  CUmodule module = nullptr;
  CUfunction scalar = nullptr;  // cc_ew / cc_sum
  CUfunction vec4 = nullptr;    // cc_ew_v4 / cc_sum_v4 (contiguous inputs)
  CUfunction vl = nullptr;      // cc_ew_vl / cc_sum_vl (float4 grouped reads; 16-byte aligned inputs)
  int block = 256;              // threads per block the kernels were generated for
  int resident_scalar = 0;      // blocks one SM holds at once, per variant
  int resident_vec4 = 0;
  int resident_vl = 0;
  int vec_unroll = 1;
  int smem_bytes = 0;           // dynamic shared memory of the scalar kernel (its load ring)
  int points = 1;               // consecutive points per thread of the scalar elementwise kernel
  std::string source;
  ~Module() {
    if (module && g_drv.ModuleUnload) g_drv.ModuleUnload(module);
  }
};

// The tunable form of programs (tunable_source); one module may serve several.
struct TuneModule {
  CUmodule module = nullptr;
  ~TuneModule() {
    if (module && g_drv.ModuleUnload) g_drv.ModuleUnload(module);
  }
};

struct TuneEntry {
  std::shared_ptr<TuneModule> mod;
  CUfunction fn[kTuneKernels] = {};
  int resident[kTuneKernels][4] = {};  // blocks per SM by kernel and block size (0: not queried yet)
  ProgramKind kind = ProgramKind::Elementwise;
  int n_inputs = 0;
  int64_t n = 0;
  bool contiguous = false;
  Ir ir;
};

// Programs compiled in their tunable form for timing (cc_tune_*).
struct TuneSet {
  std::vector<TuneEntry> entries;
  void *flush = nullptr;  // written between timed launches to empty L2
  size_t flush_cls = 0;
  size_t flush_bytes = 0;
};

// A multilayer perceptron with its Adam state and batch scratch (cc_mlp_*).
struct Mlp {
  std::vector<int> dims;  // widths, input first
  std::vector<size_t> w_off, b_off;
  size_t n_params = 0;
  void *state = nullptr;  // params, grads, Adam m, Adam v
  size_t state_cls = 0;
  int steps = 0;
  int cap = 0;             // batch the scratch holds
  void *scratch = nullptr;  // activations, deltas, column-sum partials, loss
  size_t scratch_cls = 0;
  float *params() { return static_cast<float *>(state); }
  float *grads() { return params() + n_params; }
  float *adam_m() { return params() + 2 * n_params; }
  float *adam_v() { return params() + 3 * n_params; }
};

struct Program {
  std::shared_ptr<Module> mod;
  std::unique_ptr<TuneEntry> tune;  // the tunable form (tuner on)
  int tuned_config = -1;            // the configuration the tuner chose
  ProgramKind kind = ProgramKind::Elementwise;
  Generated gen;                // shape information (its source lives in the module)
  bool is_contraction = false;  // run as a GEMM (cc_gemm_f32 mode contraction_mode)
  int contraction_mode = 0;
  Contraction con;
  bool is_row_fold = false;     // an inner-axis fold: cc_rowfold / cc_rowfold_plain of mod
  RowFold rf;
  CUfunction rf_tma = nullptr, rf_plain = nullptr;
};

struct Event {
  cudaEvent_t ev = nullptr;  // a timing event (cc_event_record), or the fence's event
  FencePtr fence;            // set for events returned by the *_ev entry points
};

// The queue pool: streams that the *_ev entry points spread independent work
// over, as the reference's CommandQueuePool spreads it over command queues
// (OpenCL.scala:423-448, 5 per device).  Streams are cheap, and every queue
// is in order, so a larger pool puts fewer unrelated operations behind one
// another: eight.
constexpr int kQueues = 8;

// Many independent programs evaluated together (cc_batch_*).
struct Batch {
  CUmodule module = nullptr;
  CUfunction persistent = nullptr;
  std::vector<CUfunction> per_structure;  // one float4 kernel per distinct program
  std::vector<int> sid;                   // structure of each program
  std::vector<int> n_inputs;              // inputs of each program
  std::vector<int64_t> length;            // points of each program
  int resident = 0;                       // persistent blocks one SM holds
  // bound buffers
  bool bound = false;
  std::vector<std::vector<uint64_t>> ptrs;  // per program: inputs..., output
  void *table = nullptr;
  size_t table_cls = 0;
  int64_t total_tiles = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  // device copy tables of recent cc_batch_upload_ev / cc_batch_download_ev
  // calls (most recent last), keyed by direction and host pointers
  struct CopyTable {
    std::vector<uint64_t> key;
    uint64_t pinned_gen = 0;
    void *dev = nullptr;
    size_t cls = 0;
    int n = 0;
    long long chunks = 0;
  };
  std::vector<CopyTable> copy_tables;
};

enum : uint64_t { kTagBuffer = 1, kTagProgram = 2, kTagEvent = 3, kTagBatch = 4, kTagTuneSet = 5, kTagMlp = 6 };

// Defaults of the batch code-generation knobs (also what the CPU-side
// compile check builds).
constexpr int kBatchInlineDefault = 1;
constexpr int kBatchRegistersDefault = 64;
constexpr int kBatchLoadsDefault = 4;
constexpr int kBatchLanesDefault = 4;
constexpr int kBatchRolledDefault = 1;
constexpr int kBatchPrefetchDefault = 0;

struct Context {
  int device = 0;
  CUcontext cuctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  size_t total_mem = 0;
  uint32_t flags = 0;

  std::recursive_mutex mu;
  std::vector<cudaEvent_t> free_events;  // of dropped fences (declared before the pool, which holds fences)
  Pool pool;
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, Buffer *> buffers;
  std::unordered_map<uint64_t, Program *> programs;   // by handle
  std::unordered_map<std::string, uint64_t> cache;    // IR text -> program handle
  std::unordered_map<std::string, std::shared_ptr<Module>> modules;  // structure key -> module
  std::unordered_map<std::string, std::shared_ptr<TuneModule>> tune_modules;  // structure key -> tunable form
  std::unordered_map<uint64_t, Event *> events;
  std::unordered_map<uint64_t, Batch *> batches;
  std::unordered_map<uint64_t, TuneSet *> tune_sets;
  std::unordered_map<uint64_t, Mlp *> mlps;
  uint64_t cost_model = 0;              // Mlp handle the learned tuner consults
  std::vector<float> cost_mean, cost_inv_std;  // its feature normalisation
  uint64_t cache_hits = 0, cache_misses = 0;
  std::mutex compile_mu;

  // Tuning knobs (cc_config_set).
  int block = 128;
  int ew_blocks_per_sm = 0;
  int sum_blocks_per_sm = 4;
  int upload_streams = 4;
  int ew_lookahead = 8;
  int ew_asm_loads = 1;
  int vec_unroll = 4;
  int64_t prefetch_min_bytes = -1;
  int sum_block = 256;
  int tc_variant = 5;  // 128x256 tiles, hi*hi restarted every 256 of K
  int contraction = 1;  // 0: generated fold kernel; else CC_GEMM_* mode + 1
  int row_fold = 1;     // inner-axis folds of at least kRowFoldMinTerms terms: 1 = TMA-staged skeleton
  int row_fold_stages = 0;  // its ring stages (0 = as many 8 KiB tiles as fit 96 KiB, at most 8)
  int batch_inline = kBatchInlineDefault;          // expressions inlined into tile functions, exp/log/tanh called
  int batch_max_registers = kBatchRegistersDefault;  // four 256-thread blocks per SM for the persistent kernel
  int batch_run_tiles = 4;                          // tiles a persistent block claims at once
  int batch_max_loads = kBatchLoadsDefault;         // float4 loads a tile function keeps in flight per thread
  int batch_lanes = kBatchLanesDefault;             // points a tile function evaluates together (0: one)
  int batch_rolled = kBatchRolledDefault;           // a tile's load groups in a loop (1) or unrolled (0)
  int batch_prefetch = kBatchPrefetchDefault;       // L2 bulk prefetch of a run's later tiles (1), and of the next run (2)
  int tuner = 0;  // 0 off, 1 exhaustive, 2 learned
  int ew_smem_ring = 0;  // generic kernels: shared-memory ring slots per thread for staged loads
  int ew_points = 1;     // generic elementwise kernels: consecutive points per thread
  int ew_vector_loads = 1;  // generic elementwise kernels: float4 grouped reads when inputs are aligned
  int ew_batch_loads = 0;   // those kernels: one predicate per group of 8 scalar loads
  int pdl = 1;           // launch generated kernels with programmatic dependent launch
  int copy_kernel = 0;   // copies between pinned host memory and the device by the SMs
  int batch_copy_kernel = 1;  // batch transfers: one SM copy kernel over a table of the copies
  // live cc_host_alloc allocations (start -> bytes); the generation changes at every free
  std::map<uintptr_t, size_t> pinned;
  uint64_t pinned_gen = 0;
  // The output range of the last generated kernel launched, and its stream: a
  // kernel that reads none of it may start its loads before that kernel ends,
  // provided nothing else was enqueued on the stream since.  Every entry point
  // that enqueues other work under the context lock clears `valid`
  // (end_pdl_chain); the sum without a context (cc_reduce_sum_f32_noalloc)
  // bumps g_foreign_enqueues instead, which `foreign` remembers.
  struct {
    cudaStream_t stream = nullptr;
    uint64_t lo = 0, hi = 0;
    uint64_t foreign = 0;
    bool valid = false;
  } last_write;
  int tc_group_m = 1;    // tensor-core GEMM: tile rows per group of the tile order (1 = row-major)
  cudaStream_t copy_streams[8] = {};
  cudaEvent_t copy_events[9] = {};

  // The queue pool, created by the first *_ev call (multi_queue then stays on).
  bool multi_queue = false;
  cudaStream_t queues[kQueues] = {};
  bool queue_dirty[kQueues] = {};  // work enqueued since the last cc_synchronize
  // copy streams with batch transfers not joined into the context stream
  // (cc_batch_*_ev) since the last cc_synchronize
  bool copy_dirty[8] = {};
  int next_queue = 0;
  void *queue_scratch[kQueues] = {};  // each queue's sum partials and counter
  size_t queue_scratch_cls[kQueues] = {};

  // Scratch of the grid sums: kMaxSumBlocks float2 partials, then the counter.
  void *sum_scratch = nullptr;
  size_t sum_scratch_cls = 0;


  uint64_t make_handle(uint64_t tag) { return (tag << 56) | (next_id++); }
  // Device error flag of the kernels with bounded waits (in the same scratch block).
  int *error_flag() {
    return reinterpret_cast<int *>(static_cast<char *>(sum_scratch) + sizeof(float2) * kMaxSumBlocks + 128);
  }
  // The word cc_probe_bounded_wait waits on (same block).
  int *probe_flag() {
    return reinterpret_cast<int *>(static_cast<char *>(sum_scratch) + sizeof(float2) * kMaxSumBlocks + 192);
  }
};

std::mutex g_init_mu;
Context *g_ctx = nullptr;

Context &ctx() {
  Context *c = g_ctx;
  if (!c) fail(CC_ERR_NOT_INITIALIZED, "cc_init has not been called");
  thread_local CUcontext bound = nullptr;
  if (bound != c->cuctx) {
    check_cuda(cudaSetDevice(c->device), "cudaSetDevice");
    check_cu(g_drv.CtxSetCurrent(c->cuctx), "cuCtxSetCurrent");
    bound = c->cuctx;
  }
  return *c;
}

uint64_t tag_of(uint64_t h) { return h >> 56; }

// Work other than a generated kernel is about to be enqueued: the next
// generated kernel must wait for it before its first load.
void end_pdl_chain(Context &c) { c.last_write.valid = false; }

// ---------------------------------------------------------------- queue pool and fences

constexpr size_t kSumScratchBytes = sizeof(float2) * kMaxSumBlocks + 256;  // partials, counter, flags

// A fence recorded on `s` now (the context lock is held).
FencePtr record_fence(Context &c, cudaStream_t s) {
  cudaEvent_t ev = nullptr;
  if (!c.free_events.empty()) {
    ev = c.free_events.back();
    c.free_events.pop_back();
  } else {
    check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
  }
  cudaError_t r = cudaEventRecord(ev, s);
  if (r != cudaSuccess) {
    c.free_events.push_back(ev);
    check_cuda(r, "cudaEventRecord");
  }
  Context *cp = &c;
  return FencePtr(new Fence{ev, s}, [cp](Fence *f) {
    cp->free_events.push_back(f->ev);
    delete f;
  });
}

// The queue pool starts after everything already enqueued on the context
// stream, so blocks that stream released earlier are safe to reuse there.
void enter_multi_queue(Context &c) {
  if (c.multi_queue) return;
  for (int i = 0; i < kQueues; ++i) {
    if (!c.queues[i]) check_cuda(cudaStreamCreateWithFlags(&c.queues[i], cudaStreamNonBlocking), "cudaStreamCreate");
    if (!c.queue_scratch[i]) {
      c.queue_scratch[i] = c.pool.alloc(kSumScratchBytes, &c.queue_scratch_cls[i]);
      check_cuda(cudaMemsetAsync(c.queue_scratch[i], 0, kSumScratchBytes, c.stream), "cudaMemsetAsync");
    }
  }
  FencePtr f = record_fence(c, c.stream);
  for (int i = 0; i < kQueues; ++i) check_cuda(cudaStreamWaitEvent(c.queues[i], f->ev, 0), "cudaStreamWaitEvent");
  c.multi_queue = true;
}

// A queue for the next operation (the reference's dispatch takes one from its
// pool): the first idle one from the round-robin position on, so that an
// operation whose wait list is already satisfied does not queue behind
// unrelated work still in flight; round robin when every queue is busy.
int pick_queue(Context &c) {
  enter_multi_queue(c);
  int q = c.next_queue;
  for (int i = 0; i < kQueues; ++i) {
    const int k = (c.next_queue + i) % kQueues;
    const cudaError_t r = cudaStreamQuery(c.queues[k]);
    if (r == cudaSuccess) {
      q = k;
      break;
    }
    if (r != cudaErrorNotReady) {
      cudaGetLastError();
      break;
    }
  }
  c.next_queue = (q + 1) % kQueues;
  return q;
}

int queue_index(const Context &c, cudaStream_t s) {
  for (int i = 0; i < kQueues; ++i)
    if (c.multi_queue && c.queues[i] == s) return i;
  return -1;
}

// Returns a block to the pool.  With the queue pool in use, work on the
// context stream and on every queue that has work pending may still use the
// block, so it is deferred behind a fence on each of them.
void release_block(Context &c, void *p, size_t cls) {
  bool copies = false;
  for (bool d : c.copy_dirty) copies = copies || d;
  if (!c.multi_queue && !copies) {
    c.pool.release(p, cls);
    return;
  }
  std::vector<FencePtr> fences;
  fences.push_back(record_fence(c, c.stream));
  for (int i = 0; i < kQueues; ++i)
    if (c.multi_queue && c.queue_dirty[i]) fences.push_back(record_fence(c, c.queues[i]));
  for (int i = 0; i < 8; ++i)
    if (c.copy_dirty[i]) fences.push_back(record_fence(c, c.copy_streams[i]));
  c.pool.release(p, cls, std::move(fences));
}

// The partials and completion counter a grid sum on stream `s` uses: the
// context's own on the context stream, each queue's own on the queues (sums on
// different streams may run at once and must not share them).  Any other
// (caller) stream gets a temporary block, zeroed on that stream; *temporary is
// then set and the caller releases it after synchronising the stream.
void *sum_scratch_for(Context &c, cudaStream_t s, size_t *temporary_cls) {
  *temporary_cls = 0;
  if (s == c.stream) return c.sum_scratch;
  const int q = queue_index(c, s);
  if (q >= 0) return c.queue_scratch[q];
  size_t cls = 0;
  void *p = c.pool.alloc(kSumScratchBytes, &cls);
  cudaError_t e = cudaMemsetAsync(static_cast<char *>(p) + sizeof(float2) * kMaxSumBlocks, 0, 256, s);
  if (e != cudaSuccess) {
    c.pool.release(p, cls);
    check_cuda(e, "cudaMemsetAsync");
  }
  *temporary_cls = cls;
  return p;
}

Buffer &buffer_of(Context &c, cc_handle h) {
  auto it = c.buffers.find(h);
  if (tag_of(h) != kTagBuffer || it == c.buffers.end())
    fail(CC_ERR_INVALID_MEM_OBJECT, "not a live buffer handle");
  return *it->second;
}

Program &program_of(Context &c, cc_handle h) {
  auto it = c.programs.find(h);
  if (tag_of(h) != kTagProgram || it == c.programs.end()) fail(CC_ERR_INVALID_PROGRAM, "not a program handle");
  return *it->second;
}

Event &event_of(Context &c, cc_handle h) {
  auto it = c.events.find(h);
  if (tag_of(h) != kTagEvent || it == c.events.end()) fail(CC_ERR_INVALID_EVENT, "not a live event handle");
  return *it->second;
}

// Makes `s` wait for every event of a wait list (Kernel.enqueue's waitingEvents).
void wait_events(Context &c, cudaStream_t s, const cc_handle *wait, int n_wait) {
  if (n_wait < 0 || (n_wait > 0 && !wait)) fail(CC_ERR_INVALID_VALUE, "bad wait list");
  for (int i = 0; i < n_wait; ++i) check_cuda(cudaStreamWaitEvent(s, event_of(c, wait[i]).ev, 0), "cudaStreamWaitEvent");
}

// A new event handle for a fence (what the *_ev entry points return).
cc_handle fence_handle(Context &c, FencePtr f) {
  auto e = std::make_unique<Event>();
  e->ev = f->ev;
  e->fence = std::move(f);
  uint64_t h = c.make_handle(kTagEvent);
  c.events[h] = e.release();
  return h;
}

// ---------------------------------------------------------------- NVRTC

std::vector<char> compile_cubin(const std::string &source, int cc_major, int cc_minor, uint32_t flags,
                                bool relocatable = false, int max_registers = 0) {
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "cc_program.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) fail(CC_ERR_BUILD_PROGRAM_FAILURE, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
  std::string arch = "-arch=sm_" + std::to_string(cc_major) + std::to_string(cc_minor) + "a";
  // Contraction is never the compiler's choice: with CC_FLAG_FMA_CONTRACT the
  // generated code holds explicit fmaf calls (FmaScope), so both modes are deterministic.
  (void)flags;
  std::vector<std::string> opts = {arch, "--std=c++17", "-default-device", "--fmad=false"};
  if (relocatable) opts.push_back("-rdc=true");
  if (max_registers > 0) opts.push_back("--maxrregcount=" + std::to_string(max_registers));
  std::vector<const char *> optp;
  for (auto &o : opts) optp.push_back(o.c_str());
  r = nvrtcCompileProgram(prog, (int)optp.size(), optp.data());
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    fail(CC_ERR_BUILD_PROGRAM_FAILURE, "NVRTC build failure (" + arch + "):\n" + log);
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  std::vector<char> cubin(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  return cubin;
}

// ---------------------------------------------------------------- launches

// Enough blocks for one element per thread, capped at what the GPU holds at
// once (the kernel then loops), so every SM gets the same share of threads.
int64_t ew_grid(int64_t work, int block, int sm_count, int resident) {
  int64_t grid = (work + block - 1) / block;
  int64_t cap = (int64_t)sm_count * (resident > 0 ? resident : 8);
  if (cap < 1) cap = 1;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return grid;
}

void encode_plane_map(CUtensorMap *map, void *base, int rows, int kcols, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)kcols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kcols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  check_cu(g_drv.TensorMapEncodeTiled(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
           "cuTensorMapEncodeTiled");
}

// C[m,n] = A[m,k] * B[k,n] with the kernels of the given CC_GEMM_* mode.
void run_gemm(Context &c, const float *A, const float *B, float *C, int m, int n, int k, int64_t lda, int64_t ldb,
              int64_t ldc, int mode, cudaStream_t s) {
  if (m == 0 || n == 0) return;
  if (mode == CC_GEMM_EXACT || mode == CC_GEMM_FP32) {
    check_cuda(launch_sgemm(A, B, C, m, n, k, lda, ldb, ldc, mode == CC_GEMM_EXACT, s), "sgemm launch");
    return;
  }
  if (mode != CC_GEMM_BF16X6) fail(CC_ERR_INVALID_VALUE, "unknown contraction mode");
  if (c.cc_major != 10) fail(CC_ERR_INVALID_OPERATION, "the tensor-core contraction needs an sm_10x GPU");
  const int Mp = (m + kTcBM - 1) / kTcBM * kTcBM;
  const int Np = (n + kTcBN - 1) / kTcBN * kTcBN;
  const int Kp = (k + kTcBK - 1) / kTcBK * kTcBK;
  size_t cls_a = 0, cls_b = 0;
  const size_t bytes_a = (size_t)3 * Mp * Kp * 2, bytes_b = (size_t)3 * Np * Kp * 2;
  void *pa = c.pool.alloc(bytes_a, &cls_a);
  void *pb = nullptr;
  try {
    pb = c.pool.alloc(bytes_b, &cls_b);
  } catch (...) {
    release_block(c, pa, cls_a);
    throw;
  }
  cudaError_t e = launch_split_a(A, lda, m, k, static_cast<__nv_bfloat16 *>(pa), Mp, Kp, c.sm_count, s);
  if (e == cudaSuccess) e = launch_split_bt(B, ldb, k, n, static_cast<__nv_bfloat16 *>(pb), Np, Kp, s);
  if (e == cudaSuccess) {
    CUtensorMap maps[9];
    const size_t plane_a = (size_t)Mp * Kp * 2, plane_b = (size_t)Np * Kp * 2;
    const int variant = gemm_tc_variant(c.tc_variant, Kp);  // the kernel that runs: its tile width
    try {
      for (int p = 0; p < 3; ++p) {
        encode_plane_map(&maps[p], static_cast<char *>(pa) + p * plane_a, Mp, Kp, kTcBM);
        encode_plane_map(&maps[3 + p], static_cast<char *>(pb) + p * plane_b, Np, Kp, gemm_tc_box_n(variant));
        encode_plane_map(&maps[6 + p], static_cast<char *>(pb) + p * plane_b, Np, Kp, gemm_tc_box_n(variant) / 2);
      }
    } catch (...) {
      release_block(c, pa, cls_a);
      release_block(c, pb, cls_b);
      throw;
    }
    e = launch_gemm_bf16x6(maps, C, m, n, Kp, ldc, c.sm_count, c.error_flag(), variant, c.tc_group_m, s);
  }
  // blocks of the pool are ordered on the context stream and the queues; wait for other streams
  if (s != c.stream && queue_index(c, s) < 0 && e == cudaSuccess) e = cudaStreamSynchronize(s);
  release_block(c, pa, cls_a);
  release_block(c, pb, cls_b);
  check_cuda(e, "bf16x6 contraction launch");
}

// Defined with the tuner, below.
void launch_tuned_program(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream);
std::shared_ptr<TuneModule> load_tune_module(const std::vector<char> &cubin);
void load_tune_entry(TuneEntry &e, const Ir &ir, std::shared_ptr<TuneModule> mod, const std::string &suffix);

// An inner-axis fold: one thread per output, 64 per block; tiles of the row
// inputs staged by TMA when every row input is 16-byte aligned, else direct loads.
void launch_row_fold(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream) {
  const RowFold &rf = p.rf;
  if (rf.rows == 0) return;
  const int nin = (int)rf.row_inputs.size();
  bool aligned = true;
  for (int k : rf.row_inputs) aligned = aligned && (in[k] & 15u) == 0;
  CUtensorMap maps[kRowFoldMaxInputs];
  if (aligned) {
    for (int i = 0; i < nin; ++i) {
      const cuuint64_t dims[2] = {(cuuint64_t)rf.cols, (cuuint64_t)rf.rows};
      const cuuint64_t strides[1] = {(cuuint64_t)rf.cols * 4};
      const cuuint32_t box[2] = {32, (cuuint32_t)kRowFoldRows};
      const cuuint32_t estr[2] = {1, 1};
      check_cu(g_drv.TensorMapEncodeTiled(&maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                          reinterpret_cast<void *>(in[rf.row_inputs[i]]), dims, strides, box, estr,
                                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
               "cuTensorMapEncodeTiled");
    }
  }
  std::vector<void *> args;
  for (int i = 0; i < nin; ++i) args.push_back(&maps[i]);
  std::vector<uint64_t> ptrs(in);
  for (auto &v : ptrs) args.push_back(&v);
  uint64_t o = out;
  long long rows = rf.rows;
  int cols = (int)rf.cols;
  uint64_t err = reinterpret_cast<uint64_t>(c.error_flag());
  args.push_back(&o);
  args.push_back(&rows);
  args.push_back(&cols);
  args.push_back(&err);
  const unsigned grid = (unsigned)((rf.rows + kRowFoldRows - 1) / kRowFoldRows);
  // With programmatic dependent launch the block set-up (barrier
  // initialisation) overlaps the previous kernel's tail; every block waits
  // (griddepcontrol.wait) before its first load.
  CUlaunchAttribute attr;
  memset(&attr, 0, sizeof attr);
  attr.id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
  attr.value.programmaticStreamSerializationAllowed = 1;
  CUlaunchConfig cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.gridDimX = grid;
  cfg.gridDimY = cfg.gridDimZ = 1;
  cfg.blockDimX = (unsigned)kRowFoldRows;
  cfg.blockDimY = cfg.blockDimZ = 1;
  cfg.sharedMemBytes = aligned ? (unsigned)row_fold_smem_bytes(nin, row_fold_stages(nin, rf.stages)) : 0u;
  cfg.hStream = (CUstream)stream;
  cfg.attrs = &attr;
  cfg.numAttrs = c.pdl ? 1 : 0;
  check_cu(g_drv.LaunchKernelEx(&cfg, aligned ? p.rf_tma : p.rf_plain, args.data(), nullptr), "cuLaunchKernelEx");
}

void launch_generated(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream);

void launch_program(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream) {
  if (p.is_contraction || p.is_row_fold) end_pdl_chain(c);
  if (p.is_row_fold) {
    launch_row_fold(c, p, in, out, stream);
    return;
  }
  if (p.tune) {
    launch_tuned_program(c, p, in, out, stream);
    return;
  }
  if (p.is_contraction) {
    const Contraction &q = p.con;
    run_gemm(c, reinterpret_cast<const float *>(in[q.a_input]), reinterpret_cast<const float *>(in[q.b_input]),
             reinterpret_cast<float *>(out), (int)q.m, (int)q.n, (int)q.k, q.k, q.n, q.n, p.contraction_mode, stream);
    return;
  }
  launch_generated(c, p, in, out, stream);
}

// The standard generated kernels (cc_ew / cc_ew_v4 / cc_ew_vl, cc_sum*) of a program.
void launch_generated(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream) {
  const Module &m = *p.mod;
  const int block = m.block;
  const int64_t n = p.gen.domain;
  bool aligned = (out & 15u) == 0;
  for (uint64_t a : in) aligned = aligned && (a & 15u) == 0;
  const bool vec = m.vec4 && aligned;
  const bool vl = !vec && m.vl && aligned;
  CUfunction f = vec ? m.vec4 : vl ? m.vl : m.scalar;
  // float4 kernels: each thread takes vec_unroll positions per batch
  // (scalar elementwise kernels: `points` consecutive points per thread)
  const int64_t work = vec ? ((n >> 2) + m.vec_unroll - 1) / m.vec_unroll : (n + m.points - 1) / m.points;
  std::vector<void *> args;
  std::vector<uint64_t> ptrs(in);
  for (auto &v : ptrs) args.push_back(&v);
  uint64_t out_ptr = out;
  int64_t nn = n;
  uint64_t partials = 0, counter = 0;
  unsigned grid;
  size_t temporary = 0;  // a sum on a caller stream: its own scratch block, released after the launch
  if (p.kind == ProgramKind::Sum) {
    char *scratch = static_cast<char *>(sum_scratch_for(c, stream, &temporary));
    partials = reinterpret_cast<uint64_t>(scratch);
    counter = reinterpret_cast<uint64_t>(scratch + sizeof(float2) * kMaxSumBlocks);
    args.push_back(&partials);
    args.push_back(&counter);
    grid = (unsigned)sum_grid_for(work, block, c.sm_count * c.sum_blocks_per_sm);
  } else {
    if (n == 0) return;
    int resident = vec ? m.resident_vec4 : vl ? m.resident_vl : m.resident_scalar;
    if (c.ew_blocks_per_sm > 0 && (resident <= 0 || c.ew_blocks_per_sm < resident)) resident = c.ew_blocks_per_sm;
    grid = (unsigned)ew_grid(work, block, c.sm_count, resident);
  }
  args.push_back(&out_ptr);
  args.push_back(&nn);
  // early start: the previous operation on the context's own stream is the
  // generated kernel last_write describes, and none of this kernel's inputs
  // overlaps what it writes (the stores still wait for it).  A caller stream
  // may carry the caller's own work, so launches there never start early.
  const uint64_t foreign = g_foreign_enqueues.load(std::memory_order_acquire);
  int early = 0;
  if (c.pdl == 1 && c.last_write.valid && c.last_write.stream == stream && stream == c.own_stream &&
      c.last_write.foreign == foreign) {
    early = 1;
    for (size_t i = 0; i < in.size(); ++i) {
      const uint64_t lo = in[i];
      const uint64_t hi = lo + (uint64_t)(i < p.gen.param_bytes.size() ? p.gen.param_bytes[i] : 0);
      if (lo < c.last_write.hi && c.last_write.lo < hi) early = 0;
    }
  }
  args.push_back(&early);
  c.last_write.stream = stream;
  c.last_write.lo = out;
  c.last_write.hi = out + (uint64_t)(p.gen.out_elems > 0 ? p.gen.out_elems : 1) * sizeof(float);
  c.last_write.foreign = foreign;
  c.last_write.valid = c.pdl == 1;
  const unsigned smem = vec || vl ? 0 : (unsigned)m.smem_bytes;
  CUresult r;
  if (c.pdl) {
    // programmatic dependent launch: this grid may be scheduled while the
    // previous kernel in the stream drains; its cc_pdl_begin / cc_pdl_gate keep the order
    CUlaunchAttribute attr;
    memset(&attr, 0, sizeof attr);
    attr.id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
    attr.value.programmaticStreamSerializationAllowed = 1;
    CUlaunchConfig cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDimX = grid;
    cfg.gridDimY = cfg.gridDimZ = 1;
    cfg.blockDimX = (unsigned)block;
    cfg.blockDimY = cfg.blockDimZ = 1;
    cfg.sharedMemBytes = smem;
    cfg.hStream = (CUstream)stream;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    r = g_drv.LaunchKernelEx(&cfg, f, args.data(), nullptr);
  } else {
    r = g_drv.LaunchKernel(f, grid, 1, 1, block, 1, 1, smem, (CUstream)stream, args.data(), nullptr);
  }
  if (temporary) {
    cudaError_t se = r == CUDA_SUCCESS ? cudaStreamSynchronize(stream) : cudaSuccess;
    c.pool.release(reinterpret_cast<void *>(partials), temporary);
    check_cuda(se, "cudaStreamSynchronize");
  }
  check_cu(r, "cuLaunchKernel");
}

// Upload striped over the context's copy streams, ordered after the work
// queued on the main stream and joined back into it.
// The device-side address of a pinned host buffer (nullptr for pageable memory).
const void *pinned_device_alias(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return a.devicePointer;
}

// Copies with the SMs (launch_copy16) when the knob is on, the host side is
// pinned and both ends are 16-byte aligned; returns false to let the caller
// use the DMA engines instead.
bool sm_copy(Context &c, void *dst, const void *src, size_t bytes, bool to_device) {
  if (!c.copy_kernel || bytes < (size_t(1) << 20)) return false;
  const void *host = to_device ? src : dst;
  const void *alias = pinned_device_alias(host);
  if (!alias) return false;
  void *d = to_device ? dst : const_cast<void *>(alias);
  const void *s = to_device ? alias : src;
  if ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(s)) & 15u) return false;
  const size_t body = bytes & ~size_t(15);
  check_cuda(launch_copy16(d, s, body, c.sm_count, c.stream), "copy kernel");
  if (body < bytes)
    check_cuda(cudaMemcpyAsync(static_cast<char *>(dst) + body, static_cast<const char *>(src) + body, bytes - body,
                               to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c.stream),
               "cudaMemcpyAsync");
  end_pdl_chain(c);
  return true;
}

void striped_upload(Context &c, char *dst, const char *src, size_t bytes) {
  if (sm_copy(c, dst, src, bytes, true)) return;
  const int k = c.upload_streams;
  if (k <= 1 || bytes < (size_t(8) << 20)) {
    check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c.stream), "cudaMemcpyAsync H2D");
    return;
  }
  check_cuda(cudaEventRecord(c.copy_events[8], c.stream), "cudaEventRecord");
  size_t chunk = ((bytes + k - 1) / k + 4095) & ~size_t(4095);
  for (int i = 0; i < k; ++i) {
    size_t off = chunk * i;
    if (off >= bytes) break;
    size_t len = bytes - off < chunk ? bytes - off : chunk;
    check_cuda(cudaStreamWaitEvent(c.copy_streams[i], c.copy_events[8], 0), "cudaStreamWaitEvent");
    check_cuda(cudaMemcpyAsync(dst + off, src + off, len, cudaMemcpyHostToDevice, c.copy_streams[i]),
               "cudaMemcpyAsync H2D");
    check_cuda(cudaEventRecord(c.copy_events[i], c.copy_streams[i]), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(c.stream, c.copy_events[i], 0), "cudaStreamWaitEvent");
  }
}

}  // namespace
}  // namespace cc

using namespace cc;

#define CC_API_BEGIN try {
#define CC_API_END                                            \
  }                                                           \
  catch (const cc::Error &e) {                                \
    cc::t_last_error = e.message;                             \
    return e.code;                                            \
  }                                                           \
  catch (const std::bad_alloc &) {                            \
    cc::t_last_error = "host allocation failed";              \
    return CC_ERR_OUT_OF_RESOURCES;                           \
  }                                                           \
  catch (const std::exception &e) {                           \
    cc::t_last_error = e.what();                              \
    return CC_ERR_INVALID_VALUE;                              \
  }                                                           \
  return CC_OK;

extern "C" {

int cc_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return CC_ERR_INVALID_VALUE;
  size_t n = t_last_error.size() < len - 1 ? t_last_error.size() : len - 1;
  memcpy(buf, t_last_error.data(), n);
  buf[n] = '\0';
  return CC_OK;
}

int cc_init(int device_ordinal, uint32_t flags) {
  CC_API_BEGIN
  std::lock_guard<std::mutex> g(g_init_mu);
  if (g_ctx) {
    if (g_ctx->device != device_ordinal) fail(CC_ERR_INVALID_OPERATION, "already initialised on another device");
    if (g_ctx->flags != flags)
      fail(CC_ERR_INVALID_OPERATION, "already initialised with flags " + std::to_string(g_ctx->flags) +
                                         " (cc_shutdown first to change them)");
    return CC_OK;
  }
  int count = 0;
  cudaError_t ce = cudaGetDeviceCount(&count);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    fail(CC_ERR_DEVICE_NOT_FOUND, std::string("no usable CUDA device: ") + cudaGetErrorString(ce));
  }
  if (device_ordinal < 0 || device_ordinal >= count) fail(CC_ERR_DEVICE_NOT_FOUND, "no CUDA device " + std::to_string(device_ordinal));
  load_driver();
  auto c = std::make_unique<Context>();
  c->device = device_ordinal;
  c->flags = flags;
  check_cuda(cudaSetDevice(device_ordinal), "cudaSetDevice");
  check_cuda(cudaFree(nullptr), "cudaFree(0)");  // creates the primary context and makes it current
  check_cu(g_drv.CtxGetCurrent(&c->cuctx), "cuCtxGetCurrent");
  check_cuda(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device_ordinal), "attr");
  check_cuda(cudaDeviceGetAttribute(&c->cc_major, cudaDevAttrComputeCapabilityMajor, device_ordinal), "attr");
  check_cuda(cudaDeviceGetAttribute(&c->cc_minor, cudaDevAttrComputeCapabilityMinor, device_ordinal), "attr");
  {
    size_t free_b = 0;
    check_cuda(cudaMemGetInfo(&free_b, &c->total_mem), "cudaMemGetInfo");
  }
  check_cuda(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  for (int i = 0; i < 8; ++i)
    check_cuda(cudaStreamCreateWithFlags(&c->copy_streams[i], cudaStreamNonBlocking), "cudaStreamCreate");
  for (int i = 0; i < 9; ++i)
    check_cuda(cudaEventCreateWithFlags(&c->copy_events[i], cudaEventDisableTiming), "cudaEventCreate");
  c->stream = c->own_stream;
  c->sum_scratch = c->pool.alloc(sizeof(float2) * kMaxSumBlocks + 256, &c->sum_scratch_cls);
  check_cuda(cudaMemsetAsync(c->sum_scratch, 0, sizeof(float2) * kMaxSumBlocks + 256, c->stream), "cudaMemsetAsync");
  check_cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  g_ctx = c.release();
  CC_API_END
}

int cc_shutdown(void) {
  CC_API_BEGIN
  std::lock_guard<std::mutex> g(g_init_mu);
  Context *c = g_ctx;
  if (!c) return CC_OK;
  cudaSetDevice(c->device);
  g_drv.CtxSetCurrent(c->cuctx);
  cudaStreamSynchronize(c->stream);
  for (int i = 0; i < kQueues; ++i)
    if (c->queues[i]) cudaStreamSynchronize(c->queues[i]);
  c->multi_queue = false;  // every stream is idle: blocks go straight back to the pool
  for (auto &kv : c->programs) delete kv.second;
  c->modules.clear();
  c->tune_modules.clear();
  for (auto &kv : c->batches) {
    Batch *b = kv.second;
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->table) release_block(*c, b->table, b->table_cls);
    if (b->module) g_drv.ModuleUnload(b->module);
    delete b;
  }
  c->batches.clear();
  for (auto &kv : c->tune_sets) {
    if (kv.second->flush) release_block(*c, kv.second->flush, kv.second->flush_cls);
    delete kv.second;
  }
  c->tune_sets.clear();
  for (auto &kv : c->mlps) {
    if (kv.second->scratch) release_block(*c, kv.second->scratch, kv.second->scratch_cls);
    if (kv.second->state) release_block(*c, kv.second->state, kv.second->state_cls);
    delete kv.second;
  }
  c->mlps.clear();
  c->cost_model = 0;
  for (auto &kv : c->buffers) {
    cudaFree(kv.second->ptr);
    delete kv.second;
  }
  for (auto &kv : c->events) {
    if (!kv.second->fence) cudaEventDestroy(kv.second->ev);
    delete kv.second;
  }
  c->events.clear();
  release_block(*c, c->sum_scratch, c->sum_scratch_cls);
  for (int i = 0; i < kQueues; ++i)
    if (c->queue_scratch[i]) release_block(*c, c->queue_scratch[i], c->queue_scratch_cls[i]);
  c->pool.trim();
  for (cudaEvent_t ev : c->free_events) cudaEventDestroy(ev);
  c->free_events.clear();
  for (int i = 0; i < kQueues; ++i)
    if (c->queues[i]) cudaStreamDestroy(c->queues[i]);
  for (int i = 0; i < 8; ++i) cudaStreamDestroy(c->copy_streams[i]);
  for (int i = 0; i < 9; ++i) cudaEventDestroy(c->copy_events[i]);
  cudaStreamDestroy(c->own_stream);
  g_ctx = nullptr;
  delete c;
  CC_API_END
}

int cc_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *total_mem) {
  CC_API_BEGIN
  Context &c = ctx();
  if (sm_count) *sm_count = c.sm_count;
  if (cc_major) *cc_major = c.cc_major;
  if (cc_minor) *cc_minor = c.cc_minor;
  if (total_mem) *total_mem = c.total_mem;
  CC_API_END
}

int cc_get_stream(uint64_t *stream) {
  CC_API_BEGIN
  if (!stream) fail(CC_ERR_INVALID_VALUE, "null pointer");
  *stream = reinterpret_cast<uint64_t>(ctx().stream);
  CC_API_END
}

int cc_set_stream(uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  // Blocks freed so far may still be read by work on the old stream.
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  c.stream = stream ? reinterpret_cast<cudaStream_t>(stream) : c.own_stream;
  CC_API_END
}

int cc_config_set(const char *key, int64_t value) {
  CC_API_BEGIN
  if (!key) fail(CC_ERR_INVALID_VALUE, "null key");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  std::string k(key);
  if (k == "block") {
    if (value != 64 && value != 128 && value != 256) fail(CC_ERR_INVALID_VALUE, "block must be 64, 128 or 256");
    c.block = (int)value;
  } else if (k == "ew_blocks_per_sm") {
    if (value < 0 || value > 32) fail(CC_ERR_INVALID_VALUE, "ew_blocks_per_sm must be in [0, 32]");
    c.ew_blocks_per_sm = (int)value;
  } else if (k == "sum_blocks_per_sm") {
    if (value < 1 || (int64_t)c.sm_count * value > kMaxSumBlocks)
      fail(CC_ERR_INVALID_VALUE, "sum_blocks_per_sm out of range for the sum scratch");
    c.sum_blocks_per_sm = (int)value;
  } else if (k == "upload_streams") {
    if (value < 1 || value > 8) fail(CC_ERR_INVALID_VALUE, "upload_streams must be in [1, 8]");
    c.upload_streams = (int)value;
  } else if (k == "ew_lookahead") {
    if (value < 0 || value > 256) fail(CC_ERR_INVALID_VALUE, "ew_lookahead must be in [0, 256]");
    c.ew_lookahead = (int)value;
  } else if (k == "prefetch_min_bytes") {
    if (value < -1) fail(CC_ERR_INVALID_VALUE, "prefetch_min_bytes must be >= -1");
    c.prefetch_min_bytes = value;
  } else if (k == "sum_block") {
    if (value != 64 && value != 128 && value != 256) fail(CC_ERR_INVALID_VALUE, "sum_block must be 64, 128 or 256");
    c.sum_block = (int)value;
  } else if (k == "copy_kernel") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "copy_kernel must be 0 or 1");
    c.copy_kernel = (int)value;
  } else if (k == "tc_group_m") {
    if (value < 1 || value > 64) fail(CC_ERR_INVALID_VALUE, "tc_group_m must be in [1, 64]");
    c.tc_group_m = (int)value;
  } else if (k == "pdl") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "pdl must be 0, 1 or 2");
    c.pdl = (int)value;
    end_pdl_chain(c);
  } else if (k == "ew_batch_loads") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "ew_batch_loads must be 0 or 1");
    c.ew_batch_loads = (int)value;
  } else if (k == "ew_vector_loads") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "ew_vector_loads must be 0 or 1");
    c.ew_vector_loads = (int)value;
  } else if (k == "ew_points") {
    if (value < 1 || value > 16) fail(CC_ERR_INVALID_VALUE, "ew_points must be in [1, 16]");
    c.ew_points = (int)value;
  } else if (k == "ew_smem_ring") {
    if (value != 0 && (value < 4 || value > 64)) fail(CC_ERR_INVALID_VALUE, "ew_smem_ring must be 0 or in [4, 64]");
    c.ew_smem_ring = (int)value;
  } else if (k == "tuner") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "tuner must be 0 (off), 1 (exhaustive) or 2 (learned)");
    c.tuner = (int)value;
  } else if (k == "batch_run_tiles") {
    if (value < 1 || value > 4096) fail(CC_ERR_INVALID_VALUE, "batch_run_tiles must be in [1, 4096]");
    c.batch_run_tiles = (int)value;
  } else if (k == "batch_max_loads") {
    if (value != 1 && value != 2 && value != 4 && value != 8 && value != 16)
      fail(CC_ERR_INVALID_VALUE, "batch_max_loads must be 1, 2, 4, 8 or 16");
    c.batch_max_loads = (int)value;
  } else if (k == "batch_max_registers") {
    if (value < 0 || value > 255) fail(CC_ERR_INVALID_VALUE, "batch_max_registers must be in [0, 255]");
    c.batch_max_registers = (int)value;
  } else if (k == "batch_inline") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "batch_inline must be 0, 1 or 2");
    c.batch_inline = (int)value;
  } else if (k == "batch_copy_kernel") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "batch_copy_kernel must be 0 or 1");
    c.batch_copy_kernel = (int)value;
  } else if (k == "batch_rolled") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "batch_rolled must be 0 or 1");
    c.batch_rolled = (int)value;
  } else if (k == "batch_prefetch") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "batch_prefetch must be 0, 1 or 2");
    c.batch_prefetch = (int)value;
  } else if (k == "batch_lanes") {
    if (value != 0 && value != 4 && value != 8) fail(CC_ERR_INVALID_VALUE, "batch_lanes must be 0, 4 or 8");
    c.batch_lanes = (int)value;
  } else if (k == "row_fold_stages") {
    if (value != 0 && (value < 2 || value > 16)) fail(CC_ERR_INVALID_VALUE, "row_fold_stages must be 0 or in [2, 16]");
    c.row_fold_stages = (int)value;
  } else if (k == "row_fold") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "row_fold must be 0 or 1");
    c.row_fold = (int)value;
  } else if (k == "contraction") {
    if (value < 0 || value > 3) fail(CC_ERR_INVALID_VALUE, "contraction must be in [0, 3]");
    c.contraction = (int)value;
  } else if (k == "tc_variant") {
    if (value < 0 || value > 5) fail(CC_ERR_INVALID_VALUE, "tc_variant must be in [0, 5]");
    c.tc_variant = (int)value;
  } else if (k == "vec_unroll") {
    if (value < 1 || value > 8) fail(CC_ERR_INVALID_VALUE, "vec_unroll must be in [1, 8]");
    c.vec_unroll = (int)value;
  } else if (k == "ew_asm_loads") {
    if (value != 0 && value != 1) fail(CC_ERR_INVALID_VALUE, "ew_asm_loads must be 0 or 1");
    c.ew_asm_loads = (int)value;
  } else {
    fail(CC_ERR_INVALID_VALUE, "unknown config key '" + k + "'");
  }
  CC_API_END
}

int cc_config_get(const char *key, int64_t *value) {
  CC_API_BEGIN
  if (!key || !value) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  std::string k(key);
  if (k == "block") *value = c.block;
  else if (k == "ew_blocks_per_sm") *value = c.ew_blocks_per_sm;
  else if (k == "sum_blocks_per_sm") *value = c.sum_blocks_per_sm;
  else if (k == "upload_streams") *value = c.upload_streams;
  else if (k == "ew_lookahead") *value = c.ew_lookahead;
  else if (k == "ew_asm_loads") *value = c.ew_asm_loads;
  else if (k == "vec_unroll") *value = c.vec_unroll;
  else if (k == "prefetch_min_bytes") *value = c.prefetch_min_bytes;
  else if (k == "sum_block") *value = c.sum_block;
  else if (k == "tc_variant") *value = c.tc_variant;
  else if (k == "contraction") *value = c.contraction;
  else if (k == "row_fold") *value = c.row_fold;
  else if (k == "row_fold_stages") *value = c.row_fold_stages;
  else if (k == "batch_inline") *value = c.batch_inline;
  else if (k == "batch_lanes") *value = c.batch_lanes;
  else if (k == "batch_rolled") *value = c.batch_rolled;
  else if (k == "batch_prefetch") *value = c.batch_prefetch;
  else if (k == "batch_copy_kernel") *value = c.batch_copy_kernel;
  else if (k == "tuner") *value = c.tuner;
  else if (k == "ew_smem_ring") *value = c.ew_smem_ring;
  else if (k == "ew_points") *value = c.ew_points;
  else if (k == "ew_vector_loads") *value = c.ew_vector_loads;
  else if (k == "ew_batch_loads") *value = c.ew_batch_loads;
  else if (k == "pdl") *value = c.pdl;
  else if (k == "tc_group_m") *value = c.tc_group_m;
  else if (k == "copy_kernel") *value = c.copy_kernel;
  else if (k == "batch_max_registers") *value = c.batch_max_registers;
  else if (k == "batch_max_loads") *value = c.batch_max_loads;
  else if (k == "batch_run_tiles") *value = c.batch_run_tiles;
  else fail(CC_ERR_INVALID_VALUE, "unknown config key '" + k + "'");
  CC_API_END
}

int cc_synchronize(void) {
  CC_API_BEGIN
  Context &c = ctx();
  cudaStream_t s;
  bool multi;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    s = c.stream;
    multi = c.multi_queue;
  }
  check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  std::lock_guard<std::recursive_mutex> g(c.mu);
  bool deferred = false;
  if (multi) {
    for (int i = 0; i < kQueues; ++i) {
      check_cuda(cudaStreamSynchronize(c.queues[i]), "cudaStreamSynchronize");
      c.queue_dirty[i] = false;
    }
    deferred = true;
  }
  for (int i = 0; i < 8; ++i)
    if (c.copy_dirty[i]) {
      check_cuda(cudaStreamSynchronize(c.copy_streams[i]), "cudaStreamSynchronize");
      c.copy_dirty[i] = false;
      deferred = true;
    }
  if (deferred) c.pool.reclaim();
  CC_API_END
}

// ---------------------------------------------------------------- buffers

int cc_buf_alloc(size_t bytes, cc_handle *out) {
  CC_API_BEGIN
  if (!out) fail(CC_ERR_INVALID_VALUE, "null handle pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  auto b = std::make_unique<Buffer>();
  b->ptr = c.pool.alloc(bytes, &b->cls);
  b->bytes = bytes;
  uint64_t h = c.make_handle(kTagBuffer);
  c.buffers[h] = b.release();
  *out = h;
  CC_API_END
}

int cc_buf_retain(cc_handle h) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  buffer_of(c, h).refs++;
  CC_API_END
}

int cc_buf_release(cc_handle h) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Buffer &b = buffer_of(c, h);
  if (--b.refs == 0) {
    release_block(c, b.ptr, b.cls);
    delete &b;
    c.buffers.erase(h);
  }
  CC_API_END
}

int cc_buf_size(cc_handle h, size_t *bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (!bytes) fail(CC_ERR_INVALID_VALUE, "null pointer");
  *bytes = buffer_of(c, h).bytes;
  CC_API_END
}

int cc_buf_device_ptr(cc_handle h, uint64_t *ptr) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (!ptr) fail(CC_ERR_INVALID_VALUE, "null pointer");
  *ptr = reinterpret_cast<uint64_t>(buffer_of(c, h).ptr);
  CC_API_END
}

int cc_buf_upload(cc_handle h, size_t offset, const void *host, size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  void *dst;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    end_pdl_chain(c);
    Buffer &b = buffer_of(c, h);
    if (offset > b.bytes || bytes > b.bytes - offset) fail(CC_ERR_INVALID_VALUE, "upload range exceeds the buffer");
    dst = static_cast<char *>(b.ptr) + offset;
  }
  if (bytes == 0) return CC_OK;
  if (!host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  striped_upload(c, static_cast<char *>(dst), static_cast<const char *>(host), bytes);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  CC_API_END
}

int cc_buf_upload_async(cc_handle h, size_t offset, const void *host, size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  void *dst;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    end_pdl_chain(c);
    Buffer &b = buffer_of(c, h);
    if (offset > b.bytes || bytes > b.bytes - offset) fail(CC_ERR_INVALID_VALUE, "upload range exceeds the buffer");
    dst = static_cast<char *>(b.ptr) + offset;
  }
  if (bytes == 0) return CC_OK;
  if (!host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  striped_upload(c, static_cast<char *>(dst), static_cast<const char *>(host), bytes);
  CC_API_END
}

int cc_buf_download(cc_handle h, size_t offset, void *host, size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  void *src;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    end_pdl_chain(c);
    Buffer &b = buffer_of(c, h);
    if (offset > b.bytes || bytes > b.bytes - offset) fail(CC_ERR_INVALID_VALUE, "download range exceeds the buffer");
    src = static_cast<char *>(b.ptr) + offset;
  }
  if (bytes == 0) return CC_OK;
  if (!host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  if (!sm_copy(c, host, src, bytes, false))
    check_cuda(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, c.stream), "cudaMemcpyAsync D2H");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  CC_API_END
}

int cc_buf_download_async(cc_handle h, size_t offset, void *host, size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  void *src;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    end_pdl_chain(c);
    Buffer &b = buffer_of(c, h);
    if (offset > b.bytes || bytes > b.bytes - offset) fail(CC_ERR_INVALID_VALUE, "download range exceeds the buffer");
    src = static_cast<char *>(b.ptr) + offset;
  }
  if (bytes == 0) return CC_OK;
  if (!host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  if (!sm_copy(c, host, src, bytes, false))
    check_cuda(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, c.stream), "cudaMemcpyAsync D2H");
  CC_API_END
}

int cc_host_alloc(size_t bytes, void **host) {
  CC_API_BEGIN
  if (!host) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  check_cuda(cudaMallocHost(host, bytes ? bytes : 1), "cudaMallocHost");
  std::lock_guard<std::recursive_mutex> g(c.mu);
  c.pinned[reinterpret_cast<uintptr_t>(*host)] = bytes ? bytes : 1;
  CC_API_END
}

int cc_host_free(void *host) {
  CC_API_BEGIN
  Context &c = ctx();
  if (!host) return CC_OK;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    c.pinned.erase(reinterpret_cast<uintptr_t>(host));
    ++c.pinned_gen;
  }
  check_cuda(cudaFreeHost(host), "cudaFreeHost");
  CC_API_END
}

int cc_pool_stats(size_t *in_use, size_t *cached, uint64_t *allocs, uint64_t *reuses) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (in_use) *in_use = c.pool.in_use_;
  if (cached) *cached = c.pool.cached_;
  if (allocs) *allocs = c.pool.allocs_;
  if (reuses) *reuses = c.pool.reuses_;
  CC_API_END
}

int cc_pool_set_limit(size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  c.pool.limit_ = bytes;
  CC_API_END
}

int cc_pool_trim(void) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  c.pool.trim();
  CC_API_END
}

// ---------------------------------------------------------------- programs

}  // extern "C"

namespace {

// The standard kernels of a program (cc_ew / cc_ew_v4 / cc_ew_vl or cc_sum*),
// compiled and loaded; contiguous programs share one module per structure.
std::shared_ptr<Module> standard_module(Context &c, const Ir &ir, CodegenOptions opt, const std::string &key,
                                        Generated *gen_out) {
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  // Contiguous programs compile once per structure; the shape only sizes the launch.
  std::string skey = contiguous_structure_key(ir);
  if (!skey.empty()) {
    skey += key.substr(key.rfind('#'));
    opt.min_blocks = 0;
  } else {
    // threads, not points: a thread of a multi-point kernel takes several
    opt.min_blocks = choose_min_blocks(domain / points_for(ir, opt.points_per_thread), opt.block, c.sm_count,
                                       -opt.min_blocks);
  }
  std::shared_ptr<Module> mod;
  if (!skey.empty()) {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    auto it = c.modules.find(skey);
    if (it != c.modules.end()) mod = it->second;
  }
  if (mod) {
    (*gen_out) = describe_program(ir);
  } else {
    (*gen_out) = generate_cuda(ir, opt);
    mod = std::make_shared<Module>();
    mod->source = (*gen_out).source;
    std::vector<char> cubin = compile_cubin(mod->source, c.cc_major, c.cc_minor, c.flags);
    check_cu(g_drv.ModuleLoadData(&mod->module, cubin.data()), "cuModuleLoadData");
    const char *sname = ir.kind == ProgramKind::Sum ? "cc_sum" : "cc_ew";
    const char *vname = ir.kind == ProgramKind::Sum ? "cc_sum_v4" : "cc_ew_v4";
    check_cu(g_drv.ModuleGetFunction(&mod->scalar, mod->module, sname), "cuModuleGetFunction");
    if ((*gen_out).has_vec4) check_cu(g_drv.ModuleGetFunction(&mod->vec4, mod->module, vname), "cuModuleGetFunction");
    if ((*gen_out).has_vl)
      check_cu(g_drv.ModuleGetFunction(&mod->vl, mod->module, ir.kind == ProgramKind::Sum ? "cc_sum_vl" : "cc_ew_vl"),
               "cuModuleGetFunction");
    mod->block = opt.block;
    mod->vec_unroll = (*gen_out).vec_unroll;
    mod->smem_bytes = (*gen_out).smem_bytes;
    mod->points = (*gen_out).points_per_thread;
    if (mod->smem_bytes > 48 * 1024)
      check_cu(g_drv.FuncSetAttribute(mod->scalar, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, mod->smem_bytes),
               "cuFuncSetAttribute");
    check_cu(g_drv.OccupancyMaxActiveBlocks(&mod->resident_scalar, mod->scalar, mod->block, mod->smem_bytes),
             "cuOccupancyMaxActiveBlocks");
    if (mod->vec4)
      check_cu(g_drv.OccupancyMaxActiveBlocks(&mod->resident_vec4, mod->vec4, mod->block, 0),
               "cuOccupancyMaxActiveBlocks");
    if (mod->vl)
      check_cu(g_drv.OccupancyMaxActiveBlocks(&mod->resident_vl, mod->vl, mod->block, 0),
               "cuOccupancyMaxActiveBlocks");
    if (!skey.empty()) {
      std::lock_guard<std::recursive_mutex> g(c.mu);
      c.modules[skey] = mod;
    }
  }
  return mod;
}

}  // namespace

extern "C" {

int cc_program_get(const char *ir_text, size_t ir_len, cc_handle *out) {
  CC_API_BEGIN
  if (!ir_text || !out) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::string key(ir_text, ir_len);
  CodegenOptions opt;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    opt.load_lookahead = c.ew_lookahead;
    opt.asm_loads = c.ew_asm_loads != 0;
    opt.min_blocks = -c.ew_blocks_per_sm;  // resolved below, once the domain is known
    opt.block = c.block;
    opt.vec_unroll = c.vec_unroll;
    opt.prefetch_min_bytes = c.prefetch_min_bytes;
    opt.smem_ring = c.ew_smem_ring;
    opt.points_per_thread = c.ew_points;
    opt.vector_loads = c.ew_vector_loads != 0;
    opt.batch_loads = c.ew_batch_loads != 0;
  }
  key += "#lookahead " + std::to_string(opt.load_lookahead) + " asm " + std::to_string((int)opt.asm_loads) +
         " blocks " + std::to_string(-opt.min_blocks) + " block " + std::to_string(opt.block) + " unroll " + std::to_string(opt.vec_unroll) +
         " prefetch " + std::to_string(opt.prefetch_min_bytes) + " ring " + std::to_string(opt.smem_ring) + " points " + std::to_string(opt.points_per_thread) + " vl " + std::to_string((int)opt.vector_loads) + " bl " + std::to_string((int)opt.batch_loads) +
         " sumblock " + std::to_string(c.sum_block) +
         " contraction " + std::to_string(c.contraction) + " rowfold " + std::to_string(c.row_fold) + "/" + std::to_string(c.row_fold_stages) +
         " tc " + std::to_string(c.tc_variant) + " tuner " +
         std::to_string(c.tuner) + " flags " + std::to_string(c.flags) + "\n";
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    auto it = c.cache.find(key);
    if (it != c.cache.end()) {
      ++c.cache_hits;
      *out = it->second;
      return CC_OK;
    }
  }
  std::lock_guard<std::mutex> cg(c.compile_mu);
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    auto it = c.cache.find(key);
    if (it != c.cache.end()) {
      ++c.cache_hits;
      *out = it->second;
      return CC_OK;
    }
  }
  Ir ir = parse_ir(ir_text, ir_len);
  if (ir.kind == ProgramKind::Sum) opt.block = c.sum_block;
  FmaScope fma_scope((c.flags & CC_FLAG_FMA_CONTRACT) != 0);
  Contraction con;
  int contraction_knob;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    contraction_knob = c.contraction;
  }
  if (contraction_knob > 0 && match_contraction(ir, &con)) {
    auto p = std::make_unique<Program>();
    p->kind = ProgramKind::Elementwise;
    p->is_contraction = true;
    p->contraction_mode = contraction_knob - 1;
    p->con = con;
    p->gen.n_inputs = ir.n_params;
    p->gen.out_elems = con.m * con.n;
    p->gen.domain = con.m * con.n;
    p->gen.source = "// contraction: C[" + std::to_string(con.m) + "," + std::to_string(con.n) + "] = A * B over " +
                    std::to_string(con.k) + " terms, cc_gemm_f32 mode " + std::to_string(p->contraction_mode) + "\n";
    std::lock_guard<std::recursive_mutex> g(c.mu);
    uint64_t h = c.make_handle(kTagProgram);
    c.programs[h] = p.release();
    c.cache[key] = h;
    ++c.cache_misses;
    *out = h;
    return CC_OK;
  }
  int row_fold_knob;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    row_fold_knob = c.row_fold;
  }
  RowFold rf;
  if (row_fold_knob && match_row_fold(ir, &rf)) {
    {
      std::lock_guard<std::recursive_mutex> g(c.mu);
      rf.stages = c.row_fold_stages;
    }
    auto p = std::make_unique<Program>();
    p->kind = ProgramKind::Elementwise;
    p->gen = describe_program(ir);
    p->is_row_fold = true;
    p->rf = rf;
    auto mod = std::make_shared<Module>();
    mod->source = row_fold_source(ir, rf);
    std::vector<char> cubin = compile_cubin(mod->source, c.cc_major, c.cc_minor, c.flags);
    check_cu(g_drv.ModuleLoadData(&mod->module, cubin.data()), "cuModuleLoadData");
    check_cu(g_drv.ModuleGetFunction(&p->rf_tma, mod->module, "cc_rowfold"), "cuModuleGetFunction");
    check_cu(g_drv.ModuleGetFunction(&p->rf_plain, mod->module, "cc_rowfold_plain"), "cuModuleGetFunction");
    check_cu(g_drv.FuncSetAttribute(p->rf_tma, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                    row_fold_smem_bytes((int)rf.row_inputs.size(),
                                                        row_fold_stages((int)rf.row_inputs.size(), rf.stages))),
             "cuFuncSetAttribute");
    p->mod = mod;
    std::lock_guard<std::recursive_mutex> g(c.mu);
    uint64_t h = c.make_handle(kTagProgram);
    c.programs[h] = p.release();
    c.cache[key] = h;
    ++c.cache_misses;
    *out = h;
    return CC_OK;
  }
  int tuner_mode;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    tuner_mode = c.tuner;
  }
  if (tuner_mode > 0 && is_tunable(ir, nullptr)) {
    // The tunable form and the standard kernels; the tuner picks among the
    // tunable configurations and the standard kernel at the first launch.
    auto p = std::make_unique<Program>();
    p->kind = ir.kind;
    // contiguous programs share one tunable module per structure (the length is an argument)
    std::string tkey = contiguous_structure_key(ir);
    std::shared_ptr<TuneModule> tmod;
    if (!tkey.empty()) {
      tkey += "#tunable flags " + std::to_string(c.flags);
      std::lock_guard<std::recursive_mutex> g(c.mu);
      auto it = c.tune_modules.find(tkey);
      if (it != c.tune_modules.end()) tmod = it->second;
    }
    if (!tmod) {
      const std::string tunable = std::string("// generated by compute.scala_gb300 for sm_103a (tunable form)\n") +
                                  kPrelude + "\n" + tunable_source(ir, "");
      tmod = load_tune_module(compile_cubin(tunable, c.cc_major, c.cc_minor, c.flags));
      if (!tkey.empty()) {
        std::lock_guard<std::recursive_mutex> g(c.mu);
        c.tune_modules[tkey] = tmod;
      }
    }
    p->tune = std::make_unique<TuneEntry>();
    load_tune_entry(*p->tune, ir, tmod, "");
    p->mod = standard_module(c, ir, opt, key, &p->gen);
    std::lock_guard<std::recursive_mutex> g(c.mu);
    uint64_t h = c.make_handle(kTagProgram);
    c.programs[h] = p.release();
    c.cache[key] = h;
    ++c.cache_misses;
    *out = h;
    return CC_OK;
  }
  auto p = std::make_unique<Program>();
  p->kind = ir.kind;
  p->mod = standard_module(c, ir, opt, key, &p->gen);
  std::lock_guard<std::recursive_mutex> g(c.mu);
  uint64_t h = c.make_handle(kTagProgram);
  c.programs[h] = p.release();
  c.cache[key] = h;
  ++c.cache_misses;
  *out = h;
  CC_API_END
}

namespace {
// "block=128 lookahead=8 ring=32 unroll=4 min_blocks=11 asm=1" (any subset; NULL = defaults).
// "rowfold=0" generates an inner-axis fold as the generic fold (default 1: the skeleton).
CodegenOptions parse_codegen_options(const char *text, bool *row_fold = nullptr, bool *fma = nullptr) {
  CodegenOptions o;
  if (row_fold) *row_fold = true;
  if (fma) *fma = false;
  if (!text) return o;
  std::istringstream in(text);
  std::string item;
  while (in >> item) {
    size_t eq = item.find('=');
    if (eq == std::string::npos) fail(CC_ERR_INVALID_VALUE, "option '" + item + "' is not key=value");
    std::string k = item.substr(0, eq);
    long long v = std::strtoll(item.c_str() + eq + 1, nullptr, 10);
    if (k == "block") o.block = (int)v;
    else if (k == "lookahead") o.load_lookahead = (int)v;
    else if (k == "ring") o.smem_ring = (int)v;
    else if (k == "unroll") o.vec_unroll = (int)v;
    else if (k == "min_blocks") o.min_blocks = (int)v;
    else if (k == "asm") o.asm_loads = v != 0;
    else if (k == "points") o.points_per_thread = (int)v;
    else if (k == "vl") o.vector_loads = v != 0;
    else if (k == "batch") o.batch_loads = v != 0;
    else if (k == "rowfold") {
      if (row_fold) *row_fold = v != 0;
    } else if (k == "fma") {
      if (fma) *fma = v != 0;
    } else fail(CC_ERR_INVALID_VALUE, "unknown code-generation option '" + k + "'");
  }
  return o;
}
}  // namespace

int cc_codegen(const char *ir_text, size_t ir_len, char *buf, size_t len, size_t *needed) {
  return cc_codegen_with(ir_text, ir_len, nullptr, buf, len, needed);
}

int cc_codegen_with(const char *ir_text, size_t ir_len, const char *options, char *buf, size_t len, size_t *needed) {
  CC_API_BEGIN
  if (!ir_text) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Ir ir = parse_ir(ir_text, ir_len);
  bool row_fold = true, fma = false;
  CodegenOptions opt = parse_codegen_options(options, &row_fold, &fma);
  FmaScope fma_scope(fma);
  RowFold rf;
  Generated gen;
  if (row_fold && match_row_fold(ir, &rf))
    gen.source = row_fold_source(ir, rf);
  else
    gen = generate_cuda(ir, opt);
  Contraction con;
  if (match_contraction(ir, &con))
    gen.source = "// contraction m=" + std::to_string(con.m) + " n=" + std::to_string(con.n) + " k=" +
                 std::to_string(con.k) + " a=" + std::to_string(con.a_input) + " b=" + std::to_string(con.b_input) +
                 "\n" + gen.source;
  if (needed) *needed = gen.source.size() + 1;
  if (buf && len) {
    size_t n = gen.source.size() < len - 1 ? gen.source.size() : len - 1;
    memcpy(buf, gen.source.data(), n);
    buf[n] = '\0';
  }
  CC_API_END
}

int cc_compile_check(const char *ir_text, size_t ir_len, int cc_major, int cc_minor, uint32_t flags) {
  return cc_compile_check_with(ir_text, ir_len, cc_major, cc_minor, flags, nullptr);
}

int cc_compile_check_with(const char *ir_text, size_t ir_len, int cc_major, int cc_minor, uint32_t flags,
                          const char *options) {
  CC_API_BEGIN
  if (!ir_text) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Ir ir = parse_ir(ir_text, ir_len);
  bool row_fold = true, fma = false;
  CodegenOptions opt = parse_codegen_options(options, &row_fold, &fma);
  FmaScope fma_scope(fma || (flags & CC_FLAG_FMA_CONTRACT) != 0);
  RowFold rf;
  if (row_fold && match_row_fold(ir, &rf))
    compile_cubin(row_fold_source(ir, rf), cc_major, cc_minor, flags);
  else
    compile_cubin(generate_cuda(ir, opt).source, cc_major, cc_minor, flags);
  CC_API_END
}

int cc_program_info(cc_handle h, int *kind, int *n_inputs, int64_t *out_elems, int *tuple_len) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, h);
  if (kind) *kind = (int)p.kind;
  if (n_inputs) *n_inputs = p.gen.n_inputs;
  if (out_elems) *out_elems = p.gen.out_elems;
  if (tuple_len) *tuple_len = p.gen.tuple_len;
  CC_API_END
}

int cc_program_source(cc_handle h, char *buf, size_t len, size_t *needed) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, h);
  const std::string &s = p.mod ? p.mod->source : p.gen.source;
  if (needed) *needed = s.size() + 1;
  if (buf && len) {
    size_t n = s.size() < len - 1 ? s.size() : len - 1;
    memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  CC_API_END
}

int cc_program_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *entries) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  if (hits) *hits = c.cache_hits;
  if (misses) *misses = c.cache_misses;
  if (entries) *entries = c.cache.size();
  CC_API_END
}

int cc_launch(cc_handle prog, const cc_handle *inputs, int n_inputs, cc_handle output) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, prog);
  if (n_inputs != p.gen.n_inputs)
    fail(CC_ERR_INVALID_KERNEL_ARGS, "program takes " + std::to_string(p.gen.n_inputs) + " inputs, got " +
                                         std::to_string(n_inputs));
  std::vector<uint64_t> ptrs;
  for (int i = 0; i < n_inputs; ++i) {
    Buffer &b = buffer_of(c, inputs[i]);
    ptrs.push_back(reinterpret_cast<uint64_t>(b.ptr));
  }
  Buffer &o = buffer_of(c, output);
  if (o.bytes < (size_t)p.gen.out_elems * sizeof(float))
    fail(CC_ERR_INVALID_VALUE, "output buffer holds " + std::to_string(o.bytes) + " bytes, the program writes " +
                                   std::to_string(p.gen.out_elems * sizeof(float)));
  launch_program(c, p, ptrs, reinterpret_cast<uint64_t>(o.ptr), c.stream);
  CC_API_END
}

int cc_launch_ptrs(cc_handle prog, const uint64_t *input_ptrs, int n_inputs, uint64_t output_ptr, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, prog);
  if (n_inputs != p.gen.n_inputs) fail(CC_ERR_INVALID_KERNEL_ARGS, "wrong number of inputs");
  if (!output_ptr || (n_inputs && !input_ptrs)) fail(CC_ERR_INVALID_VALUE, "null pointer");
  std::vector<uint64_t> ptrs(input_ptrs, input_ptrs + n_inputs);
  for (uint64_t q : ptrs)
    if (!q) fail(CC_ERR_INVALID_VALUE, "null input pointer");
  launch_program(c, p, ptrs, output_ptr, stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream);
  CC_API_END
}

// ---------------------------------------------------------------- the asynchronous DAG

int cc_launch_ev(cc_handle prog, const cc_handle *inputs, int n_inputs, cc_handle output, const cc_handle *wait,
                 int n_wait, cc_handle *event) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, prog);
  if (n_inputs != p.gen.n_inputs)
    fail(CC_ERR_INVALID_KERNEL_ARGS, "program takes " + std::to_string(p.gen.n_inputs) + " inputs, got " +
                                         std::to_string(n_inputs));
  if (n_inputs > 0 && !inputs) fail(CC_ERR_INVALID_VALUE, "null input list");
  std::vector<uint64_t> ptrs;
  for (int i = 0; i < n_inputs; ++i) ptrs.push_back(reinterpret_cast<uint64_t>(buffer_of(c, inputs[i]).ptr));
  Buffer &o = buffer_of(c, output);
  if (o.bytes < (size_t)p.gen.out_elems * sizeof(float))
    fail(CC_ERR_INVALID_VALUE, "output buffer holds " + std::to_string(o.bytes) + " bytes, the program writes " +
                                   std::to_string(p.gen.out_elems * sizeof(float)));
  if (n_wait < 0 || (n_wait > 0 && !wait)) fail(CC_ERR_INVALID_VALUE, "bad wait list");
  for (int i = 0; i < n_wait; ++i) event_of(c, wait[i]);  // every handle valid before anything is enqueued
  const int q = pick_queue(c);
  cudaStream_t s = c.queues[q];
  c.queue_dirty[q] = true;
  wait_events(c, s, wait, n_wait);
  launch_program(c, p, ptrs, reinterpret_cast<uint64_t>(o.ptr), s);
  if (event) *event = fence_handle(c, record_fence(c, s));
  CC_API_END
}

namespace {
int copy_ev(cc_handle h, size_t offset, void *host, size_t bytes, bool to_device, const cc_handle *wait, int n_wait,
            cc_handle *event) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Buffer &b = buffer_of(c, h);
  if (offset > b.bytes || bytes > b.bytes - offset)
    fail(CC_ERR_INVALID_VALUE, to_device ? "upload range exceeds the buffer" : "download range exceeds the buffer");
  if (bytes && !host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  if (n_wait < 0 || (n_wait > 0 && !wait)) fail(CC_ERR_INVALID_VALUE, "bad wait list");
  for (int i = 0; i < n_wait; ++i) event_of(c, wait[i]);
  const int q = pick_queue(c);
  cudaStream_t s = c.queues[q];
  c.queue_dirty[q] = true;
  wait_events(c, s, wait, n_wait);
  char *dev = static_cast<char *>(b.ptr) + offset;
  if (bytes)
    check_cuda(cudaMemcpyAsync(to_device ? static_cast<void *>(dev) : host, to_device ? static_cast<const void *>(host) : dev,
                               bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s),
               to_device ? "cudaMemcpyAsync H2D" : "cudaMemcpyAsync D2H");
  if (event) *event = fence_handle(c, record_fence(c, s));
  CC_API_END
}
}  // namespace

int cc_buf_upload_ev(cc_handle buf, size_t offset, const void *host, size_t bytes, const cc_handle *wait, int n_wait,
                     cc_handle *event) {
  return copy_ev(buf, offset, const_cast<void *>(host), bytes, true, wait, n_wait, event);
}

int cc_buf_download_ev(cc_handle buf, size_t offset, void *host, size_t bytes, const cc_handle *wait, int n_wait,
                       cc_handle *event) {
  return copy_ev(buf, offset, host, bytes, false, wait, n_wait, event);
}

int cc_stream_wait_events(const cc_handle *events, int n_events) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  wait_events(c, c.stream, events, n_events);
  CC_API_END
}

// ---------------------------------------------------------------- sums and random numbers

int cc_reduce_sum_f32(uint64_t in_ptr, size_t n, uint64_t out_ptr, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  if (!out_ptr || (n && !in_ptr)) fail(CC_ERR_INVALID_VALUE, "null pointer");
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  // Scratch for this call from the pool: partials, then the zeroed counter.
  size_t cls = 0;
  const size_t bytes = sizeof(float2) * kMaxSumBlocks + 256;
  void *scratch = c.pool.alloc(bytes, &cls);
  auto *partials = reinterpret_cast<float2 *>(scratch);
  auto *counter = reinterpret_cast<unsigned int *>(static_cast<char *>(scratch) + sizeof(float2) * kMaxSumBlocks);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess)
    e = launch_sum(reinterpret_cast<const float *>(in_ptr), (long long)n, partials, counter,
                   reinterpret_cast<float *>(out_ptr), c.sm_count, s);
  // blocks of the pool are ordered on the context stream and the queues; wait for other streams
  if (s != c.stream && queue_index(c, s) < 0 && e == cudaSuccess) e = cudaStreamSynchronize(s);
  release_block(c, scratch, cls);
  check_cuda(e, "sum launch");
  CC_API_END
}

int cc_gemm_f32(uint64_t a_ptr, uint64_t b_ptr, uint64_t c_ptr, int m, int n, int k, int64_t lda, int64_t ldb,
                int64_t ldc, int mode, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  if (!a_ptr || !b_ptr || !c_ptr) fail(CC_ERR_INVALID_VALUE, "null pointer");
  if (m < 0 || n < 0 || k <= 0 || lda < k || ldb < n || ldc < n) fail(CC_ERR_INVALID_VALUE, "bad matrix shape");
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  run_gemm(c, reinterpret_cast<const float *>(a_ptr), reinterpret_cast<const float *>(b_ptr),
           reinterpret_cast<float *>(c_ptr), m, n, k, lda, ldb, ldc, mode, s);
  CC_API_END
}

int cc_probe_bounded_wait(uint64_t limit_ns, int flag_value) {
  CC_API_BEGIN
  if (limit_ns > 10000000000ull) fail(CC_ERR_INVALID_VALUE, "limit_ns above 10 s");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  check_cuda(cudaMemsetAsync(c.probe_flag(), flag_value ? 1 : 0, sizeof(int), c.stream), "set probe flag");
  check_cuda(launch_flag_wait(c.probe_flag(), limit_ns, c.error_flag(), CC_DEVICE_ERR_PROBE_TIMEOUT, c.stream),
             "probe launch");
  CC_API_END
}

int cc_device_errors(int *code) {
  CC_API_BEGIN
  if (!code) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  int v = 0;
  check_cuda(cudaMemcpyAsync(&v, c.error_flag(), sizeof(int), cudaMemcpyDeviceToHost, c.stream), "read error flag");
  check_cuda(cudaMemsetAsync(c.error_flag(), 0, sizeof(int), c.stream), "clear error flag");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  *code = v;
  CC_API_END
}

int cc_random(cc_handle output, size_t n, uint32_t seed, int normal) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Buffer &b = buffer_of(c, output);
  size_t need = normal ? ((n + 1) / 2) * 2 : n;
  if (b.bytes < need * sizeof(float)) fail(CC_ERR_INVALID_VALUE, "output buffer too small for the random numbers");
  check_cuda(launch_random(static_cast<float *>(b.ptr), (long long)n, seed, normal, c.sm_count, c.stream),
             "random launch");
  CC_API_END
}

// ---------------------------------------------------------------- events

int cc_event_record(cc_handle *out) {
  CC_API_BEGIN
  if (!out) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  auto e = std::make_unique<Event>();
  check_cuda(cudaEventCreate(&e->ev), "cudaEventCreate");
  cudaError_t r = cudaEventRecord(e->ev, c.stream);
  if (r != cudaSuccess) {
    cudaEventDestroy(e->ev);
    check_cuda(r, "cudaEventRecord");
  }
  uint64_t h = c.make_handle(kTagEvent);
  c.events[h] = e.release();
  *out = h;
  CC_API_END
}

int cc_event_query(cc_handle h, int *complete) {
  CC_API_BEGIN
  Context &c = ctx();
  cudaEvent_t ev;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    ev = event_of(c, h).ev;
  }
  cudaError_t r = cudaEventQuery(ev);
  if (r == cudaErrorNotReady) {
    if (complete) *complete = 0;
    return CC_OK;
  }
  check_cuda(r, "cudaEventQuery");
  if (complete) *complete = 1;
  CC_API_END
}

int cc_event_wait(cc_handle h, uint64_t timeout_ns) {
  CC_API_BEGIN
  Context &c = ctx();
  cudaEvent_t ev;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    ev = event_of(c, h).ev;
  }
  auto t0 = std::chrono::steady_clock::now();
  int spin = 0;
  for (;;) {
    cudaError_t r = cudaEventQuery(ev);
    if (r == cudaSuccess) return CC_OK;
    if (r != cudaErrorNotReady) check_cuda(r, "cudaEventQuery");
    auto dt = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    if ((uint64_t)dt >= timeout_ns) fail(CC_ERR_TIMEOUT, "event not complete after " + std::to_string(timeout_ns) + " ns");
    if (++spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  CC_API_END
}

int cc_event_elapsed(cc_handle start, cc_handle end, float *ms) {
  CC_API_BEGIN
  if (!ms) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  check_cuda(cudaEventElapsedTime(ms, event_of(c, start).ev, event_of(c, end).ev), "cudaEventElapsedTime");
  CC_API_END
}

int cc_event_release(cc_handle h) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Event &e = event_of(c, h);
  if (!e.fence) cudaEventDestroy(e.ev);  // a fence's event goes back to the free list with the fence
  delete &e;
  c.events.erase(h);
  CC_API_END
}

}  // extern "C"

// ---------------------------------------------------------------- batches
//
// A batch evaluates many independent elementwise programs of uneven lengths.
// The reference launches one kernel per tensor (Tensors.scala:1331-1381) and
// leans on five queues per device for concurrency; here one persistent kernel
// walks all programs' tiles, with the per-program launches (and a CUDA graph
// of them) kept as the comparison and for callers that want them.

namespace cc {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kBatchUnroll = 4;
constexpr int64_t kBatchTile = (int64_t)kBatchBlock * 4 * kBatchUnroll;  // floats per tile (4096)


// The device table entry; must match the struct in the generated module.
struct BatchEntry {
  uint64_t in[kBatchMaxInputs];
  uint64_t out;
  int64_t n;
  int64_t tile_begin;
  int32_t sid;
  int32_t pad;
};
static_assert(sizeof(BatchEntry) == 64, "batch entry layout");

// A batch module is linked from separately compiled parts, because compile
// time grows faster than linearly with the size of one NVRTC program:
//   - chunk units: for kBatchChunk structures each, the structure's expression
//     (a real function), a tile function walking one tile of that structure
//     one float4 per thread at a time, and the structure's own kernel;
//   - the main unit: a device table of the tile functions and the persistent
//     kernel, which finds a tile's program by binary search and calls its tile
//     function through the table.
// The parts compile in parallel (relocatable code) and the CUDA driver API links them (cuLink*).
constexpr int kBatchChunk = 32;

// A tile function evaluates `count` consecutive tiles of one program from `base`.
const char *kTileParams =
    "(const float *__restrict__ in0, const float *__restrict__ in1, const float *__restrict__ in2, "
    "const float *__restrict__ in3, float *__restrict__ out, long long n, long long base, int count)";

// inline_level: 0 = the expression is a called function and so are exp/log/tanh;
// 1 = the expression is inlined into its tile function, exp/log/tanh called;
// 2 = everything inlined.  Higher levels run faster and compile slower.
//
// lanes (0, 4 or 8): the expression is evaluated on several points at once,
// a float4 (4) or two float4 positions (8), as a template over the value type
// (cc_f4, cc_f8; float for the ragged end), so a called exp/log/tanh computes
// 4 or 8 independent values per call.  Each lane runs the same scalar
// operation as the one-lane form (same functions, same rounding), so the
// results are identical bit for bit.
const char *kBatchLanePrelude = R"(namespace {
struct cc_f4 {
  float x, y, z, w;
  __device__ __forceinline__ cc_f4() {}
  __device__ __forceinline__ cc_f4(float s) : x(s), y(s), z(s), w(s) {}
  __device__ __forceinline__ cc_f4(float4 v) : x(v.x), y(v.y), z(v.z), w(v.w) {}
  __device__ __forceinline__ float4 f4() const { return make_float4(x, y, z, w); }
};
__device__ __forceinline__ cc_f4 operator+(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = a.x + b.x; r.y = a.y + b.y; r.z = a.z + b.z; r.w = a.w + b.w; return r; }
__device__ __forceinline__ cc_f4 operator-(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = a.x - b.x; r.y = a.y - b.y; r.z = a.z - b.z; r.w = a.w - b.w; return r; }
__device__ __forceinline__ cc_f4 operator*(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = a.x * b.x; r.y = a.y * b.y; r.z = a.z * b.z; r.w = a.w * b.w; return r; }
__device__ __forceinline__ cc_f4 operator/(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = a.x / b.x; r.y = a.y / b.y; r.z = a.z / b.z; r.w = a.w / b.w; return r; }
__device__ __forceinline__ cc_f4 operator-(cc_f4 a) { cc_f4 r; r.x = -a.x; r.y = -a.y; r.z = -a.z; r.w = -a.w; return r; }
__device__ __forceinline__ float cc_abs(float a) { return fabsf(a); }
__device__ __forceinline__ float cc_sqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ float cc_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float cc_mod(float a, float b) { return fmodf(a, b); }
__device__ __forceinline__ float cc_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float cc_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ cc_f4 cc_abs(cc_f4 a) { cc_f4 r; r.x = fabsf(a.x); r.y = fabsf(a.y); r.z = fabsf(a.z); r.w = fabsf(a.w); return r; }
__device__ __forceinline__ cc_f4 cc_sqrt(cc_f4 a) { cc_f4 r; r.x = sqrtf(a.x); r.y = sqrtf(a.y); r.z = sqrtf(a.z); r.w = sqrtf(a.w); return r; }
__device__ __forceinline__ cc_f4 cc_fma(cc_f4 a, cc_f4 b, cc_f4 c) {
  cc_f4 r; r.x = __fmaf_rn(a.x, b.x, c.x); r.y = __fmaf_rn(a.y, b.y, c.y); r.z = __fmaf_rn(a.z, b.z, c.z); r.w = __fmaf_rn(a.w, b.w, c.w); return r;
}
__device__ __forceinline__ cc_f4 cc_mod(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = fmodf(a.x, b.x); r.y = fmodf(a.y, b.y); r.z = fmodf(a.z, b.z); r.w = fmodf(a.w, b.w); return r; }
__device__ __forceinline__ cc_f4 cc_min(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = fminf(a.x, b.x); r.y = fminf(a.y, b.y); r.z = fminf(a.z, b.z); r.w = fminf(a.w, b.w); return r; }
__device__ __forceinline__ cc_f4 cc_max(cc_f4 a, cc_f4 b) { cc_f4 r; r.x = fmaxf(a.x, b.x); r.y = fmaxf(a.y, b.y); r.z = fmaxf(a.z, b.z); r.w = fmaxf(a.w, b.w); return r; }
struct cc_f8 {
  cc_f4 lo, hi;
  __device__ __forceinline__ cc_f8() {}
  __device__ __forceinline__ cc_f8(float s) : lo(s), hi(s) {}
  __device__ __forceinline__ cc_f8(float4 a, float4 b) : lo(a), hi(b) {}
};
__device__ __forceinline__ cc_f8 cc_pair(cc_f4 lo, cc_f4 hi) { cc_f8 r; r.lo = lo; r.hi = hi; return r; }
__device__ __forceinline__ cc_f8 operator+(cc_f8 a, cc_f8 b) { return cc_pair(a.lo + b.lo, a.hi + b.hi); }
__device__ __forceinline__ cc_f8 operator-(cc_f8 a, cc_f8 b) { return cc_pair(a.lo - b.lo, a.hi - b.hi); }
__device__ __forceinline__ cc_f8 operator*(cc_f8 a, cc_f8 b) { return cc_pair(a.lo * b.lo, a.hi * b.hi); }
__device__ __forceinline__ cc_f8 operator/(cc_f8 a, cc_f8 b) { return cc_pair(a.lo / b.lo, a.hi / b.hi); }
__device__ __forceinline__ cc_f8 operator-(cc_f8 a) { return cc_pair(-a.lo, -a.hi); }
__device__ __forceinline__ cc_f8 cc_abs(cc_f8 a) { return cc_pair(cc_abs(a.lo), cc_abs(a.hi)); }
__device__ __forceinline__ cc_f8 cc_sqrt(cc_f8 a) { return cc_pair(cc_sqrt(a.lo), cc_sqrt(a.hi)); }
__device__ __forceinline__ cc_f8 cc_fma(cc_f8 a, cc_f8 b, cc_f8 c) { return cc_pair(cc_fma(a.lo, b.lo, c.lo), cc_fma(a.hi, b.hi, c.hi)); }
__device__ __forceinline__ cc_f8 cc_mod(cc_f8 a, cc_f8 b) { return cc_pair(cc_mod(a.lo, b.lo), cc_mod(a.hi, b.hi)); }
__device__ __forceinline__ cc_f8 cc_min(cc_f8 a, cc_f8 b) { return cc_pair(cc_min(a.lo, b.lo), cc_min(a.hi, b.hi)); }
__device__ __forceinline__ cc_f8 cc_max(cc_f8 a, cc_f8 b) { return cc_pair(cc_max(a.lo, b.lo), cc_max(a.hi, b.hi)); }
)";

// L2 bulk prefetch of [p, p + bytes): p 16-byte aligned, bytes a multiple of 16.
const char *kBatchPrefetchPrelude =
    "static __device__ __forceinline__ void cc_l2_prefetch(const float *p, unsigned bytes) {\n"
    "  asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], %1;\" ::\"l\"(p), \"r\"(bytes) : \"memory\");\n"
    "}\n";

// exp, log and tanh over one lane and over four: called functions (shared by
// every structure of the part) below inline level 2, else inlined.
std::string batch_lane_transcendentals(int inline_level) {
  std::ostringstream o;
  const char *fq = inline_level >= 2 ? "__forceinline__" : "__noinline__";
  for (const char *f : {"exp", "log", "tanh"}) {
    const std::string F = std::string(f) + "f(";
    o << "__device__ " << fq << " float cc_" << f << "(float a) { return " << F << "a); }\n"
      << "__device__ " << fq << " cc_f4 cc_" << f << "(cc_f4 a) { cc_f4 r; r.x = " << F << "a.x); r.y = " << F
      << "a.y); r.z = " << F << "a.z); r.w = " << F << "a.w); return r; }\n"
      << "__device__ " << fq << " cc_f8 cc_" << f << "(cc_f8 a) { cc_f8 r; r.lo.x = " << F << "a.lo.x); r.lo.y = "
      << F << "a.lo.y); r.lo.z = " << F << "a.lo.z); r.lo.w = " << F << "a.lo.w); r.hi.x = " << F
      << "a.hi.x); r.hi.y = " << F << "a.hi.y); r.hi.z = " << F << "a.hi.z); r.hi.w = " << F
      << "a.hi.w); return r; }\n";
  }
  return o.str();
}

std::string batch_chunk_source(const std::vector<Ir> &structs, const std::vector<int> &struct_inputs, size_t first,
                               size_t last, int inline_level, int max_loads, int lane_width, bool rolled,
                               int prefetch) {
  const bool lanes = lane_width > 0;
  std::ostringstream o;
  o << "// generated batch part for sm_103a\n"
    << kBatchPrefetchPrelude
    << "static __device__ __noinline__ float cc_expf(float x) { return expf(x); }\n"
       "static __device__ __noinline__ float cc_logf(float x) { return logf(x); }\n"
       "static __device__ __noinline__ float cc_tanhf(float x) { return tanhf(x); }\n";
  if (lanes) o << kBatchLanePrelude << batch_lane_transcendentals(inline_level) << "}  // namespace\n";
  const std::string B = std::to_string(kBatchBlock);
  for (size_t s = first; s < last; ++s) {
    const int nin = struct_inputs[s];
    const std::string S = std::to_string(s);
    std::string pf = point_function(structs[s], "cc_point_" + S, inline_level >= 1, inline_level <= 1, lanes);
    o << (lanes ? "namespace {\n" + pf + "}  // namespace\n" : "static " + pf);
    // one lane (`suffix` names a float: ".x", "_0.y", ...) or, with lanes, a
    // whole float4 (`suffix` names the float4 itself and `four` is set)
    auto call = [&](const std::string &suffix, bool four = false) {
      std::string c = "cc_point_" + S + (lanes ? (four ? "<cc_f4>(" : "<float>(") : "(");
      for (int i = 0; i < kBatchMaxInputs; ++i) {
        std::string v = i < nin ? "v" + std::to_string(i) + suffix : std::string("0.0f");
        if (four) v = "cc_f4(" + v + ")";
        c += (i ? ", " : "") + v;
      }
      return c + ")" + (four ? ".f4()" : "");
    };
    // eight lanes: the float4s at positions u and u + 1 of every input
    auto call8 = [&](int u) {
      std::string c = "cc_point_" + S + "<cc_f8>(";
      for (int i = 0; i < kBatchMaxInputs; ++i) {
        const std::string I = std::to_string(i);
        c += (i ? ", " : "") + (i < nin ? "cc_f8(v" + I + "_" + std::to_string(u) + ", v" + I + "_" +
                                              std::to_string(u + 1) + ")"
                                        : std::string("cc_f8(0.0f)"));
      }
      return c + ")";
    };
    // A full tile loads its float4s before computing any: all kBatchUnroll
    // positions per input at once, or, when that is more than max_loads float4
    // loads, in groups of positions (fewer registers held by loads in flight;
    // eight lanes take positions in pairs); the ragged last tile of a program
    // takes the plain loops.
    const int min_group = lane_width == 8 ? 2 : 1;
    int group = kBatchUnroll;
    while (group > min_group && nin * group > max_loads) group /= 2;
    o << "extern \"C\" __device__ __noinline__ void cc_tile_" << S << kTileParams << " {\n";
    // prefetch: one thread asks L2 for the run's later tiles of every input
    // (one bulk prefetch per input) before the first tile's loads, so only
    // the first tile of a run waits for DRAM
    if (prefetch >= 1 && nin > 0) {
      o << "  if (threadIdx.x == 0 && count > 1) {\n"
        << "    const long long ps = base + " << kBatchTile << "LL;\n"
        << "    long long pe = base + (long long)count * " << kBatchTile << "LL;\n"
        << "    if (pe > n) pe = n;\n"
        << "    if (pe - ps >= 4) {\n"
        << "      const unsigned bytes = (unsigned)(((pe - ps) & ~3LL) * 4);\n";
      for (int i = 0; i < nin; ++i) o << "      cc_l2_prefetch(in" << i << " + ps, bytes);\n";
      o << "    }\n  }\n";
    }
    o << "  for (; count > 0; --count, base += " << kBatchTile << "LL) {\n"
      << "  if (base + " << kBatchTile << "LL <= n) {\n"
      << "    const long long q0 = (base >> 2) + threadIdx.x;\n";
    // rolled: one copy of the group's code in a loop over the groups (a
    // smaller tile function) instead of one copy per group
    const int copies = rolled ? group : kBatchUnroll;
    if (rolled && group < kBatchUnroll)
      o << "    #pragma unroll 1\n"
        << "    for (int k_ = 0; k_ < " << kBatchUnroll << "; k_ += " << group << ") {\n"
        << "    const long long qk = q0 + (long long)k_ * " << kBatchBlock << ";\n";
    else
      o << "    {\n    const long long qk = q0;\n";
    for (int g0 = 0; g0 < copies; g0 += group) {
      o << "    {\n";
      for (int i = 0; i < nin; ++i)
        for (int u = g0; u < g0 + group; ++u)
          o << "    const float4 v" << i << "_" << u << " = __ldg(reinterpret_cast<const float4 *>(in" << i
            << ") + qk + " << u * kBatchBlock << ");\n";
      if (lane_width == 8) {
        for (int u = g0; u < g0 + group; u += 2)
          o << "    const cc_f8 r8_" << u << " = " << call8(u) << ";\n"
            << "    const float4 r_" << u << " = r8_" << u << ".lo.f4(), r_" << u + 1 << " = r8_" << u
            << ".hi.f4();\n";
      }
      for (int u = g0; u < g0 + group && lane_width != 8; ++u) {
        const std::string U = "_" + std::to_string(u);
        if (lanes) {
          o << "    const float4 r" << U << " = " << call(U, true) << ";\n";
          continue;
        }
        o << "    float4 r" << U << ";\n";
        for (const char *lane : {".x", ".y", ".z", ".w"})
          o << "    r" << U << lane << " = " << call(U + lane) << ";\n";
      }
      for (int u = g0; u < g0 + group; ++u)
        o << "    reinterpret_cast<float4 *>(out)[qk + " << u * kBatchBlock << "] = r_" << u << ";\n";
      o << "    }\n";
    }
    o << "    }\n";
    o << "    continue;\n  }\n"
      << "  const long long end = base + " << kBatchTile << "LL < n ? base + " << kBatchTile << "LL : n;\n"
      << "  const long long end4 = end & ~3LL;\n"
      << "  for (long long q = (base >> 2) + threadIdx.x; (q << 2) < end4; q += " << B << ") {\n";
    for (int i = 0; i < nin; ++i)
      o << "    const float4 v" << i << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q);\n";
    if (lanes) {
      o << "    const float4 r = " << call("", true) << ";\n";
    } else {
      o << "    float4 r;\n";
      for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    r" << lane << " = " << call(lane) << ";\n";
    }
    o << "    reinterpret_cast<float4 *>(out)[q] = r;\n  }\n"
      << "  for (long long i = end4 + threadIdx.x; i < end; i += " << B << ") {\n";
    for (int i = 0; i < nin; ++i) o << "    const float v" << i << " = __ldg(in" << i << " + i);\n";
    o << "    out[i] = " << call("") << ";\n  }\n  }\n}\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << B << ") cc_prog_" << S
      << "(const float *__restrict__ in0, const float *__restrict__ in1, const float *__restrict__ in2, "
         "const float *__restrict__ in3, float *__restrict__ out, long long n) {\n"
      << "  const long long tiles = (n + " << kBatchTile - 1 << "LL) / " << kBatchTile << "LL;\n"
      << "  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) cc_tile_" << S
      << "(in0, in1, in2, in3, out, n, t * " << kBatchTile << "LL, 1);\n}\n";
  }
  return o.str();
}

std::string batch_main_source(size_t n_structs, int prefetch) {
  std::ostringstream o;
  o << "// generated batch main part for sm_103a\n"
    << kBatchPrefetchPrelude
    << "struct cc_entry { const float *in[4]; float *out; long long n; long long tile_begin; int sid; int pad; };\n"
    << "typedef void (*cc_tile_fn)" << kTileParams << ";\n";
  for (size_t s = 0; s < n_structs; ++s) o << "extern \"C\" __device__ void cc_tile_" << s << kTileParams << ";\n";
  o << "__device__ cc_tile_fn const cc_tiles[" << n_structs << "] = {\n";
  for (size_t s = 0; s < n_structs; ++s) o << "  cc_tile_" << s << ",\n";
  o << "};\n"
    // Blocks claim runs of `run` consecutive tiles from a work
    // counter (zeroed before each launch): a block stays in one program's code
    // for a run, and the uneven per-point cost of programs still balances.
    << "extern \"C\" __global__ void __launch_bounds__(" << kBatchBlock
    << ") cc_batch(const cc_entry *__restrict__ table, int nprog, long long total_tiles,\n"
    << "                unsigned long long *__restrict__ work, int run) {\n"
    << "  extern __shared__ long long s_begin[];\n"
    << "  __shared__ long long s_run;\n"
    << "  for (int i = threadIdx.x; i < nprog; i += blockDim.x) s_begin[i] = table[i].tile_begin;\n";
  if (prefetch >= 2) {
    // The block claims its next run one run ahead and, while it works on the
    // current one, L2 prefetches the next run's first tile (the tile
    // functions prefetch the later tiles of a run themselves).
    o << "  __shared__ long long s_next;\n"
      << "  if (threadIdx.x == 0) s_next = (long long)atomicAdd(work, (unsigned long long)run);\n"
      << "  for (;;) {\n"
      << "    __syncthreads();\n"
      << "    if (threadIdx.x == 0) {\n"
      << "      s_run = s_next;\n"
      << "      const long long tn = s_run < total_tiles ? (long long)atomicAdd(work, (unsigned long long)run) : total_tiles;\n"
      << "      s_next = tn;\n"
      << "      if (tn < total_tiles) {\n"
      << "        int a = 0, z = nprog - 1;\n"
      << "        while (a < z) {\n          const int m = (a + z + 1) >> 1;\n"
      << "          if (s_begin[m] <= tn) a = m; else z = m - 1;\n        }\n"
      << "        const cc_entry &f = table[a];\n"
      << "        const long long b0 = (tn - f.tile_begin) * " << kBatchTile << "LL;\n"
      << "        long long b1 = b0 + " << kBatchTile << "LL;\n"
      << "        if (b1 > f.n) b1 = f.n;\n"
      << "        if (b1 - b0 >= 4) {\n"
      << "          const unsigned bytes = (unsigned)(((b1 - b0) & ~3LL) * 4);\n"
      << "          for (int k = 0; k < 4; ++k)\n"
      << "            if (f.in[k]) cc_l2_prefetch(f.in[k] + b0, bytes);\n"
      << "        }\n"
      << "      }\n"
      << "    }\n"
      << "    __syncthreads();\n";
  } else {
    o << "  for (;;) {\n"
      << "    __syncthreads();\n"
      << "    if (threadIdx.x == 0) s_run = (long long)atomicAdd(work, (unsigned long long)run);\n"
      << "    __syncthreads();\n";
  }
  o
    << "    const long long t0 = s_run;\n"
    << "    if (t0 >= total_tiles) break;\n"
    << "    const long long t1 = t0 + run < total_tiles ? t0 + run : total_tiles;\n"
    << "    int lo = 0, hi = nprog - 1;\n"
    << "    while (lo < hi) {\n      const int mid = (lo + hi + 1) >> 1;\n"
    << "      if (s_begin[mid] <= t0) lo = mid; else hi = mid - 1;\n    }\n"
    << "    long long next = lo + 1 < nprog ? s_begin[lo + 1] : total_tiles;\n"
    // one call per program the run touches, for all of its tiles in the run
    << "    for (long long t = t0; t < t1;) {\n"
    << "      while (t >= next && lo + 1 < nprog) {\n        ++lo;\n"
    << "        next = lo + 1 < nprog ? s_begin[lo + 1] : total_tiles;\n      }\n"
    << "      const long long stop = next < t1 ? next : t1;\n"
    << "      const cc_entry e = table[lo];\n"
    << "      const long long base = (t - e.tile_begin) * " << kBatchTile << "LL;\n"
    << "      if (e.sid >= 0 && e.sid < " << n_structs << ") cc_tiles[e.sid](e.in[0], e.in[1], e.in[2], e.in[3], e.out, e.n, base, (int)(stop - t));\n"
    << "      t = stop;\n"
    << "    }\n"
    << "  }\n}\n";
  return o.str();
}

// NVRTC-compiles the sources on all host threads; the first failure is raised.
std::vector<std::vector<char>> compile_parallel(const std::vector<std::string> &sources, int cc_major, int cc_minor,
                                                uint32_t flags, bool relocatable, int max_registers) {
  std::vector<std::vector<char>> parts(sources.size());
  std::vector<std::string> errors(sources.size());
  std::atomic<size_t> next{0};
  unsigned nthreads = std::thread::hardware_concurrency();
  if (nthreads == 0) nthreads = 4;
  if (nthreads > sources.size()) nthreads = (unsigned)sources.size();
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nthreads; ++t) {
    pool.emplace_back([&]() {
      for (size_t i; (i = next.fetch_add(1)) < sources.size();) {
        try {
          parts[i] = compile_cubin(sources[i], cc_major, cc_minor, flags, relocatable, max_registers);
        } catch (const Error &e) {
          errors[i] = e.message;
        }
      }
    });
  }
  for (auto &th : pool) th.join();
  for (auto &e : errors)
    if (!e.empty()) fail(CC_ERR_BUILD_PROGRAM_FAILURE, e);
  return parts;
}

// Compiles the parts in parallel and links them into one loadable image.
std::vector<char> build_batch_image(const std::vector<Ir> &structs, const std::vector<int> &struct_inputs,
                                    int cc_major, int cc_minor, uint32_t flags, bool link, int inline_level,
                                    int max_registers, int max_loads, int lane_width, bool rolled,
                                    int prefetch) {
  std::vector<std::string> sources;
  FmaScope fma_scope((flags & CC_FLAG_FMA_CONTRACT) != 0);
  for (size_t first = 0; first < structs.size(); first += kBatchChunk)
    sources.push_back(batch_chunk_source(structs, struct_inputs, first,
                                         std::min(structs.size(), first + (size_t)kBatchChunk), inline_level,
                                         max_loads, lane_width, rolled, prefetch));
  sources.push_back(batch_main_source(structs.size(), prefetch));
  std::vector<std::vector<char>> parts = compile_parallel(sources, cc_major, cc_minor, flags, true, max_registers);
  if (!link) return {};
  CUlinkState state;
  check_cu(g_drv.LinkCreate(0, nullptr, nullptr, &state), "cuLinkCreate");
  try {
    for (size_t i = 0; i < parts.size(); ++i) {
      std::string name = "batch_part_" + std::to_string(i);
      check_cu(g_drv.LinkAddData(state, CU_JIT_INPUT_CUBIN, parts[i].data(), parts[i].size(), name.c_str(), 0,
                                 nullptr, nullptr),
               "cuLinkAddData");
    }
    void *image = nullptr;
    size_t size = 0;
    check_cu(g_drv.LinkComplete(state, &image, &size), "cuLinkComplete");
    std::vector<char> out(static_cast<char *>(image), static_cast<char *>(image) + size);
    g_drv.LinkDestroy(state);
    return out;
  } catch (...) {
    g_drv.LinkDestroy(state);
    throw;
  }
}

Batch &batch_of(Context &c, cc_handle h) {
  auto it = c.batches.find(h);
  if (tag_of(h) != kTagBatch || it == c.batches.end()) fail(CC_ERR_INVALID_VALUE, "not a live batch handle");
  return *it->second;
}

void batch_drop_graph(Batch &b) {
  if (b.graph_exec) cudaGraphExecDestroy(b.graph_exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.graph_exec = nullptr;
  b.graph = nullptr;
}

struct BatchCopy {
  void *dst;
  const void *src;
  size_t bytes;
};

// Copies between pinned host memory and a batch's buffers, host to device on
// copy streams 0-3 and device to host on copy streams 4-7 (so one step's reads
// and the next step's uploads overlap on the link), each stream taking the
// next copy when it holds the fewest bytes.  Every stream first waits for the
// wait list; the returned event completes when every copy has.  The streams are
// not joined into the context stream: the caller orders later work by the event.
// Whether [p, p + bytes) lies inside one live cc_host_alloc allocation.
bool in_pinned(const Context &c, const void *p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  auto it = c.pinned.upper_bound(a);
  if (it == c.pinned.begin()) return false;
  --it;
  return a - it->first <= it->second && bytes <= it->second - (a - it->first);
}

// The device copy table of these copies (built and cached on first use), or
// nullptr when a host end is not memory of cc_host_alloc (then the DMA engines copy).
const Batch::CopyTable *batch_copy_table(Context &c, Batch &b, const std::vector<BatchCopy> &copies, bool to_device) {
  std::vector<uint64_t> key;
  key.reserve(1 + 3 * copies.size());
  key.push_back(to_device ? 1 : 0);
  for (const BatchCopy &cp : copies) {
    key.push_back(reinterpret_cast<uint64_t>(cp.dst));
    key.push_back(reinterpret_cast<uint64_t>(cp.src));
    key.push_back(cp.bytes);
  }
  for (auto it = b.copy_tables.begin(); it != b.copy_tables.end(); ++it)
    if (it->pinned_gen == c.pinned_gen && it->key == key) {
      if (it + 1 != b.copy_tables.end()) std::rotate(it, it + 1, b.copy_tables.end());  // most recent last
      return &b.copy_tables.back();
    }
  std::vector<CopyEntry> table;
  long long chunks = 0;
  for (const BatchCopy &cp : copies) {
    const void *host = to_device ? cp.src : cp.dst;
    if (cp.bytes == 0) continue;
    if (!in_pinned(c, host, cp.bytes)) return nullptr;
    const void *alias = pinned_device_alias(host);
    if (!alias) return nullptr;
    CopyEntry e;
    e.dst = reinterpret_cast<uint64_t>(to_device ? cp.dst : alias);
    e.src = reinterpret_cast<uint64_t>(to_device ? alias : cp.src);
    e.bytes = cp.bytes;
    e.chunk_begin = chunks;
    chunks += (long long)((cp.bytes + kCopyChunk - 1) / kCopyChunk);
    table.push_back(e);
  }
  if (table.empty()) return nullptr;
  Batch::CopyTable t;
  t.key = std::move(key);
  t.pinned_gen = c.pinned_gen;
  t.n = (int)table.size();
  t.chunks = chunks;
  t.dev = c.pool.alloc(sizeof(CopyEntry) * table.size(), &t.cls);
  // ordered after the context stream's work (the block may have served it) and
  // complete before the host's table goes away: built once per pointer list
  cudaError_t e = cudaMemcpyAsync(t.dev, table.data(), sizeof(CopyEntry) * table.size(), cudaMemcpyHostToDevice,
                                  c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    release_block(c, t.dev, t.cls);
    check_cuda(e, "cudaMemcpy copy table");
  }
  constexpr size_t kKeep = 4;
  if (b.copy_tables.size() >= kKeep) {
    release_block(c, b.copy_tables.front().dev, b.copy_tables.front().cls);
    b.copy_tables.erase(b.copy_tables.begin());
  }
  b.copy_tables.push_back(std::move(t));
  return &b.copy_tables.back();
}

void batch_drop_copy_tables(Context &c, Batch &b) {
  for (auto &t : b.copy_tables) release_block(c, t.dev, t.cls);
  b.copy_tables.clear();
}

cc_handle batch_copies(Context &c, Batch &b, const std::vector<BatchCopy> &copies, bool to_device,
                       const cc_handle *wait, int n_wait) {
  const int first = to_device ? 0 : 4, n = 4;
  if (c.batch_copy_kernel) {
    // one kernel over the whole table on the direction's first copy stream
    const Batch::CopyTable *t = batch_copy_table(c, b, copies, to_device);
    if (t) {
      cudaStream_t s = c.copy_streams[first];
      wait_events(c, s, wait, n_wait);
      check_cuda(launch_copy_table(static_cast<const CopyEntry *>(t->dev), t->n, t->chunks, c.sm_count * 2, s),
                 "copy table kernel");
      c.copy_dirty[first] = true;
      return fence_handle(c, record_fence(c, s));
    }
  }
  for (int i = 0; i < n; ++i) wait_events(c, c.copy_streams[first + i], wait, n_wait);
  size_t load[4] = {0, 0, 0, 0};
  for (const BatchCopy &cp : copies) {
    if (!cp.bytes) continue;
    int s = 0;
    for (int i = 1; i < n; ++i)
      if (load[i] < load[s]) s = i;
    load[s] += cp.bytes;
    check_cuda(cudaMemcpyAsync(cp.dst, cp.src, cp.bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                               c.copy_streams[first + s]),
               to_device ? "cudaMemcpyAsync H2D" : "cudaMemcpyAsync D2H");
  }
  cudaStream_t lead = c.copy_streams[first];
  for (int i = 1; i < n; ++i) {
    FencePtr f = record_fence(c, c.copy_streams[first + i]);
    check_cuda(cudaStreamWaitEvent(lead, f->ev, 0), "cudaStreamWaitEvent");
  }
  for (int i = 0; i < n; ++i) c.copy_dirty[first + i] = true;
  return fence_handle(c, record_fence(c, lead));
}

void batch_launch_each(Context &c, Batch &b, cudaStream_t s) {
  for (size_t p = 0; p < b.sid.size(); ++p) {
    if (b.length[p] == 0) continue;
    uint64_t in[kBatchMaxInputs] = {0, 0, 0, 0};
    for (int i = 0; i < b.n_inputs[p]; ++i) in[i] = b.ptrs[p][i];
    uint64_t out = b.ptrs[p][b.n_inputs[p]];
    long long n = b.length[p];
    void *args[] = {&in[0], &in[1], &in[2], &in[3], &out, &n};
    int64_t tiles = (n + kBatchTile - 1) / kBatchTile;
    int64_t cap = (int64_t)c.sm_count * 8;
    unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
    check_cu(g_drv.LaunchKernel(b.per_structure[b.sid[p]], grid, 1, 1, kBatchBlock, 1, 1, 0, (CUstream)s, args, nullptr),
             "cuLaunchKernel");
  }
}

}  // namespace
}  // namespace cc

extern "C" {

int cc_batch_create(const char *const *irs, const size_t *lens, int n_programs, cc_handle *out) {
  CC_API_BEGIN
  if (!irs || !lens || !out || n_programs <= 0) fail(CC_ERR_INVALID_VALUE, "empty batch");
  Context &c = ctx();
  auto b = std::make_unique<Batch>();
  std::unordered_map<std::string, int> seen;
  std::vector<Ir> structs;
  std::vector<int> struct_inputs;
  for (int p = 0; p < n_programs; ++p) {
    if (!irs[p]) fail(CC_ERR_INVALID_VALUE, "null program text");
    std::string text(irs[p], lens[p]);
    Ir ir = parse_ir(text.data(), text.size());
    std::string why;
    if (!is_batchable(ir, &why)) fail(CC_ERR_INVALID_PROGRAM, "program " + std::to_string(p) + ": " + why);
    int64_t n = 1;
    for (int64_t d : ir.out_shape) n *= d;
    // programs differing only in length share code
    std::string key = contiguous_structure_key(ir);
    if (key.empty()) key = text;
    auto it = seen.find(key);
    int sid;
    if (it == seen.end()) {
      sid = (int)structs.size();
      seen.emplace(key, sid);
      struct_inputs.push_back(ir.n_params);
      structs.push_back(std::move(ir));
    } else {
      sid = it->second;
    }
    b->sid.push_back(sid);
    b->n_inputs.push_back(struct_inputs[sid]);
    b->length.push_back(n);
  }
  std::vector<char> cubin;
  {
    std::lock_guard<std::mutex> cg(c.compile_mu);
    cubin = build_batch_image(structs, struct_inputs, c.cc_major, c.cc_minor, c.flags, true, c.batch_inline,
                              c.batch_max_registers, c.batch_max_loads, c.batch_lanes, c.batch_rolled != 0,
                              c.batch_prefetch);
  }
  check_cu(g_drv.ModuleLoadData(&b->module, cubin.data()), "cuModuleLoadData");
  check_cu(g_drv.ModuleGetFunction(&b->persistent, b->module, "cc_batch"), "cuModuleGetFunction");
  for (size_t s = 0; s < structs.size(); ++s) {
    CUfunction f;
    check_cu(g_drv.ModuleGetFunction(&f, b->module, ("cc_prog_" + std::to_string(s)).c_str()), "cuModuleGetFunction");
    b->per_structure.push_back(f);
  }
  const size_t smem = sizeof(int64_t) * (size_t)n_programs;
  if (smem > 48 * 1024)
    check_cu(g_drv.FuncSetAttribute(b->persistent, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem),
             "cuFuncSetAttribute");
  check_cu(g_drv.OccupancyMaxActiveBlocks(&b->resident, b->persistent, kBatchBlock, smem), "occupancy");
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  uint64_t h = c.make_handle(kTagBatch);
  c.batches[h] = b.release();
  *out = h;
  CC_API_END
}

int cc_batch_compile_check(const char *const *irs, const size_t *lens, int n_programs, int cc_major, int cc_minor,
                           int *n_structures, double *seconds) {
  CC_API_BEGIN
  if (!irs || !lens || n_programs <= 0) fail(CC_ERR_INVALID_VALUE, "empty batch");
  std::unordered_map<std::string, int> seen;
  std::vector<Ir> structs;
  std::vector<int> struct_inputs;
  for (int p = 0; p < n_programs; ++p) {
    Ir ir = parse_ir(irs[p], lens[p]);
    std::string why;
    if (!is_batchable(ir, &why)) fail(CC_ERR_INVALID_PROGRAM, "program " + std::to_string(p) + ": " + why);
    std::string key = contiguous_structure_key(ir);
    if (key.empty()) key = std::string(irs[p], lens[p]);
    if (seen.emplace(key, (int)structs.size()).second) {
      struct_inputs.push_back(ir.n_params);
      structs.push_back(std::move(ir));
    }
  }
  auto t0 = std::chrono::steady_clock::now();
  // a context's default settings; linking needs a driver
  build_batch_image(structs, struct_inputs, cc_major, cc_minor, 0, false, kBatchInlineDefault, kBatchRegistersDefault,
                    kBatchLoadsDefault, kBatchLanesDefault, kBatchRolledDefault != 0, kBatchPrefetchDefault);
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (n_structures) *n_structures = (int)structs.size();
  CC_API_END
}

int cc_batch_info(cc_handle batch, int *n_programs, int *n_structures, int *registers, int *resident_blocks) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  if (n_programs) *n_programs = (int)b.sid.size();
  if (n_structures) *n_structures = (int)b.per_structure.size();
  if (registers) check_cu(g_drv.FuncGetAttribute(registers, CU_FUNC_ATTRIBUTE_NUM_REGS, b.persistent), "cuFuncGetAttribute");
  if (resident_blocks) *resident_blocks = b.resident;
  CC_API_END
}

int cc_batch_bind(cc_handle batch, const uint64_t *ptrs, size_t n_ptrs) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Batch &b = batch_of(c, batch);
  size_t need = 0;
  for (size_t p = 0; p < b.sid.size(); ++p) need += b.n_inputs[p] + 1;
  if (!ptrs || n_ptrs != need)
    fail(CC_ERR_INVALID_KERNEL_ARGS, "the batch needs " + std::to_string(need) + " pointers (inputs, then the output, per program)");
  std::vector<BatchEntry> table(b.sid.size());
  std::vector<std::vector<uint64_t>> bound(b.sid.size());
  size_t k = 0;
  int64_t tiles = 0;
  for (size_t p = 0; p < b.sid.size(); ++p) {
    BatchEntry &e = table[p];
    memset(&e, 0, sizeof e);
    for (int i = 0; i <= b.n_inputs[p]; ++i) {
      uint64_t q = ptrs[k++];
      if (!q || (q & 15u)) fail(CC_ERR_INVALID_VALUE, "batch buffers must be non-null and 16-byte aligned");
      bound[p].push_back(q);
      if (i < b.n_inputs[p]) e.in[i] = q; else e.out = q;
    }
    e.n = b.length[p];
    e.tile_begin = tiles;
    e.sid = b.sid[p];
    tiles += (b.length[p] + kBatchTile - 1) / kBatchTile;
  }
  // one extra entry at the end holds the persistent kernel's work counter
  if (!b.table) b.table = c.pool.alloc(sizeof(BatchEntry) * (table.size() + 1), &b.table_cls);
  check_cuda(cudaMemcpyAsync(b.table, table.data(), sizeof(BatchEntry) * table.size(), cudaMemcpyHostToDevice, c.stream),
             "upload batch table");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  b.ptrs = std::move(bound);
  b.total_tiles = tiles;
  b.bound = true;
  batch_drop_graph(b);
  batch_drop_copy_tables(c, b);
  CC_API_END
}

int cc_batch_run(cc_handle batch, int mode, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Batch &b = batch_of(c, batch);
  if (!b.bound) fail(CC_ERR_INVALID_OPERATION, "bind the batch's buffers first");
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  if (mode == CC_BATCH_PERSISTENT) {
    if (b.total_tiles == 0) return CC_OK;
    uint64_t table = reinterpret_cast<uint64_t>(b.table);
    int nprog = (int)b.sid.size();
    long long total = b.total_tiles;
    uint64_t work = table + sizeof(BatchEntry) * b.sid.size();
    check_cuda(cudaMemsetAsync(reinterpret_cast<void *>(work), 0, sizeof(unsigned long long), s), "cudaMemsetAsync");
    int run = c.batch_run_tiles;
    void *args[] = {&table, &nprog, &total, &work, &run};
    int64_t cap = (int64_t)c.sm_count * (b.resident > 0 ? b.resident : 4);
    unsigned grid = (unsigned)(b.total_tiles < cap ? b.total_tiles : cap);
    check_cu(g_drv.LaunchKernel(b.persistent, grid, 1, 1, kBatchBlock, 1, 1, (unsigned)(sizeof(int64_t) * nprog),
                                (CUstream)s, args, nullptr),
             "cuLaunchKernel");
  } else if (mode == CC_BATCH_PER_PROGRAM) {
    batch_launch_each(c, b, s);
  } else if (mode == CC_BATCH_GRAPH) {
    if (!b.graph_exec) {
      cudaStream_t cap_stream;
      check_cuda(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking), "cudaStreamCreate");
      cudaError_t e = cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        try {
          batch_launch_each(c, b, cap_stream);
        } catch (...) {
          cudaGraph_t broken = nullptr;
          cudaStreamEndCapture(cap_stream, &broken);
          if (broken) cudaGraphDestroy(broken);
          cudaStreamDestroy(cap_stream);
          throw;
        }
        e = cudaStreamEndCapture(cap_stream, &b.graph);
      }
      cudaStreamDestroy(cap_stream);
      check_cuda(e, "graph capture");
      check_cuda(cudaGraphInstantiate(&b.graph_exec, b.graph, 0), "cudaGraphInstantiate");
    }
    check_cuda(cudaGraphLaunch(b.graph_exec, s), "cudaGraphLaunch");
  } else {
    fail(CC_ERR_INVALID_VALUE, "unknown batch mode");
  }
  CC_API_END
}

int cc_batch_run_ev(cc_handle batch, int mode, const cc_handle *wait, int n_wait, cc_handle *event) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  batch_of(c, batch);
  for (int i = 0; i < n_wait; ++i) event_of(c, wait[i]);  // every handle valid before anything is enqueued
  end_pdl_chain(c);
  wait_events(c, c.stream, wait, n_wait);
  const int r = cc_batch_run(batch, mode, 0);
  if (r != CC_OK) return r;
  if (event) *event = fence_handle(c, record_fence(c, c.stream));
  CC_API_END
}

int cc_batch_upload_ev(cc_handle batch, const void *const *hosts, size_t n_hosts, const cc_handle *wait, int n_wait,
                       cc_handle *event) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  if (!b.bound) fail(CC_ERR_INVALID_OPERATION, "bind the batch's buffers first");
  size_t need = 0;
  for (size_t p = 0; p < b.sid.size(); ++p) need += b.n_inputs[p];
  if (!hosts || n_hosts != need)
    fail(CC_ERR_INVALID_VALUE, "the batch has " + std::to_string(need) + " inputs, got " + std::to_string(n_hosts) +
                                   " host pointers");
  for (int i = 0; i < n_wait; ++i) event_of(c, wait[i]);
  std::vector<BatchCopy> copies;
  size_t k = 0;
  for (size_t p = 0; p < b.sid.size(); ++p)
    for (int i = 0; i < b.n_inputs[p]; ++i, ++k) {
      const size_t bytes = (size_t)b.length[p] * sizeof(float);
      if (bytes && !hosts[k]) fail(CC_ERR_INVALID_VALUE, "null host pointer");
      copies.push_back({reinterpret_cast<void *>(b.ptrs[p][i]), hosts[k], bytes});
    }
  end_pdl_chain(c);  // the context stream's generated kernels do not see these writes as their own
  *event = batch_copies(c, b, copies, true, wait, n_wait);
  CC_API_END
}

int cc_batch_download_ev(cc_handle batch, void *const *hosts, size_t n_hosts, const cc_handle *wait, int n_wait,
                         cc_handle *event) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  if (!b.bound) fail(CC_ERR_INVALID_OPERATION, "bind the batch's buffers first");
  if (!hosts || n_hosts != b.sid.size())
    fail(CC_ERR_INVALID_VALUE, "the batch has " + std::to_string(b.sid.size()) + " outputs, got " +
                                   std::to_string(n_hosts) + " host pointers");
  for (int i = 0; i < n_wait; ++i) event_of(c, wait[i]);
  std::vector<BatchCopy> copies;
  for (size_t p = 0; p < b.sid.size(); ++p) {
    const size_t bytes = (size_t)b.length[p] * sizeof(float);
    if (bytes && !hosts[p]) fail(CC_ERR_INVALID_VALUE, "null host pointer");
    copies.push_back({hosts[p], reinterpret_cast<const void *>(b.ptrs[p][b.n_inputs[p]]), bytes});
  }
  *event = batch_copies(c, b, copies, false, wait, n_wait);
  CC_API_END
}

int cc_batch_release(cc_handle batch) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  batch_drop_graph(b);
  batch_drop_copy_tables(c, b);
  if (b.table) release_block(c, b.table, b.table_cls);
  g_drv.ModuleUnload(b.module);
  delete &b;
  c.batches.erase(batch);
  CC_API_END
}

}  // extern "C"

// ---------------------------------------------------------------- tuner
//
// A program's tunable form (tunable_source) runs in any of kTuneConfigs launch
// configurations.  The exhaustive tuner times them all on the program's own
// buffers at its first launch; the learned tuner asks a cost model (an Mlp
// trained on such timings) for the configuration with the least predicted
// log-runtime.  Tuning sets (cc_tune_*) compile many programs' tunable forms
// at once and time configurations on request: the data the model learns from.

namespace cc {
namespace {

constexpr int kTuneChunk = 16;                     // programs per NVRTC unit of a tuning set
constexpr size_t kFlushBytes = size_t(256) << 20;  // written between timed launches: twice L2

void wait_event_bounded(cudaEvent_t ev, uint64_t timeout_ns, const char *what) {
  auto t0 = std::chrono::steady_clock::now();
  int spin = 0;
  for (;;) {
    cudaError_t r = cudaEventQuery(ev);
    if (r == cudaSuccess) return;
    if (r != cudaErrorNotReady) check_cuda(r, what);
    auto dt = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
    if ((uint64_t)dt >= timeout_ns) fail(CC_ERR_TIMEOUT, std::string(what) + ": not complete in time");
    if (++spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

bool tune_config_fits(const TuneEntry &e, int config, const std::vector<uint64_t> &in, uint64_t out) {
  if (tune_config(config).vec != 4) return true;
  if (e.kind == ProgramKind::Elementwise && (out & 15u)) return false;
  if (e.contiguous)
    for (uint64_t a : in)
      if (a & 15u) return false;
  return true;
}

void launch_tune_entry(Context &c, TuneEntry &e, int config, const std::vector<uint64_t> &in, uint64_t out,
                       cudaStream_t s) {
  if (config < 0 || config >= kTuneConfigs) fail(CC_ERR_INVALID_VALUE, "configuration index out of range");
  if (!tune_config_fits(e, config, in, out))
    fail(CC_ERR_INVALID_VALUE, "a float4 configuration needs 16-byte aligned buffers");
  const TuneConfig t = tune_config(config);
  const int k = tune_kernel_index(t), bi = config % 4;
  if (e.resident[k][bi] <= 0) {
    check_cu(g_drv.OccupancyMaxActiveBlocks(&e.resident[k][bi], e.fn[k], t.block, 0), "cuOccupancyMaxActiveBlocks");
    if (e.resident[k][bi] <= 0) fail(CC_ERR_OUT_OF_RESOURCES, "the configuration's block does not fit on an SM");
  }
  const bool sum = e.kind == ProgramKind::Sum;
  const int64_t grid = tune_grid(e.n, t, sum, c.sm_count, e.resident[k][bi]);
  std::vector<uint64_t> ptrs(in);
  std::vector<void *> args;
  for (auto &v : ptrs) args.push_back(&v);
  size_t temporary = 0;
  char *scratch = sum ? static_cast<char *>(sum_scratch_for(c, s, &temporary)) : nullptr;
  uint64_t partials = reinterpret_cast<uint64_t>(scratch);
  uint64_t counter = reinterpret_cast<uint64_t>(scratch + sizeof(float2) * kMaxSumBlocks);
  uint64_t o = out;
  long long n = e.n;
  if (sum) {
    args.push_back(&partials);
    args.push_back(&counter);
  }
  args.push_back(&o);
  args.push_back(&n);
  // programmatic dependent launch (the tunable kernels wait at entry)
  CUlaunchAttribute attr;
  memset(&attr, 0, sizeof attr);
  attr.id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
  attr.value.programmaticStreamSerializationAllowed = 1;
  CUlaunchConfig cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.gridDimX = (unsigned)grid;
  cfg.gridDimY = cfg.gridDimZ = 1;
  cfg.blockDimX = (unsigned)t.block;
  cfg.blockDimY = cfg.blockDimZ = 1;
  cfg.hStream = (CUstream)s;
  cfg.attrs = &attr;
  cfg.numAttrs = c.pdl ? 1 : 0;
  CUresult r = g_drv.LaunchKernelEx(&cfg, e.fn[k], args.data(), nullptr);
  if (temporary) {
    cudaError_t se = r == CUDA_SUCCESS ? cudaStreamSynchronize(s) : cudaSuccess;
    c.pool.release(scratch, temporary);
    check_cuda(se, "cudaStreamSynchronize");
  }
  check_cu(r, "cuLaunchKernel");
}

// Median device time (ms) over `reps` launches of each configuration, after
// one untimed launch; with a flush buffer, a write twice the size of L2
// precedes every timed launch.  Configurations that do not apply to these
// buffers get -1.
void time_tune_entry(Context &c, TuneEntry &e, const int *configs, int n_configs, const std::vector<uint64_t> &in,
                     uint64_t out, int reps, void *flush, size_t flush_bytes, float *ms) {
  if (reps < 1) reps = 1;
  cudaStream_t s = c.stream;
  std::vector<cudaEvent_t> ev(2 * (size_t)reps, nullptr);
  for (auto &x : ev) check_cuda(cudaEventCreate(&x), "cudaEventCreate");
  auto destroy = [&]() {
    for (auto &x : ev)
      if (x) cudaEventDestroy(x);
  };
  try {
    std::vector<float> t(reps);
    for (int i = 0; i < n_configs; ++i) {
      if (configs[i] < 0 || configs[i] >= kTuneConfigs) fail(CC_ERR_INVALID_VALUE, "configuration index out of range");
      if (!tune_config_fits(e, configs[i], in, out)) {
        ms[i] = -1.0f;
        continue;
      }
      launch_tune_entry(c, e, configs[i], in, out, s);
      for (int r = 0; r < reps; ++r) {
        if (flush) check_cuda(cudaMemsetAsync(flush, r & 0xff, flush_bytes, s), "cudaMemsetAsync");
        check_cuda(cudaEventRecord(ev[2 * r], s), "cudaEventRecord");
        launch_tune_entry(c, e, configs[i], in, out, s);
        check_cuda(cudaEventRecord(ev[2 * r + 1], s), "cudaEventRecord");
      }
      wait_event_bounded(ev[2 * reps - 1], 60ull * 1000000000ull, "timing a configuration");
      for (int r = 0; r < reps; ++r) check_cuda(cudaEventElapsedTime(&t[r], ev[2 * r], ev[2 * r + 1]), "cudaEventElapsedTime");
      std::sort(t.begin(), t.end());
      ms[i] = t[reps / 2];
    }
  } catch (...) {
    destroy();
    throw;
  }
  destroy();
}

Mlp &mlp_of(Context &c, uint64_t h) {
  auto it = c.mlps.find(h);
  if (tag_of(h) != kTagMlp || it == c.mlps.end()) fail(CC_ERR_INVALID_VALUE, "not a live network handle");
  return *it->second;
}

int mlp_max_width(const Mlp &m) { return *std::max_element(m.dims.begin(), m.dims.end()); }

// Scratch layout for a batch of `cap`: activations h_1..h_L, two deltas, the
// column-sum partials, the loss.
void mlp_reserve(Context &c, Mlp &m, int batch) {
  if (batch <= m.cap) return;
  size_t acts = 0;
  for (size_t l = 1; l < m.dims.size(); ++l) acts += (size_t)m.dims[l];
  const size_t w = (size_t)mlp_max_width(m);
  const size_t floats = (size_t)batch * acts + 2 * (size_t)batch * w + (size_t)colsum_chunks(batch) * w + 64;
  if (m.scratch) {
    check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
    release_block(c, m.scratch, m.scratch_cls);
    m.scratch = nullptr;
    m.cap = 0;
  }
  m.scratch = c.pool.alloc(floats * sizeof(float), &m.scratch_cls);
  m.cap = batch;
}

float *mlp_act(Mlp &m, size_t l) {  // h_l, l >= 1
  size_t off = 0;
  for (size_t j = 1; j < l; ++j) off += (size_t)m.dims[j] * m.cap;
  return static_cast<float *>(m.scratch) + off;
}
float *mlp_delta(Mlp &m, int which) {
  return mlp_act(m, m.dims.size()) + (size_t)which * m.cap * mlp_max_width(m);
}
float *mlp_partial(Mlp &m) { return mlp_delta(m, 2); }
float *mlp_loss(Mlp &m) { return mlp_partial(m) + (size_t)colsum_chunks(m.cap) * mlp_max_width(m); }

void mlp_forward(Context &c, Mlp &m, const float *x, int batch, float *y, cudaStream_t s) {
  const size_t L = m.dims.size() - 1;
  for (size_t l = 1; l <= L; ++l) {
    const float *in = l == 1 ? x : mlp_act(m, l - 1);
    float *o = (l == L && y) ? y : mlp_act(m, l);
    const int k = m.dims[l - 1], n = m.dims[l];
    check_cuda(launch_mlp_gemm(false, false, in, m.params() + m.w_off[l], o, batch, n, k, k, n, n,
                               m.params() + m.b_off[l], l < L ? kMlpBiasRelu : kMlpBias, nullptr, s),
               "network forward");
  }
}

// Forward, loss and every parameter's gradient (into m.grads()).
void mlp_backward(Context &c, Mlp &m, const float *x, const float *t, int batch, cudaStream_t s) {
  const size_t L = m.dims.size() - 1;
  mlp_forward(c, m, x, batch, nullptr, s);
  int cur = 0;
  check_cuda(launch_mse(mlp_act(m, L), t, batch, mlp_delta(m, cur), mlp_loss(m), s), "loss");
  for (size_t l = L; l >= 1; --l) {
    const float *in = l == 1 ? x : mlp_act(m, l - 1);
    const int k = m.dims[l - 1], n = m.dims[l];
    float *d = mlp_delta(m, cur);
    check_cuda(launch_mlp_gemm(true, false, in, d, m.grads() + m.w_off[l], k, n, batch, k, n, n, nullptr, kMlpNone,
                               nullptr, s),
               "weight gradient");
    check_cuda(launch_colsum(d, batch, n, mlp_partial(m), m.grads() + m.b_off[l], s), "bias gradient");
    if (l > 1) {
      check_cuda(launch_mlp_gemm(false, true, d, m.params() + m.w_off[l], mlp_delta(m, 1 - cur), batch, k, n, n, n, k,
                                 nullptr, kMlpReluMask, mlp_act(m, l - 1), s),
                 "delta");
      cur = 1 - cur;
    }
  }
}

// Median device time (ms) of `reps` runs of launch() on the context stream,
// after one untimed run; with a flush buffer, a write twice the size of L2
// precedes every timed run.
float time_launches(Context &c, const std::function<void()> &launch, int reps, void *flush, size_t flush_bytes) {
  if (reps < 1) reps = 1;
  cudaStream_t s = c.stream;
  std::vector<cudaEvent_t> ev(2 * (size_t)reps, nullptr);
  auto destroy = [&]() {
    for (auto &x : ev)
      if (x) cudaEventDestroy(x);
  };
  std::vector<float> t(reps);
  try {
    for (auto &x : ev) check_cuda(cudaEventCreate(&x), "cudaEventCreate");
    launch();
    for (int r = 0; r < reps; ++r) {
      if (flush) check_cuda(cudaMemsetAsync(flush, r & 0xff, flush_bytes, s), "cudaMemsetAsync");
      check_cuda(cudaEventRecord(ev[2 * r], s), "cudaEventRecord");
      launch();
      check_cuda(cudaEventRecord(ev[2 * r + 1], s), "cudaEventRecord");
    }
    wait_event_bounded(ev[2 * reps - 1], 60ull * 1000000000ull, "timing a launch");
    for (int r = 0; r < reps; ++r) check_cuda(cudaEventElapsedTime(&t[r], ev[2 * r], ev[2 * r + 1]), "cudaEventElapsedTime");
  } catch (...) {
    destroy();
    throw;
  }
  destroy();
  std::sort(t.begin(), t.end());
  return t[reps / 2];
}

// The standard generated kernel of a tuned program, timed like a configuration.
float time_standard(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, int reps, void *flush,
                    size_t flush_bytes) {
  return time_launches(
      c,
      [&]() {
        end_pdl_chain(c);
        launch_generated(c, p, in, out, c.stream);
      },
      reps, flush, flush_bytes);
}

// Every configuration of the tunable form and the standard kernel, timed
// (3 runs each after an L2 flush); the fastest is kept, so a tuned program is
// never slower than the standard kernel it would otherwise run.
int choose_exhaustive(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out) {
  TuneEntry &e = *p.tune;
  std::vector<int> configs(kTuneConfigs);
  for (int i = 0; i < kTuneConfigs; ++i) configs[i] = i;
  std::vector<float> ms(kTuneConfigs + 1);
  size_t cls = 0;
  void *flush = c.pool.alloc(kFlushBytes, &cls);
  try {
    time_tune_entry(c, e, configs.data(), kTuneConfigs, in, out, 3, flush, kFlushBytes, ms.data());
    ms[kStdConfig] = time_standard(c, p, in, out, 3, flush, kFlushBytes);
  } catch (...) {
    release_block(c, flush, cls);
    throw;
  }
  release_block(c, flush, cls);
  int best = kStdConfig;
  for (int i = 0; i < kTuneConfigs; ++i)
    if (ms[i] >= 0.0f && ms[i] < ms[best]) best = i;
  return best;
}

// The cost model ranks the configurations of the tunable form; its first
// choice and the standard kernel are then timed (3 runs each after an L2
// flush) and the faster is kept.
int choose_learned(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out) {
  TuneEntry &e = *p.tune;
  if (!c.cost_model) fail(CC_ERR_INVALID_OPERATION, "the learned tuner needs a cost model (cc_tuner_set_model)");
  Mlp &m = mlp_of(c, c.cost_model);
  std::vector<float> x((size_t)kTuneConfigs * kFeatures);
  for (int i = 0; i < kTuneConfigs; ++i) {
    float *f = &x[(size_t)i * kFeatures];
    program_features(e.ir, i, c.sm_count, f);
    for (int j = 0; j < kFeatures; ++j) f[j] = (f[j] - c.cost_mean[j]) * c.cost_inv_std[j];
  }
  size_t cls = 0;
  float *dx = static_cast<float *>(c.pool.alloc((x.size() + kTuneConfigs) * sizeof(float), &cls));
  std::vector<float> y(kTuneConfigs);
  try {
    mlp_reserve(c, m, kTuneConfigs);
    check_cuda(cudaMemcpyAsync(dx, x.data(), x.size() * sizeof(float), cudaMemcpyHostToDevice, c.stream), "upload");
    mlp_forward(c, m, dx, kTuneConfigs, dx + x.size(), c.stream);
    check_cuda(cudaMemcpyAsync(y.data(), dx + x.size(), y.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream),
               "download");
    check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  } catch (...) {
    release_block(c, dx, cls);
    throw;
  }
  release_block(c, dx, cls);
  int pick = -1;
  for (int i = 0; i < kTuneConfigs; ++i)
    if (tune_config_fits(e, i, in, out) && (pick < 0 || y[i] < y[pick])) pick = i;
  if (pick < 0) return kStdConfig;
  float t_pick = 0.0f, t_std = 0.0f;
  void *flush = c.pool.alloc(kFlushBytes, &cls);
  try {
    time_tune_entry(c, e, &pick, 1, in, out, 3, flush, kFlushBytes, &t_pick);
    t_std = time_standard(c, p, in, out, 3, flush, kFlushBytes);
  } catch (...) {
    release_block(c, flush, cls);
    throw;
  }
  release_block(c, flush, cls);
  return (t_pick >= 0.0f && t_pick < t_std) ? pick : kStdConfig;
}

TuneSet &tune_set_of(Context &c, uint64_t h) {
  auto it = c.tune_sets.find(h);
  if (tag_of(h) != kTagTuneSet || it == c.tune_sets.end()) fail(CC_ERR_INVALID_VALUE, "not a live tuning set handle");
  return *it->second;
}

std::vector<Ir> parse_tunable(const char *const *irs, const size_t *lens, int n) {
  if (!irs || !lens || n <= 0) fail(CC_ERR_INVALID_VALUE, "no programs");
  std::vector<Ir> out;
  out.reserve(n);
  for (int p = 0; p < n; ++p) {
    if (!irs[p]) fail(CC_ERR_INVALID_VALUE, "null program text");
    out.push_back(parse_ir(irs[p], lens[p]));
    std::string why;
    if (!is_tunable(out.back(), &why)) fail(CC_ERR_INVALID_PROGRAM, "program " + std::to_string(p) + ": " + why);
  }
  return out;
}

std::vector<std::string> tune_sources(const std::vector<Ir> &irs) {
  std::vector<std::string> sources;
  for (size_t first = 0; first < irs.size(); first += kTuneChunk) {
    std::ostringstream o;
    o << "// generated by compute.scala_gb300 for sm_103a (tunable forms)\n" << kPrelude << "\n";
    for (size_t p = first; p < irs.size() && p < first + kTuneChunk; ++p) o << tunable_source(irs[p], "_" + std::to_string(p));
    sources.push_back(o.str());
  }
  return sources;
}

std::shared_ptr<TuneModule> load_tune_module(const std::vector<char> &cubin) {
  auto m = std::make_shared<TuneModule>();
  check_cu(g_drv.ModuleLoadData(&m->module, cubin.data()), "cuModuleLoadData");
  return m;
}

void load_tune_entry(TuneEntry &e, const Ir &ir, std::shared_ptr<TuneModule> mod, const std::string &suffix) {
  e.mod = std::move(mod);
  int k = 0;
  for (int V : {1, 4})
    for (int E : {1, 2, 4}) {
      std::string name = "cc_t" + suffix + "_v" + std::to_string(V) + "_e" + std::to_string(E);
      check_cu(g_drv.ModuleGetFunction(&e.fn[k++], e.mod->module, name.c_str()), "cuModuleGetFunction");
    }
  e.kind = ir.kind;
  e.n_inputs = ir.n_params;
  e.n = 1;
  for (int64_t d : ir.out_shape) e.n *= d;
  e.contiguous = !contiguous_structure_key(ir).empty();
  e.ir = ir;
}

void launch_tuned_program(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream) {
  TuneEntry &e = *p.tune;
  if (p.tuned_config < 0 || (p.tuned_config < kTuneConfigs && !tune_config_fits(e, p.tuned_config, in, out))) {
    if (stream != c.stream) check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    end_pdl_chain(c);
    p.tuned_config = c.tuner == 2 ? choose_learned(c, p, in, out) : choose_exhaustive(c, p, in, out);
    end_pdl_chain(c);
  }
  if (p.tuned_config == kStdConfig) {
    launch_generated(c, p, in, out, stream);  // keeps the early-start chain going
  } else {
    end_pdl_chain(c);
    launch_tune_entry(c, e, p.tuned_config, in, out, stream);
  }
}

}  // namespace
}  // namespace cc

extern "C" {

int cc_tune_config(int index, int *block, int *vec, int *ept, int *split) {
  CC_API_BEGIN
  if (index < 0 || index >= kTuneConfigs) fail(CC_ERR_INVALID_VALUE, "configuration index out of range");
  TuneConfig t = tune_config(index);
  if (block) *block = t.block;
  if (vec) *vec = t.vec;
  if (ept) *ept = t.ept;
  if (split) *split = t.split;
  CC_API_END
}

int cc_program_features(const char *ir_text, size_t ir_len, int config, int sm_count, float *out) {
  CC_API_BEGIN
  if (!ir_text || !out) fail(CC_ERR_INVALID_VALUE, "null pointer");
  if (config < 0 || config >= kTuneConfigs) fail(CC_ERR_INVALID_VALUE, "configuration index out of range");
  Ir ir = parse_ir(ir_text, ir_len);
  std::string why;
  if (!is_tunable(ir, &why)) fail(CC_ERR_INVALID_PROGRAM, why);
  program_features(ir, config, sm_count, out);
  CC_API_END
}

int cc_tune_compile_check(const char *const *irs, const size_t *lens, int n_programs, int cc_major, int cc_minor,
                          double *seconds) {
  CC_API_BEGIN
  auto t0 = std::chrono::steady_clock::now();
  std::vector<Ir> parsed = parse_tunable(irs, lens, n_programs);
  compile_parallel(tune_sources(parsed), cc_major, cc_minor, 0, false, 0);
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  CC_API_END
}

int cc_tune_create(const char *const *irs, const size_t *lens, int n_programs, cc_handle *set) {
  CC_API_BEGIN
  if (!set) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::vector<Ir> parsed = parse_tunable(irs, lens, n_programs);
  std::vector<std::vector<char>> cubins;
  {
    std::lock_guard<std::mutex> cg(c.compile_mu);
    FmaScope fma_scope((c.flags & CC_FLAG_FMA_CONTRACT) != 0);
    cubins = compile_parallel(tune_sources(parsed), c.cc_major, c.cc_minor, c.flags, false, 0);
  }
  auto ts = std::make_unique<TuneSet>();
  ts->entries.resize(parsed.size());
  for (size_t u = 0; u < cubins.size(); ++u) {
    auto mod = load_tune_module(cubins[u]);
    for (size_t p = u * kTuneChunk; p < parsed.size() && p < (u + 1) * kTuneChunk; ++p)
      load_tune_entry(ts->entries[p], parsed[p], mod, "_" + std::to_string(p));
  }
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  uint64_t h = c.make_handle(kTagTuneSet);
  c.tune_sets[h] = ts.release();
  *set = h;
  CC_API_END
}

namespace {
std::vector<uint64_t> tune_ptrs(const TuneEntry &e, const uint64_t *ptrs, size_t n_ptrs) {
  if (!ptrs || n_ptrs != (size_t)e.n_inputs + 1)
    fail(CC_ERR_INVALID_KERNEL_ARGS, "the program needs " + std::to_string(e.n_inputs + 1) + " pointers (inputs, then the output)");
  for (size_t i = 0; i < n_ptrs; ++i)
    if (!ptrs[i]) fail(CC_ERR_INVALID_VALUE, "null pointer");
  return std::vector<uint64_t>(ptrs, ptrs + e.n_inputs);
}
}  // namespace

int cc_tune_info(cc_handle set, int *n_programs) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  TuneSet &ts = tune_set_of(c, set);
  if (n_programs) *n_programs = (int)ts.entries.size();
  CC_API_END
}

int cc_tune_launch(cc_handle set, int program, const uint64_t *ptrs, size_t n_ptrs, int config, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  TuneSet &ts = tune_set_of(c, set);
  if (program < 0 || program >= (int)ts.entries.size()) fail(CC_ERR_INVALID_VALUE, "program index out of range");
  TuneEntry &e = ts.entries[program];
  std::vector<uint64_t> in = tune_ptrs(e, ptrs, n_ptrs);
  launch_tune_entry(c, e, config, in, ptrs[e.n_inputs], stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream);
  CC_API_END
}

int cc_tune_time(cc_handle set, int program, const uint64_t *ptrs, size_t n_ptrs, const int *configs, int n_configs,
                 int reps, int flush_l2, float *ms) {
  CC_API_BEGIN
  if (!configs || !ms || n_configs <= 0) fail(CC_ERR_INVALID_VALUE, "no configurations");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  TuneSet &ts = tune_set_of(c, set);
  if (program < 0 || program >= (int)ts.entries.size()) fail(CC_ERR_INVALID_VALUE, "program index out of range");
  TuneEntry &e = ts.entries[program];
  std::vector<uint64_t> in = tune_ptrs(e, ptrs, n_ptrs);
  if (flush_l2 && !ts.flush) {
    ts.flush = c.pool.alloc(kFlushBytes, &ts.flush_cls);
    ts.flush_bytes = kFlushBytes;
  }
  time_tune_entry(c, e, configs, n_configs, in, ptrs[e.n_inputs], reps, flush_l2 ? ts.flush : nullptr, ts.flush_bytes,
                  ms);
  CC_API_END
}

int cc_tune_release(cc_handle set) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  TuneSet &ts = tune_set_of(c, set);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  if (ts.flush) release_block(c, ts.flush, ts.flush_cls);
  delete &ts;
  c.tune_sets.erase(set);
  CC_API_END
}

int cc_tuner_choice(cc_handle prog, int *config) {
  CC_API_BEGIN
  if (!config) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Program &p = program_of(c, prog);
  *config = p.tune ? p.tuned_config : -1;
  CC_API_END
}

// ---- the cost model's network

int cc_mlp_create(const int *dims, int n_dims, cc_handle *mlp) {
  CC_API_BEGIN
  if (!dims || !mlp || n_dims < 2 || n_dims > 16) fail(CC_ERR_INVALID_VALUE, "a network has 2 to 16 widths");
  Context &c = ctx();
  auto m = std::make_unique<Mlp>();
  m->dims.assign(dims, dims + n_dims);
  m->w_off.assign(n_dims, 0);
  m->b_off.assign(n_dims, 0);
  size_t off = 0;
  for (int l = 1; l < n_dims; ++l) {
    if (dims[l - 1] <= 0 || dims[l] <= 0 || dims[l] > 65536) fail(CC_ERR_INVALID_VALUE, "widths must be in [1, 65536]");
    m->w_off[l] = off;
    off += (size_t)dims[l - 1] * dims[l];
    m->b_off[l] = off;
    off += (size_t)dims[l];
  }
  m->n_params = off;
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  m->state = c.pool.alloc(4 * off * sizeof(float), &m->state_cls);
  check_cuda(cudaMemsetAsync(m->state, 0, 4 * off * sizeof(float), c.stream), "cudaMemsetAsync");
  uint64_t h = c.make_handle(kTagMlp);
  c.mlps[h] = m.release();
  *mlp = h;
  CC_API_END
}

int cc_mlp_info(cc_handle mlp, size_t *n_params, int *steps) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Mlp &m = mlp_of(c, mlp);
  if (n_params) *n_params = m.n_params;
  if (steps) *steps = m.steps;
  CC_API_END
}

int cc_mlp_set_params(cc_handle mlp, const float *host, size_t n) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Mlp &m = mlp_of(c, mlp);
  if (!host || n != m.n_params) fail(CC_ERR_INVALID_VALUE, "expected " + std::to_string(m.n_params) + " parameters");
  check_cuda(cudaMemcpyAsync(m.params(), host, n * sizeof(float), cudaMemcpyHostToDevice, c.stream), "upload");
  check_cuda(cudaMemsetAsync(m.adam_m(), 0, 2 * n * sizeof(float), c.stream), "cudaMemsetAsync");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  m.steps = 0;
  CC_API_END
}

int cc_mlp_get_params(cc_handle mlp, float *host, size_t n) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Mlp &m = mlp_of(c, mlp);
  if (!host || n != m.n_params) fail(CC_ERR_INVALID_VALUE, "expected " + std::to_string(m.n_params) + " parameters");
  check_cuda(cudaMemcpyAsync(host, m.params(), n * sizeof(float), cudaMemcpyDeviceToHost, c.stream), "download");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  CC_API_END
}

int cc_mlp_forward(cc_handle mlp, uint64_t x, int batch, uint64_t y, uint64_t stream) {
  CC_API_BEGIN
  if (!x || !y || batch <= 0) fail(CC_ERR_INVALID_VALUE, "null pointer or empty batch");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Mlp &m = mlp_of(c, mlp);
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  if (s != c.stream) check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  mlp_reserve(c, m, batch);
  mlp_forward(c, m, reinterpret_cast<const float *>(x), batch, reinterpret_cast<float *>(y), s);
  if (s != c.stream) check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");  // the scratch is the context's
  CC_API_END
}

int cc_mlp_gradients(cc_handle mlp, uint64_t x, uint64_t t, int batch, float *loss, float *grads) {
  CC_API_BEGIN
  if (!x || !t || batch <= 0) fail(CC_ERR_INVALID_VALUE, "null pointer or empty batch");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Mlp &m = mlp_of(c, mlp);
  mlp_reserve(c, m, batch);
  mlp_backward(c, m, reinterpret_cast<const float *>(x), reinterpret_cast<const float *>(t), batch, c.stream);
  if (loss)
    check_cuda(cudaMemcpyAsync(loss, mlp_loss(m), sizeof(float), cudaMemcpyDeviceToHost, c.stream), "download");
  if (grads)
    check_cuda(cudaMemcpyAsync(grads, m.grads(), m.n_params * sizeof(float), cudaMemcpyDeviceToHost, c.stream),
               "download");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  CC_API_END
}

int cc_mlp_train_step(cc_handle mlp, uint64_t x, uint64_t t, int batch, float lr, float beta1, float beta2, float eps,
                      float *loss) {
  CC_API_BEGIN
  if (!x || !t || batch <= 0) fail(CC_ERR_INVALID_VALUE, "null pointer or empty batch");
  if (!(lr > 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
    fail(CC_ERR_INVALID_VALUE, "Adam needs lr > 0, betas in [0, 1) and eps > 0");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  Mlp &m = mlp_of(c, mlp);
  mlp_reserve(c, m, batch);
  mlp_backward(c, m, reinterpret_cast<const float *>(x), reinterpret_cast<const float *>(t), batch, c.stream);
  ++m.steps;
  const float c1 = (float)(1.0 - std::pow((double)beta1, (double)m.steps));
  const float c2 = (float)(1.0 - std::pow((double)beta2, (double)m.steps));
  check_cuda(launch_adam(m.params(), m.grads(), m.adam_m(), m.adam_v(), (long long)m.n_params, lr, beta1, beta2, eps,
                         c1, c2, c.sm_count, c.stream),
             "adam");
  if (loss) {
    check_cuda(cudaMemcpyAsync(loss, mlp_loss(m), sizeof(float), cudaMemcpyDeviceToHost, c.stream), "download");
    check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  }
  CC_API_END
}

int cc_mlp_release(cc_handle mlp) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Mlp &m = mlp_of(c, mlp);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  if (m.scratch) release_block(c, m.scratch, m.scratch_cls);
  release_block(c, m.state, m.state_cls);
  if (c.cost_model == mlp) c.cost_model = 0;
  delete &m;
  c.mlps.erase(mlp);
  CC_API_END
}

int cc_tuner_set_model(cc_handle mlp, const float *mean, const float *inv_std) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  end_pdl_chain(c);
  if (!mlp) {
    c.cost_model = 0;
    return CC_OK;
  }
  Mlp &m = mlp_of(c, mlp);
  if (m.dims.front() != kFeatures || m.dims.back() != 1)
    fail(CC_ERR_INVALID_VALUE, "a cost model maps " + std::to_string(kFeatures) + " features to one value");
  if (!mean || !inv_std) fail(CC_ERR_INVALID_VALUE, "null pointer");
  c.cost_mean.assign(mean, mean + kFeatures);
  c.cost_inv_std.assign(inv_std, inv_std + kFeatures);
  c.cost_model = mlp;
  CC_API_END
}

}  // extern "C"
