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
#include <cstring>
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

namespace cc {

namespace {
thread_local std::string t_last_error;
}

void fail(int code, const std::string &message) { throw Error{code, message}; }

void record_error(const std::string &message) { t_last_error = message; }

// Driver API entry points, resolved through the CUDA runtime at cc_init so the
// library loads (and its GPU-free entry points work) on hosts without a driver.
Driver g_drv;

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

// ---------------------------------------------------------------- buffer pool
//
// Blocks are binned by size class (eight classes per power of two above 4 KiB,
// so at most 12.5% slack).  A released block goes back to its class's free
// list; work is ordered on the context stream, so a later allocation may reuse
// it at once.  A cap (cc_pool_set_limit) turns allocations past it into
// CC_ERR_OUT_OF_MEMORY, the reference's MemObjectAllocationFailure.
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

  void release(void *p, size_t cls) {
    in_use_ -= cls;
    cached_ += cls;
    free_[cls].push_back(p);
  }

  void trim() {
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
  std::map<size_t, std::vector<void *>> free_;
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
  int block = 256;              // threads per block the kernels were generated for
  int resident_scalar = 0;      // blocks one SM holds at once, per variant
  int resident_vec4 = 0;
  int vec_unroll = 1;
  std::string source;
  ~Module() {
    if (module && g_drv.ModuleUnload) g_drv.ModuleUnload(module);
  }
};

struct Program {
  std::shared_ptr<Module> mod;
  ProgramKind kind = ProgramKind::Elementwise;
  Generated gen;                // shape information (its source lives in the module)
  bool is_contraction = false;  // run as a GEMM (cc_gemm_f32 mode contraction_mode)
  int contraction_mode = 0;
  Contraction con;
};

struct Event {
  cudaEvent_t ev = nullptr;
};

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
};

enum : uint64_t { kTagBuffer = 1, kTagProgram = 2, kTagEvent = 3, kTagBatch = 4 };

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
  Pool pool;
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, Buffer *> buffers;
  std::unordered_map<uint64_t, Program *> programs;   // by handle
  std::unordered_map<std::string, uint64_t> cache;    // IR text -> program handle
  std::unordered_map<std::string, std::shared_ptr<Module>> modules;  // structure key -> module
  std::unordered_map<uint64_t, Event *> events;
  std::unordered_map<uint64_t, Batch *> batches;
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
  int tc_variant = 0;
  int contraction = 1;  // 0: generated fold kernel; else CC_GEMM_* mode + 1
  int batch_inline = 0;
  int batch_max_registers = 0;
  cudaStream_t copy_streams[8] = {};
  cudaEvent_t copy_events[9] = {};

  // Scratch of the grid sums: kMaxSumBlocks float2 partials, then the counter.
  void *sum_scratch = nullptr;
  size_t sum_scratch_cls = 0;

  uint64_t make_handle(uint64_t tag) { return (tag << 56) | (next_id++); }
  float2 *partials() { return reinterpret_cast<float2 *>(sum_scratch); }
  unsigned int *counter() {
    return reinterpret_cast<unsigned int *>(static_cast<char *>(sum_scratch) + sizeof(float2) * kMaxSumBlocks);
  }
  // Device error flag of the kernels with bounded waits (in the same scratch block).
  int *error_flag() {
    return reinterpret_cast<int *>(static_cast<char *>(sum_scratch) + sizeof(float2) * kMaxSumBlocks + 128);
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

// ---------------------------------------------------------------- NVRTC

std::vector<char> compile_cubin(const std::string &source, int cc_major, int cc_minor, uint32_t flags,
                                bool relocatable = false, int max_registers = 0) {
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "cc_program.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) fail(CC_ERR_BUILD_PROGRAM_FAILURE, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
  std::string arch = "-arch=sm_" + std::to_string(cc_major) + std::to_string(cc_minor) + "a";
  std::vector<std::string> opts = {arch, "--std=c++17", "-default-device",
                                   (flags & CC_FLAG_FMA_CONTRACT) ? "--fmad=true" : "--fmad=false"};
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
    c.pool.release(pa, cls_a);
    throw;
  }
  cudaError_t e = launch_split_a(A, lda, m, k, static_cast<__nv_bfloat16 *>(pa), Mp, Kp, c.sm_count, s);
  if (e == cudaSuccess) e = launch_split_bt(B, ldb, k, n, static_cast<__nv_bfloat16 *>(pb), Np, Kp, s);
  if (e == cudaSuccess) {
    CUtensorMap maps[6];
    const size_t plane_a = (size_t)Mp * Kp * 2, plane_b = (size_t)Np * Kp * 2;
    try {
      for (int p = 0; p < 3; ++p) {
        encode_plane_map(&maps[p], static_cast<char *>(pa) + p * plane_a, Mp, Kp, kTcBM);
        encode_plane_map(&maps[3 + p], static_cast<char *>(pb) + p * plane_b, Np, Kp, gemm_tc_box_n(c.tc_variant));
      }
    } catch (...) {
      c.pool.release(pa, cls_a);
      c.pool.release(pb, cls_b);
      throw;
    }
    e = launch_gemm_bf16x6(maps, C, m, n, Kp, ldc, c.sm_count, c.error_flag(), c.tc_variant, s);
  }
  if (s != c.stream && e == cudaSuccess) e = cudaStreamSynchronize(s);  // the pool is ordered on the context stream
  c.pool.release(pa, cls_a);
  c.pool.release(pb, cls_b);
  check_cuda(e, "bf16x6 contraction launch");
}

void launch_program(Context &c, Program &p, const std::vector<uint64_t> &in, uint64_t out, cudaStream_t stream) {
  if (p.is_contraction) {
    const Contraction &q = p.con;
    run_gemm(c, reinterpret_cast<const float *>(in[q.a_input]), reinterpret_cast<const float *>(in[q.b_input]),
             reinterpret_cast<float *>(out), (int)q.m, (int)q.n, (int)q.k, q.k, q.n, q.n, p.contraction_mode, stream);
    return;
  }
  const Module &m = *p.mod;
  const int block = m.block;
  const int64_t n = p.gen.domain;
  bool aligned = (out & 15u) == 0;
  for (uint64_t a : in) aligned = aligned && (a & 15u) == 0;
  const bool vec = m.vec4 && aligned;
  CUfunction f = vec ? m.vec4 : m.scalar;
  // float4 kernels: each thread takes vec_unroll positions per batch
  const int64_t work = vec ? ((n >> 2) + m.vec_unroll - 1) / m.vec_unroll : n;
  std::vector<void *> args;
  std::vector<uint64_t> ptrs(in);
  for (auto &v : ptrs) args.push_back(&v);
  uint64_t out_ptr = out;
  int64_t nn = n;
  uint64_t partials = 0, counter = 0;
  unsigned grid;
  if (p.kind == ProgramKind::Sum) {
    partials = reinterpret_cast<uint64_t>(c.partials());
    counter = reinterpret_cast<uint64_t>(c.counter());
    args.push_back(&partials);
    args.push_back(&counter);
    grid = (unsigned)sum_grid_for(work, block, c.sm_count * c.sum_blocks_per_sm);
  } else {
    if (n == 0) return;
    int resident = vec ? m.resident_vec4 : m.resident_scalar;
    if (c.ew_blocks_per_sm > 0 && (resident <= 0 || c.ew_blocks_per_sm < resident)) resident = c.ew_blocks_per_sm;
    grid = (unsigned)ew_grid(work, block, c.sm_count, resident);
  }
  args.push_back(&out_ptr);
  args.push_back(&nn);
  check_cu(g_drv.LaunchKernel(f, grid, 1, 1, block, 1, 1, 0, (CUstream)stream, args.data(), nullptr),
           "cuLaunchKernel");
}

// Upload striped over the context's copy streams, ordered after the work
// queued on the main stream and joined back into it.
void striped_upload(Context &c, char *dst, const char *src, size_t bytes) {
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
    g_ctx->flags = flags;
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
  for (auto &kv : c->programs) delete kv.second;
  c->modules.clear();
  for (auto &kv : c->buffers) {
    cudaFree(kv.second->ptr);
    delete kv.second;
  }
  for (auto &kv : c->events) {
    cudaEventDestroy(kv.second->ev);
    delete kv.second;
  }
  c->pool.release(c->sum_scratch, c->sum_scratch_cls);
  c->pool.trim();
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
  } else if (k == "batch_max_registers") {
    if (value < 0 || value > 255) fail(CC_ERR_INVALID_VALUE, "batch_max_registers must be in [0, 255]");
    c.batch_max_registers = (int)value;
  } else if (k == "batch_inline") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "batch_inline must be 0, 1 or 2");
    c.batch_inline = (int)value;
  } else if (k == "contraction") {
    if (value < 0 || value > 3) fail(CC_ERR_INVALID_VALUE, "contraction must be in [0, 3]");
    c.contraction = (int)value;
  } else if (k == "tc_variant") {
    if (value < 0 || value > 2) fail(CC_ERR_INVALID_VALUE, "tc_variant must be 0, 1 or 2");
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
  else if (k == "batch_inline") *value = c.batch_inline;
  else if (k == "batch_max_registers") *value = c.batch_max_registers;
  else fail(CC_ERR_INVALID_VALUE, "unknown config key '" + k + "'");
  CC_API_END
}

int cc_synchronize(void) {
  CC_API_BEGIN
  check_cuda(cudaStreamSynchronize(ctx().stream), "cudaStreamSynchronize");
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
    c.pool.release(b.ptr, b.cls);
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

int cc_buf_download(cc_handle h, size_t offset, void *host, size_t bytes) {
  CC_API_BEGIN
  Context &c = ctx();
  void *src;
  {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    Buffer &b = buffer_of(c, h);
    if (offset > b.bytes || bytes > b.bytes - offset) fail(CC_ERR_INVALID_VALUE, "download range exceeds the buffer");
    src = static_cast<char *>(b.ptr) + offset;
  }
  if (bytes == 0) return CC_OK;
  if (!host) fail(CC_ERR_INVALID_VALUE, "null host pointer");
  check_cuda(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, c.stream), "cudaMemcpyAsync D2H");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  CC_API_END
}

int cc_host_alloc(size_t bytes, void **host) {
  CC_API_BEGIN
  if (!host) fail(CC_ERR_INVALID_VALUE, "null pointer");
  ctx();
  check_cuda(cudaMallocHost(host, bytes ? bytes : 1), "cudaMallocHost");
  CC_API_END
}

int cc_host_free(void *host) {
  CC_API_BEGIN
  ctx();
  if (host) check_cuda(cudaFreeHost(host), "cudaFreeHost");
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
  }
  key += "#lookahead " + std::to_string(opt.load_lookahead) + " asm " + std::to_string((int)opt.asm_loads) +
         " blocks " + std::to_string(-opt.min_blocks) + " block " + std::to_string(opt.block) + " unroll " + std::to_string(opt.vec_unroll) +
         " prefetch " + std::to_string(opt.prefetch_min_bytes) + " sumblock " + std::to_string(c.sum_block) +
         " contraction " + std::to_string(c.contraction) + " tc " + std::to_string(c.tc_variant) + "\n";
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
  int64_t domain = 1;
  for (int64_t d : ir.out_shape) domain *= d;
  // Contiguous programs compile once per structure; the shape only sizes the launch.
  std::string skey = contiguous_structure_key(ir);
  if (!skey.empty()) {
    skey += key.substr(key.rfind('#'));
    opt.min_blocks = 0;
  } else {
    opt.min_blocks = choose_min_blocks(domain, opt.block, c.sm_count, -opt.min_blocks);
  }
  auto p = std::make_unique<Program>();
  p->kind = ir.kind;
  std::shared_ptr<Module> mod;
  if (!skey.empty()) {
    std::lock_guard<std::recursive_mutex> g(c.mu);
    auto it = c.modules.find(skey);
    if (it != c.modules.end()) mod = it->second;
  }
  if (mod) {
    p->gen = describe_program(ir);
  } else {
    p->gen = generate_cuda(ir, opt);
    mod = std::make_shared<Module>();
    mod->source = p->gen.source;
    std::vector<char> cubin = compile_cubin(mod->source, c.cc_major, c.cc_minor, c.flags);
    check_cu(g_drv.ModuleLoadData(&mod->module, cubin.data()), "cuModuleLoadData");
    const char *sname = ir.kind == ProgramKind::Sum ? "cc_sum" : "cc_ew";
    const char *vname = ir.kind == ProgramKind::Sum ? "cc_sum_v4" : "cc_ew_v4";
    check_cu(g_drv.ModuleGetFunction(&mod->scalar, mod->module, sname), "cuModuleGetFunction");
    if (p->gen.has_vec4) check_cu(g_drv.ModuleGetFunction(&mod->vec4, mod->module, vname), "cuModuleGetFunction");
    mod->block = opt.block;
    mod->vec_unroll = p->gen.vec_unroll;
    check_cu(g_drv.OccupancyMaxActiveBlocks(&mod->resident_scalar, mod->scalar, mod->block, 0),
             "cuOccupancyMaxActiveBlocks");
    if (mod->vec4)
      check_cu(g_drv.OccupancyMaxActiveBlocks(&mod->resident_vec4, mod->vec4, mod->block, 0),
               "cuOccupancyMaxActiveBlocks");
    if (!skey.empty()) {
      std::lock_guard<std::recursive_mutex> g(c.mu);
      c.modules[skey] = mod;
    }
  }
  p->mod = mod;
  std::lock_guard<std::recursive_mutex> g(c.mu);
  uint64_t h = c.make_handle(kTagProgram);
  c.programs[h] = p.release();
  c.cache[key] = h;
  ++c.cache_misses;
  *out = h;
  CC_API_END
}

int cc_codegen(const char *ir_text, size_t ir_len, char *buf, size_t len, size_t *needed) {
  CC_API_BEGIN
  if (!ir_text) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Ir ir = parse_ir(ir_text, ir_len);
  Generated gen = generate_cuda(ir, CodegenOptions{});
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
  CC_API_BEGIN
  if (!ir_text) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Ir ir = parse_ir(ir_text, ir_len);
  Generated gen = generate_cuda(ir, CodegenOptions{});
  compile_cubin(gen.source, cc_major, cc_minor, flags);
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

// ---------------------------------------------------------------- sums and random numbers

int cc_reduce_sum_f32(uint64_t in_ptr, size_t n, uint64_t out_ptr, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  if (!out_ptr || (n && !in_ptr)) fail(CC_ERR_INVALID_VALUE, "null pointer");
  std::lock_guard<std::recursive_mutex> g(c.mu);
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
  if (s != c.stream && e == cudaSuccess) e = cudaStreamSynchronize(s);  // the pool is ordered on the context stream
  c.pool.release(scratch, cls);
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
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  run_gemm(c, reinterpret_cast<const float *>(a_ptr), reinterpret_cast<const float *>(b_ptr),
           reinterpret_cast<float *>(c_ptr), m, n, k, lda, ldb, ldc, mode, s);
  CC_API_END
}

int cc_device_errors(int *code) {
  CC_API_BEGIN
  if (!code) fail(CC_ERR_INVALID_VALUE, "null pointer");
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
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
  cudaEventDestroy(e.ev);
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
extern const char *kPrelude;
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
// The parts compile in parallel (relocatable code) and the driver links them.
constexpr int kBatchChunk = 32;

const char *kTileParams =
    "(const float *__restrict__ in0, const float *__restrict__ in1, const float *__restrict__ in2, "
    "const float *__restrict__ in3, float *__restrict__ out, long long n, long long base)";

// inline_level: 0 = the expression is a called function and so are exp/log/tanh;
// 1 = the expression is inlined into its tile function, exp/log/tanh called;
// 2 = everything inlined.  Higher levels run faster and compile slower.
std::string batch_chunk_source(const std::vector<Ir> &structs, const std::vector<int> &struct_inputs, size_t first,
                               size_t last, int inline_level) {
  std::ostringstream o;
  o << "// generated batch part for sm_103a\n"
    << "static __device__ __noinline__ float cc_expf(float x) { return expf(x); }\n"
       "static __device__ __noinline__ float cc_logf(float x) { return logf(x); }\n"
       "static __device__ __noinline__ float cc_tanhf(float x) { return tanhf(x); }\n";
  const std::string B = std::to_string(kBatchBlock);
  for (size_t s = first; s < last; ++s) {
    const int nin = struct_inputs[s];
    const std::string S = std::to_string(s);
    std::string pf = point_function(structs[s], "cc_point_" + S, inline_level >= 1, inline_level <= 1);
    o << "static " << pf;
    auto call = [&](const std::string &suffix) {
      std::string c = "cc_point_" + S + "(";
      for (int i = 0; i < kBatchMaxInputs; ++i)
        c += (i ? ", " : "") + (i < nin ? "v" + std::to_string(i) + suffix : std::string("0.0f"));
      return c + ")";
    };
    // A full tile loads all its float4s before computing any, so every thread
    // has kBatchUnroll loads per input in flight; the ragged last tile of a
    // program takes the plain loops.
    o << "extern \"C\" __device__ __noinline__ void cc_tile_" << S << kTileParams << " {\n"
      << "  if (base + " << kBatchTile << "LL <= n) {\n"
      << "    const long long q0 = (base >> 2) + threadIdx.x;\n";
    for (int i = 0; i < nin; ++i)
      for (int u = 0; u < kBatchUnroll; ++u)
        o << "    const float4 v" << i << "_" << u << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q0 + "
          << u * kBatchBlock << ");\n";
    for (int u = 0; u < kBatchUnroll; ++u) {
      const std::string U = "_" + std::to_string(u);
      o << "    float4 r" << U << ";\n";
      for (const char *lane : {".x", ".y", ".z", ".w"})
        o << "    r" << U << lane << " = " << call(U + lane) << ";\n";
    }
    for (int u = 0; u < kBatchUnroll; ++u)
      o << "    reinterpret_cast<float4 *>(out)[q0 + " << u * kBatchBlock << "] = r_" << u << ";\n";
    o << "    return;\n  }\n"
      << "  const long long end = base + " << kBatchTile << "LL < n ? base + " << kBatchTile << "LL : n;\n"
      << "  const long long end4 = end & ~3LL;\n"
      << "  for (long long q = (base >> 2) + threadIdx.x; (q << 2) < end4; q += " << B << ") {\n";
    for (int i = 0; i < nin; ++i)
      o << "    const float4 v" << i << " = __ldg(reinterpret_cast<const float4 *>(in" << i << ") + q);\n";
    o << "    float4 r;\n";
    for (const char *lane : {".x", ".y", ".z", ".w"}) o << "    r" << lane << " = " << call(lane) << ";\n";
    o << "    reinterpret_cast<float4 *>(out)[q] = r;\n  }\n"
      << "  for (long long i = end4 + threadIdx.x; i < end; i += " << B << ") {\n";
    for (int i = 0; i < nin; ++i) o << "    const float v" << i << " = __ldg(in" << i << " + i);\n";
    o << "    out[i] = " << call("") << ";\n  }\n}\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << B << ") cc_prog_" << S
      << "(const float *__restrict__ in0, const float *__restrict__ in1, const float *__restrict__ in2, "
         "const float *__restrict__ in3, float *__restrict__ out, long long n) {\n"
      << "  const long long tiles = (n + " << kBatchTile - 1 << "LL) / " << kBatchTile << "LL;\n"
      << "  for (long long t = blockIdx.x; t < tiles; t += gridDim.x) cc_tile_" << S
      << "(in0, in1, in2, in3, out, n, t * " << kBatchTile << "LL);\n}\n";
  }
  return o.str();
}

std::string batch_main_source(size_t n_structs) {
  std::ostringstream o;
  o << "// generated batch main part for sm_103a\n"
    << "struct cc_entry { const float *in[4]; float *out; long long n; long long tile_begin; int sid; int pad; };\n"
    << "typedef void (*cc_tile_fn)" << kTileParams << ";\n";
  for (size_t s = 0; s < n_structs; ++s) o << "extern \"C\" __device__ void cc_tile_" << s << kTileParams << ";\n";
  o << "__device__ cc_tile_fn const cc_tiles[" << n_structs << "] = {\n";
  for (size_t s = 0; s < n_structs; ++s) o << "  cc_tile_" << s << ",\n";
  o << "};\n"
    << "extern \"C\" __global__ void __launch_bounds__(" << kBatchBlock
    << ") cc_batch(const cc_entry *__restrict__ table, int nprog, long long total_tiles) {\n"
    << "  extern __shared__ long long s_begin[];\n"
    << "  for (int i = threadIdx.x; i < nprog; i += blockDim.x) s_begin[i] = table[i].tile_begin;\n"
    << "  __syncthreads();\n"
    << "  for (long long t = blockIdx.x; t < total_tiles; t += gridDim.x) {\n"
    << "    int lo = 0, hi = nprog - 1;\n"
    << "    while (lo < hi) {\n      const int mid = (lo + hi + 1) >> 1;\n"
    << "      if (s_begin[mid] <= t) lo = mid; else hi = mid - 1;\n    }\n"
    << "    const cc_entry e = table[lo];\n"
    << "    const long long base = (t - e.tile_begin) * " << kBatchTile << "LL;\n"
    << "    if (e.sid >= 0 && e.sid < " << n_structs << ") cc_tiles[e.sid](e.in[0], e.in[1], e.in[2], e.in[3], e.out, e.n, base);\n"
    << "  }\n}\n";
  return o.str();
}

// Compiles the parts in parallel and links them into one loadable image.
std::vector<char> build_batch_image(const std::vector<Ir> &structs, const std::vector<int> &struct_inputs,
                                    int cc_major, int cc_minor, uint32_t flags, bool link, int inline_level,
                                    int max_registers) {
  std::vector<std::string> sources;
  for (size_t first = 0; first < structs.size(); first += kBatchChunk)
    sources.push_back(batch_chunk_source(structs, struct_inputs, first,
                                         std::min(structs.size(), first + (size_t)kBatchChunk), inline_level));
  sources.push_back(batch_main_source(structs.size()));
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
          parts[i] = compile_cubin(sources[i], cc_major, cc_minor, flags, true, max_registers);
        } catch (const Error &e) {
          errors[i] = e.message;
        }
      }
    });
  }
  for (auto &th : pool) th.join();
  for (auto &e : errors)
    if (!e.empty()) fail(CC_ERR_BUILD_PROGRAM_FAILURE, e);
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
                              c.batch_max_registers);
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
  build_batch_image(structs, struct_inputs, cc_major, cc_minor, 0, false, 0, 0);  // linking needs a driver
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
  if (!b.table) b.table = c.pool.alloc(sizeof(BatchEntry) * table.size(), &b.table_cls);
  check_cuda(cudaMemcpyAsync(b.table, table.data(), sizeof(BatchEntry) * table.size(), cudaMemcpyHostToDevice, c.stream),
             "upload batch table");
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  b.ptrs = std::move(bound);
  b.total_tiles = tiles;
  b.bound = true;
  batch_drop_graph(b);
  CC_API_END
}

int cc_batch_run(cc_handle batch, int mode, uint64_t stream) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  if (!b.bound) fail(CC_ERR_INVALID_OPERATION, "bind the batch's buffers first");
  cudaStream_t s = stream ? reinterpret_cast<cudaStream_t>(stream) : c.stream;
  if (mode == CC_BATCH_PERSISTENT) {
    if (b.total_tiles == 0) return CC_OK;
    uint64_t table = reinterpret_cast<uint64_t>(b.table);
    int nprog = (int)b.sid.size();
    long long total = b.total_tiles;
    void *args[] = {&table, &nprog, &total};
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

int cc_batch_release(cc_handle batch) {
  CC_API_BEGIN
  Context &c = ctx();
  std::lock_guard<std::recursive_mutex> g(c.mu);
  Batch &b = batch_of(c, batch);
  check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
  batch_drop_graph(b);
  if (b.table) c.pool.release(b.table, b.table_cls);
  g_drv.ModuleUnload(b.module);
  delete &b;
  c.batches.erase(batch);
  CC_API_END
}

}  // extern "C"
