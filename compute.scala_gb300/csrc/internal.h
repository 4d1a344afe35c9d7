// Internal declarations shared by the runtime translation units.
#pragma once

#include <cuda.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/compute_cuda.h"

namespace cc {

// A failure carried to the C ABI boundary, where it becomes a status code and
// the thread's last-error message.
struct Error {
  int code;
  std::string message;
};

[[noreturn]] void fail(int code, const std::string &message);

// Stores `message` as the calling thread's last error (what cc_last_error returns).
void record_error(const std::string &message);

// Driver API functions the runtime uses, resolved at cc_init through
// cudaGetDriverEntryPointByVersion (the library itself does not link libcuda).
struct Driver {
  bool loaded = false;
  decltype(&::cuModuleLoadData) ModuleLoadData = nullptr;
  decltype(&::cuModuleGetFunction) ModuleGetFunction = nullptr;
  decltype(&::cuModuleUnload) ModuleUnload = nullptr;
  decltype(&::cuLaunchKernel) LaunchKernel = nullptr;
  decltype(&::cuLaunchKernelEx) LaunchKernelEx = nullptr;
  decltype(&::cuGetErrorName) GetErrorName = nullptr;
  decltype(&::cuGetErrorString) GetErrorString = nullptr;
  decltype(&::cuCtxGetCurrent) CtxGetCurrent = nullptr;
  decltype(&::cuCtxSetCurrent) CtxSetCurrent = nullptr;
  decltype(&::cuFuncSetAttribute) FuncSetAttribute = nullptr;
  decltype(&::cuFuncGetAttribute) FuncGetAttribute = nullptr;
  decltype(&::cuTensorMapEncodeTiled) TensorMapEncodeTiled = nullptr;
  decltype(&::cuOccupancyMaxActiveBlocksPerMultiprocessor) OccupancyMaxActiveBlocks = nullptr;
  decltype(&::cuLinkCreate) LinkCreate = nullptr;
  decltype(&::cuLinkAddData) LinkAddData = nullptr;
  decltype(&::cuLinkComplete) LinkComplete = nullptr;
  decltype(&::cuLinkDestroy) LinkDestroy = nullptr;
};
extern Driver g_drv;

// Operations enqueued by entry points that run without the context lock (the
// sum without a context, cc_reduce_sum_f32_noalloc): a generated kernel starts
// its loads early only if this count has not moved since the previous
// generated kernel was launched.
extern std::atomic<uint64_t> g_foreign_enqueues;

// ---- IR (the alpha-converted expression tree; format documented in compute/trees.py)
enum class NodeKind : uint8_t { Param, Literal, Extract, View, Unary, Binary, Tuple };
enum class UnOp : uint8_t { Neg, Exp, Log, Tanh, Abs, Sqrt };
enum class BinOp : uint8_t { Add, Sub, Mul, Div, Mod, Min, Max };

struct IrNode {
  NodeKind kind;
  uint8_t op = 0;              // UnOp / BinOp
  int a = -1, b = -1;          // operands; Extract: a = param node; View: a = sub node
  std::vector<int64_t> dims;   // Param / View: the viewed tensor's shape
  uint32_t bits = 0;           // Literal value / Param or View padding (binary32 bits)
  int cols = 0;                // Extract / View: matrix columns (= frame rank + 1)
  std::vector<double> m;       // Extract / View: row-major view matrix
  std::vector<int> elems;      // Tuple
  int param_index = -1;        // Param: kernel input number
};

enum class ProgramKind : int { Elementwise = 0, Sum = 1 };

struct Ir {
  ProgramKind kind = ProgramKind::Elementwise;
  std::vector<int64_t> out_shape;
  std::vector<IrNode> nodes;
  int root = -1;
  int n_params = 0;
  std::vector<int> param_nodes;
};

Ir parse_ir(const char *text, size_t len);

// Device helpers every generated module starts with (device_common.cuh).
extern const char *kPrelude;

struct CodegenOptions {
  int block = 256;
  int load_lookahead = 8;   // loads kept in flight ahead of the arithmetic (generic kernels)
  bool asm_loads = true;    // emit those loads as volatile inline PTX so their order holds
  int min_blocks = 0;       // __launch_bounds__ minimum blocks per SM of the generic kernels (0: none)
  int vec_unroll = 4;       // float4 positions per thread per batch in the contiguous kernels
  int64_t prefetch_min_bytes = -1;  // L2-prefetch loads from inputs at least this large (-1: never)
  int smem_ring = 0;        // generic kernels: shared-memory ring slots per thread for staged loads (0: none)
  int points_per_thread = 1;  // generic elementwise kernels: consecutive points a thread computes together
  bool vector_loads = true;   // generic kernels: also cc_ew_vl / cc_sum_vl, with float4 grouped reads
  bool batch_loads = false;   // those kernels: scalar loads of one condition share one predicate, 8 at a time
};

// Minimum resident blocks per SM to request for a generic kernel over `domain`
// points (one per thread, `block` threads per block) on `sm_count` SMs: the
// blocks one wave needs when the whole grid fits in one wave, else 4 (the
// kernel then loops over the domain with a resident grid).  More registers per
// thread let the compiler keep more loads in flight.
int choose_min_blocks(int64_t domain, int block, int sm_count, int override_blocks);
// Points per thread a generic elementwise kernel takes for `requested`: 1 for
// sums, contiguous programs and last extents that `requested` does not divide.
int points_for(const Ir &ir, int requested);

struct Generated {
  std::string source;
  bool has_vec4 = false;   // a float4 variant of the kernel exists (all inputs contiguous)
  int tuple_len = 1;
  int n_inputs = 0;
  int64_t out_elems = 0;   // floats written (1 for a sum)
  int64_t domain = 0;      // points evaluated
  bool uses_fp64_index = false;
  int vec_unroll = 1;      // positions per thread per batch of the float4 variant
  int smem_bytes = 0;      // dynamic shared memory of the generic kernel (its load ring)
  std::vector<int64_t> param_bytes;  // bytes of each input buffer the kernel may read
  int points_per_thread = 1;         // of the generic elementwise kernel
  bool has_vl = false;               // cc_ew_vl / cc_sum_vl exists (float4 grouped reads; aligned inputs)
};

// FMA contraction of the code generated on this thread (CC_FLAG_FMA_CONTRACT):
// every + or - with a product operand becomes one fmaf of that product (the
// left one when both operands are products), rounded once.  Set it around
// generate_cuda, row_fold_source, point_function and tunable_source with
// FmaScope.
extern thread_local bool g_codegen_fma;
struct FmaScope {
  bool saved;
  explicit FmaScope(bool on) : saved(g_codegen_fma) { g_codegen_fma = on; }
  ~FmaScope() { g_codegen_fma = saved; }
};

Generated generate_cuda(const Ir &ir, const CodegenOptions &opt);
// The shape information of generate_cuda without generating code.
Generated describe_program(const Ir &ir);
// For a program that reads every input contiguously with the output's shape
// (no views): a key that identifies its code whatever the shape.  Empty otherwise.
std::string contiguous_structure_key(const Ir &ir);

// The library's matmul idiom (TensorsSpec.scala:468-485, README.md:336-343):
//   A.broadcast([I,J,K]) * B.reshape([1,J,K]).broadcast([I,J,K]), then
//   split(1).reduce(_ + _)
// which, with the product fused, arrives as a left fold over j of views that
// select j from one product node A[i][j] * B[j][k].  On a match, C[I,K] =
// A[I,J] * B[J,K] with A and B the given kernel inputs (row-major, dense).
struct Contraction {
  int a_input = -1, b_input = -1;
  int64_t m = 0, k = 0, n = 0;  // C is m x n, the folded dimension has k terms
};
bool match_contraction(const Ir &ir, Contraction *out);

// The inner-axis fold `t.split(last).reduce(_ + _)` (Tensors.scala:1035-1074
// with Scala's left-to-right reduce): after fusion, a left fold over j of J
// terms that are one template -- the viewed tensor t at coordinates
// (g_0..g_{r-1}, j) -- so out[g] = ((t(g,0) + t(g,1)) + t(g,2)) + ...  The
// template reads "row inputs" (tensors of t's shape, read at (g, j)), "column
// inputs" (one-dimensional tensors of J elements, read at j) and literals.
// On a match the runtime stages tiles of the row inputs through shared memory
// by TMA and each thread folds one output's terms in the reference's order.
struct RowFold {
  int term = -1;                  // the template node, evaluated in frame `term_frame`
  std::vector<int64_t> term_frame;  // t's shape (a fused view), or the output's (a parameter read directly)
  int64_t rows = 0, cols = 0;     // outputs, and J
  std::vector<int> row_inputs;    // parameter indices read as rows, in order
  std::vector<bool> is_row;       // per parameter: a row input (else a column input)
  int stages = 0;                 // shared-memory ring stages (row_fold_stages)
};
// Terms below this count stay on the generic fold (a short fold is cheap to unroll).
constexpr int64_t kRowFoldMinTerms = 32;
constexpr int kRowFoldRows = 64;       // outputs (threads) per block
constexpr int kRowFoldMaxInputs = 4;   // row inputs staged per tile
constexpr int kRowFoldWaitCode = 31;   // device error code: a tile's barrier wait ran out
bool match_row_fold(const Ir &ir, RowFold *out, std::string *why = nullptr);
// Stages of the shared-memory ring for `row_inputs` staged inputs: `requested`
// (2..16) if it fits, else as many 8 KiB tiles per input as fit in 96 KiB
// (two blocks per SM), 2 to 12.
int row_fold_stages(int row_inputs, int requested = 0);
// Dynamic shared memory of cc_rowfold (ring + alignment slack).
int row_fold_smem_bytes(int row_inputs, int stages);
// Kernels cc_rowfold (TMA-staged tiles) and cc_rowfold_plain (direct loads,
// for row inputs that are not 16-byte aligned), with the prelude.
std::string row_fold_source(const Ir &ir, const RowFold &rf);

// Batching: a program is batchable when it is an elementwise program whose
// inputs are all read contiguously with the output's shape (the float4 form)
// and it has at most kBatchMaxInputs inputs.
constexpr int kBatchMaxInputs = 4;
bool is_batchable(const Ir &ir, std::string *why);
// `__device__ float <name>(float a0, ..., float a<kBatchMaxInputs-1>)`: the
// program's value at one point from its inputs' values there (unused
// arguments are ignored).  With shared_transcendentals, exp/log/tanh go through
// the module's cc_expf/cc_logf/cc_tanhf (the same functions, called, which keeps
// the code of thousands of structures small).  With lanes, the function is a
// template over the value type T (`template <class T> T <name>(T a0, ...)`):
// its operations are + - * / and negation on T and the overloaded helpers
// cc_exp, cc_log, cc_tanh, cc_abs, cc_sqrt, cc_fma, cc_mod, cc_min and cc_max,
// which the including module defines for each T it evaluates.
std::string point_function(const Ir &ir, const std::string &name, bool inline_it = true,
                           bool shared_transcendentals = false, bool lanes = false);

// ---- tuning
// A launch configuration of a program's tunable form: threads per block,
// points per work item (1, or 4 consecutive points with float4 access),
// work items per thread per loop iteration (their loads issued together), and
// the grid: split 1 = at most one resident wave (the threads loop), split 2 =
// one work batch per thread (sums: up to kMaxSumBlocks partials).
struct TuneConfig {
  int block = 256, vec = 1, ept = 1, split = 1;
};
constexpr int kTuneConfigs = 48;
constexpr int kTuneMaxNodes = 64;  // larger programs are not tuned
// The tuner's choice "the program's standard generated kernel" (no tunable configuration).
constexpr int kStdConfig = kTuneConfigs;
constexpr int kTuneKernels = 6;  // (vec, ept) pairs compiled per program
constexpr int kFeatures = 64;
TuneConfig tune_config(int index);
int tune_kernel_index(const TuneConfig &c);
int64_t tune_grid(int64_t n, const TuneConfig &c, bool sum, int sm_count, int resident);
bool is_tunable(const Ir &ir, std::string *why);
// Kernels cc_t<suffix>_v<1|4>_e<1|2|4> (arguments as the program's cc_ew /
// cc_sum) and their point function; the module needs the prelude first.
std::string tunable_source(const Ir &ir, const std::string &suffix);
// The cost model's input for (program, configuration): kFeatures floats.
void program_features(const Ir &ir, int config, int sm_count, float *out);

// The literal text DecimalFormat gives a view coefficient (at most three
// fraction digits, HALF_EVEN, no grouping), as OpenCLKernelBuilder.toLiteral.
std::string decimal_format3(double v);

}  // namespace cc
