/*
 * compute_cuda.h -- C ABI of the GB300 (sm_103a) back-end for Compute.scala's
 * fused-tensor path.
 *
 * A `cuda` device object (a sibling of Compute.scala's `gpu` and `cpu`
 * objects) binds these entry points through JNI or Panama; the Python mirror
 * of the Tensor API in this repository binds them through ctypes.  Every
 * entry point replaces one member of the OpenCL layer that `Tensors` calls
 * (paths below are inside the Compute.scala project):
 *
 *   OpenCL/src/main/scala/com/thoughtworks/compute/OpenCL.scala      ("OpenCL.scala")
 *   Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala    ("Tensors.scala")
 *
 * Conventions
 *   - Every function returns a status: 0 on success, otherwise a negative
 *     code.  Codes that have an OpenCL counterpart use its value, so the
 *     reference's `OpenCL.Exceptions.fromErrorCode` (OpenCL.scala:251-303)
 *     maps them to the same exception types.  The message of the last failure
 *     on the calling thread is returned by cc_last_error.
 *   - Handles are opaque 64-bit values (0 is never a valid handle).
 *   - All functions are thread-safe.  Work is ordered on one CUDA stream per
 *     context (cc_get_stream / cc_set_stream), except the *_ev entry points,
 *     which spread work over a pool of streams ordered by event wait lists.
 *   - Completion is reported by polling or by blocking waits with a timeout;
 *     the library never calls back into the caller from a driver thread.
 */
#ifndef COMPUTE_CUDA_H
#define COMPUTE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t cc_handle;

/* ---- status codes -------------------------------------------------------- */
#define CC_OK                         0
#define CC_ERR_DEVICE_NOT_FOUND      (-1)    /* CL_DEVICE_NOT_FOUND */
#define CC_ERR_OUT_OF_MEMORY         (-4)    /* CL_MEM_OBJECT_ALLOCATION_FAILURE */
#define CC_ERR_OUT_OF_RESOURCES      (-5)    /* CL_OUT_OF_RESOURCES */
#define CC_ERR_BUILD_PROGRAM_FAILURE (-11)   /* CL_BUILD_PROGRAM_FAILURE; message = NVRTC log */
#define CC_ERR_INVALID_VALUE         (-30)   /* CL_INVALID_VALUE */
#define CC_ERR_INVALID_MEM_OBJECT    (-38)   /* CL_INVALID_MEM_OBJECT */
#define CC_ERR_INVALID_PROGRAM       (-44)   /* CL_INVALID_PROGRAM */
#define CC_ERR_INVALID_KERNEL_ARGS   (-52)   /* CL_INVALID_KERNEL_ARGS */
#define CC_ERR_INVALID_EVENT         (-58)   /* CL_INVALID_EVENT */
#define CC_ERR_INVALID_OPERATION     (-59)   /* CL_INVALID_OPERATION */
#define CC_ERR_TIMEOUT               (-1001) /* a bounded wait ran out */
#define CC_ERR_NOT_INITIALIZED       (-1002) /* cc_init has not succeeded */
#define CC_ERR_CUDA                  (-1003) /* CUDA runtime/driver error; see cc_last_error */
#define CC_ERR_DEVICE_REPORTED       (-1004) /* a kernel set its error flag (bounded wait expired) */

/* ---- flags for cc_init ----------------------------------------------------- */
#define CC_FLAG_FMA_CONTRACT   0x1u  /* FMA contraction, as a vendor compiler under the reference's
                                        -cl-unsafe-math-optimizations (OpenCL.scala:1131-1135) may
                                        apply it: every + or - with a product operand is one fmaf of
                                        that product (the left one when both operands are products),
                                        rounded once; the compiler itself never contracts.  Off (the
                                        default): every SSA statement rounds separately, as written */
#define CC_FLAG_NO_FUSION_SUM  0x2u  /* reserved */

/* ---- context: replaces OpenCL.UseAllDevicesByType + context + CommandQueuePool
 *      (OpenCL.scala:340-374, :423-448, :1375-1393) ------------------------- */
/* Initialises the context on a device; calling it again with the same device
 * and flags does nothing, other flags are refused (CC_ERR_INVALID_OPERATION). */
int cc_init(int device_ordinal, uint32_t flags);
int cc_shutdown(void);
/* Copies the message of this thread's last failure (NUL-terminated, truncated to len). */
int cc_last_error(char *buf, size_t len);
/* deviceId.maxComputeUnits / deviceType (OpenCL.scala:451-470). */
int cc_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *total_mem);
int cc_get_stream(uint64_t *stream);            /* the context's cudaStream_t */
int cc_set_stream(uint64_t stream);             /* order later work on a caller-owned stream */
int cc_synchronize(void);
/* Runtime tuning knobs (no reference counterpart: the reference leaves launch
 * geometry to the OpenCL runtime, Tensors.scala:1360-1375, :697-753).  Keys:
 *   "block"             threads per block of generated kernels (64, 128 or 256; default 128)
 *   "ew_blocks_per_sm"  cap on resident blocks per SM for elementwise grids (0 = occupancy; default 0)
 *   "sum_blocks_per_sm" blocks per SM of the grid sums (default 4)
 *   "sum_block"         threads per block of the generated sums (64, 128 or 256; default 256)
 *   "prefetch_min_bytes" generated kernels L2-prefetch every load from an input at least this large
 *                       before loading (-1: never; default -1)
 *   "upload_streams"    copy streams a large cc_buf_upload is striped over (1..8; default 4)
 *   "ew_lookahead"      loads a generated kernel keeps in flight ahead of its arithmetic (0..256; default 8)
 *   "ew_asm_loads"      1: those loads are volatile inline PTX so the compiler keeps their order (default 1)
 *   "row_fold"          1 (default) = a program that folds the last axis of a tensor, t.split(last).reduce(_ + _)
 *                       with at least 32 terms whose term reads inputs of t's shape at (g, j), one-dimensional
 *                       inputs at j and literals, runs as a skeleton that stages tiles of those inputs in
 *                       shared memory by TMA and folds each output's terms in order (bit-identical to the
 *                       generated fold); 0 = the generated fold
 *   "row_fold_stages"   that skeleton's ring of 8 KiB tiles per staged input (2..16; 0 = as many as fit
 *                       96 KiB, at most 12; default 0)
 *   "contraction"       how a program that is the library's matmul idiom runs (a left fold over j
 *                       of split(1) views of A.broadcast * B.reshape.broadcast): 0 = the generated
 *                       fold kernel, 1 = CC_GEMM_EXACT (bit-identical to 0, default), 2 = CC_GEMM_FP32,
 *                       3 = CC_GEMM_BF16X6
 *   "copy_kernel"       1 = cc_buf_upload / cc_buf_download of 1 MiB or more between pinned host memory
 *                       (cc_host_alloc) and the device are done by a copy kernel on the SMs instead of
 *                       the DMA engines (16-byte aligned ends; default 0)
 *   "tc_group_m"        tensor-core GEMM: output tiles visited in groups of this many tile rows, so the
 *                       CTAs running together share A and B panels in L2 (1 = row-major; default 1)
 *   "pdl"               1 (default) = launch generated kernels with programmatic dependent launch: a kernel is
 *                       scheduled while the previous one drains and waits (griddepcontrol.wait)
 *                       before its first memory access, so results and ordering are unchanged; on the
 *                       context's own stream, a kernel that follows another generated kernel (nothing
 *                       else enqueued by this library in between) and reads none of its output loads
 *                       early and waits before its first store.  A caller that enqueues its own work on
 *                       that stream between launches (cc_get_stream) sets 2: programmatic launch, every
 *                       kernel waiting before its first load.  0 = ordinary launches
 *   "ew_smem_ring"      generic kernels: per-thread slots of a shared-memory ring through which loads
 *                       with zero padding are staged by cp.async (0 = loads into registers; 4..64)
 *   "ew_vector_loads"   1 (default) = generic elementwise kernels whose reads at a constant innermost index
 *                       (a channel split, also through views) group into 16-byte loads also get
 *                       cc_ew_vl, launched when every input and the output are 16-byte aligned
 *                       (bit-identical); 0 = cc_ew only
 *   "ew_batch_loads"    1 = in cc_ew_vl / cc_sum_vl, scalar loads under one bounds condition share one
 *                       predicate, 8 per inline-PTX block, issued 8 at a time (faster from L2, slower
 *                       from DRAM: default 0)
 *   "ew_points"         generic elementwise kernels: consecutive points per thread along the last output
 *                       dimension (when it divides that extent), with index arithmetic, loads and
 *                       arithmetic common to the points done once (1 = one point; default 1; 1..16)
 *   "tuner"             0 = generated kernels with the fixed launch shape (default), 1 = exhaustive
 *                       tuner, 2 = learned tuner (see the tuner section)
 *   "batch_max_registers" batch modules: register cap per thread of every compiled part (0 = none;
 *                       default 64: four blocks per SM; the indirect calls of the persistent kernel
 *                       otherwise take the largest part's registers and one block per SM)
 *   "batch_run_tiles"   consecutive 4096-float tiles a block of the persistent batch kernel claims at once
 *                       (default 4)
 *   "batch_max_loads"   float4 loads a batch tile function keeps in flight per thread (1, 2, 4, 8 or 16;
 *                       default 4); programs with more inputs load their four positions per input in groups
 *   "batch_rolled"      batch tile functions: 1 = the load groups of a tile run in a loop over one copy of
 *                       the group's code (default), 0 = one copy per group
 *   "batch_prefetch"    persistent batch kernel: 1 = a tile function asks L2 for the later tiles of its run
 *                       (one bulk prefetch per input) before loading the first; 2 = also, a block claims
 *                       its next run one run ahead and prefetches that run's first tile (default 0)
 *   "batch_lanes"       points a batch tile function evaluates per expression call: 4 = a float4's four
 *                       (default; a called exp/log/tanh computes four values), 8 = two float4s, 0 = one
 *                       point per call.  Every setting gives the same bits.
 *   "batch_inline"      batch modules: 0 = expressions and exp/log/tanh are called functions,
 *                       1 = expressions inlined, exp/log/tanh called (default), 2 = all inlined
 *   "tc_variant"        tensor-core contraction: 0 = 128x128 tiles, K in chunks of 128 summed in
 *                       registers (error ~1.6e-7 at any K), 1 = 128x256 tiles, one accumulator
 *                       per tile (error grows with K), 2 = 128x128, one per tile, 3 = as 0 with
 *                       chunks of 256 (~2.4e-7), 4 = chunks of 512 (~4.7e-7), 5 (default) =
 *                       128x256 tiles, hi*hi in chunks of 256, the five small products over
 *                       the whole K (~2.5e-7)
 *   "vec_unroll"        float4 positions a thread of a contiguous kernel loads before computing (1..8; default 4)
 * Unknown keys or values out of range return CC_ERR_INVALID_VALUE. */
int cc_config_set(const char *key, int64_t value);
int cc_config_get(const char *key, int64_t *value);

/* ---- device buffers: replace allocateBuffer / allocateBufferFrom
 *      (OpenCL.scala:1397-1431) and DeviceBuffer.retain/release/numberOfBytes/
 *      toHostBuffer (OpenCL.scala:633-717).  Buffers come from a size-binned,
 *      stream-ordered pool; the reference count mirrors retain/release. ------ */
int cc_buf_alloc(size_t bytes, cc_handle *buf);
int cc_buf_retain(cc_handle buf);
int cc_buf_release(cc_handle buf);
int cc_buf_size(cc_handle buf, size_t *bytes);
int cc_buf_device_ptr(cc_handle buf, uint64_t *device_ptr);
/* Host -> device copy into [offset, offset+bytes).  Returns when the host memory may be reused. */
int cc_buf_upload(cc_handle buf, size_t offset, const void *host, size_t bytes);
/* The same, ordered on the context stream without waiting for it (OpenCL's
 * non-blocking enqueueWriteBuffer): the host memory must stay unchanged until
 * the copy is complete (cc_synchronize, or an event recorded after it). */
int cc_buf_upload_async(cc_handle buffer, size_t offset, const void *host, size_t bytes);
/* Device -> host copy of [offset, offset+bytes) after all work queued so far; blocking. */
int cc_buf_download(cc_handle buf, size_t offset, void *host, size_t bytes);
/* The same, ordered on the context stream without waiting (OpenCL's non-blocking
 * enqueueReadBuffer): the host memory holds the data once the copy is complete
 * (cc_synchronize, or an event recorded after it); pinned host memory
 * (cc_host_alloc) makes the copy asynchronous to the host. */
int cc_buf_download_async(cc_handle buf, size_t offset, void *host, size_t bytes);
/* Page-locked host memory for fast transfers (the staging of Tensor.apply / flatArray). */
int cc_host_alloc(size_t bytes, void **host);
int cc_host_free(void *host);
/* Pool accounting and an optional cap (bytes in use + cached); 0 = no cap. */
int cc_pool_stats(size_t *in_use, size_t *cached, uint64_t *allocs, uint64_t *reuses);
int cc_pool_set_limit(size_t bytes);
int cc_pool_trim(void);

/* ---- programs: replace createProgramWithSource + Program.build
 *      (OpenCL.scala:885-932, :1266-1294) and the kernel cache keyed by the
 *      alpha-converted tree (Tensors.scala:1267-1293).  `ir` is the
 *      alpha-converted expression tree in the text form documented in
 *      compute/trees.py; the runtime generates CUDA C for sm_103a, compiles it
 *      with NVRTC to a cubin and caches it by the IR text.  A compile failure
 *      returns CC_ERR_BUILD_PROGRAM_FAILURE with the NVRTC log as the message
 *      (the reference's BuildProgramFailure, OpenCL.scala:172-181). --------- */
int cc_program_get(const char *ir, size_t ir_len, cc_handle *program);
/* kind: 0 = elementwise store, 1 = full sum.  out_elems = number of floats written. */
int cc_program_info(cc_handle program, int *kind, int *n_inputs, int64_t *out_elems, int *tuple_len);
/* The generated CUDA C source, NUL-terminated; *needed gets the size required. */
int cc_program_source(cc_handle program, char *buf, size_t len, size_t *needed);
int cc_program_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *entries);
/* GPU-free checks of the same path (no cc_init needed): the CUDA C generated
 * for `ir`, and an NVRTC compile of it for sm_<cc_major><cc_minor>a whose
 * failure carries the NVRTC log, like cc_program_get. */
int cc_codegen(const char *ir, size_t ir_len, char *buf, size_t len, size_t *needed);
int cc_compile_check(const char *ir, size_t ir_len, int cc_major, int cc_minor, uint32_t flags);
/* The same with code-generation options as "key=value" words (NULL = defaults):
 * block, lookahead, ring (shared-memory ring slots), unroll, min_blocks, asm,
 * points (consecutive points per thread of a generic elementwise kernel),
 * vl (1, the default as in the runtime: also the float4 grouped-read kernel cc_ew_vl),
 * batch (1: its scalar loads in predicate-sharing blocks of 8). */
int cc_codegen_with(const char *ir, size_t ir_len, const char *options, char *buf, size_t len, size_t *needed);
int cc_compile_check_with(const char *ir, size_t ir_len, int cc_major, int cc_minor, uint32_t flags,
                          const char *options);

/* ---- launch: replaces Kernel.update + Kernel.enqueue + dispatch
 *      (OpenCL.scala:751-844, :1298-1329) as driven by CompiledKernel.run
 *      (Tensors.scala:1331-1381).  Inputs are in the program's parameter
 *      order; the output must hold out_elems floats (1 for a sum). --------- */
int cc_launch(cc_handle program, const cc_handle *inputs, int n_inputs, cc_handle output);
/* The same on raw device pointers and a caller stream (0 = the context stream). */
int cc_launch_ptrs(cc_handle program, const uint64_t *input_ptrs, int n_inputs, uint64_t output_ptr,
                   uint64_t stream);

/* ---- the asynchronous DAG: Kernel.enqueue(commandQueue, ..., waitingEvents) returning an Event
 *      (OpenCL.scala:787-844), dispatched to a queue of the CommandQueuePool (:423-448, :1298-1329),
 *      and the non-blocking enqueueWriteBuffer / enqueueReadBuffer with their events (:1206-1244,
 *      :1415-1431), as CompiledKernel.run drives them: each kernel waits for the events of the
 *      buffers it reads (Tensors.scala:1331-1381, PendingBuffer / EventBuffer :253-299).
 *      Each call takes a stream of a pool of eight (the first idle one from a round-robin position,
 *      else the next one round robin: each stream runs its work in order), makes it wait for every
 *      event of `wait` (n_wait of them; NULL when 0), enqueues its work there and, when `event` is
 *      not NULL, returns an event that completes with it (release it with cc_event_release; it
 *      has no timing, so cc_event_elapsed refuses it).  Work without a chain of events between it
 *      runs concurrently.  Work on the context stream (cc_launch, cc_buf_upload, ...) is ordered
 *      after the pool's work only through cc_stream_wait_events.  Once the pool is in use, a
 *      released buffer is reused only after every stream that may still use it has passed it.
 *      A host copy must leave `host` unchanged (upload) or unread (download) until the event
 *      completes; pinned memory (cc_host_alloc) makes the copy asynchronous to the host. --------- */
int cc_launch_ev(cc_handle program, const cc_handle *inputs, int n_inputs, cc_handle output, const cc_handle *wait,
                 int n_wait, cc_handle *event);
int cc_buf_upload_ev(cc_handle buf, size_t offset, const void *host, size_t bytes, const cc_handle *wait, int n_wait,
                     cc_handle *event);
int cc_buf_download_ev(cc_handle buf, size_t offset, void *host, size_t bytes, const cc_handle *wait, int n_wait,
                       cc_handle *event);
/* Later work on the context stream waits for these events (also those of cc_event_record). */
int cc_stream_wait_events(const cc_handle *events, int n_events);

/* ---- reductions: Tensor.sum -> reduce(PlusPrograms) (Tensors.scala:303-392,
 *      :673-771).  A fused sum is a kind-1 program run by cc_launch; this is the
 *      plain sum of n floats at a device address, written to one float at
 *      `out`.  Scratch (block partials and a completion counter) comes from the
 *      context's buffer pool. ------------------------------------------------ */
int cc_reduce_sum_f32(uint64_t in_ptr, size_t n, uint64_t out_ptr, uint64_t stream);

/* The same sum for callers that cannot allocate device memory.  It has no
 * counterpart in the reference.  Some callers cannot call cudaMalloc (or
 * cc_init, whose pool does): a host framework that has already reserved the
 * device's memory for its own allocator and forbids side allocations, or a
 * latency-critical caller that cannot accept cudaMalloc's device-wide
 * synchronisation.  This entry point allocates nothing: its scratch (one
 * compensated partial per block and a completion counter, 128 KiB + 256 B) is a
 * fixed array in device memory that every GPU loading this library holds until
 * the process exits.  It needs no cc_init and runs on the calling thread's
 * current device; in_ptr and out_ptr must be on that device, and stream 0 is
 * that device's default stream.
 *   - n may be at most 134,217,728 floats (16384 blocks of 8192); larger n is
 *     rejected with CC_ERR_INVALID_VALUE and nothing is launched.
 *   - The array's device address belongs to the CUDA context current on the
 *     calling thread (the device's primary context, or a driver-API context
 *     of the caller's own).  The first call in each context looks it up
 *     (cudaGetSymbolAddress) and keeps it under the context's unique ID
 *     (cuCtxGetId), so a context created after cudaDeviceReset, or another
 *     context on the same device, gets its own address.  Make that first call
 *     in a context before any stream capture.
 *   - Every call shares the one array, which keeps the last call's contents:
 *     each call zeroes the counter on `stream` first, so calls ordered on one
 *     stream are safe, but calls that can overlap on the GPU (on different
 *     streams of one device) race and give wrong sums. */
int cc_reduce_sum_f32_noalloc(uint64_t in_ptr, size_t n, uint64_t out_ptr, uint64_t stream);

/* ---- contraction: the library's matmul, `A.broadcast([i,j,k]) * B.reshape([1,j,k]).broadcast(...)`
 *      followed by `split(1).reduce(_ + _)` (TensorsSpec.scala:468-485, README.md:311-343), as one
 *      kernel.  C[M,N] = A[M,K] * B[K,N], float, row-major, leading dimensions in elements.
 *      mode CC_GEMM_EXACT: FP32 on the CUDA cores, every output the sequential left fold over k of
 *        separately rounded products: bit-identical to the reference's result;
 *      mode CC_GEMM_FP32: FP32 on the CUDA cores with fused multiply-adds;
 *      mode CC_GEMM_BF16X6: each operand split into three bfloat16 planes, the six leading
 *        products accumulated in FP32 by the tcgen05 tensor cores (FP32-level error).
 *      The bfloat16 planes (6*(M*K + K*N) bytes, padded) come from the buffer pool. ---------- */
#define CC_GEMM_EXACT 0
#define CC_GEMM_FP32 1
#define CC_GEMM_BF16X6 2
int cc_gemm_f32(uint64_t a_ptr, uint64_t b_ptr, uint64_t c_ptr, int m, int n, int k, int64_t lda, int64_t ldb,
                int64_t ldc, int mode, uint64_t stream);
/* Reads and clears the device error flag that kernels with bounded waits set
 * when a wait expires (0 = none); blocking. */
int cc_device_errors(int *code);
/* Diagnostic of the bounded waits themselves: enqueues on the context stream
 * one thread that waits for a device word, which is set beforehand when
 * flag_value != 0 (the wait ends at once) and never otherwise, so the wait
 * gives up after limit_ns (at most 10 s) and the device error flag reads
 * CC_DEVICE_ERR_PROBE_TIMEOUT.  Asynchronous: an event recorded after it
 * completes once the wait has ended; the context stays usable. */
#define CC_DEVICE_ERR_PROBE_TIMEOUT 90
int cc_probe_bounded_wait(uint64_t limit_ns, int flag_value);

/* ---- batches: many independent elementwise programs of uneven lengths evaluated
 *      together (no reference counterpart: the reference launches one kernel per
 *      tensor, Tensors.scala:1331-1381).  A batch compiles once; each distinct
 *      program structure gets a point function shared by all three run modes, so
 *      every mode gives the same bits.  Programs must be contiguous elementwise
 *      programs (inputs read without views) with at most 4 inputs. ------------- */
#define CC_BATCH_PERSISTENT 0   /* one persistent kernel over every program's 4096-float tiles */
#define CC_BATCH_PER_PROGRAM 1  /* one launch per program, back to back */
#define CC_BATCH_GRAPH 2        /* the per-program launches, captured once into a CUDA graph and replayed */
int cc_batch_create(const char *const *irs, const size_t *ir_lens, int n_programs, cc_handle *batch);
/* registers: per thread of the persistent kernel; resident_blocks: its blocks per SM.  Any pointer may be NULL. */
int cc_batch_info(cc_handle batch, int *n_programs, int *n_structures, int *registers, int *resident_blocks);
/* ptrs: for each program, its inputs in parameter order, then its output (16-byte aligned). */
int cc_batch_bind(cc_handle batch, const uint64_t *ptrs, size_t n_ptrs);
int cc_batch_run(cc_handle batch, int mode, uint64_t stream);
/* The batch with host transfers in the event model of the launch API
 * (Kernel.enqueue with waitingEvents, OpenCL.scala:787-844; enqueueWriteBuffer /
 * enqueueReadBuffer with wait lists, OpenCL.scala:1206-1244, 1415-1431): each
 * call waits for exactly its wait list and returns an event (release it with
 * cc_event_release).
 *   cc_batch_upload_ev: every bound input from pinned host memory; hosts: for
 *     each program its inputs in parameter order (length of the program floats
 *     each); copies spread over four copy streams.
 *   cc_batch_run_ev: cc_batch_run on the context stream after the wait list.
 *   cc_batch_download_ev: every program's output into hosts[p] (pinned), on four
 *     other copy streams, so the reads of one step overlap the uploads of the
 *     next when their wait lists allow it (uploads after the previous run; the
 *     next run after these reads and the new uploads).
 * The copies are ordered by their wait lists only: a caller that writes a bound
 * buffer otherwise must wait for the events itself.  cc_synchronize waits for
 * them too, and a buffer released meanwhile returns to the pool after them. */
int cc_batch_upload_ev(cc_handle batch, const void *const *hosts, size_t n_hosts, const cc_handle *wait, int n_wait,
                       cc_handle *event);
int cc_batch_run_ev(cc_handle batch, int mode, const cc_handle *wait, int n_wait, cc_handle *event);
int cc_batch_download_ev(cc_handle batch, void *const *hosts, size_t n_hosts, const cc_handle *wait, int n_wait,
                         cc_handle *event);
int cc_batch_release(cc_handle batch);
/* GPU-free: generates and NVRTC-compiles a batch module for sm_<cc_major><cc_minor>a. */
int cc_batch_compile_check(const char *const *irs, const size_t *ir_lens, int n_programs, int cc_major, int cc_minor,
                           int *n_structures, double *seconds);

/* ---- tuner.  No reference counterpart: the reference lets the OpenCL runtime
 *      choose the local size (Tensors.scala:1360-1375) and sizes reduction
 *      groups as min(length, CL_KERNEL_WORK_GROUP_SIZE) (Tensors.scala:700).
 *      A program's tunable form runs in CC_TUNE_CONFIGS launch configurations:
 *      index i -> block {64,128,256,512}[i%4], vector width {1,4}[(i/4)%2],
 *      work items per thread {1,2,4}[(i/8)%3], grid split {1,2}[(i/24)%2]
 *      (1: at most one resident wave of blocks, the threads loop; 2: one batch
 *      of work items per thread; for a sum, the number of partial sums).
 *      Elementwise results are identical in every configuration; sums differ
 *      in the order of their compensated partials.
 *      Programs of more than 64 IR nodes (beyond the cost model's training
 *      workloads) and tuple-valued programs are not tuned: they run their
 *      standard kernel whatever the knob.
 *      With the "tuner" knob at 1 (exhaustive), cc_program_get compiles the
 *      tunable form beside the standard kernels, and the first launch times
 *      all configurations and the standard kernel on its own buffers (3
 *      launches each after an L2 flush) and keeps the fastest; at 2 (learned)
 *      the cost model installed by cc_tuner_set_model predicts each
 *      configuration's log-runtime, and its first choice and the standard
 *      kernel are timed the same way; the faster is kept. -------------------- */
#define CC_TUNE_CONFIGS 48
#define CC_FEATURES 64
int cc_tune_config(int index, int *block, int *vec, int *ept, int *split);
/* The cost model's features of (program, configuration) for a GPU of sm_count SMs: CC_FEATURES floats. */
int cc_program_features(const char *ir, size_t ir_len, int config, int sm_count, float *out);
/* The configuration the tuner chose for a program (-1: not launched yet or not tuned;
 * CC_TUNE_STANDARD: the program's standard generated kernel, which the tuner times beside
 * the tunable configurations, so a tuned program is never slower than it). */
#define CC_TUNE_STANDARD CC_TUNE_CONFIGS
int cc_tuner_choice(cc_handle program, int *config);
/* Installs network `mlp` (CC_FEATURES inputs, one output) as the learned tuner's
 * model; inputs are normalised as (feature - mean) * inv_std.  mlp = 0 removes it. */
int cc_tuner_set_model(cc_handle mlp, const float *mean, const float *inv_std);
/* Tuning sets: many programs' tunable forms compiled together (NVRTC units of
 * 16 programs, compiled on all host threads) and timed on request. */
int cc_tune_create(const char *const *irs, const size_t *ir_lens, int n_programs, cc_handle *set);
int cc_tune_info(cc_handle set, int *n_programs);
/* ptrs: the program's inputs in parameter order, then its output. */
int cc_tune_launch(cc_handle set, int program, const uint64_t *ptrs, size_t n_ptrs, int config, uint64_t stream);
/* ms[i]: median device time of `reps` launches of configs[i] (after one untimed
 * launch; with flush_l2, a 256 MiB write precedes each); -1 where a float4
 * configuration meets a buffer that is not 16-byte aligned. */
int cc_tune_time(cc_handle set, int program, const uint64_t *ptrs, size_t n_ptrs, const int *configs, int n_configs,
                 int reps, int flush_l2, float *ms);
int cc_tune_release(cc_handle set);
/* GPU-free: generates and NVRTC-compiles the tunable forms for sm_<cc_major><cc_minor>a. */
int cc_tune_compile_check(const char *const *irs, const size_t *ir_lens, int n_programs, int cc_major, int cc_minor,
                          double *seconds);

/* ---- the cost model's network: a multilayer perceptron with ReLU hidden
 *      layers, trained by its own CUDA kernels (forward, backward, Adam) on a
 *      mean-squared-error loss.  dims: widths, input first (the cost model is
 *      {64, 256, 256, 256, 1}).  Parameters are packed per layer as W (rows =
 *      inputs, row-major) then b.  x: batch x dims[0] floats, row-major, and
 *      t / y: batch floats, all device pointers. ----------------------------- */
int cc_mlp_create(const int *dims, int n_dims, cc_handle *mlp);
int cc_mlp_info(cc_handle mlp, size_t *n_params, int *steps);
/* Also zeroes the Adam moments and the step count. */
int cc_mlp_set_params(cc_handle mlp, const float *host, size_t n);
int cc_mlp_get_params(cc_handle mlp, float *host, size_t n);
int cc_mlp_forward(cc_handle mlp, uint64_t x, int batch, uint64_t y, uint64_t stream);
/* Loss (mean squared error) and the gradient of every parameter, copied to the host (either may be NULL). */
int cc_mlp_gradients(cc_handle mlp, uint64_t x, uint64_t t, int batch, float *loss, float *grads);
/* One Adam step on the batch's gradients; loss (may be NULL) is the loss before the step. */
int cc_mlp_train_step(cc_handle mlp, uint64_t x, uint64_t t, int batch, float lr, float beta1, float beta2, float eps,
                      float *loss);
int cc_mlp_release(cc_handle mlp);

/* ---- random numbers: Tensor.random / Tensor.randomNormal with the Wang hash
 *      (Tensors.scala:106-117, :397-524).  normal=0: uniform [0,1]; normal=1:
 *      Box-Muller pairs (the buffer must hold n rounded up to even floats). -- */
int cc_random(cc_handle output, size_t n, uint32_t seed, int normal);

/* ---- events: replace Event.waitFor / waitForStatus / release
 *      (OpenCL.scala:565-611, :1246-1263).  Waits are bounded and return
 *      CC_ERR_TIMEOUT instead of hanging. ---------------------------------- */
int cc_event_record(cc_handle *event);
int cc_event_query(cc_handle event, int *complete);
int cc_event_wait(cc_handle event, uint64_t timeout_ns);
int cc_event_elapsed(cc_handle start, cc_handle end, float *ms);
int cc_event_release(cc_handle event);

#ifdef __cplusplus
}
#endif

#endif /* COMPUTE_CUDA_H */
