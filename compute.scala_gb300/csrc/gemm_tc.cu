// Split-BF16 contraction on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C = A * B for float A[M,K], B[K,N].  Each operand is split into three
// bfloat16 planes (x = hi + mid + lo, gemm.cu) and C accumulates, in FP32 in
// tensor memory, the six products whose order of magnitude is at least
// 2^-16 of the leading one: hi*hi, hi*mid, mid*hi, mid*mid, hi*lo, lo*hi.  The
// dropped products (mid*lo, lo*mid, lo*lo) are below 2^-24 relative.  hi*hi
// accumulates in one TMEM accumulator and the five small products in a second
// one, added once in the epilogue: adding a product 2^-8 smaller into the big
// accumulator would cost up to an ulp of it each time.
//
// Kernel structure (one CTA per SM, persistent over 128 x BN output tiles):
//   warp 0      TMA producer: per k-block of 32, loads the 3 A planes (128x32)
//               and the 3 B^T planes (BNx32) into a shared-memory ring of
//               STAGES, 64-byte swizzled, completing on the stage's "full"
//               mbarrier;
//   warp 1      allocates 512 TMEM columns (ACC_BUFS pairs of BN-column FP32
//               accumulators), and one thread issues the 12 tcgen05.mma (6
//               products x 2 k-steps of 16) per stage, committing to the stage's
//               "empty" mbarrier and, after a tile's last stage, to the
//               accumulator pair's "full";
//   warps 2..5  epilogue: tcgen05.ld both accumulators (each warp reads its own
//               32-lane quarter of TMEM, in the 16x256b shape so that four
//               threads hold 32 consecutive bytes of a row and every store
//               fills whole sectors), add, store to C, release the pair;
//               kernels that sum K chunks in registers have a second group,
//               warps 6..9, and each group takes half of the columns.
// With one accumulator pair of 256 columns (TMEM holds no second pair) and K
// chunks, only hi*hi restarts per chunk: the five small products, 2^-8 of it
// and smaller, accumulate over the whole K (their rounding stays far below
// the chunked hi*hi's), and at a chunk boundary the MMA thread issues the next
// k-block's small products before it waits for the epilogue to drain hi*hi, so
// the drain overlaps tensor work.
// Every mbarrier wait gives up after kWaitNs of %globaltimer time: it records
// an error code in *err, raises the CTA's abort flag, and all roles leave their
// loops, so the CTA still frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gemm.h"

namespace cc {
namespace {

constexpr int BM = 128, BK = 32;  // BK bf16 = 64 bytes = one 64-byte swizzle row
constexpr int kAPlaneBytes = BM * BK * 2;  // 8 KiB
constexpr int kTmemCols = 512;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s
// Warps: 0 = TMA, 1 = MMA and TMEM allocation, then the epilogue: one group of
// four warps (one per 32-lane quarter of TMEM) for kernels that store each
// accumulator pair directly, two groups splitting the columns for kernels that
// keep a running sum per row (half the registers each).
__host__ __device__ constexpr int epilogue_groups(int kc) { return kc > 0 ? 2 : 1; }
__host__ __device__ constexpr int threads_for(int kc) { return 64 + 128 * epilogue_groups(kc); }

template <int BN, int STAGES, int ACC_BUFS>
struct TcCfg {
  static_assert(ACC_BUFS * 2 * BN == kTmemCols, "two accumulators per buffer fill TMEM");
  static constexpr int kBPlaneBytes = BN * BK * 2;
  static constexpr int kStageBytes = 3 * kAPlaneBytes + 3 * kBPlaneBytes;
  // Shared memory after the stage ring (offsets from the 1 KiB-aligned base):
  // full[STAGES], empty[STAGES], acc_full[ACC_BUFS], acc_empty[ACC_BUFS], drain,
  // big_full, big_empty (kernels whose hi*hi chunks drain separately).
  static constexpr int kBarOffset = STAGES * kStageBytes;
  static constexpr int kNumBars = 2 * STAGES + 2 * ACC_BUFS + 3;
  static constexpr int kTmemSlotOffset = kBarOffset + kNumBars * 8;
  static constexpr int kAbortOffset = kTmemSlotOffset + 4;
  static constexpr int kSmemBytes = kAbortOffset + 4 + 1024;  // + slack to align the base to 1 KiB
  // Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M=128, N=BN.
  static constexpr uint32_t kIdesc =
      (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  // The same with N = BN / 2 (a tile split into column halves).
  static constexpr uint32_t kIdescHalf =
      (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 4) << 17) | ((uint32_t)(BM >> 4) << 24);
  static_assert(kSmemBytes <= 232448, "shared memory");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and the error recorded, the abort flag raised) on timeout
// or when another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err,
                                          int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > kWaitNs) {
      atomicCAS(err, 0, code);
      *abort_flag = 1;
      return false;
    }
    __nanosleep(64);
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// tcgen05 shared-memory descriptor: K-major operand, 64-byte swizzle, 8-row
// groups 512 bytes apart (SBO), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);        // start address, 16-byte units
  d |= (uint64_t)(16u >> 4) << 16;                // leading byte offset (unused for this layout)
  d |= (uint64_t)(512u >> 4) << 32;               // stride byte offset
  d |= (uint64_t)1 << 46;                         // descriptor version
  d |= (uint64_t)4 << 61;                         // SWIZZLE_64B
  return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 columns of the 32 TMEM lanes of this warp's subpartition, read as two
// 16x256b.x4 loads (lanes 0-15, then 16-31).  Thread t receives, for h = 0, 1 and
// k = 0..3: v[16h + 4k + {0,1}] = lane 16h + t/4, columns 8k + 2(t%4) + {0,1};
// v[16h + 4k + {2,3}] = lane 16h + t/4 + 8, the same columns.  Four threads hold
// 32 consecutive bytes of a row, so the stores below fill whole 32-byte sectors.
__device__ __forceinline__ void tmem_ld_block32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
#pragma unroll
  for (int h = 0; h < 2; ++h)
    asm volatile(
        "tcgen05.ld.sync.aligned.16x256b.x4.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[16 * h + 0]), "=r"(r[16 * h + 1]), "=r"(r[16 * h + 2]), "=r"(r[16 * h + 3]), "=r"(r[16 * h + 4]),
          "=r"(r[16 * h + 5]), "=r"(r[16 * h + 6]), "=r"(r[16 * h + 7]), "=r"(r[16 * h + 8]), "=r"(r[16 * h + 9]),
          "=r"(r[16 * h + 10]), "=r"(r[16 * h + 11]), "=r"(r[16 * h + 12]), "=r"(r[16 * h + 13]),
          "=r"(r[16 * h + 14]), "=r"(r[16 * h + 15])
        : "r"(taddr + ((uint32_t)(16 * h) << 16)));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Stores a block read by tmem_ld_block32: row0 is the output row of the
// subpartition's lane 0, col0 the block's first column (masked to M and N).
// vec2: C and ldc allow 8-byte stores.
__device__ __forceinline__ void store_block32(float *C, int row0, int col0, int M, int N, long long ldc, bool vec2,
                                              const float *v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int row = row0 + 16 * h + (lane >> 2) + 8 * g;
        const int col = col0 + 8 * k + 2 * (lane & 3);
        const float a = v[16 * h + 4 * k + 2 * g], b = v[16 * h + 4 * k + 2 * g + 1];
        if (row >= M) continue;
        float *p = C + (long long)row * ldc + col;
        if (vec2 && col + 1 < N) {
          *reinterpret_cast<float2 *>(p) = make_float2(a, b);
        } else {
          if (col < N) p[0] = a;
          if (col + 1 < N) p[1] = b;
        }
      }
}

// Origin of output tile `tile` in tile units.  Tiles are numbered in groups of
// `group_m` tile rows, columns outermost within a group, so the CTAs working at
// the same time share a few A and B panels in L2 (group_m = 1: row-major).
__device__ __forceinline__ void tile_origin(int tile, int tiles_m, int tiles_n, int group_m, int &tm, int &tn) {
  const int per_group = group_m * tiles_n;
  const int first = (tile / per_group) * group_m;
  const int rows = tiles_m - first < group_m ? tiles_m - first : group_m;
  const int in = tile - (tile / per_group) * per_group;
  tm = first + in % rows;
  tn = in / rows;
}

// Work item `item` of a persistent grid whose last tiles run as two column
// halves: items below `full` are whole tiles, then two per remaining tile, so
// the last round of a grid that does not divide the tiles is half as long.
// half: -1 for a whole tile, else 0 or 1.
__device__ __forceinline__ void item_origin(int item, int full, int tiles_m, int tiles_n, int group_m, int bn,
                                            int &m0, int &n0, int &half) {
  int tile = item;
  half = -1;
  if (item >= full) {
    tile = full + ((item - full) >> 1);
    half = (item - full) & 1;
  }
  int tm, tn;
  tile_origin(tile, tiles_m, tiles_n, group_m, tm, tn);
  m0 = tm * BM;
  n0 = tn * bn + (half > 0 ? bn / 2 : 0);
}

// The six (A plane, B plane) products, largest first: (0,0) (0,1) (1,0) (1,1)
// (0,2) (2,0).  Compile-time functions, so the unrolled issue loop folds them.
__host__ __device__ constexpr int prod_a(int p) { return p == 2 || p == 3 ? 1 : p == 5 ? 2 : 0; }
__host__ __device__ constexpr int prod_b(int p) { return p == 1 || p == 3 ? 1 : p == 4 ? 2 : 0; }

template <int BN, int STAGES, int ACC_BUFS, int KC>
__global__ void __launch_bounds__(threads_for(KC), 1)
    gemm_bf16x6_kernel(const __grid_constant__ CUtensorMap ta0, const __grid_constant__ CUtensorMap ta1,
                       const __grid_constant__ CUtensorMap ta2, const __grid_constant__ CUtensorMap tb0,
                       const __grid_constant__ CUtensorMap tb1, const __grid_constant__ CUtensorMap tb2,
                       const __grid_constant__ CUtensorMap th0, const __grid_constant__ CUtensorMap th1,
                       const __grid_constant__ CUtensorMap th2, float *__restrict__ C, int M, int N, long long ldc,
                       int num_kb, int tiles_n, int num_tiles, int full_tiles, int group_m, int *err) {
  using Cfg = TcCfg<BN, STAGES, ACC_BUFS>;
  constexpr int kStages = STAGES;
  constexpr int kStageBytes = Cfg::kStageBytes;
  constexpr int kBPlaneBytes = Cfg::kBPlaneBytes;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t base = smem_u32(smem);
  const uint32_t bar_full = base + Cfg::kBarOffset;            // + 8*s
  const uint32_t bar_empty = bar_full + 8 * kStages;           // + 8*s
  const uint32_t bar_accfull = bar_empty + 8 * kStages;        // + 8*a
  const uint32_t bar_accempty = bar_accfull + 8 * ACC_BUFS;    // + 8*a
  const uint32_t bar_drain = bar_accempty + 8 * ACC_BUFS;
  const uint32_t bar_bigfull = bar_drain + 8;   // (late-small kernels) a hi*hi chunk is complete
  const uint32_t bar_bigempty = bar_drain + 16; // (late-small kernels) the epilogue has read it
  // One 256-column pair and K chunks: hi*hi drains per chunk, the rest per tile.
  constexpr bool kLate = ACC_BUFS == 1 && KC > 0;
  // items: whole tiles, then column halves of the rest (only kLate kernels are given full_tiles < num_tiles)
  const int num_items = full_tiles + 2 * (num_tiles - full_tiles);
  const int tiles_m = num_tiles / tiles_n;
  volatile uint32_t *tmem_slot = reinterpret_cast<volatile uint32_t *>(smem + Cfg::kTmemSlotOffset);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + Cfg::kAbortOffset);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_empty + 8 * s, 1);
    }
    for (int a = 0; a < ACC_BUFS; ++a) {
      mbar_init(bar_accfull + 8 * a, 1);
      mbar_init(bar_accempty + 8 * a, 128 * epilogue_groups(KC));
    }
    mbar_init(bar_drain, 1);
    mbar_init(bar_bigfull, 1);
    mbar_init(bar_bigempty, 128 * epilogue_groups(KC));
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((const void *)tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      const CUtensorMap *ta[3] = {&ta0, &ta1, &ta2};
      const CUtensorMap *tb[3] = {&tb0, &tb1, &tb2};
      const CUtensorMap *th[3] = {&th0, &th1, &th2};  // B planes, half-width boxes
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      uint32_t fill_parity[kStages];
      bool filled[kStages];
#pragma unroll
      for (int s = 0; s < kStages; ++s) filled[s] = false;
      for (int item = blockIdx.x; item < num_items && ok; item += gridDim.x) {
        int m0, n0, half;
        item_origin(item, full_tiles, tiles_m, tiles_n, group_m, BN, m0, n0, half);
        const CUtensorMap *const *tbs = half < 0 ? tb : th;
        // a half tile fills the first half of each B plane slot
        const uint32_t bytes = half < 0 ? (uint32_t)kStageBytes : (uint32_t)(3 * kAPlaneBytes + 3 * (kBPlaneBytes / 2));
        for (int kb = 0; kb < num_kb; ++kb) {
          if (!mbar_wait(bar_empty + 8 * stage, phase ^ 1u, abort_flag, err, 1)) {
            ok = false;
            break;
          }
          const uint32_t sbase = base + stage * kStageBytes;
          filled[stage] = true;
          fill_parity[stage] = phase;
          mbar_arrive_expect_tx(bar_full + 8 * stage, bytes);
#pragma unroll
          for (int p = 0; p < 3; ++p) tma_load_2d(sbase + p * kAPlaneBytes, ta[p], kb * BK, m0, bar_full + 8 * stage);
#pragma unroll
          for (int p = 0; p < 3; ++p)
            tma_load_2d(sbase + 3 * kAPlaneBytes + p * kBPlaneBytes, tbs[p], kb * BK, n0, bar_full + 8 * stage);
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1u;
          }
        }
      }
      // Before the CTA may exit, every load this thread issued must have landed
      // (a normal run's consumer has already waited for all of them; after an
      // abort they may still be in flight).  The last fill of each stage
      // completes the phase of its recorded parity; the wait is bounded.
      if (!ok) {
        for (int s = 0; s < kStages; ++s) {
          if (!filled[s]) continue;
          const unsigned long long t0 = globaltimer();
          while (!mbar_try_wait(bar_full + 8 * s, fill_parity[s]) && globaltimer() - t0 < kWaitNs) __nanosleep(64);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0 && kLate) {
      int stage = 0;
      uint32_t phase = 0, small_phase = 0, big_phase = 0;
      bool ok = true;
      const uint32_t d_big = tmem_base, d_small = tmem_base + BN;
      for (int item = blockIdx.x; item < num_items && ok; item += gridDim.x) {
        int m0, n0, half;
        item_origin(item, full_tiles, tiles_m, tiles_n, group_m, BN, m0, n0, half);
        const uint32_t idesc = half < 0 ? Cfg::kIdesc : Cfg::kIdescHalf;
        for (int kb = 0; kb < num_kb; ++kb) {
          if (!mbar_wait(bar_full + 8 * stage, phase, abort_flag, err, 3)) {
            ok = false;
            break;
          }
          if (kb == 0 && !mbar_wait(bar_accempty, small_phase ^ 1u, abort_flag, err, 2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint64_t sdesc = smem_desc(base + stage * kStageBytes);
#pragma unroll
          for (int k16 = 0; k16 < BK / 16; ++k16) {
#pragma unroll
            for (int prod = 1; prod < 6; ++prod) {
              const uint64_t adesc = sdesc + (uint64_t)((prod_a(prod) * kAPlaneBytes + k16 * 32) >> 4);
              const uint64_t bdesc =
                  sdesc + (uint64_t)((3 * kAPlaneBytes + prod_b(prod) * kBPlaneBytes + k16 * 32) >> 4);
              mma_bf16(d_small, adesc, bdesc, idesc, (kb == 0 && k16 == 0 && prod == 1) ? 0u : 1u);
            }
          }
          const bool chunk_start = kb % KC == 0;
          if (chunk_start) {
            if (!mbar_wait(bar_bigempty, big_phase ^ 1u, abort_flag, err, 2)) {
              ok = false;
              break;
            }
            tc_fence_after();
          }
#pragma unroll
          for (int k16 = 0; k16 < BK / 16; ++k16) {
            const uint64_t adesc = sdesc + (uint64_t)((k16 * 32) >> 4);
            const uint64_t bdesc = sdesc + (uint64_t)((3 * kAPlaneBytes + k16 * 32) >> 4);
            mma_bf16(d_big, adesc, bdesc, idesc, (chunk_start && k16 == 0) ? 0u : 1u);
          }
          mma_commit(bar_empty + 8 * stage);
          if (++stage == kStages) {
            stage = 0;
            phase ^= 1u;
          }
          if ((kb + 1) % KC == 0 || kb + 1 == num_kb) {
            mma_commit(bar_bigfull);  // this hi*hi chunk is complete
            big_phase ^= 1u;
          }
        }
        if (!ok) break;
        mma_commit(bar_accfull);  // the small products of the tile are complete
        small_phase ^= 1u;
      }
      mma_commit(bar_drain);
      const unsigned long long t0 = globaltimer();
      while (!mbar_try_wait(bar_drain, 0) && globaltimer() - t0 < kWaitNs) __nanosleep(64);
    } else if (lane == 0) {
      int stage = 0, acc = 0;
      uint32_t phase = 0, acc_phase = 0;
      bool ok = true;
      // K is processed in chunks of KC k-blocks (the whole K when KC == 0); each
      // chunk accumulates into a fresh accumulator pair.
      const int kc = KC > 0 ? KC : num_kb;
      for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
        for (int kb0 = 0; kb0 < num_kb && ok; kb0 += kc) {
          if (!mbar_wait(bar_accempty + 8 * acc, acc_phase ^ 1u, abort_flag, err, 2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d_big = tmem_base + (uint32_t)(acc * 2 * BN);  // hi*hi
          const uint32_t d_small = d_big + BN;                           // the five small products
          const int kend = kb0 + kc < num_kb ? kb0 + kc : num_kb;
          for (int kb = kb0; kb < kend; ++kb) {
            if (!mbar_wait(bar_full + 8 * stage, phase, abort_flag, err, 3)) {
              ok = false;
              break;
            }
            tc_fence_after();
            // One descriptor per stage; each operand's is that plus a constant
            // (16-byte units: shared addresses stay below 256 KiB, so the
            // 14-bit start-address field never carries).
            const uint64_t sdesc = smem_desc(base + stage * kStageBytes);
            const uint32_t fresh = kb == kb0 ? 1u : 0u;
#pragma unroll
            for (int k16 = 0; k16 < BK / 16; ++k16) {
#pragma unroll
              for (int prod = 0; prod < 6; ++prod) {
                const uint64_t adesc = sdesc + (uint64_t)((prod_a(prod) * kAPlaneBytes + k16 * 32) >> 4);
                const uint64_t bdesc =
                    sdesc + (uint64_t)((3 * kAPlaneBytes + prod_b(prod) * kBPlaneBytes + k16 * 32) >> 4);
                // the first product into each accumulator of a chunk overwrites it
                const uint32_t overwrite = (k16 == 0 && (prod == 0 || prod == 1)) ? fresh : 0u;
                mma_bf16(prod == 0 ? d_big : d_small, adesc, bdesc, Cfg::kIdesc, overwrite ^ 1u);
              }
            }
            mma_commit(bar_empty + 8 * stage);  // the stage is free once these MMAs have read it
            if (++stage == kStages) {
              stage = 0;
              phase ^= 1u;
            }
          }
          if (!ok) break;
          mma_commit(bar_accfull + 8 * acc);  // the accumulator pair is complete
          if (++acc == ACC_BUFS) {
            acc = 0;
            acc_phase ^= 1u;
          }
        }
      }
      // Every MMA this thread issued must be complete before TMEM is freed.
      mma_commit(bar_drain);
      const unsigned long long t0 = globaltimer();
      while (!mbar_try_wait(bar_drain, 0) && globaltimer() - t0 < kWaitNs) __nanosleep(64);
    }
    __syncwarp();
  } else {
    // Epilogue: warp w reads TMEM lanes 32*(w%4) .. 32*(w%4)+31 (one row each).
    const int quarter = warp & 3;
    const int row_block = quarter * 32;  // the tile row of this subpartition's lane 0
    int acc = 0;
    uint32_t acc_phase = 0;
    const uint32_t lane_tmem = tmem_base + ((uint32_t)(quarter * 32) << 16);
    const bool vec2 = (ldc & 1) == 0 && (reinterpret_cast<uintptr_t>(C) & 7) == 0;
    if constexpr (kLate) {
      // hi*hi per chunk into a running sum of the row; the small products once
      // per tile, added last.
      const int nchunks = (num_kb + KC - 1) / KC;
      constexpr int kCols = BN / epilogue_groups(KC);  // columns of a group in a whole tile
      const int group = (warp - 2) >> 2;
      uint32_t big_phase = 0, small_phase = 0;
      bool ok = true;
      for (int item = blockIdx.x; item < num_items && ok; item += gridDim.x) {
        int m0, n0, half;
        item_origin(item, full_tiles, tiles_m, tiles_n, group_m, BN, m0, n0, half);
        const int cols = half < 0 ? kCols : kCols / 2;  // this group's columns of the item
        const int col0 = group * cols;
        float sum[kCols];
#pragma unroll
        for (int j = 0; j < kCols; ++j) sum[j] = 0.0f;
        for (int ch = 0; ch < nchunks; ++ch) {
          if (!mbar_wait(bar_bigfull, big_phase, abort_flag, err, 4)) {
            ok = false;
            break;
          }
          big_phase ^= 1u;
          tc_fence_after();
#pragma unroll
          for (int c32 = 0; c32 < kCols / 32; ++c32) {
            if (c32 * 32 >= cols) break;
            float v[32];
            tmem_ld_block32(lane_tmem + (uint32_t)(col0 + c32 * 32), v);
#pragma unroll
            for (int j = 0; j < 32; ++j) sum[c32 * 32 + j] = __fadd_rn(sum[c32 * 32 + j], v[j]);
          }
          tc_fence_before();
          mbar_arrive(bar_bigempty);
        }
        if (!ok) break;
        if (!mbar_wait(bar_accfull, small_phase, abort_flag, err, 4)) break;
        small_phase ^= 1u;
        tc_fence_after();
#pragma unroll
        for (int c32 = 0; c32 < kCols / 32; ++c32) {
          if (c32 * 32 >= cols) break;
          float w[32];
          tmem_ld_block32(lane_tmem + (uint32_t)(BN + col0 + c32 * 32), w);
#pragma unroll
          for (int j = 0; j < 32; ++j) w[j] = __fadd_rn(sum[c32 * 32 + j], w[j]);
          store_block32(C, m0 + row_block, n0 + col0 + c32 * 32, M, N, ldc, vec2, w);
        }
        tc_fence_before();
        mbar_arrive(bar_accempty);
      }
    } else if constexpr (KC == 0) {
      // One accumulator pair per tile: add the pair and store, 32 columns at a time.
      for (int tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
        if (!mbar_wait(bar_accfull + 8 * acc, acc_phase, abort_flag, err, 4)) break;
        tc_fence_after();
        int tm, tn;
        tile_origin(tile, num_tiles / tiles_n, tiles_n, group_m, tm, tn);
        const int m0 = tm * BM, n0 = tn * BN;
#pragma unroll 1
        for (int chunk = 0; chunk < BN / 32; ++chunk) {
          float v[32], w[32];
          const uint32_t t = lane_tmem + (uint32_t)(acc * 2 * BN + chunk * 32);
          tmem_ld_block32(t, v);
          tmem_ld_block32(t + BN, w);
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = __fadd_rn(v[j], w[j]);
          store_block32(C, m0 + row_block, n0 + chunk * 32, M, N, ldc, vec2, v);
        }
        tc_fence_before();
        mbar_arrive(bar_accempty + 8 * acc);
        if (++acc == ACC_BUFS) {
          acc = 0;
          acc_phase ^= 1u;
        }
      }
    } else {
      // A pair per K chunk: fold each into a running sum of the row (in
      // registers, round-to-nearest), so no FP32 accumulator inside the tensor
      // core takes more than KC k-blocks of additions.
      const int nchunks = (num_kb + KC - 1) / KC;
      constexpr int kCols = BN / epilogue_groups(KC);      // columns of this thread's group
      const int col0 = ((warp - 2) >> 2) * kCols;           // group 0: warps 2-5, group 1: warps 6-9
      bool ok = true;
      for (int tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x) {
        float sum[kCols];
#pragma unroll
        for (int j = 0; j < kCols; ++j) sum[j] = 0.0f;
        for (int ch = 0; ch < nchunks; ++ch) {
          if (!mbar_wait(bar_accfull + 8 * acc, acc_phase, abort_flag, err, 4)) {
            ok = false;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int c32 = 0; c32 < kCols / 32; ++c32) {
            float v[32], w[32];
            const uint32_t t = lane_tmem + (uint32_t)(acc * 2 * BN + col0 + c32 * 32);
            tmem_ld_block32(t, v);
            tmem_ld_block32(t + BN, w);
#pragma unroll
            for (int j = 0; j < 32; ++j) sum[c32 * 32 + j] = __fadd_rn(sum[c32 * 32 + j], __fadd_rn(v[j], w[j]));
          }
          tc_fence_before();
          mbar_arrive(bar_accempty + 8 * acc);
          if (++acc == ACC_BUFS) {
            acc = 0;
            acc_phase ^= 1u;
          }
        }
        if (!ok) break;
        int tm, tn;
        tile_origin(tile, num_tiles / tiles_n, tiles_n, group_m, tm, tn);
        const int m0 = tm * BM, n0 = tn * BN;
#pragma unroll
        for (int c32 = 0; c32 < kCols / 32; ++c32)
          store_block32(C, m0 + row_block, n0 + col0 + c32 * 32, M, N, ldc, vec2, sum + c32 * 32);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols) : "memory");
  }
}

template <int BN, int STAGES, int ACC_BUFS, int KC>
cudaError_t launch_variant(const CUtensorMap *maps, float *C, int M, int N, int K_padded, long long ldc, int sm_count,
                           int group_m, int *err, cudaStream_t stream) {
  using Cfg = TcCfg<BN, STAGES, ACC_BUFS>;
  // The dynamic shared-memory limit is a per-device attribute of the kernel; set
  // it on every launch (a cheap host call) so a second device, or another thread,
  // never launches without it.
  cudaError_t e = cudaFuncSetAttribute(gemm_bf16x6_kernel<BN, STAGES, ACC_BUFS, KC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmemBytes);
  if (e != cudaSuccess) return e;
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int num_tiles = tiles_m * tiles_n;
  const int num_kb = K_padded / BK;
  const int grid = num_tiles < sm_count ? num_tiles : sm_count;
  // Kernels with one 256-column accumulator pair and K chunks split the tiles
  // of a last, partial round into column halves when those fit one round.
  int full = num_tiles;
  const int rem = num_tiles % grid;
  if (ACC_BUFS == 1 && KC > 0 && num_tiles > grid && rem > 0 && 2 * rem <= grid) full = num_tiles - rem;
  gemm_bf16x6_kernel<BN, STAGES, ACC_BUFS, KC><<<grid, threads_for(KC), Cfg::kSmemBytes, stream>>>(
      maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], maps[6], maps[7], maps[8], C, M, N, ldc, num_kb,
      tiles_n, num_tiles, full, group_m < 1 ? 1 : group_m, err);
  return cudaGetLastError();
}

}  // namespace

int gemm_tc_box_n(int variant) { return variant == 1 || variant == 5 ? 256 : 128; }

int gemm_tc_variant(int variant, int K_padded) {
  // When K fits in one chunk the running sum only adds the pair to zero, which
  // changes no value (at most the sign of a zero result): a one-pair-per-tile
  // kernel computes the same without the running sum's registers.  The
  // 128-column one holds two accumulator pairs, so the epilogue of one tile
  // overlaps the products of the next (K = 256, 16384 x 16384: 241.7 against
  // 208.0 TFLOP/s for the 256-column kernel with one pair).
  const int num_kb = K_padded / BK;
  if ((variant == 0 && num_kb <= 4) || (variant == 3 && num_kb <= 8) || (variant == 4 && num_kb <= 16)) return 2;
  if (variant == 5 && num_kb <= 8) return 2;
  return variant;
}

cudaError_t launch_gemm_bf16x6(const CUtensorMap *maps, float *C, int M, int N, int K_padded, long long ldc,
                               int sm_count, int *err, int variant, int group_m, cudaStream_t stream) {
  // the maps were encoded for the resolved variant's tile width
  if (variant != gemm_tc_variant(variant, K_padded)) return cudaErrorInvalidValue;
  if (variant == 5) return launch_variant<256, 3, 1, 8>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
  if (variant == 1) return launch_variant<256, 3, 1, 0>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
  if (variant == 2) return launch_variant<128, 4, 2, 0>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
  if (variant == 3) return launch_variant<128, 4, 2, 8>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
  if (variant == 4) return launch_variant<128, 4, 2, 16>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
  return launch_variant<128, 4, 2, 4>(maps, C, M, N, K_padded, ldc, sm_count, group_m, err, stream);
}

}  // namespace cc
