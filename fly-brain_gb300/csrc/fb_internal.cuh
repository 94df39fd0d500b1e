// Internal device structures and helpers of the GB300 brain step. Not part of the C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/flybrain.h"

namespace fb {

constexpr int kBlock = 512;          // threads per block of the persistent step kernel
constexpr int kNPT = 2;              // neurons per thread in the update phase
constexpr int kTile = kBlock * kNPT; // neurons per update tile
constexpr int kSub = 64;             // neurons per warp sub-tile (a warp's share of a tile, 2 per lane)
constexpr int kSubPerTile = kTile / kSub;  // the unit of spike staging, one per warp of the block
static_assert(kSubPerTile * 32 == kBlock, "one warp per sub-tile");
constexpr int kDrivenPer = 8;        // driven-list entries per thread and round
constexpr int kChunk = 32;           // edges per delivery work item (one per lane)
constexpr int kBucket = 8;           // in-place contribution slots per target and step
constexpr int kSortMax = 64;         // contributions per target sorted in local memory
constexpr uint32_t kNil = 0xffffffffu;
// A row may name one target up to kMaxRepeat + 1 times; a contribution's key is
// (arrival rank << 3) | (repeat index << 1) | inhibitory, so repeats sort in row order.
constexpr int kMaxRepeat = 3;

// Per-brain flags (Trial::flags).
constexpr int32_t kHasBg = 1;        // background events enabled (bgEvents > 0)
constexpr int32_t kHasDep = 2;       // synaptic depression enabled (depU != 0)
// Constant state: with adaptInc == 0 an adapt field that is exactly 0 everywhere stays 0
// (0 * dA = 0, 0 + 0 = 0), and with depU == 0 a res field that is exactly 1 stays 1
// (1 + (1 - 1) kRec = 1): the update neither reads nor writes it. Set at reset, cleared when the
// host writes the field.
constexpr int32_t kAdaptZero = 8;
constexpr int32_t kResRest = 16;
constexpr int32_t kHasPreInh = 4;    // presynaptic inhibition (forces sequential delivery)
// Zero parameters: a bias (thr) field whose every word is +0.0f, as at creation, is not read; the
// update adds the literal +0.0f in its place, the same IEEE operation on the same operands.
// Cleared when the host stores a word other than +0.0f into the field.
constexpr int32_t kBiasZero = 32;
constexpr int32_t kThrZero = 64;

// One brain of a batch: header constants (f32, rounded once from f64 on the host, the values
// LIFWasm._writeHeader stores), graph and state pointers, delivery scratch, dynamic scalars.
struct Trial {
  int32_t N, nslots, coba, mode;
  int64_t E;
  float dt, vRest, vThresh, vReset, tRef, adaptInc, depU, dE, dTr, dA, kRec, kM, dtS;
  float eExc, eInh, cE, cI, bgEvents, bgAmp, preInh;
  int32_t tileBase, nTiles, flags, pad0;
  int64_t chunkCap;  // delivery work items per ring slot
  // graph (shared, read-only during a step)
  const uint32_t *indptr, *indices;
  const float *W, *sign;
  const uint8_t *dup;  // per edge: its repeat index in its row (null: no row repeats a target)
  // state, SoA, N each
  float *v, *gE, *gI, *refr, *trace, *adapt, *res, *bias, *thr, *drive;
  uint32_t *spikeCount;
  // delay ring: nslots lists of N, counts, per-arrival edge offsets (N+1 per slot) and row starts
  // (N per slot), each slot's total edge count, and per 32-edge delivery work item (chunkCap per
  // slot) its first arrival: {rank k, presynaptic neuron, end of k's edges, row start - offset}
  int32_t *ring, *ringCount;
  uint32_t *ringOff, *ringRow, *slotEdges;
  uint4 *chunkK;
  int32_t *driven;
  // delivery scratch: contribution counts and buckets per target, overflow list heads,
  // background hits, arrival marks
  uint32_t *cnt;
  uint2 *bucket;
  uint32_t *ovfHead, *bgHits;
  uint8_t *arrived;
  // threshold-spike staging per update tile (compacted list + out-degree prefix)
  int32_t *stage;
  uint32_t *stageDeg;
  int32_t *tileCnt;    // [nTiles * kSubPerTile], indexed by the brain-local warp sub-tile
  uint32_t *tileDeg;
  // forced-spike staging per driven-list chunk of kBlock entries, two step parities:
  // dStage/dStageDeg [2][maxDch * kBlock], dCnt/dDeg [2][maxDch]; liveTag[maxDch] publishes each
  // chunk's count of non-refractory entries (high word: step + 1) for the chunks after it
  int32_t *dStage;
  uint32_t *dStageDeg;
  int32_t *dCnt;
  uint32_t *dDeg;
  unsigned long long *liveTag;
  int32_t maxDch, pad1;
  // optional per-step log of fired counts and fired lists
  int32_t *logCount;
  int32_t *logRaster;
  int64_t logCap, logRasterCap;
  // dynamic scalars (device-written). The RNG state and background accumulator at the start of
  // global step g are rngP[g & 1] and bgAccP[g & 1]; step g writes the other halves.
  uint32_t rngP[2];
  float bgAccP[2];
  int32_t head;
  int32_t nDriven;
  int32_t nFired, lastSlot;
  int64_t stepsDone;
  int64_t logStart;       // first logged step (global step index)
  int64_t logRasterLen[2];
};

// Overflow record of a target that received more than kBucket contributions in one step.
struct OvfRec {
  uint32_t key, bits, next, pad;
};

struct StepArgs {
  Trial *trials;
  int32_t B, maxSteps;
  const int32_t *steps;      // per-brain steps of this launch
  const int32_t *tileTrial;  // update tile -> brain
  int32_t nTilesTotal, pad0;
  const uint32_t *jump;      // xorshift32 jump tables [32][8][16]
  uint32_t *barCount;         // the barrier word
  unsigned long long *phaseNs;  // optional per-phase time accumulators (null: off)
  int32_t *err;
  OvfRec *ovf[2];
  uint32_t *ovfTop;          // [2]
  uint32_t ovfCap;
  int32_t log;               // 1: record per-step fired counts / lists
  int32_t itemChunks;        // kChunk-edge delivery chunks per warp work item (>= 1)
  int32_t subGrab;           // update sub-tiles per dynamic grab (0: every sub-tile dealt statically)
  uint32_t *subNext;         // [2] per step parity: next dynamically dealt sub-tile
  int64_t timeoutNs;
  uint32_t *dbg;             // checked builds: [site, value, value, count] of the first bad index
};

// Index checks of the checked build (-DFB_CHECK): a failed check records its site and values in
// a.dbg (the first one only), sets FB_EINVAL and skips the access. Compiled out otherwise.
#ifdef FB_CHECK
#define FB_GUARD(a, cond, site, v1, v2, skip)                                    \
  do {                                                                           \
    if (!(cond)) {                                                               \
      if ((a).dbg && atomicCAS((a).dbg, 0u, (uint32_t)(site)) == 0u) {         \
        (a).dbg[1] = (uint32_t)(v1);                                            \
        (a).dbg[2] = (uint32_t)(v2);                                            \
      }                                                                          \
      if ((a).dbg) atomicAdd((a).dbg + 3, 1u);                                  \
      atomicCAS((a).err, 0, FB_EINVAL);                                          \
      skip;                                                                      \
    }                                                                            \
  } while (0)
#else
#define FB_GUARD(a, cond, site, v1, v2, skip) \
  do {                                        \
  } while (0)
#endif

// ---- memory helpers --------------------------------------------------------------------------
// Data written by other blocks during the same launch is read through L2 (ld.global.cg): L1 is
// not coherent across SMs.
template <typename T>
__device__ __forceinline__ T ldcg(const T *p) { return __ldcg(p); }

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int32_t ld_volatile(const int32_t *p) {
  return *(const volatile int32_t *)p;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a co-resident (cooperative) grid on one counter word: block 0 adds
// 0x80000000 - (grid - 1), every other block adds 1, so bit 31 of the word flips exactly when the
// last block arrives (sense reversal by overflow: the word never needs resetting). A block waits
// until bit 31 differs from the value its own arrival returned. Every wait is bounded, by
// %globaltimer (timeoutNs) and by an iteration cap: a waiter that gives up records FB_ETIMEOUT in
// *err and returns false; every block returns false once *err is set, so all blocks leave the
// kernel at the same barrier.
__device__ __forceinline__ bool grid_sync(const StepArgs &a) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const uint32_t add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    __threadfence();
    const uint32_t old = atomicAdd(a.barCount, add);
    const uint64_t t0 = global_ns();
    uint32_t it = 0;
    while (((ld_relaxed(a.barCount) ^ old) & 0x80000000u) == 0) {
      ++it;
      if ((it & 63u) == 0) {
        if (ld_volatile(a.err) != 0) { ok = 0; break; }
        if (global_ns() - t0 > (uint64_t)a.timeoutNs || it > (1u << 30)) {
          atomicCAS(a.err, 0, FB_ETIMEOUT);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    if (ok && ld_volatile(a.err) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---- xorshift32 ------------------------------------------------------------------------------
// lif.c's generator (src/wasm/lif.c:27). It is linear over GF(2): the state after d draws is
// M^d s. jump[j] holds M^(2^j) as 8 nibble tables of 16 words, so applying it costs 8 lookups.
__device__ __forceinline__ uint32_t xs_next(uint32_t x) {
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  return x;
}

__device__ __forceinline__ uint32_t xs_apply(const uint32_t *tab, uint32_t x) {
  uint32_t y = 0;
#pragma unroll
  for (int n = 0; n < 8; n++) y ^= tab[n * 16 + ((x >> (4 * n)) & 15u)];
  return y;
}

// State after d draws from s.
__device__ __forceinline__ uint32_t xs_jump(const uint32_t *jump, uint32_t s, uint32_t d) {
  while (d) {
    const int j = __ffs(d) - 1;
    s = xs_apply(jump + j * 128, s);
    d &= d - 1;
  }
  return s;
}

// ---- block scans -----------------------------------------------------------------------------
// Exclusive prefix over the block (blockDim.x a multiple of 32, <= 1024). *total receives the
// block sum. Uses scratch[32].
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T x, T *total, T *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  __syncthreads();
  if (lane == 31) scratch[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? scratch[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < nw) scratch[lane] = wi - w;
    if (lane == 31) scratch[32] = wi;
  }
  __syncthreads();
  const T res = scratch[warp] + inc - x;
  *total = scratch[32];
  __syncthreads();
  return res;
}

// Sum over the block; every thread receives it. Uses scratch[33].
template <typename T>
__device__ __forceinline__ T block_sum(T x, T *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  __syncthreads();
  if (lane == 0) scratch[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < nw ? scratch[lane] : T(0);
#pragma unroll
    for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (lane == 0) scratch[32] = w;
  }
  __syncthreads();
  const T r = scratch[32];
  __syncthreads();
  return r;
}

// Write the "first arrival" index k into every delivery work item that starts inside arrival
// k's edge range [o, o + deg).
__device__ __forceinline__ void mark_chunks(uint4 *chunkK, uint32_t o, uint32_t deg, uint32_t k,
                                            uint32_t pre, uint32_t row) {
  const uint32_t end = o + deg;
  const uint4 rec = make_uint4(k, pre, end, row - o);  // edge e of arrival k is row + (e - o)
  for (uint32_t c = (o + kChunk - 1) / kChunk; c * kChunk < end; c++) chunkK[c] = rec;  // c < chunkCap: end <= E
}

}  // namespace fb
