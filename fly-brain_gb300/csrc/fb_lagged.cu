// The brain step without a per-step grid barrier, for one brain advanced by many steps: the exact
// semantics of lif_step (src/wasm/lif.c:29-80), scheduled by the synaptic delay.
//
// A spike emitted at step s arrives D = nslots - 1 steps later (lif.c:44-45, 77-79). Its
// contributions are known at emission, so they are pushed then into per-arrival-step buckets;
// a block updating step t only needs every block to have finished step t - D (plus the helper
// delay below), not step t - 1. Blocks therefore advance on their own and synchronise through
// per-step completion counters with up to L = D - help steps of slack.
//
//  - Tile blocks (all but block 0) own fixed sets of non-driven neurons (contiguous ascending id
//    ranges), their state held in shared memory for the whole launch.
//  - The driven block (block 0) owns every Poisson-driven neuron and the generator: the
//    background draws and one draw per non-refractory driven neuron in list order (lif.c:46-52),
//    then those neurons' updates. Its spikes are pushed by the tile blocks `help` steps later.
//  - The summation order of lif.c is kept per target: each contribution carries its arrival's
//    rank in the fired list (forced spikes first in list order, then threshold spikes by
//    ascending id, lif.c:51-52, 73-76), and the target adds them in rank order.
//  - The amplitude sign*res of an arrival (lif.c:37) is fixed at emission by replaying the
//    presynaptic neuron's own depression and recovery up to the arrival step (its earlier spikes
//    in flight are known to its owner); the result is the value lif.c reads at delivery.
//  - At launch start the spikes already in flight (the ring) are pushed the same way; at the end
//    the last D fired lists are written back into the ring, so either kernel can continue.
//
// Not covered (the two-phase kernel runs these): presynaptic inhibition (its amplitude depends on
// the target state at delivery), sequential and fast delivery modes, batches, per-step logging.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "fb_internal.cuh"
#include "fb_lagged.cuh"

namespace fb {

constexpr int kLB = kLagThreads;
constexpr int kBgChunk = 1024;
constexpr int kHexLevels = 3;           // hexadecimal digits by table; beyond, M^4096 repeated
constexpr int kHexWords = (kHexLevels * 15 + 1) * 128;
constexpr int kOffWords = 32 * 128;

__device__ __forceinline__ void red_release(uint32_t *p, uint32_t v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int kMaxPer = kLagPer;

// Tile blocks: warps 0 .. kTW/32 - 1 update neurons; the last two warps serve them. The
// publisher warp releases the block's completion of each step and checks the lag for the next
// one; the helper warp loads the next step's share of the driven block's spikes into shared
// memory. Both do this while the workers run a step, so neither a release's wait for the block's
// writes nor the list's L2 round trips lies on the workers' path; the workers synchronise among
// themselves on named barrier 1 and with the service warps once per step (barrier 0).
constexpr int kTW = kLagTileWorkers;
constexpr int kTWarps = kTW / 32;
constexpr int kHelpMax = kLagHelpMax;  // the host keeps ceil(driven / tile blocks) within it

__device__ __forceinline__ void wbar() { asm volatile("bar.sync 1, %0;" ::"n"(kTW) : "memory"); }
__device__ __forceinline__ bool wbar_or(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p), "n"(kTW)
      : "memory");
  return r != 0;
}
// Exclusive prefix over the worker threads of a tile block; *total receives their sum.
__device__ __forceinline__ uint64_t worker_exclusive_scan(uint64_t x, uint64_t *total, uint64_t *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  wbar();
  if (lane == 31) scratch[warp] = inc;
  wbar();
  if (warp == 0) {
    const uint64_t w = lane < kTWarps ? scratch[lane] : 0ull;
    uint64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kTWarps) scratch[lane] = wi - w;
    if (lane == 31) scratch[32] = wi;
  }
  wbar();
  const uint64_t res = scratch[warp] + inc - x;
  *total = scratch[32];
  wbar();
  return res;
}

// Loads issued a step or two before their values are used (the count and first-entry prefetch).
// A plain load may be scheduled at any point before its first use, which for a prefetch can be
// the end of the step, exposing the whole L2 latency at the next step's start; these stay where
// they are written.
__device__ __forceinline__ uint32_t ld_early(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint2 ld_early(const uint2 *p) {
  uint2 v;
  asm volatile("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p) : "memory");
  return v;
}

struct LagShared {
  int32_t nLocal;  // neurons owned by this block
  int32_t dLo;     // driven block: list position of its first entry
  int32_t m;       // driven block: entries per thread
  int32_t idLo, idHi;
  int32_t stop;
  int32_t stopP[2];  // the lag check's verdict, by step parity (the driven block's steps have one
                     // barrier, so thread 0 may write step s + 1's before a slow warp reads step s's)
  uint32_t rng;
  float bgAcc;
  int32_t nbg;
  int32_t known;   // highest step known finished by every block
  int32_t head0;   // ring head at launch
  int64_t steps0;  // steps done before the launch
  int64_t logBase;
  uint32_t scan[33];
  uint64_t scan64[33];
  uint32_t dbCount;               // epilogue scratch
  // driven block, by step parity: each step prepares the next one's inputs while it runs, so a
  // step needs one block barrier. Live entries per warp and round (ballots after the previous
  // update), the generator at the step's start, its states at every 32nd driven draw, the
  // background draws, the accumulator after them, and the step's spike count.
  uint32_t wcnt[2][kMaxPer * 32];
  uint32_t cst[2][kLagMaxDB * kMaxPer * kLagThreads / 32];  // every 32nd draw of the whole list
  uint32_t rngP[2];
  int32_t nbgP[2];
  float bgAccP[2];
  uint32_t dbCnt2[2];
  // tile blocks, by step parity: the service warps' verdicts for the step and the helper warp's
  // share of the driven block's spikes ({row start, row end, rank key, amplitude})
  int32_t stopQ[2];
  int32_t helpN[2];
  uint4 help[2][kHelpMax];
};


__device__ __forceinline__ bool lag_timeout(const LagArgs &a, uint64_t t0, uint32_t &it) {
  if ((++it & 63u) == 0) {
    if (ld_volatile(a.err) != 0) return true;
    if (global_ns() - t0 > (uint64_t)a.timeoutNs || it > (1u << 30)) {
      atomicCAS(a.err, 0, FB_ETIMEOUT);
      return true;
    }
  }
  return false;
}

// Grid barrier of a cooperative launch (same scheme as grid_sync).
__device__ bool lag_grid_sync(const LagArgs &a) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const uint32_t add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    __threadfence();
    const uint32_t old = atomicAdd(a.barCount, add);
    const uint64_t t0 = global_ns();
    uint32_t it = 0;
    while (((ld_relaxed(a.barCount) ^ old) & 0x80000000u) == 0)
      if (lag_timeout(a, t0, it)) {
        ok = 0;
        break;
      }
    __threadfence();
    if (ok && ld_volatile(a.err) != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Waits (thread 0) until *p >= target (acquire); false on timeout or a recorded error. *seen
// (optional) receives the value observed.
__device__ __forceinline__ bool wait_geq(const LagArgs &a, const uint32_t *p, uint32_t target,
                                         uint32_t *seen = nullptr) {
  uint32_t v = ld_acquire(p);
  if (v < target) {
    const uint64_t t0 = global_ns();
    uint32_t it = 0;
    while ((v = ld_acquire(p)) < target)
      if (lag_timeout(a, t0, it)) return false;
  }
  if (seen) *seen = v;
  return true;
}

// A driven block's count of live entries at step s (its share of the step's draws), published
// as one word (s + 1) << 32 | count: the step tag makes the value self-describing, so neither side
// needs a fence.
__device__ __forceinline__ void live_put(const LagArgs &a, int s, int d, uint32_t n) {
  const unsigned long long v = ((unsigned long long)(uint32_t)(s + 1) << 32) | n;
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(a.liveTag + (s & (kLagRing - 1)) * kLagMaxDB + d), "l"(v)
               : "memory");
}
// Driven block d's count for step s; false on a timeout or a recorded error.
__device__ __forceinline__ bool live_get(const LagArgs &a, int s, int d, uint32_t &n) {
  const unsigned long long *p = a.liveTag + (s & (kLagRing - 1)) * kLagMaxDB + d;
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  if ((uint32_t)(v >> 32) != (uint32_t)(s + 1)) {
    const uint64_t t0 = global_ns();
    uint32_t it = 0;
    do {
      if (lag_timeout(a, t0, it)) return false;
      asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    } while ((uint32_t)(v >> 32) != (uint32_t)(s + 1));
  }
  n = (uint32_t)v;
  return true;
}

// Jump-ahead for the driven block. hex[(i * 15 + v - 1) * 128 ...] holds M^(v * 16^i) (v = 1..15,
// i = 0..2) as 8 nibble tables, followed by M^4096; for a warp-uniform d every lane reads the same
// words (broadcast). d < 65536.
__device__ __forceinline__ uint32_t xs_jump_hex(const uint32_t *hex, uint32_t s, uint32_t d) {
#pragma unroll
  for (int i = 0; i < kHexLevels; i++) {
    const uint32_t v = (d >> (4 * i)) & 15u;
    if (v) s = xs_apply(hex + (i * 15 + v - 1) * 128, s);
  }
  for (uint32_t q = d >> (4 * kHexLevels); q; q--) s = xs_apply(hex + kHexLevels * 15 * 128, s);
  return s;
}
// off holds M^l (l = 0..31) interleaved by lane: word (n * 16 + nibble) * 32 + l, so lane l
// applying M^l reads bank l only.
__device__ __forceinline__ uint32_t xs_apply_lane(const uint32_t *off, uint32_t lane, uint32_t x) {
  uint32_t y = 0;
#pragma unroll
  for (int n = 0; n < 8; n++) y ^= off[((uint32_t)n * 16 + ((x >> (4 * n)) & 15u)) * 32 + lane];
  return y;
}

// Phase timer: thread 0 of the first driven block and of the first tile block adds the time
// since its last lap to slot k.
__device__ __forceinline__ void lap(const LagArgs &a, int k, uint64_t &tp) {
  if (a.prof != nullptr && (blockIdx.x == 0 || blockIdx.x == (unsigned)a.nDB) && threadIdx.x == 0) {
    const uint64_t now = global_ns();
    atomicAdd(a.prof + k, (unsigned long long)(now - tp));
    tp = now;
  }
}

// Every block has finished step `s`: its completion counter reached grid * (epoch + 1).
__device__ __forceinline__ uint32_t done_target(int s, int grid) { return (uint32_t)grid * (uint32_t)(s / kLagRing + 1); }

// Amplitude sign*res that lif.c reads when this neuron's spike arrives, replayed from its state
// now: `r` is res after this step's update, bit w of `pend` marks an earlier spike of the neuron
// arriving w+1 steps from now; `steps` steps of delivery (depression, lif.c:37-39) and
// recovery (lif.c:71) precede the arrival.
__device__ __forceinline__ float predict_amp(const LagArgs &a, float sign, float r, uint32_t pend, int steps) {
  if (sign == 0.f) return 0.f;
  if (a.depU == 0.f && r == 1.f) return sign;
  for (int w = 0; w < steps; w++) {
    if ((pend >> w) & 1u)
      if (__fmul_rn(sign, r) != 0.f) r = __fsub_rn(r, __fmul_rn(a.depU, r));
    r = __fadd_rn(r, __fmul_rn(__fsub_rn(1.f, r), a.kRec));
  }
  return __fmul_rn(sign, r);
}

// One warp pushes the contributions W[j]*amp (lif.c:41-42) of edges [lo, hi) of one presynaptic
// neuron into the buckets of arrival slot `slot`, keyed by (rank << 3) | (repeat << 1) | inhibitory
// (the edge record's repeat index orders a row's edges to one target); of the row's
// 32-edge chunks it takes c0, c0 + cs, ... (several warps can share a row). Each edge's record
// holds its target's count slot, its first bucket entry and their end. Up to kPushChunks edges per
// lane are in flight at once: their loads, then their slot claims, then their stores.
constexpr int kPushChunks = 1;
__device__ __forceinline__ void push_edges(const LagArgs &a, uint32_t lo, uint32_t hi, uint32_t rank, float amp,
                                           int slot, uint32_t c0 = 0, uint32_t cs = 1) {
  if (amp == 0.f) return;  // lif.c:37: nothing delivered, no depression
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t key0 = (rank << 3) | (amp > 0 ? 0u : 1u);
  uint32_t *cnt = a.cnt + (int64_t)slot * a.cntStride;
  uint2 *buf = a.buf + (int64_t)slot * a.E;
  for (uint32_t j0 = lo + 32u * kPushChunks * c0; j0 < hi; j0 += 32u * kPushChunks * cs) {
    uint4 er[kPushChunks];
    float w[kPushChunks];
    uint32_t pos[kPushChunks];
#pragma unroll
    for (int c = 0; c < kPushChunks; c++) {
      const uint32_t j = j0 + lane + 32 * c;
      if (j < hi) {
        er[c] = __ldg(a.edgeRec + j);
        w[c] = __ldg(a.W + j);
      }
    }
#pragma unroll
    for (int c = 0; c < kPushChunks; c++)
      if (j0 + lane + 32 * c < hi) pos[c] = atomicAdd(cnt + er[c].x, 1u);
#pragma unroll
    for (int c = 0; c < kPushChunks; c++) {
      if (j0 + lane + 32 * c < hi) {
        if (er[c].y + pos[c] < er[c].z)
          buf[er[c].y + pos[c]] = make_uint2(key0 | (er[c].w << 1), __float_as_uint(__fmul_rn(w[c], amp)));
        else atomicCAS(a.err, 0, FB_EOVERFLOW);
      }
    }
  }
}

__device__ __forceinline__ void push_row(const LagArgs &a, int32_t pre, uint32_t rank, float amp, int slot) {
  if (amp == 0.f) return;
  push_edges(a, __ldg(a.indptr + pre), __ldg(a.indptr + pre + 1), rank, amp, slot);
}

// Adds target i's n contributions of a slot in ascending key order (lif.c's order); up to
// kSortMax are sorted in registers at a time, in windows of ascending keys beyond that.
__device__ void apply_slot(const LagArgs &a, const uint2 *e0, uint32_t n, float &ge, float &gi) {
  if (n == 1) {
    const uint2 x = ldcg(e0);
    if (x.x & 1u) gi = __fadd_rn(gi, __uint_as_float(x.y));
    else ge = __fadd_rn(ge, __uint_as_float(x.y));
    return;
  }
  uint2 e[kSortMax];
  bool any = false;
  uint32_t last = 0;
  for (uint32_t done = 0; done < n;) {
    uint32_t m = 0;
    for (uint32_t u = 0; u < n; u++) {
      const uint2 x = ldcg(e0 + u);
      if (any && x.x <= last) continue;
      if (m == (uint32_t)kSortMax && x.x >= e[m - 1].x) continue;
      uint32_t w = m < (uint32_t)kSortMax ? m++ : m - 1;
      while (w > 0 && e[w - 1].x > x.x) {
        e[w] = e[w - 1];
        w--;
      }
      e[w] = x;
    }
    if (m == 0) {
      atomicCAS(a.err, 0, FB_EOVERFLOW);
      break;
    }
    for (uint32_t u = 0; u < m; u++) {
      if (e[u].x & 1u) gi = __fadd_rn(gi, __uint_as_float(e[u].y));
      else ge = __fadd_rn(ge, __uint_as_float(e[u].y));
    }
    last = e[m - 1].x;
    any = true;
    done += m;
  }
}

// Shared-memory state of the block's neurons (structure of arrays, `cap` entries each): the
// model state, launch constants (bias, thr, drive, sign, bucket offset and in-degree), the
// amplitude of a spike of this step, the in-flight arrival mask and background hit counts.
constexpr int kStateWords = 20;
struct LagState {
  float *v, *ge, *gi, *r, *tr, *ad, *rs, *bias, *thr, *drive, *amp, *sign;
  uint32_t *sc, *pend, *hits, *off, *deg, *row0, *row1;
  int32_t *id;
};

__device__ __forceinline__ LagState carve(unsigned char *sm, int cap) {
  LagState s;
  float *f = (float *)sm;
  s.v = f; f += cap;
  s.ge = f; f += cap;
  s.gi = f; f += cap;
  s.r = f; f += cap;
  s.tr = f; f += cap;
  s.ad = f; f += cap;
  s.rs = f; f += cap;
  s.bias = f; f += cap;
  s.thr = f; f += cap;
  s.drive = f; f += cap;
  s.amp = f; f += cap;
  s.sign = f; f += cap;
  s.sc = (uint32_t *)f; f += cap;
  s.pend = (uint32_t *)f; f += cap;
  s.hits = (uint32_t *)f; f += cap;
  s.off = (uint32_t *)f; f += cap;
  s.deg = (uint32_t *)f; f += cap;
  s.row0 = (uint32_t *)f; f += cap;
  s.row1 = (uint32_t *)f; f += cap;
  s.id = (int32_t *)f;
  return s;
}

// Delivery side of one step for local neuron k with n contributions in slot `slot`: the
// contributions, then background hits (lif.c:48), then the neuron's own depression if its spike
// arrives now (lif.c:37-39).
__device__ __forceinline__ void receive(const LagArgs &a, const LagState &S, int k, uint32_t n, uint32_t ci,
                                        int slot, bool haveE, uint2 e0) {
  float ge = S.ge[k], gi = S.gi[k];
  if (n) {
    const uint32_t deg = S.deg[k];
    if (n > deg) {  // cannot happen with one contribution per presynaptic neuron and step
      atomicCAS(a.err, 0, FB_EOVERFLOW);
      n = deg;
    }
    if (n == 1 && haveE) {  // the prefetched entry
      if (e0.x & 1u) gi = __fadd_rn(gi, __uint_as_float(e0.y));
      else ge = __fadd_rn(ge, __uint_as_float(e0.y));
    } else {
      apply_slot(a, a.buf + (int64_t)slot * a.E + S.off[k], n, ge, gi);
    }
    a.cnt[(int64_t)slot * a.cntStride + ci] = 0;
  }
  const uint32_t h = S.hits[k];
  if (h) {
    for (uint32_t u = 0; u < h; u++) ge = __fadd_rn(ge, a.bgAmp);
    S.hits[k] = 0;
  }
  S.ge[k] = ge;
  S.gi[k] = gi;
  if (S.pend[k] & 1u) {
    const float rs = S.rs[k];
    if (!(__fmul_rn(S.sign[k], rs) == 0.f)) S.rs[k] = __fsub_rn(rs, __fmul_rn(a.depU, rs));
  }
}

// lif.c:53-76 for local neuron k: membrane, decays, threshold. Returns whether it crossed the
// threshold; pend advances one step and, on a spike, marks the new arrival D steps ahead.
__device__ __forceinline__ bool integrate(const LagArgs &a, const LagState &S, int k) {
  float v = S.v[k], r = S.r[k], ge = S.ge[k], gi = S.gi[k];
  float acc = __fsub_rn(a.vRest, v);
  if (a.coba) {
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(ge, __fsub_rn(a.eExc, v)), a.cE));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(gi, __fsub_rn(v, a.eInh)), a.cI));
  } else {
    acc = __fadd_rn(acc, ge);
    acc = __fadd_rn(acc, gi);
  }
  acc = __fadd_rn(acc, S.bias[k]);
  const float dv = __fmul_rn(acc, a.kM);
  const bool refractory = r > 0;
  v = refractory ? a.vReset : __fadd_rn(v, dv);
  r = refractory ? __fsub_rn(r, a.dt) : r;
  S.ge[k] = __fmul_rn(ge, a.dE);
  S.gi[k] = __fmul_rn(gi, a.dE);
  float tr = __fmul_rn(S.tr[k], a.dTr);
  float ad = __fmul_rn(S.ad[k], a.dA);
  const float rs0 = S.rs[k];
  S.rs[k] = __fadd_rn(rs0, __fmul_rn(__fsub_rn(1.f, rs0), a.kRec));
  bool fired = false;
  if (v >= __fadd_rn(__fadd_rn(a.vThresh, ad), S.thr[k]) && r <= 0) {
    v = a.vReset;
    r = a.tRef;
    tr = 1.f;
    ad = __fadd_rn(ad, a.adaptInc);
    S.sc[k] += 1u;
    fired = true;
  }
  S.v[k] = v;
  S.r[k] = r;
  S.tr[k] = tr;
  S.ad[k] = ad;
  return fired;
}

// After a step: the arrival mask shifts; a spike of this step arrives D steps ahead (bit D-1)
// and its amplitude is fixed now.
__device__ __forceinline__ void emit(const LagArgs &a, const LagState &S, int k, bool spiked) {
  const uint32_t p = S.pend[k] >> 1;
  if (spiked) S.amp[k] = predict_amp(a, S.sign[k], S.rs[k], p, a.D - 1);
  S.pend[k] = spiked ? p | (1u << (a.D - 1)) : p;
}

// Background targets of the step that fall on this block's neurons: a hit count per neuron.
template <bool kWorkers>
__device__ void collect_bg(const LagArgs &a, LagShared &sh, const LagState &S, uint32_t *sBg, int s,
                           bool driven) {
  const int nbg = ldcg(a.bgCount + (s & (kLagRing - 1)));
  const uint32_t *list = a.bgList + (int64_t)(s & (kLagRing - 1)) * a.bgCap;
  const int nT = kWorkers ? kTW : (int)blockDim.x;
  for (int c0 = 0; c0 < nbg; c0 += kBgChunk) {
    const int m = min(kBgChunk, nbg - c0);
    for (int k = threadIdx.x; k < m; k += nT) sBg[k] = ldcg(list + c0 + k);
    if (kWorkers) wbar();
    else __syncthreads();
    for (int k = threadIdx.x; k < m; k += nT) {
      const int32_t x = (int32_t)sBg[k];
      if (driven) {  // the target's place in the driven list, if this block owns it
        const int32_t p = __ldg(a.drvPosOf + x) - sh.dLo;
        if (p >= 0 && p < sh.nLocal) atomicAdd(S.hits + p, 1u);
        continue;
      }
      if (x < sh.idLo || x > sh.idHi) continue;
      int lo = 0, hi = sh.nLocal;
      while (lo < hi) {  // first entry >= x
        const int mid = (lo + hi) >> 1;
        if (S.id[mid] < x) lo = mid + 1;
        else hi = mid;
      }
      if (lo < sh.nLocal && S.id[lo] == x) atomicAdd(S.hits + lo, 1u);
    }
    if (kWorkers) wbar();
    else __syncthreads();
  }
}

// The driven block's generator work for step t, done by one warp while the others update the
// step before: the state at the start of step t (`s0`), its background draw count (the
// accumulator advanced by lane 0, lif.c:46-47) and the states M^(32 q) M^(nbg+1) s0 at every 32nd
// driven draw (lane j: q = j, 32 + j, ...).
__device__ __forceinline__ void driven_prepare(const LagArgs &a, LagShared &sh, const uint32_t *sHex, int par,
                                               uint32_t s0, float accIn) {
  const uint32_t j = threadIdx.x & 31u;
  uint32_t nbg = 0;
  if (a.hasBg) {
    if (j == 0) {
      const float acc = __fadd_rn(accIn, a.bgEvents);
      const int32_t n = (int32_t)acc;
      sh.bgAccP[par] = __fsub_rn(acc, (float)n);
      if (n > a.bgCap) atomicCAS(a.err, 0, FB_EOVERFLOW);
      nbg = (uint32_t)min(n, a.bgCap);
    }
    nbg = __shfl_sync(0xffffffffu, nbg, 0);
  }
  if (j == 0) {
    sh.nbgP[par] = (int32_t)nbg;
    sh.rngP[par] = s0;
  }
  const uint32_t b0 = xs_jump_hex(sHex, s0, nbg + 1u);
  const uint32_t nq = (uint32_t)(a.nD + 31) / 32;
  uint32_t c = xs_jump_hex(sHex, b0, 32u * j);
  for (uint32_t q = j; q < nq; q += 32) {
    sh.cst[par][q] = c;
    c = xs_apply(sHex + (2 * 15 + 4 - 1) * 128, c);  // M^1024 = M^(4 * 16^2)
  }
}

// The driven block's live entries per warp and round for the coming step (ballots over the
// refractory state, lif.c:50).
__device__ __forceinline__ void driven_ballots(const LagArgs &a, LagShared &sh, const LagState &S, int par) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < kMaxPer; r++) {
    const int k = threadIdx.x + r * kLB;
    const bool live = r < sh.m && k < sh.nLocal && !(S.r[k] > 0);
    const uint32_t wm = __ballot_sync(0xffffffffu, live);
    if (lane == 0 && r < sh.m) sh.wcnt[par][r * 32 + warp] = __popc(wm);
  }
}

__global__ void __launch_bounds__(kLB, 1) lagged_kernel(LagArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ LagShared sh;
  const int tid = threadIdx.x;
  const int nDB = a.nDB;
  const bool drivenBlock = (int)blockIdx.x < nDB;
  const int dIdx = drivenBlock ? (int)blockIdx.x : 0;  // driven block: its part of the list
  const int cap = drivenBlock ? a.nDcap : a.cap;
  LagState S = carve(smraw, cap);
  unsigned char *tail = smraw + (size_t)kStateWords * 4 * cap;
  uint32_t *sBg = (uint32_t *)tail;
  uint32_t *sHex = sBg + kBgChunk;
  uint32_t *sOff = sHex + kHexWords;
  int32_t *sThr = (int32_t *)(sOff + kOffWords);  // driven block: threshold spikes of a step
  const int b = (int)blockIdx.x - nDB;  // tile index of a tile block

  // ---------------- prologue: own state into shared memory ----------------
  if (tid == 0) {
    sh.stop = 0;
    sh.stopP[0] = sh.stopP[1] = 0;
    sh.known = -1;
    sh.dbCount = 0;
    sh.head0 = ldcg(&a.G->head);
    sh.steps0 = ldcg(&a.G->stepsDone);
    sh.dLo = 0;
    if (drivenBlock) {
      sh.dLo = a.dLo[dIdx];
      sh.nLocal = a.dLo[dIdx + 1] - a.dLo[dIdx];
      sh.m = (sh.nLocal + kLB - 1) / kLB;
      sh.idLo = 0;
      sh.idHi = -1;
      sh.rng = ldcg(&a.G->rngP[sh.steps0 & 1]);
      sh.bgAcc = ldcg(&a.G->bgAccP[sh.steps0 & 1]);
    } else {
      const int lo = a.ndLo[b], hi = a.ndLo[b + 1];
      sh.nLocal = hi - lo;
      sh.idLo = hi > lo ? a.ndIds[lo] : 0;
      sh.idHi = hi > lo ? a.ndIds[hi - 1] : -1;
    }
  }
  __syncthreads();
  const int nLocal = sh.nLocal;
  const int head0 = sh.head0;
  const int64_t steps0 = sh.steps0;
  for (int k = tid; k < nLocal; k += blockDim.x) {
    const int32_t i = drivenBlock ? a.driven[sh.dLo + k] : a.ndIds[a.ndLo[b] + k];
    S.id[k] = i;
    S.v[k] = a.v[i];
    S.ge[k] = a.gE[i];
    S.gi[k] = a.gI[i];
    S.r[k] = a.refr[i];
    S.tr[k] = a.trace[i];
    S.ad[k] = a.adapt[i];
    S.rs[k] = a.res[i];
    S.bias[k] = a.bias[i];
    S.thr[k] = a.thr[i];
    S.drive[k] = drivenBlock ? a.drive[i] : 0.f;
    S.sc[k] = a.spikeCount[i];
    S.hits[k] = 0;
    S.sign[k] = a.sign[i];
    const uint32_t o = a.inOff[i];
    S.off[k] = o;
    S.deg[k] = a.inOff[i + 1] - o;
    S.row0[k] = a.indptr[i];
    S.row1[k] = a.indptr[i + 1];
  }
  if (drivenBlock) {
    for (int k = tid; k < kHexWords + kOffWords; k += blockDim.x) sHex[k] = a.jumpHex[k];
  }
  // spikes in flight at launch: mark each presynaptic neuron's arrival steps
  const int ns = a.D + 1;
  for (int u = 0; u < a.D; u++) {
    const int rslot = (head0 + u) % ns;
    const int32_t na = min(max(a.ringCount[rslot], 0), a.N);
    for (int k = blockIdx.x * blockDim.x + tid; k < na; k += gridDim.x * blockDim.x) {
      const int32_t pre = a.ring[(int64_t)rslot * a.N + k];
      if (pre >= 0 && pre < a.N) atomicOr(a.pend0 + pre, 1u << u);
      else atomicCAS(a.err, 0, FB_EINVAL);
    }
  }
  if (!lag_grid_sync(a)) return;
  for (int k = tid; k < nLocal; k += blockDim.x) S.pend[k] = ldcg(a.pend0 + S.id[k]);
  // push them: one warp per in-flight arrival, ranked by its place in the ring list
  {
    int32_t *sPre = (int32_t *)sBg;  // prefix of the in-flight counts over arrival steps
    if (tid == 0) {
      int32_t c = 0;
      for (int u = 0; u < a.D; u++) {
        sPre[u] = c;
        c += min(max(a.ringCount[(head0 + u) % ns], 0), a.N);
      }
      sPre[a.D] = c;
    }
    __syncthreads();
    const int lane = tid & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t f = ((int64_t)blockIdx.x * blockDim.x + tid) >> 5; f < sPre[a.D]; f += nw) {
      int u = 0;
      while (sPre[u + 1] <= f) u++;
      const int64_t w = f - sPre[u];
      const int32_t pre = a.ring[(int64_t)((head0 + u) % ns) * a.N + w];
      if (pre < 0 || pre >= a.N) continue;  // recorded in the marking pass above
      float amp = 0.f;
      if (lane == 0) {
        const float sg = __ldg(a.sign + pre);
        if (sg != 0.f) {
          float r = a.res[pre];
          const uint32_t p = ldcg(a.pend0 + pre);
          if (a.depU == 0.f && r == 1.f) {
            amp = sg;
          } else {  // u steps of delivery and recovery before the arrival
            for (int x = 0; x < u; x++) {
              if ((p >> x) & 1u)
                if (__fmul_rn(sg, r) != 0.f) r = __fsub_rn(r, __fmul_rn(a.depU, r));
              r = __fadd_rn(r, __fmul_rn(__fsub_rn(1.f, r), a.kRec));
            }
            amp = __fmul_rn(sg, r);
          }
        }
      }
      amp = __shfl_sync(0xffffffffu, amp, 0);
      push_row(a, pre, (uint32_t)w, amp, u % a.S);
    }
  }
  if (!lag_grid_sync(a)) return;
  if (drivenBlock) {  // step 0's inputs
    driven_ballots(a, sh, S, 0);
    if ((int)tid >= (int)blockDim.x - 32) driven_prepare(a, sh, sHex, 0, sh.rng, sh.bgAcc);
    if (tid == 0) sh.dbCnt2[0] = sh.dbCnt2[1] = 0;
  }

  // ---------------- the steps ----------------
  // driven block: this thread's entries are k = tid + r * kLB (r < per), the list in order,
  // round by round
  const int per = sh.m;
  auto kOf = [&](int r) { return tid + r * kLB; };
  // count slot of local neuron k: driven neurons have their own slots after the N neuron ids
  auto cOf = [&](int k) { return drivenBlock ? (uint32_t)(a.N + sh.dLo + k) : (uint32_t)S.id[k]; };
  // contribution counts are loaded two steps ahead and, where a neuron has one, its first bucket
  // entry one step ahead (the lag guarantees those buckets are complete): nA / eA hold step s's,
  // nB step s + 1's
  uint32_t nA[kMaxPer], nB[kMaxPer];
  uint2 eA[kMaxPer];
  bool haveA = false, haveB = false;
  uint64_t tp = a.prof != nullptr ? global_ns() : 0;
  const int pb = 0;                    // phase slots of the driven block (tile blocks: 5 ..)
  int sEnd = a.T;                      // the steps run (fewer after a failed wait)
  const int publisher = (int)blockDim.x - 64;
  if (drivenBlock) {
   for (int s = 0; s < a.T; s++) {
    const int slot = s % a.S;
    const int ring = s & (kLagRing - 1);
    // lag: every block has finished step s - L (and, for the background, the driven block has
    // published this step's draws)
    if (tid == 0) {
      // every block has finished step s + ahead - L, so the counts prefetched two steps ahead
      // are final (ahead = 2 unless the lag is too short; a block's own completion of step s - 1
      // is published only after this wait, so need <= s - 2). One look further ahead first: its
      // round trip, when it succeeds, covers the next few steps as well.
      bool ok = true;
      const int need = s + min(2, a.L - 2) - a.L;
      if (need >= 0 && sh.known < need) {
        const int far = min(need + 4, s - 2);
        if (far > need && ld_acquire(a.done + (far & (kLagRing - 1))) >= done_target(far, gridDim.x)) {
          sh.known = far;
        } else {
          ok = wait_geq(a, a.done + (need & (kLagRing - 1)), done_target(need, gridDim.x));
          if (ok) sh.known = need;
        }
      }
      if (ok && dIdx > 0 && a.hasBg) ok = wait_geq(a, a.bgReady, (uint32_t)(s + 1));
      sh.stopP[s & 1] = ok ? 0 : 1;
    }
    __syncthreads();
    if (sh.stopP[s & 1]) {
      sEnd = s;
      break;
    }
    // step s - 1 is complete in this block (the barrier above): its completion is published now,
    // so the release's wait for the block's writes overlaps this step's work. The publishing
    // thread is in the second-last warp, which has few neurons (thread 0 checks the lag; in the
    // driven block the last warp prepares the next step's generator states: with both duties in
    // one warp that warp set the driven block's pace, 4.65 against 4.26 us per step)
    if ((int)tid == publisher && s > 0) {
      const int sp = s - 1;
      {
        const uint32_t n = sh.dbCnt2[sp & 1];
        sh.dbCnt2[sp & 1] = 0;
        a.dbCnt[(sp & (kLagRing - 1)) * nDB + dIdx] = (int32_t)n;
        if (a.log) atomicAdd(a.stepTot + sp, (int32_t)n);
        // the spike lists and counts of the steps before s, released every other step: the
        // release holds up its warp about as long as the rest of a step, and the tile blocks push
        // these spikes `help` steps later
        if (s % a.dbPub == 0) st_release(a.dbDone + dIdx, (uint32_t)s);
        atomicAdd(a.done + (sp & (kLagRing - 1)), 1u);  // the driven block pushes nothing itself
      }
      if ((sp & 3) == 3) {  // now and then: a later step known finished everywhere, which keeps
        // the count prefetch two steps ahead going (it needs step s + 2 - L finished)
        const int probe = sp - 5;
        if (probe > sh.known && ld_acquire(a.done + (probe & (kLagRing - 1))) >= done_target(probe, gridDim.x))
          sh.known = probe;
      }
    }
    lap(a, pb + 0, tp);
    // this step's counts and first entries (prefetched when the lag allowed it)
    uint32_t nCur[kMaxPer];
    uint2 eCur[kMaxPer];
    const bool haveE = haveA;
#pragma unroll
    for (int r = 0; r < kMaxPer; r++) {
      const int k = kOf(r);
      nCur[r] = haveA ? nA[r] : ((r < per && k < nLocal) ? ldcg(a.cnt + (int64_t)slot * a.cntStride + cOf(k)) : 0u);
      eCur[r] = eA[r];
    }
    // step s + 1: its counts (loaded last step) and their first entries
    haveA = haveB && s + 1 < a.T;
    if (haveA) {
      const int slot1 = (s + 1) % a.S;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        nA[r] = nB[r];
        if (nB[r]) eA[r] = ld_early(a.buf + (int64_t)slot1 * a.E + S.off[kOf(r)]);
      }
    }
    // step s + 2: its counts
    haveB = s + 2 < a.T && sh.known >= s + 2 - a.L;
    if (haveB) {
      const int slot2 = (s + 2) % a.S;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        const int k = kOf(r);
        nB[r] = (r < per && k < nLocal) ? ld_early(a.cnt + (int64_t)slot2 * a.cntStride + cOf(k)) : 0u;
      }
    }

    {
      const int par = s & 1, parN = par ^ 1;
      const int m = sh.m, nLoc = sh.nLocal, dLo = sh.dLo;
      const uint32_t nbg = (uint32_t)sh.nbgP[par], s0 = sh.rngP[par];
      // background draws 1..nbg (lif.c:46-48), published for every block by driven block 0 (the
      // other driven blocks waited for them in their lag check)
      if (a.hasBg) {
        if (dIdx == 0) {
          if (tid == 0) a.bgCount[ring] = (int32_t)nbg;
          for (int d = 1 + tid; d <= (int)nbg; d += blockDim.x)
            a.bgList[(int64_t)ring * a.bgCap + d - 1] = xs_jump_hex(sHex, s0, (uint32_t)d) % (uint32_t)a.N;
          __syncthreads();
          if (tid == 0) st_release(a.bgReady, (uint32_t)(s + 1));
        }
        collect_bg<false>(a, sh, S, sBg, s, true);
      }
      // each warp's first draw among the step's live entries, from the ballots taken at the end
      // of the last step: (live entries of earlier rounds) + (live entries of earlier warps)
      const uint32_t lane = tid & 31u, warp = tid >> 5, ltMask = (1u << lane) - 1u;
      const uint32_t nwarps = blockDim.x >> 5;
      uint32_t totLive = 0, wfirst[kMaxPer];
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        wfirst[r] = totLive;
        if (r >= m) continue;
        const uint32_t v = lane < nwarps ? sh.wcnt[par][r * 32 + lane] : 0u;
        wfirst[r] = totLive + __reduce_add_sync(0xffffffffu, lane < warp ? v : 0u);
        totLive += __reduce_add_sync(0xffffffffu, v);
      }
      // with the list split over driven blocks: this block's share of the step's draws goes to
      // the others, whose shares before it offset its draws (pre), and the step's draws in all
      // (all) fix the generator state of the next step (lif.c:49-52 draws the list in order)
      uint32_t pre = 0, all = totLive;
      if (nDB > 1) {
        if (tid == 0) live_put(a, s, dIdx, totLive);
        if (dIdx > 0) {
          uint32_t x = 0;
          if (lane == 0)
            for (int d2 = 0; d2 < dIdx; d2++) {
              uint32_t n = 0;
              if (!live_get(a, s, d2, n)) break;
              x += n;
            }
          pre = __shfl_sync(0xffffffffu, x, 0);
        }
      }
      // the last warp prepares the next step's generator states: after this step's nbg
      // background and all driven draws
      if ((int)tid >= (int)blockDim.x - 32) {
        if (nDB > 1) {
          uint32_t x = 0;
          if (lane == 0)
            for (int d2 = dIdx + 1; d2 < nDB; d2++) {
              uint32_t n = 0;
              if (!live_get(a, s, d2, n)) break;
              x += n;
            }
          all = pre + totLive + __shfl_sync(0xffffffffu, x, 0);
        }
        driven_prepare(a, sh, sHex, parN, xs_jump_hex(sHex, s0, nbg + all), a.hasBg ? sh.bgAccP[par] : 0.f);
      }
      // entries k = tid + r * kLB (r < m), the driven list in order round by round
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        const int k = tid + r * kLB;
        if (r < m && k < nLoc) receive(a, S, k, nCur[r], a.N + dLo + k, slot, haveE, eCur[r]);
      }
      lap(a, 1, tp);
      // the draws in list order: one per non-refractory entry (lif.c:49-52). Entry k's draw is
      // its rank p among the live entries: M^(p mod 32) C_(p / 32) (lane tables M^l)
      uint32_t firedMask = 0;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        if (r >= m) break;
        const int k = tid + r * kLB;
        const bool live = k < nLoc && !(S.r[k] > 0);
        const uint32_t wmask = __ballot_sync(0xffffffffu, live);
        if (live) {
          const uint32_t p = pre + wfirst[r] + __popc(wmask & ltMask);
          const uint32_t x = xs_apply_lane(sOff, p & 31u, sh.cst[par][p >> 5]);  // lanes hold distinct p mod 32
          const float u = __fmul_rn((float)(x >> 8), 1.0f / 16777216.0f);
          if (u < __fmul_rn(S.drive[k], a.dtS)) {  // lif.c:52
            S.v[k] = a.vReset;
            S.r[k] = __fadd_rn(a.tRef, a.dt);
            S.sc[k] += 1u;
            S.tr[k] = 1.f;
            S.ad[k] = __fadd_rn(S.ad[k], a.adaptInc);
            firedMask |= 1u << r;
          }
        }
      }
      lap(a, 2, tp);
      uint32_t thrMask = 0;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        const int k = tid + r * kLB;
        if (r < m && k < nLoc) {
          const bool f = integrate(a, S, k);
          if (f) thrMask |= 1u << r;
          emit(a, S, k, f || ((firedMask >> r) & 1u));
        }
      }
      // the step's spikes in any order, each with its rank key (the list position of a forced
      // spike, nD + id of a threshold spike): sorted by key they are lif.c's fired order
      uint4 *out = a.dbList + ((int64_t)ring * a.nDall + dLo) * 2;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        const int k = tid + r * kLB;
        const bool forced = (firedMask >> r) & 1u, thr = (thrMask >> r) & 1u;
        if (forced || thr) {
          const uint32_t e = atomicAdd(&sh.dbCnt2[par], 1u);
          out[2 * e] = make_uint4((uint32_t)S.id[k], forced ? (uint32_t)(dLo + k) : (uint32_t)(a.nD + S.id[k]),
                                  __float_as_uint(S.amp[k]), 0u);
          out[2 * e + 1] = make_uint4(S.row0[k], S.row1[k], 0u, 0u);
        }
      }
      lap(a, 3, tp);
      // the next step's live entries (the count is published at the next step's start)
      driven_ballots(a, sh, S, parN);
      lap(a, 4, tp);
      }
  }
  } else {
    // ---------------- tile blocks ----------------
    const int lane = tid & 31, warp = tid >> 5;
    const int perT = (nLocal + kTW - 1) / kTW;
    auto kT = [&](int r) { return tid + r * kTW; };
    auto mineT = [&](int r) { return tid < kTW && r < perT && kT(r) < nLocal; };
    // the lag check for step s1 (publisher lane): every block has finished step s1 + ahead - L so
    // the counts prefetched two steps ahead are final (this block's completion is published up
    // to s1 - 2 when the check runs); the background draws of step s1 are published
    auto lag_ok = [&](int s1) -> bool {
      bool ok = true;
      const int need = s1 + min(2, a.L - 2) - a.L;
      if (need >= 0 && sh.known < need) {
        const int far = min(need + 4, s1 - 2);
        if (far > need && ld_acquire(a.done + (far & (kLagRing - 1))) >= done_target(far, gridDim.x)) {
          sh.known = far;
        } else {
          ok = wait_geq(a, a.done + (need & (kLagRing - 1)), done_target(need, gridDim.x));
          if (ok) sh.known = need;
        }
      }
      if (ok && a.hasBg) ok = wait_geq(a, a.bgReady, (uint32_t)(s1 + 1));
      // test hook: a wait that nothing satisfies (the background progress word never reaches
      // 2^32 - 1), so it runs out after timeoutNs and the launch ends with FB_ETIMEOUT
      if (ok && s1 == a.tripStep && b == 0) ok = wait_geq(a, a.bgReady, 0xffffffffu);
      return ok;
    };
    // the driven block's spikes of step s1 - help that fall to this block (spike e goes to tile
    // block (e + 61 sp) mod nTB: the assignment rotates, so no block carries a push every step),
    // one per lane of the helper warp, into the shared list of step s1's parity
    uint32_t dbKnown = 0;  // helper warp, lane d < nDB: steps driven block d is known to have released
    auto help_load = [&](int s1) -> bool {
      const int par1 = s1 & 1;
      int n = 0;
      bool ok = true;
      if (s1 >= a.help && s1 < a.T) {
        const int sp = s1 - a.help, rp = sp & (kLagRing - 1);
        if (lane < nDB && dbKnown < (uint32_t)(sp + 1)) ok = wait_geq(a, a.dbDone + lane, (uint32_t)(sp + 1), &dbKnown);
        ok = __all_sync(0xffffffffu, ok);
        if (ok) {
          // the step's spikes are the driven blocks' lists one after the other: spike e of the
          // concatenation is entry e - first[d] of block d's list
          const int nd = lane < nDB ? ldcg(a.dbCnt + rp * nDB + lane) : 0;
          int first = nd;
#pragma unroll
          for (int o = 1; o < kLagMaxDB; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, first, o);
            if (lane >= o) first += y;
          }
          const int nsp = __shfl_sync(0xffffffffu, first, nDB - 1);
          first -= nd;  // exclusive prefix
          int e0 = b - (int)(((int64_t)sp * 61) % a.nTB);
          if (e0 < 0) e0 += a.nTB;
          n = nsp > e0 ? (nsp - e0 + a.nTB - 1) / a.nTB : 0;
          if (n > kHelpMax) {
            if (lane == 0) atomicCAS(a.err, 0, FB_EOVERFLOW);
            n = kHelpMax;
          }
          const int e = e0 + lane * a.nTB;
          int seg = 0;  // the block whose list holds spike e
          for (int d2 = 1; d2 < nDB; d2++) seg += e >= __shfl_sync(0xffffffffu, first, d2) ? 1 : 0;
          const int f = __shfl_sync(0xffffffffu, first, seg);
          if (lane < n) {
            const int64_t at = (int64_t)rp * a.nDall + a.dLo[seg] + (e - f);
            const uint4 x = ldcg(a.dbList + at * 2);
            const uint4 row = ldcg(a.dbList + at * 2 + 1);
            sh.help[par1][lane] = make_uint4(row.x, row.y, x.y, x.z);
          }
        }
      }
      if (lane == 0) {
        sh.helpN[par1] = n;
        sh.stopQ[par1] = ok ? 0 : 1;
      }
      return ok;
    };
    if (warp == kTWarps && lane == 0) sh.stopP[0] = lag_ok(0) ? 0 : 1;
    if (warp == kTWarps + 1) help_load(0);
    uint32_t nA[kMaxPer], nB[kMaxPer];
    uint2 eA[kMaxPer];
    bool haveA = false, haveB = false;
    uint64_t tp = a.prof != nullptr ? global_ns() : 0;
    for (int s = 0; s < a.T; s++) {
      const int slot = s % a.S;
      const int ring = s & (kLagRing - 1);
      const int par = s & 1;
      __syncthreads();  // the workers finished step s - 1; the service warps prepared step s
      if (sh.stopP[par] | sh.stopQ[par]) {
        sEnd = s;
        break;
      }
      // the service warps' own time per step (phase timer, first tile block)
      const bool svcTimed = a.prof != nullptr && b == 0 && lane == 0 && warp >= kTWarps;
      const uint64_t svc0 = svcTimed ? global_ns() : 0;
      if (warp == kTWarps) {  // publisher: step s - 1 complete, then the lag for step s + 1
        if (lane == 0) {
          if (s > 0) {
            const int sp = s - 1;
            red_release(a.done + (sp & (kLagRing - 1)), 1u);
            if ((sp & 3) == 3) {  // now and then: a later step known finished everywhere
              const int probe = sp - 5;
              if (probe > sh.known && ld_acquire(a.done + (probe & (kLagRing - 1))) >= done_target(probe, gridDim.x))
                sh.known = probe;
            }
          }
          if (s + 1 < a.T) sh.stopP[par ^ 1] = lag_ok(s + 1) ? 0 : 1;
          if (svcTimed) atomicAdd(a.prof + 10, (unsigned long long)(global_ns() - svc0));
        }
        continue;
      }
      if (warp == kTWarps + 1) {  // helper: the next step's share of the driven spikes
        help_load(s + 1);
        if (svcTimed) atomicAdd(a.prof + 11, (unsigned long long)(global_ns() - svc0));
        continue;
      }
      lap(a, 5, tp);
      // this step's counts and first entries (prefetched when the lag allowed it)
      uint32_t nCur[kMaxPer];
      uint2 eCur[kMaxPer];
      const bool haveE = haveA;
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        nCur[r] = haveA ? nA[r] : (mineT(r) ? ldcg(a.cnt + (int64_t)slot * a.cntStride + S.id[kT(r)]) : 0u);
        eCur[r] = eA[r];
      }
      haveA = haveB && s + 1 < a.T;
      if (haveA) {
        const int slot1 = (s + 1) % a.S;
#pragma unroll
        for (int r = 0; r < kMaxPer; r++) {
          nA[r] = nB[r];
          if (nB[r]) eA[r] = ld_early(a.buf + (int64_t)slot1 * a.E + S.off[kT(r)]);
        }
      }
      haveB = s + 2 < a.T && *(volatile int32_t *)&sh.known >= s + 2 - a.L;
      if (haveB) {
        const int slot2 = (s + 2) % a.S;
#pragma unroll
        for (int r = 0; r < kMaxPer; r++)
          nB[r] = mineT(r) ? ld_early(a.cnt + (int64_t)slot2 * a.cntStride + S.id[kT(r)]) : 0u;
      }
      if (a.hasBg) collect_bg<true>(a, sh, S, sBg, s, false);
      uint64_t flags = 0;  // bit 16 r: neuron r of this thread crossed the threshold
#pragma unroll
      for (int r = 0; r < kMaxPer; r++) {
        if (mineT(r)) {
          const int k = kT(r);
          receive(a, S, k, nCur[r], (uint32_t)S.id[k], slot, haveE, eCur[r]);
          const bool f = integrate(a, S, k);
          emit(a, S, k, f);
          if (f) flags |= (uint64_t)1 << (16 * r);
        }
      }
      lap(a, 9, tp);
      // compaction in ascending local index: neurons r = 0 (k = tid) first, then r = 1, ...
      uint32_t fired = 0;
      if (wbar_or(flags != 0)) {
        uint64_t tot;
        const uint64_t pos = worker_exclusive_scan(flags, &tot, sh.scan64);
        int32_t *st = a.tStage + ((int64_t)ring * a.nTB + b) * a.cap;
        uint32_t before = 0;
#pragma unroll
        for (int r = 0; r < kMaxPer; r++) {
          const uint32_t c = (uint32_t)(tot >> (16 * r)) & 0xffffu;
          if ((flags >> (16 * r)) & 1u) st[before + ((uint32_t)(pos >> (16 * r)) & 0xffffu)] = kT(r);
          before += c;
        }
        fired = before;
      }
      lap(a, 6, tp);
      // own spikes into the slot of step s + D: their 32-edge chunks dealt round-robin over the
      // worker warps, so a large row is spread over the block
      const uint32_t nw = kTWarps;
      if (fired) {
        wbar();
        const int32_t *st = a.tStage + ((int64_t)ring * a.nTB + b) * a.cap;
        uint32_t base = 0;
        for (uint32_t f = 0; f < fired; f++) {
          const int k = ldcg(st + f);
          const uint32_t lo = S.row0[k], hi = S.row1[k];
          push_edges(a, lo, hi, (uint32_t)(a.nD + S.id[k]), S.amp[k], (s + a.D) % a.S,
                     ((uint32_t)warp + nw - base % nw) % nw, nw);
          base += (hi - lo + 31) / 32;
        }
      }
      lap(a, 7, tp);
      // the driven block's spikes of step s - help that fall to this block (listed by the helper
      // warp during the last step)
      if (s >= a.help) {
        const int sp = s - a.help;
        const int n = sh.helpN[par];
        uint32_t base = 0;
        for (int j = 0; j < n; j++) {
          const uint4 h = sh.help[par][j];
          push_edges(a, h.x, h.y, h.z, __uint_as_float(h.w), (sp + a.D) % a.S,
                     ((uint32_t)warp + nw - base % nw) % nw, nw);
          base += (h.y - h.x + 31) / 32;
        }
      }
      if (tid == 0) {
        a.tCnt[(int64_t)ring * a.nTB + b] = (int32_t)fired;
        if (a.log && fired) atomicAdd(a.stepTot + s, (int32_t)fired);
      }
      lap(a, 8, tp);
    }
  }

  // ---------------- epilogue ----------------
  __syncthreads();
  if (drivenBlock && (int)tid == publisher && a.T > 0 && sEnd == a.T) {  // the last step's count
    const int sp = a.T - 1;
    a.dbCnt[(sp & (kLagRing - 1)) * nDB + dIdx] = (int32_t)sh.dbCnt2[sp & 1];
    if (a.log) atomicAdd(a.stepTot + sp, (int32_t)sh.dbCnt2[sp & 1]);
  }
  const bool ok = lag_grid_sync(a);
  if (!ok) return;
  for (int k = tid; k < nLocal; k += blockDim.x) {
    const int32_t i = S.id[k];
    a.v[i] = S.v[k];
    a.gE[i] = S.ge[k];
    a.gI[i] = S.gi[k];
    a.refr[i] = S.r[k];
    a.trace[i] = S.tr[k];
    a.adapt[i] = S.ad[k];
    a.res[i] = S.rs[k];
    a.spikeCount[i] = S.sc[k];
  }
  // slots delivered during the launch are empty (lif.c:44) unless refilled below
  if (blockIdx.x == 0)
    for (int u = tid; u < min(a.T, ns); u += blockDim.x) a.ringCount[(head0 + u) % ns] = 0;
  if (!lag_grid_sync(a)) return;
  if (tid == 0) sh.dbCount = 0;
  __syncthreads();
  // fired lists (lif.c:77-79), one block per step: the last D steps into their ring slots (the
  // arrivals still in flight), and with logging every step of the launch into the log
  const int first = a.log ? 0 : max(0, a.T - a.D);
  for (int s = first + (int)blockIdx.x; s < a.T; s += gridDim.x) {
    const int ring = s & (kLagRing - 1);
    const int rslot = (head0 + s + ns - 1) % ns;
    const bool toRing = s >= a.T - a.D;
    int32_t *out = a.ring + (int64_t)rslot * a.N;
    // the driven blocks' spike lists one after the other (each in any order)
    int first[kLagMaxDB + 1];
    first[0] = 0;
    for (int d2 = 0; d2 < nDB; d2++) first[d2 + 1] = first[d2] + ldcg(a.dbCnt + ring * nDB + d2);
    const int nSp = first[nDB];
    auto dbe = [&](int e) -> uint4 {
      int d2 = 0;
      while (d2 + 1 < nDB && e >= first[d2 + 1]) d2++;
      return ldcg(a.dbList + ((int64_t)ring * a.nDall + a.dLo[d2] + (e - first[d2])) * 2);
    };
    // the driven spikes in key order into sThr (ids): forced (key < nD) in list order, then
    // threshold spikes by ascending id
    for (int e = tid; e < nSp; e += blockDim.x) {
      const uint4 x = dbe(e);
      uint32_t rank = 0;
      for (int o = 0; o < nSp; o++) rank += dbe(o).y < x.y ? 1u : 0u;
      sThr[rank] = (int32_t)x.x;
      if (x.y < (uint32_t)a.nD) atomicAdd(&sh.dbCount, 1u);
    }
    __syncthreads();
    const int nF = (int)sh.dbCount;
    int32_t *tOff = (int32_t *)sBg;  // tile spike prefix over tile blocks (nTB + 1 <= kBgChunk)
    uint32_t carry = 0;
    for (int t0 = 0; t0 < a.nTB; t0 += blockDim.x) {
      const int t = t0 + tid;
      const uint32_t c = t < a.nTB ? (uint32_t)ldcg(a.tCnt + (int64_t)ring * a.nTB + t) : 0u;
      uint32_t tot;
      const uint32_t pre = block_exclusive_scan(c, &tot, sh.scan);
      if (t < a.nTB) tOff[t] = (int32_t)(carry + pre);
      carry += tot;
    }
    if (tid == 0) {
      tOff[a.nTB] = (int32_t)carry;
      int64_t rb = 0;
      if (a.log) {  // launches with logging have at most kLagRing steps
        rb = ldcg(&a.G->logRasterLen[steps0 & 1]);
        for (int x = 0; x < s; x++) rb += ldcg(a.stepTot + x);
      }
      sh.logBase = rb;
    }
    __syncthreads();
    const int64_t rbase = sh.logBase;
    const bool logR = a.log && a.logRaster != nullptr;
    auto put = [&](int k, int32_t id) {
      if (toRing) out[k] = id;
      if (logR && rbase + k < a.logRasterCap) a.logRaster[rbase + k] = id;
    };
    const int nDT = nSp - nF;
    for (int k = tid; k < nF; k += blockDim.x) put(k, sThr[k]);
    // driven threshold spikes (ascending) merged with the tile spikes (ascending)
    for (int j = tid; j < nDT; j += blockDim.x) {
      const int32_t y = sThr[nF + j];
      int32_t below = 0;
      for (int t = 0; t < a.nTB; t++) {
        const int lo0 = a.ndLo[t], hi0 = a.ndLo[t + 1];
        if (hi0 == lo0) continue;
        if (a.ndIds[lo0] > y) break;
        const int n = tOff[t + 1] - tOff[t];
        const int32_t *st = a.tStage + ((int64_t)ring * a.nTB + t) * a.cap;
        int lo = 0, hi = n;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (a.ndIds[lo0 + ldcg(st + mid)] < y) lo = mid + 1;
          else hi = mid;
        }
        below += lo;
      }
      put(nF + j + below, y);
    }
    for (int t = 0; t < a.nTB; t++) {
      const int n = tOff[t + 1] - tOff[t];
      const int32_t *st = a.tStage + ((int64_t)ring * a.nTB + t) * a.cap;
      const int lo0 = a.ndLo[t];
      for (int p = tid; p < n; p += blockDim.x) {
        const int32_t y = a.ndIds[lo0 + ldcg(st + p)];
        int lo = 0, hi = nDT;  // driven threshold spikes below y
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (sThr[nF + mid] < y) lo = mid + 1;
          else hi = mid;
        }
        put(nF + tOff[t] + p + lo, y);
      }
    }
    if (tid == 0) {
      const int total = nSp + (int)carry;
      if (toRing) a.ringCount[rslot] = total;
      if (a.log && a.logCount) {
        const int64_t lb = steps0 + s - ldcg(&a.G->logStart);
        if (lb >= 0 && lb < a.logCap) a.logCount[lb] = total;
      }
      if (s == a.T - 1) {
        a.G->nFired = total;
        a.G->lastSlot = rslot;
        if (a.log && a.logRaster) a.G->logRasterLen[(steps0 + a.T) & 1] = rbase + total;
      }
      sh.dbCount = 0;
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && tid == 0) {  // every driven block holds the same generator state
    const int64_t g = steps0 + a.T;
    a.G->head = (head0 + a.T) % ns;
    a.G->stepsDone = g;
    a.G->rngP[g & 1] = sh.rngP[a.T & 1];  // the state at the start of step T
    a.G->bgAccP[g & 1] = (a.hasBg && a.T > 0) ? sh.bgAccP[(a.T - 1) & 1] : sh.bgAcc;
  }
}

// ---- host side -------------------------------------------------------------------------------

namespace {
// 32x32 matrices over GF(2) by columns: col[b] = A e_b.
uint32_t mat_apply(const uint32_t *col, uint32_t x) {
  uint32_t y = 0;
  for (int b = 0; b < 32; b++)
    if (x >> b & 1u) y ^= col[b];
  return y;
}
void mat_mul(const uint32_t *A, const uint32_t *B, uint32_t *C) {  // C = A B
  uint32_t t[32];
  for (int b = 0; b < 32; b++) t[b] = mat_apply(A, B[b]);
  for (int b = 0; b < 32; b++) C[b] = t[b];
}
uint32_t nibble_entry(const uint32_t *col, int n, uint32_t v) {
  uint32_t y = 0;
  for (int b = 0; b < 4; b++)
    if (v >> b & 1u) y ^= col[4 * n + b];
  return y;
}
}  // namespace

void lagged_jump_tables(std::vector<uint32_t> &tab) {
  tab.assign(kHexWords + kOffWords, 0);
  uint32_t M[32], I[32];
  for (int b = 0; b < 32; b++) {
    uint32_t x = 1u << b;  // one xorshift32 step (src/wasm/lif.c:27) is linear over GF(2)
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    M[b] = x;
    I[b] = 1u << b;
  }
  uint32_t P[32];  // M^(16^i)
  memcpy(P, M, sizeof P);
  for (int i = 0; i < kHexLevels; i++) {
    uint32_t A[32];
    memcpy(A, P, sizeof A);  // M^(v 16^i), v = 1..15
    for (int v = 1; v <= 15; v++) {
      for (int n = 0; n < 8; n++)
        for (uint32_t x = 0; x < 16; x++) tab[(i * 15 + v - 1) * 128 + n * 16 + x] = nibble_entry(A, n, x);
      mat_mul(A, P, A);
    }
    for (int r = 0; r < 4; r++) mat_mul(P, P, P);  // M^(16^(i+1))
  }
  for (int n = 0; n < 8; n++)  // M^(16^kHexLevels)
    for (uint32_t x = 0; x < 16; x++) tab[kHexLevels * 15 * 128 + n * 16 + x] = nibble_entry(P, n, x);
  uint32_t A[32];
  memcpy(A, I, sizeof A);  // M^l, l = 0..31
  for (int l = 0; l < 32; l++) {
    for (int n = 0; n < 8; n++)
      for (uint32_t x = 0; x < 16; x++) tab[kHexWords + ((uint32_t)n * 16 + x) * 32 + l] = nibble_entry(A, n, x);
    mat_mul(M, A, A);
  }
}

__global__ void edge_records_kernel(const uint32_t *indices, const uint8_t *dup, const uint32_t *inOff,
                                    const int32_t *posOf, int32_t N, int64_t E, uint4 *out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < E; j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q = indices[j];
    const int32_t p = posOf[q];
    out[j] = make_uint4(p >= 0 ? (uint32_t)(N + p) : q, inOff[q], inOff[q + 1], dup ? (uint32_t)dup[j] : 0u);
  }
}

cudaError_t launch_edge_records(const uint32_t *indices, const uint8_t *dup, const uint32_t *inOff,
                                const int32_t *posOf, int32_t N, int64_t E, uint4 *out, cudaStream_t st) {
  if (E > 0) edge_records_kernel<<<1024, 256, 0, st>>>(indices, dup, inOff, posOf, N, E, out);
  return cudaGetLastError();
}

size_t lagged_smem_bytes(int cap, int nDcap, int nDall) {
  const int c = cap > nDcap ? cap : nDcap;
  return (size_t)kStateWords * 4 * c + (size_t)(kBgChunk + kHexWords + kOffWords) * 4 + (size_t)4 * nDall;
}

int lagged_blocks_per_sm(size_t smem) {
  if (cudaFuncSetAttribute(lagged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lagged_kernel, kLB, smem) != cudaSuccess) return 0;
  return n;
}

cudaError_t launch_lagged(const LagArgs &a, int grid, size_t smem, cudaStream_t st) {
  void *args[] = {(void *)&a};
  return cudaLaunchCooperativeKernel((const void *)lagged_kernel, dim3(grid), dim3(kLB), args, smem, st);
}

}  // namespace fb
