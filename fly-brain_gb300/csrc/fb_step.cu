// The brain step on sm_103a: one persistent cooperative launch advances a batch of brains by many
// steps. Semantics are those of the reference kernel lif_step (src/wasm/lif.c:29-80), bit for bit
// in the default (exact) delivery mode.
//
// Per step, two phases separated by grid barriers:
//
//  A. deliver   - warps walk the arriving spikes' CSR rows 32 edges at a time (one edge per lane)
//                 and push each contribution W*s, keyed by the arrival's rank in the ring list,
//                 into a small bucket of its target (atomic slot claim, no float atomics);
//               - one block per brain runs the brain's serial parts: the background accumulator
//                 and draws, the Poisson-driven draws (xorshift32 jump-ahead, one draw per
//                 non-refractory driven neuron in driven-list order, lif.c:49-52), the forced
//                 spikes, and (sequential mode) the whole delivery in list order;
//               - blocks copy the previous step's per-tile threshold spikes into the ring slot in
//                 ascending order, with each arrival's edge offset and the work-item map that
//                 delivery uses when that slot arrives nslots-1 steps later.
//  B. update    - one thread per neuron: sort its bucket by arrival rank and add the
//                 contributions in that order (the reference's per-target summation order),
//                 then the background hits, the membrane update and decays (lif.c:53-72) and
//                 the threshold (lif.c:73-76); each tile compacts its spikes in ascending order.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "fb_internal.cuh"

namespace fb {

// ---------------------------------------------------------------------------------------------
// Phase A pieces
// ---------------------------------------------------------------------------------------------

// Phase timer (fb_profile): thread 0 of block 0 adds the time since its last lap to counter k.
__device__ __forceinline__ void prof_lap(const StepArgs &a, int k, uint64_t &tp) {
  if (a.phaseNs != nullptr && blockIdx.x == 0 && threadIdx.x == 0) {
    const uint64_t now = global_ns();
    atomicAdd(a.phaseNs + k, (unsigned long long)(now - tp));
    tp = now;
  }
}

__device__ __forceinline__ void st_relaxed64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Phase A for chunk c (entries c*kBlock ... +kBlock) of one brain's driven list. Chunk 0 also runs
// the brain's other serial parts of lif.c's step: sequential delivery or arrival marks, the
// ring-count clear, the background accumulator and draws (lif.c:34-48).
//
// Draw order is lif.c's (lif.c:48-52): draws 1..nbg go to the background, then one draw per
// non-refractory driven entry in list order. A chunk's first draw index needs the non-refractory
// count of every earlier chunk: each chunk publishes its count tagged with the step, and reads
// the earlier ones (a bounded wait; chunks only wait on lower chunks, which never wait on higher
// ones, and the grid is co-resident). xorshift32 is linear over GF(2), so each entry jumps to its
// draw with the M^(2^j) tables. Forced spikes are staged per chunk; the next phase places them
// at the head of the ring list.
__device__ void driven_item(const StepArgs &a, const Trial &T, Trial *G, int c, int nDch, int32_t nD,
                            uint64_t gstep, int head, uint32_t *scan, uint64_t *scan64,
                            const uint32_t *jump, uint64_t &tp) {
  __shared__ uint32_t sh_base;
  __shared__ float sh_amp;
  __shared__ bool sh_go;
  const int tid = threadIdx.x;
  const int N = T.N;
  const uint32_t par = (uint32_t)(gstep & 1);
  // lif.c:47 on this step's copy: bgAcc += bgEvents; nbg = (int)bgAcc; bgAcc -= nbg (f32)
  const float acc = __fadd_rn(ldcg(G->bgAccP + par), T.bgEvents);
  const int32_t nbgI = (int32_t)acc;
  const uint32_t nbg = (uint32_t)nbgI;
  const uint32_t s0 = ldcg(G->rngP + par);
  // this chunk's entries: one per thread
  const int32_t k = c * kBlock + tid;
  const bool valid = k < nD;
  int32_t i = valid ? ldcg(T.driven + k) : 0;
  FB_GUARD(a, i >= 0 && i < N, 5, i, k, i = 0);
  const float rf = ldcg(T.refr + i), dr = ldcg(T.drive + i);

  if (c == 0) {
    if (tid == 0) G->bgAccP[par ^ 1u] = __fsub_rn(acc, (float)nbgI);
    const int32_t *arr = T.ring + (int64_t)head * N;
    if (T.mode == FB_DELIVER_SEQUENTIAL) {
      // Sequential delivery (exact also with presynaptic inhibition, lif.c:36-43): arrivals one
      // at a time in list order; each row's targets are distinct, so a row scatters in parallel.
      const int32_t na = ldcg(T.ringCount + head);
      for (int32_t q0 = 0; q0 < na; q0++) {
        const int32_t pre = ldcg(arr + q0);
        if (tid == 0) {
          const float r = ldcg(T.res + pre);
          float amp = __fmul_rn(__ldg(T.sign + pre), r);
          sh_go = amp != 0.f;  // lif.c:37 skips only a zero sign*res, not a zero after :38
          if (sh_go) {
            if (T.preInh > 0.f && ldcg(T.drive + pre) > 0.f) {
              const float gi = ldcg(T.gI + pre);
              amp = __fdiv_rn(amp, __fadd_rn(1.f, __fmul_rn(T.preInh, gi < 0.f ? -gi : 0.f)));
            }
            T.res[pre] = __fsub_rn(r, __fmul_rn(T.depU, r));
          }
          sh_amp = amp;
        }
        __syncthreads();
        const float amp = sh_amp;
        if (sh_go) {
          const uint32_t lo = __ldg(T.indptr + pre), hi = __ldg(T.indptr + pre + 1);
          float *g = amp > 0 ? T.gE : T.gI;
          for (uint32_t j = lo + tid; j < hi; j += blockDim.x) {
            const uint32_t q = __ldg(T.indices + j);
            g[q] = __fadd_rn(ldcg(g + q), __fmul_rn(__ldg(T.W + j), amp));
          }
        }
        __syncthreads();
      }
    } else if (T.flags & kHasDep) {
      // Mark arrivals so the update phase applies the depression res -= depU*res (lif.c:39).
      const int32_t na = ldcg(T.ringCount + head);
      for (int32_t q0 = tid; q0 < na; q0 += blockDim.x) T.arrived[ldcg(arr + q0)] = 1;
    }
    __syncthreads();  // every thread has read ringCount[head] above
    if (tid == 0) T.ringCount[head] = 0;  // lif.c:44
    // background draws 1..nbg (lif.c:48): target = draw % N, counted per target; the update
    // phase adds bgAmp once per hit after the synaptic contributions, as lif.c orders them
    for (uint32_t d = 1 + tid; d <= nbg; d += blockDim.x) {
      const uint32_t x = xs_jump(jump, s0, d);
      atomicAdd(T.bgHits + (x % (uint32_t)N), 1u);
    }
  }
  prof_lap(a, 5, tp);

  const uint32_t live = (valid && !(rf > 0)) ? 1u : 0u;  // refractory entries draw nothing
  uint32_t L;
  const uint32_t lp = block_exclusive_scan(live, &L, scan);
  if (tid == 0) {
    const unsigned long long tag = (unsigned long long)(gstep + 1) << 32;
    st_relaxed64(T.liveTag + c, tag | L);
    uint32_t base = 0;
    const uint64_t t0 = global_ns();
    uint32_t it = 0;
    for (int c2 = 0; c2 < c; c2++) {
      unsigned long long x;
      while (((x = ld_relaxed64(T.liveTag + c2)) >> 32) != (gstep + 1)) {
        if ((++it & 63u) == 0 && (global_ns() - t0 > (uint64_t)a.timeoutNs || it > (1u << 30) ||
                                  ld_volatile(a.err) != 0)) {
          atomicCAS(a.err, 0, FB_ETIMEOUT);
          break;
        }
      }
      base += (uint32_t)x;
    }
    sh_base = base;
  }
  __syncthreads();
  prof_lap(a, 6, tp);
  const uint32_t base = sh_base;
  uint32_t fire = 0, dg = 0;
  if (live) {
    const uint32_t x = xs_jump(jump, s0, nbg + base + lp + 1);
    const float u = __fmul_rn((float)(x >> 8), 1.0f / 16777216.0f);
    if (u < __fmul_rn(dr, T.dtS)) {
      fire = 1;
      dg = __ldg(T.indptr + i + 1) - __ldg(T.indptr + i);
    }
  }
  if (c == nDch - 1 && tid == 0) G->rngP[par ^ 1u] = xs_jump(jump, s0, nbg + base + L);
  prof_lap(a, 7, tp);
  const int64_t cidx = (int64_t)par * T.maxDch + c;
  if (__syncthreads_or(fire)) {
    uint64_t tot;
    const uint64_t pre = block_exclusive_scan(((uint64_t)fire << 32) | dg, &tot, scan64);
    if (fire) {
      const int64_t o = cidx * kBlock + (int64_t)(pre >> 32);
      T.dStage[o] = i;
      T.dStageDeg[o] = (uint32_t)pre;
      // lif.c:52
      T.v[i] = T.vReset;
      T.refr[i] = __fadd_rn(T.tRef, T.dt);
      T.spikeCount[i] = ldcg(T.spikeCount + i) + 1u;
      T.trace[i] = 1.f;
      T.adapt[i] = __fadd_rn(ldcg(T.adapt + i), T.adaptInc);
    }
    if (tid == 0) {
      T.dCnt[cidx] = (int32_t)(tot >> 32);
      T.dDeg[cidx] = (uint32_t)tot;
    }
  } else if (tid == 0) {
    T.dCnt[cidx] = 0;
    T.dDeg[cidx] = 0;
  }
  prof_lap(a, 8, tp);
}

// Materializes brain b's fired list of step `gstep` into its ring slot, one block per brain. The
// staging units are the driven-list chunks (forced spikes, list order) followed by the update
// tiles (threshold spikes, ascending), so the slot holds lif.c's order (lif.c:51-52 then
// :74-76). Units are scanned blockDim at a time: counts and out-degree sums give each unit's
// offset, the non-empty ones are compacted, and the block copies their spikes with each arrival's
// edge offset, row start and delivery work-item records.
__device__ void materialize_brain(const StepArgs &a, const Trial &T, Trial *G, int nDch, uint64_t gstep,
                                  int slot, int64_t logBase, uint64_t *scan64, uint32_t *scan) {
  __shared__ uint32_t uIdx[kBlock];   // non-empty units of the round (compacted)
  __shared__ uint32_t uCnt[kBlock], uOff[kBlock], uDeg[kBlock];
  const int tid = threadIdx.x;
  const int N = T.N;
  const int64_t dpar = (int64_t)(gstep & 1) * T.maxDch;
  const int nUnits = nDch + T.nTiles * kSubPerTile;
  int32_t *out = T.ring + (int64_t)slot * N;
  uint32_t *outOff = T.ringOff + (int64_t)slot * (N + 1);
  uint32_t *outRow = T.ringRow + (int64_t)slot * N;
  uint4 *chunkK = T.chunkK + (int64_t)slot * T.chunkCap;
  const bool logging = a.log && T.logRaster != nullptr;
  const int64_t rbase = logging ? ldcg(G->logRasterLen + (gstep & 1)) : 0;
  uint32_t cntBase = 0, degBase = 0;
  for (int u0 = 0; u0 < nUnits; u0 += blockDim.x) {
    const int u = u0 + tid;
    uint32_t m = 0, dsum = 0;
    if (u < nUnits) {
      if (u < nDch) {
        m = (uint32_t)ldcg(T.dCnt + dpar + u);
        dsum = ldcg(T.dDeg + dpar + u);
      } else {
        m = (uint32_t)ldcg(T.tileCnt + (u - nDch));  // brain-local warp sub-tile
        dsum = ldcg(T.tileDeg + (u - nDch));
      }
    }
    uint64_t tot;
    const uint64_t pre = block_exclusive_scan(((uint64_t)m << 32) | dsum, &tot, scan64);
    uint32_t nz;
    const uint32_t zpos = block_exclusive_scan(m ? 1u : 0u, &nz, scan);
    if (m) {
      uIdx[zpos] = (uint32_t)u;
      uCnt[zpos] = m;
      uOff[zpos] = cntBase + (uint32_t)(pre >> 32);
      uDeg[zpos] = degBase + (uint32_t)pre;
    }
    __syncthreads();
    // each warp copies whole units, warps striding over the non-empty units
    for (uint32_t z = tid >> 5; z < nz; z += blockDim.x >> 5) {
      const uint32_t uu = uIdx[z], mm = uCnt[z], before = uOff[z], dbefore = uDeg[z];
      const bool drv = (int)uu < nDch;
      const int32_t *stage = drv ? T.dStage + (dpar + uu) * kBlock : T.stage + (int64_t)(uu - nDch) * kSub;
      const uint32_t *stageDeg = drv ? T.dStageDeg + (dpar + uu) * kBlock : T.stageDeg + (int64_t)(uu - nDch) * kSub;
      for (uint32_t p = tid & 31; p < mm; p += 32) {
        const int32_t i = ldcg(stage + p);
        const uint32_t k = before + p, o = dbefore + ldcg(stageDeg + p);
        FB_GUARD(a, i >= 0 && i < N && k < (uint32_t)N, 6, i, k, continue);
        const uint32_t r0 = __ldg(T.indptr + i), r1 = __ldg(T.indptr + i + 1);
        out[k] = i;
        outOff[k] = o;
        outRow[k] = r0;
        mark_chunks(chunkK, o, r1 - r0, k, (uint32_t)i, r0);
        if (logging && rbase + k < T.logRasterCap) T.logRaster[rbase + k] = i;
      }
    }
    cntBase += (uint32_t)(tot >> 32);
    degBase += (uint32_t)tot;
    __syncthreads();
  }
  if (tid == 0) {
    const uint32_t nf = cntBase, F = degBase;
    outOff[nf] = F;
    T.ringCount[slot] = (int32_t)nf;
    T.slotEdges[slot] = F;
    G->nFired = (int32_t)nf;
    G->lastSlot = slot;
    if (a.log) {
      if (T.logCount && logBase >= 0 && logBase < T.logCap) T.logCount[logBase] = (int32_t)nf;
      if (T.logRaster) G->logRasterLen[(gstep + 1) & 1] = rbase + nf;
    }
  }
}

// One delivery work item: 32 consecutive edges of the concatenated rows of the arrivals in
// `slot`, starting at edge c * 32. Lane l takes edge c*32+l. The item's record names its first
// arrival; lanes past that arrival's edges find theirs through the offsets. The delivery is split
// in two so a warp can keep two items' loads in flight: load_edge gathers the edge, its target,
// key and contribution W*s; claim_edge takes the target's bucket slot and stores the entry (the
// order of the claims does not matter: the update adds a target's entries in key order).
struct DEdge {
  uint32_t q, key;
  float w;
  bool valid;
};

__device__ __forceinline__ DEdge load_edge(const StepArgs &a, const Trial &T, int slot, uint32_t F, uint32_t c) {
  DEdge d;
  d.valid = false;
  const int lane = threadIdx.x & 31;
  const uint32_t e = c * kChunk + lane;
  if (e >= F) return d;
  const int N = T.N;
  FB_GUARD(a, (int64_t)c < T.chunkCap, 1, c, slot, return d);
  const uint4 ck = ldcg(T.chunkK + (int64_t)slot * T.chunkCap + c);
  uint32_t k = ck.x, pre = ck.y, j = ck.w + e;
  if (e >= ck.z) {  // a later arrival of this item
    const uint32_t *off = T.ringOff + (int64_t)slot * (N + 1);
    k++;
    while (k < (uint32_t)N && ldcg(off + k + 1) <= e) k++;
    FB_GUARD(a, k < (uint32_t)N, 2, k, e, return d);
    pre = (uint32_t)ldcg(T.ring + (int64_t)slot * N + k);
    j = ldcg(T.ringRow + (int64_t)slot * N + k) + (e - ldcg(off + k));
  }
  FB_GUARD(a, pre < (uint32_t)N && (int64_t)j < T.E, 3, pre, j, return d);
  // the edge's loads are issued with the presynaptic ones, before the zero-amplitude test
  const uint32_t q = __ldg(T.indices + j);
  const float wj = __ldg(T.W + j);
  const float amp = __fmul_rn(__ldg(T.sign + pre), (T.flags & kResRest) ? 1.f : ldcg(T.res + pre));  // lif.c:37
  if (amp == 0.f) return d;
  FB_GUARD(a, q < (uint32_t)N, 4, q, j, return d);
  d.q = q;
  d.w = __fmul_rn(wj, amp);  // lif.c:41-42, one rounding
  const bool inh = !(amp > 0);
  d.key = (k << 3) | ((T.dup ? (uint32_t)__ldg(T.dup + j) : 0u) << 1) | (inh ? 1u : 0u);
  d.valid = true;
  return d;
}

__device__ __forceinline__ void claim_edge(const StepArgs &a, const Trial &T, const DEdge &d, uint32_t gparity) {
  if (!d.valid) return;
  const uint32_t q = d.q;
  if (T.mode == FB_DELIVER_FAST) {
    atomicAdd((d.key & 1u) ? T.gI + q : T.gE + q, d.w);
    return;
  }
  const uint32_t pos = atomicAdd(T.cnt + q, 1u);
  if (pos < (uint32_t)kBucket) {
    T.bucket[(int64_t)q * kBucket + pos] = make_uint2(d.key, __float_as_uint(d.w));
  } else {
    const uint32_t r = atomicAdd(a.ovfTop + gparity, 1u);
    if (r >= a.ovfCap) {
      atomicCAS(a.err, 0, FB_EOVERFLOW);
      return;
    }
    OvfRec rec;
    rec.key = d.key;
    rec.bits = __float_as_uint(d.w);
    rec.pad = q;
    rec.next = atomicExch(T.ovfHead + q, r);
    a.ovf[gparity][r] = rec;
  }
}

// ---------------------------------------------------------------------------------------------
// Phase B: the update of one tile of one brain
// ---------------------------------------------------------------------------------------------

// Adds target i's contributions in ascending key (arrival rank) order; inhibitory keys go to gI.
// Up to kSortMax contributions are sorted in local memory; beyond that they are applied in
// successive windows of the kSortMax smallest keys above the last one applied (keys are unique
// per target: one contribution per arrival).
__device__ void apply_contributions(const StepArgs &a, const Trial &T, Trial *G, int i, uint32_t n,
                                    uint32_t gparity, float &ge, float &gi) {
  const uint2 *bk = T.bucket + (int64_t)i * kBucket;
  if (n == 1) {
    const uint2 x = ldcg(bk);
    if (x.x & 1u) gi = __fadd_rn(gi, __uint_as_float(x.y));
    else ge = __fadd_rn(ge, __uint_as_float(x.y));
    return;
  }
  uint2 e[kSortMax];
  const uint32_t nb = n < (uint32_t)kBucket ? n : (uint32_t)kBucket;
  bool any = false;
  uint32_t last = 0;
  for (uint32_t done = 0; done < n;) {
    uint32_t m = 0;
    auto offer = [&](uint2 x) {  // keep the kSortMax smallest keys above `last`, sorted
      if (any && x.x <= last) return;
      if (m == (uint32_t)kSortMax && x.x >= e[m - 1].x) return;
      uint32_t w = m < (uint32_t)kSortMax ? m++ : m - 1;
      while (w > 0 && e[w - 1].x > x.x) {
        e[w] = e[w - 1];
        w--;
      }
      e[w] = x;
    };
    for (uint32_t u = 0; u < nb; u++) offer(ldcg(bk + u));
    if (n > (uint32_t)kBucket)
      for (uint32_t r = ldcg(T.ovfHead + i), hops = 0; r != kNil && hops < n; hops++) {
        FB_GUARD(a, r < a.ovfCap, 7, r, i, break);
        const OvfRec rec = a.ovf[gparity][r];
        offer(make_uint2(rec.key, rec.bits));
        r = rec.next;
      }
    if (m == 0) {  // fewer entries than counted: the overflow pool ran out
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
  if (n > (uint32_t)kBucket) T.ovfHead[i] = kNil;
}

// A neuron's state as loaded at the start of the update phase.
struct NState {
  float v, r, ge, gi, tr, ad, rs, bias, thr;
  uint32_t n, hits;
  uint8_t arrived;
};

__device__ __forceinline__ NState load_neuron(const Trial &T, int i) {
  NState x;
  x.v = ldcg(T.v + i);
  x.r = ldcg(T.refr + i);
  x.ge = ldcg(T.gE + i);
  x.gi = ldcg(T.gI + i);
  x.tr = ldcg(T.trace + i);
  x.ad = (T.flags & kAdaptZero) ? 0.f : ldcg(T.adapt + i);
  x.rs = (T.flags & kResRest) ? 1.f : ldcg(T.res + i);
  x.bias = (T.flags & kBiasZero) ? 0.f : ldcg(T.bias + i);
  x.thr = (T.flags & kThrZero) ? 0.f : ldcg(T.thr + i);
  x.n = T.mode == FB_DELIVER_EXACT ? ldcg(T.cnt + i) : 0u;
  x.hits = (T.flags & kHasBg) ? ldcg(T.bgHits + i) : 0u;
  x.arrived = ((T.flags & kHasDep) && T.mode != FB_DELIVER_SEQUENTIAL) ? ldcg(T.arrived + i) : (uint8_t)0;
  return x;
}

// One neuron's step after delivery: contributions in order, background hits, depression,
// membrane and decays (lif.c:55-72), threshold (lif.c:73-76). Returns the out-degree + 1 if it
// fired, 0 otherwise.
__device__ __forceinline__ uint32_t update_neuron(const StepArgs &a, const Trial &T, Trial *G, int i,
                                                  NState x, uint32_t gparity) {
  float v = x.v, r = x.r, ge = x.ge, gi = x.gi, tr = x.tr, ad = x.ad, rs = x.rs;
  if (x.n) {
    apply_contributions(a, T, G, i, x.n, gparity, ge, gi);
    T.cnt[i] = 0;
  }
  if (x.hits) {  // lif.c:48, after every synaptic contribution
    for (uint32_t u = 0; u < x.hits; u++) ge = __fadd_rn(ge, T.bgAmp);
    T.bgHits[i] = 0;
  }
  if (x.arrived) {  // lif.c:37-39: depressed at delivery unless sign*res == 0
    T.arrived[i] = 0;
    if (!(__fmul_rn(__ldg(T.sign + i), rs) == 0.f)) rs = __fsub_rn(rs, __fmul_rn(T.depU, rs));
  }
  // lif.c:55-72, one IEEE f32 operation per C operation, in C order
  float acc = __fsub_rn(T.vRest, v);
  if (T.coba) {
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(ge, __fsub_rn(T.eExc, v)), T.cE));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(gi, __fsub_rn(v, T.eInh)), T.cI));
  } else {
    acc = __fadd_rn(acc, ge);
    acc = __fadd_rn(acc, gi);
  }
  acc = __fadd_rn(acc, x.bias);
  const float dv = __fmul_rn(acc, T.kM);
  const bool refractory = r > 0;
  v = refractory ? T.vReset : __fadd_rn(v, dv);
  r = refractory ? __fsub_rn(r, T.dt) : r;
  ge = __fmul_rn(ge, T.dE);
  gi = __fmul_rn(gi, T.dE);
  tr = __fmul_rn(tr, T.dTr);
  ad = __fmul_rn(ad, T.dA);
  rs = __fadd_rn(rs, __fmul_rn(__fsub_rn(1.f, rs), T.kRec));
  uint32_t fired = 0;
  // lif.c:74-75: threshold against the decayed adapt
  if (v >= __fadd_rn(__fadd_rn(T.vThresh, ad), x.thr) && r <= 0) {
    v = T.vReset;
    r = T.tRef;
    tr = 1.f;
    ad = __fadd_rn(ad, T.adaptInc);
    T.spikeCount[i] = ldcg(T.spikeCount + i) + 1u;
    fired = 1 + __ldg(T.indptr + i + 1) - __ldg(T.indptr + i);
  }
  // Words that provably keep their bits are not stored, so sectors no neuron changed cost no DRAM
  // write: the refractory count of a neuron neither refractory nor firing (r = r), a trace of +0
  // without a spike (0 * dTr = +0), a conductance of +0 with no contribution or background hit
  // (0 * dE = +0), a membrane potential that came out bit-identical.
  const bool input = x.n != 0u || x.hits != 0u;
  if (__float_as_uint(v) != __float_as_uint(x.v)) T.v[i] = v;
  if (refractory || fired) T.refr[i] = r;
  if (__float_as_uint(x.ge) != 0u || input) T.gE[i] = ge;
  if (__float_as_uint(x.gi) != 0u || input) T.gI[i] = gi;
  if (__float_as_uint(x.tr) != 0u || fired) T.trace[i] = tr;
  if (!(T.flags & kAdaptZero)) T.adapt[i] = ad;
  if (!(T.flags & kResRest)) T.res[i] = rs;
  return fired;
}

// Warp sub-tile w (kSub neurons) of tile t: lane l updates the sub-tile's neurons l and l + 32,
// both loaded before either is stored. Each warp stages its
// spikes in ascending order with their out-degree prefix (ballots and a warp scan), so no block
// barrier paces the tile loop; materialization concatenates the sub-tiles in order.
__device__ void update_tile(const StepArgs &a, const Trial &T, Trial *G, int t, int w, uint32_t gparity) {
  const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  const int local = t - T.tileBase;
  FB_GUARD(a, local >= 0 && local < T.nTiles, 8, local, t, return);
  const int sub = local * kSubPerTile + w;
  const int i0 = sub * kSub + (int)lane, i1 = i0 + 32;
  const int N = T.N;
  // both neurons' loads are issued before either is stored (the stores could alias them)
  const NState x0 = load_neuron(T, i0 < N ? i0 : 0);
  const NState x1 = load_neuron(T, i1 < N ? i1 : 0);
  const uint32_t f0 = i0 < N ? update_neuron(a, T, G, i0, x0, gparity) : 0;
  const uint32_t f1 = i1 < N ? update_neuron(a, T, G, i1, x1, gparity) : 0;
  const uint32_t b0 = __ballot_sync(0xffffffffu, f0 != 0), b1 = __ballot_sync(0xffffffffu, f1 != 0);
  if (!(b0 | b1)) {
    if (lane == 0) {
      T.tileCnt[sub] = 0;
      T.tileDeg[sub] = 0;
    }
    return;
  }
  // out-degree prefix in ascending order: the lanes' first neurons, then their second ones
  const uint32_t d0 = f0 ? f0 - 1 : 0u, d1 = f1 ? f1 - 1 : 0u;
  uint32_t s0 = d0, s1 = d1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y0 = __shfl_up_sync(0xffffffffu, s0, o), y1 = __shfl_up_sync(0xffffffffu, s1, o);
    if ((int)lane >= o) {
      s0 += y0;
      s1 += y1;
    }
  }
  const uint32_t tot0 = __shfl_sync(0xffffffffu, s0, 31), tot1 = __shfl_sync(0xffffffffu, s1, 31);
  const uint32_t n0 = __popc(b0);
  int32_t *stage = T.stage + (int64_t)sub * kSub;
  uint32_t *stageDeg = T.stageDeg + (int64_t)sub * kSub;
  if (f0) {
    const uint32_t p = __popc(b0 & lt);
    stage[p] = i0;
    stageDeg[p] = s0 - d0;
  }
  if (f1) {
    const uint32_t p = n0 + __popc(b1 & lt);
    stage[p] = i1;
    stageDeg[p] = tot0 + s1 - d1;
  }
  if (lane == 0) {
    T.tileCnt[sub] = (int32_t)(n0 + __popc(b1));
    T.tileDeg[sub] = tot0 + tot1;
  }
}

// ---------------------------------------------------------------------------------------------
// The persistent kernel
// ---------------------------------------------------------------------------------------------

// Brain headers of the first kTrialCache brains of a batch are copied to shared memory once per
// launch: the acquire fence that ends every grid barrier invalidates L1, so constants read from
// global memory would be refetched from L2 at every step.
constexpr int kTrialCache = 4;

__global__ void __launch_bounds__(kBlock, 2) step_kernel(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  // per-brain launch constants (layout mirrors step_smem_bytes): step count and log start at
  // launch, start head, ring depth, steps of this launch, first tile; then the prefix of this
  // step's delivery work items over brains
  int64_t *sDone = (int64_t *)smraw;
  int64_t *sLog = sDone + a.B;
  int32_t *sHead0 = (int32_t *)(sLog + a.B);
  int32_t *sNs = sHead0 + a.B;
  int32_t *sSteps = sNs + a.B;
  int32_t *sND = sSteps + a.B;             // driven-list length at launch
  int32_t *sTile0 = sND + a.B;             // B + 1: first update tile of each brain
  int32_t *sDch0 = sTile0 + a.B + 1;       // B + 1: first driven chunk item of each brain
  uint32_t *sPre = (uint32_t *)(sDch0 + a.B + 1);  // B + 1
  __shared__ uint32_t scan[33];
  __shared__ uint64_t scan64[33];
  __shared__ uint32_t sJump[32 * 128];
  __shared__ Trial sTr[kTrialCache];
  const int tid = threadIdx.x;
  for (int k = tid; k < 32 * 128; k += blockDim.x) sJump[k] = a.jump[k];
  {
    const int nc = min(a.B, kTrialCache);
    const uint32_t *src = (const uint32_t *)a.trials;
    uint32_t *dst = (uint32_t *)sTr;
    for (int k = tid; k < nc * (int)(sizeof(Trial) / 4); k += blockDim.x) dst[k] = ldcg(src + k);
  }
  for (int b = tid; b < a.B; b += blockDim.x) {
    const Trial *G = a.trials + b;
    sDone[b] = ldcg(&G->stepsDone);
    sLog[b] = ldcg(&G->logStart);
    sHead0[b] = ldcg(&G->head);
    sNs[b] = G->nslots;
    sSteps[b] = a.steps[b];
    sND[b] = ldcg(&G->nDriven);
    sTile0[b] = G->tileBase;
  }
  __syncthreads();
  if (tid == 0) {
    sTile0[a.B] = a.nTilesTotal;
    int dc = 0;
    for (int b = 0; b < a.B; b++) {
      sDch0[b] = dc;
      dc += max(1, (sND[b] + kBlock - 1) / kBlock);
    }
    sDch0[a.B] = dc;
  }
  __syncthreads();
  auto hdr = [&](int b) -> const Trial & {
    const Trial *p = b < kTrialCache ? (const Trial *)sTr + b : (const Trial *)a.trials + b;
    return *p;
  };
  auto find = [&](const int32_t *first, int x) {  // b with first[b] <= x < first[b+1]
    int lo = 0, hi = a.B;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (first[mid] <= x) lo = mid;
      else hi = mid;
    }
    return lo;
  };
  const int nDItems = sDch0[a.B];
  const int warpsPerBlock = blockDim.x >> 5;
  const uint32_t gwarp = blockIdx.x * warpsPerBlock + (tid >> 5);
  const uint32_t nwarps = gridDim.x * warpsPerBlock;

  // the first step's grab counter; later ones are cleared a step ahead in the update phase
  if (blockIdx.x == 0 && tid == 0 && a.subGrab) a.subNext[0] = 0;
  uint64_t tp = a.phaseNs != nullptr ? global_ns() : 0;
  auto lap = [&](int k) { prof_lap(a, k, tp); };
  for (int s = 0; s <= a.maxSteps; s++) {
    // ---------------- phase A: materialize step s-1, control + deliver step s ----------------
    for (int item = blockIdx.x; item < nDItems + a.B; item += gridDim.x) {
      if (item < nDItems) {
        const int b = find(sDch0, item);
        if (s < sSteps[b]) {
          const int ns = sNs[b];
          const int head = (sHead0[b] + s) % ns;
          driven_item(a, hdr(b), a.trials + b, item - sDch0[b], sDch0[b + 1] - sDch0[b], sND[b],
                      (uint64_t)(sDone[b] + s), head, scan, scan64, sJump, tp);
          __syncthreads();
        }
      } else {
        const int b = item - nDItems;
        if (s >= 1 && s <= sSteps[b]) {
          const int ns = sNs[b];
          const int head = (sHead0[b] + s - 1) % ns;
          const uint64_t g = (uint64_t)(sDone[b] + s - 1);
          materialize_brain(a, hdr(b), a.trials + b, sDch0[b + 1] - sDch0[b], g, (head + ns - 1) % ns,
                            (int64_t)g - sLog[b], scan64, scan);
          __syncthreads();
        }
      }
    }
    if (s == a.maxSteps) break;
    lap(0);
    // delivery work items of every brain still stepping, enumerated through a prefix over brains
    {
      uint32_t carry = 0;
      for (int b0 = 0; b0 < a.B; b0 += blockDim.x) {
        const int b = b0 + tid;
        uint32_t n = 0;
        if (b < a.B && s < sSteps[b]) {
          const Trial &T = hdr(b);
          if (T.mode != FB_DELIVER_SEQUENTIAL) {
            const int head = (sHead0[b] + s) % sNs[b];
            const uint32_t per = (uint32_t)kChunk * (uint32_t)a.itemChunks;
            n = (ldcg(T.slotEdges + head) + per - 1) / per;
          }
        }
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(n, &tot, scan);
        if (b < a.B) sPre[b] = carry + ex;
        carry += tot;
      }
      if (tid == 0) sPre[a.B] = carry;
      __syncthreads();
    }
    // work items go to warps from the far end of the grid, whose blocks have the fewest items;
    // a warp takes two at a time (w and w + nwarps): both items' loads, then both items' claims
    const uint32_t total = sPre[a.B];
    auto brain_of = [&](uint32_t w) {  // brain b with sPre[b] <= w < sPre[b+1]
      int lo = 0, hi = a.B;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sPre[mid] <= w) lo = mid;
        else hi = mid;
      }
      return lo;
    };
    for (uint32_t w = nwarps - 1 - gwarp; w < total; w += 2 * nwarps) {
      const uint32_t w2 = w + nwarps;
      const bool two = w2 < total;
      const int b1 = brain_of(w), b2 = two ? brain_of(w2) : b1;
      const Trial &T1 = hdr(b1);
      const Trial &T2 = hdr(b2);
      const int h1 = (sHead0[b1] + s) % sNs[b1], h2 = (sHead0[b2] + s) % sNs[b2];
      const uint32_t F1 = ldcg(T1.slotEdges + h1), F2 = two ? ldcg(T2.slotEdges + h2) : 0u;
      const uint32_t c1 = (w - sPre[b1]) * (uint32_t)a.itemChunks;
      const uint32_t c2 = two ? (w2 - sPre[b2]) * (uint32_t)a.itemChunks : 0u;
      for (int u = 0; u < a.itemChunks; u++) {
        const bool on1 = (c1 + u) * (uint32_t)kChunk < F1, on2 = two && (c2 + u) * (uint32_t)kChunk < F2;
        if (!on1 && !on2) break;
        DEdge d1, d2;
        d1.valid = d2.valid = false;
        if (on1) d1 = load_edge(a, T1, h1, F1, c1 + u);
        if (on2) d2 = load_edge(a, T2, h2, F2, c2 + u);
        claim_edge(a, T1, d1, (uint32_t)(s & 1));
        claim_edge(a, T2, d2, (uint32_t)(s & 1));
      }
    }
    lap(1);
    if (!grid_sync(a)) return;
    lap(2);

    // ---------------- phase B: update every neuron of every brain still stepping --------------
    // the overflow pool alternates with the launch-local step parity; the half used next step
    // was last read in the update phase of the step before this one
    if (blockIdx.x == 0 && tid == 0) a.ovfTop[(s + 1) & 1] = 0;
    if (blockIdx.x == 0 && tid == 0 && a.subGrab) a.subNext[(s + 1) & 1] = 0;
    // warp sub-tiles (a warp per sub-tile, no block barrier) of the brains still stepping, numbered
    // through a prefix over brains (sPre, free again after the delivery). With many sub-tiles per
    // warp the first 5/8 go to the warps as equal contiguous runs (a run stays within few brains,
    // whose headers stay in L1, and a warp keeps the brain of its last sub-tile) and the rest is
    // taken subGrab at a time from a counter, so warps that drew slow sub-tiles take fewer of the
    // rest; otherwise every warp takes every nwarps-th
    {
      int64_t total;
      if (a.B > 1) {
        uint32_t carry = 0;
        for (int b0 = 0; b0 < a.B; b0 += blockDim.x) {
          const int b = b0 + tid;
          const uint32_t n = (b < a.B && s < sSteps[b]) ? (uint32_t)(sTile0[b + 1] - sTile0[b]) * kSubPerTile : 0u;
          uint32_t tot;
          const uint32_t ex = block_exclusive_scan(n, &tot, scan);
          if (b < a.B) sPre[b] = carry + ex;
          carry += tot;
        }
        if (tid == 0) sPre[a.B] = carry;
        __syncthreads();
        total = carry;
      } else {
        total = s < sSteps[0] ? (int64_t)a.nTilesTotal * kSubPerTile : 0;
      }
      const bool dyn = a.subGrab > 0 && total >= 8 * (int64_t)nwarps;
      const int64_t s0 = dyn ? total * 5 / 8 : total, run = (s0 + nwarps - 1) / nwarps;
      int64_t gs = dyn ? (int64_t)gwarp * run : gwarp, end = dyn ? min(s0, gs + run) : total,
              stride = dyn ? 1 : nwarps;
      int cb = 0;
      int64_t cLo = 0, cHi = a.B > 1 ? 0 : total;  // the brain of the last sub-tile and its range
      for (;;) {
        if (gs >= end) {
          if (!dyn) break;
          uint32_t g0 = 0;
          if ((tid & 31) == 0) g0 = atomicAdd(a.subNext + (s & 1), (uint32_t)a.subGrab);
          gs = s0 + (int64_t)__shfl_sync(0xffffffffu, g0, 0);
          end = min(total, gs + a.subGrab);
          stride = 1;
          if (gs >= total) break;
        }
        if (gs < cLo || gs >= cHi) {  // largest b with sPre[b] <= gs (brains with no sub-tile skipped)
          int lo = 0, hi = a.B;
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if ((int64_t)sPre[mid] <= gs) lo = mid;
            else hi = mid;
          }
          cb = lo;
          cLo = sPre[lo];
          cHi = sPre[lo + 1];
        }
        const int64_t local = gs - cLo;
        update_tile(a, hdr(cb), a.trials + cb, sTile0[cb] + (int)(local / kSubPerTile), (int)(local % kSubPerTile),
                    (uint32_t)(s & 1));
        gs += stride;
      }
    }
    lap(3);
    if (!grid_sync(a)) return;
    lap(4);
  }
  // per-brain scalars after the launch: ring head and step count
  __syncthreads();
  if (!grid_sync(a)) return;
  for (int b = blockIdx.x * blockDim.x + tid; b < a.B; b += gridDim.x * blockDim.x) {
    Trial *G = a.trials + b;
    G->head = (sHead0[b] + sSteps[b]) % sNs[b];
    G->stepsDone = sDone[b] + sSteps[b];
  }
  if (blockIdx.x == 0 && tid == 0) {  // the next launch starts with an empty overflow pool
    a.ovfTop[0] = 0;
    a.ovfTop[1] = 0;
  }
}

// ---------------------------------------------------------------------------------------------
// Small kernels around the step
// ---------------------------------------------------------------------------------------------

struct Delta {
  int32_t brain, field, idx, pad;
  double val;
};

// Applies queued host writes in call order. Deltas arrive grouped by (brain, field, index) with
// the call order kept inside a group (stable sort on the host); one thread runs one group.
__global__ void apply_deltas_kernel(Trial *trials, const Delta *d, const int32_t *groupStart,
                                    int32_t nGroups) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nGroups) return;
  const int32_t lo = groupStart[g], hi = groupStart[g + 1];
  const Delta d0 = d[lo];
  Trial *T = trials + d0.brain;
  float *dst;
  switch (d0.field) {
    case FB_FIELD_GE: dst = T->gE; break;
    case FB_FIELD_GI: dst = T->gI; break;
    case FB_FIELD_BIAS: dst = T->bias; break;
    case FB_FIELD_THR: dst = T->thr; break;
    default: dst = T->drive; break;
  }
  float x = dst[d0.idx];
  const bool add = d0.field == FB_FIELD_GE || d0.field == FB_FIELD_GI;
  for (int32_t k = lo; k < hi; k++) {
    // a JS number into a Float32Array element: formed in f64, rounded once on the store
    x = add ? __double2float_rn((double)x + d[k].val) : __double2float_rn(d[k].val);
  }
  dst[d0.idx] = x;
}

// State back to rest for brain b (src/lifwasm.js:78).
__global__ void reset_kernel(Trial *trials, int32_t b0, int32_t b1) {
  for (int32_t b = b0; b < b1; b++) {
    Trial *T = trials + b;
    const int N = T->N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
      T->v[i] = T->vRest;
      T->gE[i] = 0.f;
      T->gI[i] = 0.f;
      T->refr[i] = 0.f;
      T->trace[i] = 0.f;
      T->adapt[i] = 0.f;
      T->res[i] = 1.f;
      T->spikeCount[i] = 0u;
    }
    if (blockIdx.x == 0)
      for (int k = threadIdx.x; k < T->nslots; k += blockDim.x) {
        T->ringCount[k] = 0;
        T->slotEdges[k] = 0;
      }
  }
}

// Rebuilds, for every ring slot, the per-arrival edge offsets and row starts, the slot's edge
// total and its delivery work-item records from the caller's ring lists (one block per slot).
__global__ void rebuild_slots_kernel(Trial *Tp, int32_t *err) {
  __shared__ uint32_t scan[33];
  const Trial &T = *Tp;
  const int slot = blockIdx.x, tid = threadIdx.x;
  const int N = T.N;
  const int32_t na = T.ringCount[slot];
  if (na < 0 || na > N) {
    if (tid == 0) atomicCAS(err, 0, FB_EINVAL);
    return;
  }
  const int32_t *list = T.ring + (int64_t)slot * N;
  uint32_t *off = T.ringOff + (int64_t)slot * (N + 1);
  uint32_t *row = T.ringRow + (int64_t)slot * N;
  uint4 *chunkK = T.chunkK + (int64_t)slot * T.chunkCap;
  uint32_t carry = 0;
  for (int32_t k0 = 0; k0 < na; k0 += blockDim.x) {
    const int32_t k = k0 + tid;
    int32_t i = 0;
    uint32_t r0 = 0, deg = 0;
    if (k < na) {
      i = list[k];
      if (i < 0 || i >= N) {
        atomicCAS(err, 0, FB_EINVAL);
        i = 0;
      } else {
        r0 = T.indptr[i];
        deg = T.indptr[i + 1] - r0;
      }
    }
    uint32_t tot;
    const uint32_t pre = block_exclusive_scan(deg, &tot, scan);
    if (k < na) {
      const uint32_t o = carry + pre;
      off[k] = o;
      row[k] = r0;
      mark_chunks(chunkK, o, deg, (uint32_t)k, (uint32_t)i, r0);
    }
    carry += tot;
  }
  if (tid == 0) {
    off[na] = carry;
    T.slotEdges[slot] = carry;
  }
}

}  // namespace fb

// ---------------------------------------------------------------------------------------------
// Host-side launch glue (internal; called from fb_api.cu)
// ---------------------------------------------------------------------------------------------
namespace fb {

size_t step_smem_bytes(int B) {
  return (size_t)B * 8 * 2 + (size_t)B * 4 * 4 + (size_t)(B + 1) * 4 * 3;
}

// The kernel's dynamic shared-memory limit, raised (never lowered) per device to the largest
// size asked for, so a batch's launch never runs under a limit another batch set lower.
cudaError_t set_step_smem(size_t bytes) {
  static std::mutex mu;
  static size_t limit[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[dev & 63];
  if (bytes <= cur || bytes <= 48 * 1024) return cudaSuccess;
  e = cudaFuncSetAttribute(step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

int step_kernel_blocks_per_sm(size_t smem) {
  if (set_step_smem(smem) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel, kBlock, smem) != cudaSuccess) return 0;
  return n;
}

cudaError_t launch_step(const StepArgs &a, int grid, size_t smem, cudaStream_t st) {
  const cudaError_t e = set_step_smem(smem);
  if (e != cudaSuccess) return e;
  void *args[] = {(void *)&a};
  return cudaLaunchCooperativeKernel((const void *)step_kernel, dim3(grid), dim3(kBlock), args, smem, st);
}

cudaError_t launch_deltas(Trial *trials, const Delta *d, const int32_t *gs, int32_t nGroups, cudaStream_t st) {
  if (nGroups <= 0) return cudaSuccess;
  apply_deltas_kernel<<<(nGroups + 255) / 256, 256, 0, st>>>(trials, d, gs, nGroups);
  return cudaGetLastError();
}


cudaError_t launch_rebuild_slots(Trial *Td, int nslots, int32_t *err, cudaStream_t st) {
  rebuild_slots_kernel<<<nslots, kBlock, 0, st>>>(Td, err);
  return cudaGetLastError();
}

cudaError_t launch_reset(Trial *trials, int32_t b0, int32_t b1, cudaStream_t st) {
  reset_kernel<<<304, 256, 0, st>>>(trials, b0, b1);
  return cudaGetLastError();
}

}  // namespace fb
