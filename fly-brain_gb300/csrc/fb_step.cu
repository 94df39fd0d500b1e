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

#include "fb_internal.cuh"

namespace fb {

// ---------------------------------------------------------------------------------------------
// Phase A pieces
// ---------------------------------------------------------------------------------------------

// The serial parts of one brain's step, executed by one block (lif.c:35-52 minus the scatter).
__device__ void brain_control(const StepArgs &a, Trial *T, int s, uint64_t gstep, int head,
                              int slot, uint32_t *scan) {
  __shared__ uint32_t sh_s0, sh_nbg;
  __shared__ float sh_amp;
  __shared__ bool sh_go;
  const int tid = threadIdx.x;
  const int N = T->N;
  const int mode = T->mode;
  if (tid == 0) {
    // lif.c:47: bgAcc += bgEvents; nbg = (int)bgAcc; bgAcc -= nbg (f32 throughout)
    float acc = __fadd_rn(ldcg(&T->bgAcc), T->bgEvents);
    const int32_t nbg = (int32_t)acc;
    acc = __fsub_rn(acc, (float)nbg);
    T->bgAcc = acc;
    sh_nbg = (uint32_t)nbg;
    sh_s0 = ldcg(&T->rng);
  }
  __syncthreads();
  const uint32_t s0 = sh_s0, nbg = sh_nbg;
  const int32_t *arr = T->ring + (int64_t)head * N;

  // Sequential delivery (exact also with presynaptic inhibition, lif.c:36-43): arrivals one at a
  // time in list order; each row's targets are distinct, so a row scatters in parallel.
  if (mode == FB_DELIVER_SEQUENTIAL) {
    const int32_t na = ldcg(T->ringCount + head);
    for (int32_t k = 0; k < na; k++) {
      const int32_t pre = ldcg(arr + k);
      if (tid == 0) {
        float r = ldcg(T->res + pre);
        float amp = __fmul_rn(__ldg(T->sign + pre), r);
        sh_go = amp != 0.f;  // lif.c:37 skips only a zero sign*res, not a zero after :38
        if (sh_go) {
          if (T->preInh > 0.f && ldcg(T->drive + pre) > 0.f) {
            const float gi = ldcg(T->gI + pre);
            amp = __fdiv_rn(amp, __fadd_rn(1.f, __fmul_rn(T->preInh, gi < 0.f ? -gi : 0.f)));
          }
          T->res[pre] = __fsub_rn(r, __fmul_rn(T->depU, r));
        }
        sh_amp = amp;
      }
      __syncthreads();
      const float amp = sh_amp;
      if (sh_go) {
        const uint32_t lo = __ldg(T->indptr + pre), hi = __ldg(T->indptr + pre + 1);
        float *g = amp > 0 ? T->gE : T->gI;
        for (uint32_t j = lo + tid; j < hi; j += blockDim.x) {
          const uint32_t q = __ldg(T->indices + j);
          g[q] = __fadd_rn(ldcg(g + q), __fmul_rn(__ldg(T->W + j), amp));
        }
      }
      __syncthreads();
    }
  } else if (T->flags & kHasDep) {
    // Mark arrivals so the update phase applies the depression res -= depU*res (lif.c:39).
    const int32_t na = ldcg(T->ringCount + head);
    for (int32_t k = tid; k < na; k += blockDim.x) T->arrived[ldcg(arr + k)] = 1;
  }
  __syncthreads();  // every thread has read ringCount[head] above
  if (tid == 0) T->ringCount[head] = 0;  // lif.c:44

  // Background draws 1..nbg (lif.c:48): target = draw % N, counted per target; the update phase
  // adds bgAmp once per hit after the synaptic contributions, as lif.c orders them.
  for (uint32_t d = 1 + tid; d <= nbg; d += blockDim.x) {
    const uint32_t x = xs_jump(a.jump, s0, d);
    atomicAdd(T->bgHits + (x % (uint32_t)N), 1u);
  }

  // Poisson-driven forced spikes (lif.c:49-52), in driven-list order, blockDim at a time.
  const int32_t nD = ldcg(&T->nDriven);
  int32_t *out = T->ring + (int64_t)slot * N;
  uint32_t *outOff = T->ringOff + (int64_t)slot * (N + 1);
  uint32_t *chunkK = T->chunkK + (int64_t)slot * T->chunkCap;
  uint32_t draws = 0, nd = 0, deg = 0;
  for (int32_t r0 = 0; r0 < nD; r0 += blockDim.x) {
    const int32_t k = r0 + tid;
    int32_t i = 0;
    uint32_t live = 0;
    if (k < nD) {
      i = ldcg(T->driven + k);
      live = ldcg(T->refr + i) > 0 ? 0u : 1u;  // refractory neurons draw nothing
    }
    uint32_t nlive;
    const uint32_t dpos = block_exclusive_scan(live, &nlive, scan);
    uint32_t fire = 0;
    if (live) {
      const uint32_t x = xs_jump(a.jump, s0, nbg + draws + dpos + 1);
      const float u = __fmul_rn((float)(x >> 8), 1.0f / 16777216.0f);
      const float p = __fmul_rn(ldcg(T->drive + i), T->dtS);
      fire = u < p ? 1u : 0u;
    }
    uint32_t nfire;
    const uint32_t fpos = block_exclusive_scan(fire, &nfire, scan);
    uint32_t dg = 0;
    if (fire) dg = __ldg(T->indptr + i + 1) - __ldg(T->indptr + i);
    uint32_t dsum;
    const uint32_t opos = block_exclusive_scan(dg, &dsum, scan);
    if (fire) {
      const uint32_t kk = nd + fpos, o = deg + opos;
      out[kk] = i;
      outOff[kk] = o;
      mark_chunks(chunkK, o, dg, kk);
      T->v[i] = T->vReset;
      T->refr[i] = __fadd_rn(T->tRef, T->dt);
      T->spikeCount[i] = ldcg(T->spikeCount + i) + 1u;
      T->trace[i] = 1.f;
      T->adapt[i] = __fadd_rn(ldcg(T->adapt + i), T->adaptInc);
    }
    draws += nlive;
    nd += nfire;
    deg += dsum;
  }
  if (tid == 0) {
    T->rng = xs_jump(a.jump, s0, nbg + draws);
    T->nForced[gstep & 1] = (int32_t)nd;
    T->forcedDeg[gstep & 1] = deg;
  }
}

// Copies tile t's threshold spikes of step `gstep` (staged in the update phase) into the ring
// slot, after the driven spikes and all lower tiles: ascending neuron order (lif.c:74-76).
__device__ void materialize_tile(const StepArgs &a, Trial *T, int t, uint64_t gstep, int slot,
                                 int64_t logBase) {
  __shared__ uint32_t sh_cnt, sh_deg;
  const int tid = threadIdx.x;
  const int local = t - T->tileBase;
  const bool last = local == T->nTiles - 1;
  const int32_t m = ldcg(T->tileCnt + t);
  if (m == 0 && !last && !(local == 0 && a.log)) return;  // uniform across the block
  // counts and out-degrees of the lower tiles of this brain (the last tile also needs its own)
  if (tid < 32) {
    uint32_t c = 0, d = 0;
    for (int u = tid; u < local; u += 32) {
      c += (uint32_t)ldcg(T->tileCnt + T->tileBase + u);
      d += ldcg(T->tileDeg + T->tileBase + u);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, o);
      d += __shfl_xor_sync(0xffffffffu, d, o);
    }
    if (tid == 0) { sh_cnt = c; sh_deg = d; }
  }
  __syncthreads();
  const int N = T->N;
  const uint32_t nd = (uint32_t)ldcg(T->nForced + (gstep & 1));
  const uint32_t Fd = ldcg(T->forcedDeg + (gstep & 1));
  const uint32_t before = nd + sh_cnt, dbefore = Fd + sh_deg;
  int32_t *out = T->ring + (int64_t)slot * N;
  uint32_t *outOff = T->ringOff + (int64_t)slot * (N + 1);
  uint32_t *chunkK = T->chunkK + (int64_t)slot * T->chunkCap;
  const int32_t *stage = T->stage + (int64_t)local * kTile;
  const uint32_t *stageDeg = T->stageDeg + (int64_t)local * kTile;
  const bool logging = a.log && T->logRaster != nullptr;
  const int64_t rbase = logging ? ldcg(T->logRasterLen + (gstep & 1)) : 0;
  for (int p = tid; p < m; p += blockDim.x) {
    const int32_t i = ldcg(stage + p);
    const uint32_t k = before + p, o = dbefore + ldcg(stageDeg + p);
    out[k] = i;
    outOff[k] = o;
    mark_chunks(chunkK, o, __ldg(T->indptr + i + 1) - __ldg(T->indptr + i), k);
    if (logging && rbase + k < T->logRasterCap) T->logRaster[rbase + k] = i;
  }
  if (logging && local == 0) {  // the driven spikes head the list
    for (uint32_t p = tid; p < nd; p += blockDim.x)
      if (rbase + p < T->logRasterCap) T->logRaster[rbase + p] = ldcg(out + p);
  }
  if (last && tid == 0) {
    const uint32_t nf = before + (uint32_t)m;
    const uint32_t F = dbefore + ldcg(T->tileDeg + t);
    outOff[nf] = F;
    T->ringCount[slot] = (int32_t)nf;
    T->slotEdges[slot] = F;
    T->nFired = (int32_t)nf;
    T->lastSlot = slot;
    if (a.log) {
      if (T->logCount && logBase >= 0 && logBase < T->logCap) T->logCount[logBase] = (int32_t)nf;
      if (T->logRaster) T->logRasterLen[(gstep + 1) & 1] = rbase + nf;
    }
  }
}

// One delivery work item: 32 consecutive edges of the concatenated rows of the arrivals in
// `slot`, starting at edge c * 32. Lane l takes edge c*32+l.
__device__ __forceinline__ void deliver_chunk(const StepArgs &a, Trial *T, int slot, uint32_t F,
                                              uint32_t c, uint32_t gparity) {
  const int lane = threadIdx.x & 31;
  const uint32_t e = c * kChunk + lane;
  if (e >= F) return;
  const int N = T->N;
  const int32_t *arr = T->ring + (int64_t)slot * N;
  const uint32_t *off = T->ringOff + (int64_t)slot * (N + 1);
  uint32_t k = ldcg(T->chunkK + (int64_t)slot * T->chunkCap + c);
  while (ldcg(off + k + 1) <= e) k++;
  const int32_t pre = ldcg(arr + k);
  const float amp = __fmul_rn(__ldg(T->sign + pre), ldcg(T->res + pre));  // lif.c:37
  if (amp == 0.f) return;
  const uint32_t j = __ldg(T->indptr + pre) + (e - ldcg(off + k));
  const uint32_t q = __ldg(T->indices + j);
  const float w = __fmul_rn(__ldg(T->W + j), amp);  // lif.c:41-42, one rounding
  const bool inh = !(amp > 0);
  if (T->mode == FB_DELIVER_FAST) {
    atomicAdd(inh ? T->gI + q : T->gE + q, w);
    return;
  }
  const uint32_t key = (k << 1) | (inh ? 1u : 0u);
  const uint32_t pos = atomicAdd(T->cnt + q, 1u);
  if (pos < (uint32_t)kBucket) {
    T->bucket[(int64_t)q * kBucket + pos] = make_uint2(key, __float_as_uint(w));
  } else {
    const uint32_t r = atomicAdd(a.ovfTop + gparity, 1u);
    if (r >= a.ovfCap) {
      atomicCAS(a.err, 0, FB_EOVERFLOW);
      return;
    }
    OvfRec rec;
    rec.key = key;
    rec.bits = __float_as_uint(w);
    rec.pad = q;
    rec.next = atomicExch(T->ovfHead + q, r);
    a.ovf[gparity][r] = rec;
  }
}

// ---------------------------------------------------------------------------------------------
// Phase B: the update of one tile of one brain
// ---------------------------------------------------------------------------------------------

// Adds target i's contributions in ascending key (arrival rank) order; inhibitory keys go to gI.
__device__ __forceinline__ void apply_contributions(const StepArgs &a, Trial *T, int i, uint32_t n,
                                                    uint32_t gparity, float &ge, float &gi) {
  const uint2 *bk = T->bucket + (int64_t)i * kBucket;
  if (n == 1) {
    const uint2 x = ldcg(bk);
    if (x.x & 1u) gi = __fadd_rn(gi, __uint_as_float(x.y));
    else ge = __fadd_rn(ge, __uint_as_float(x.y));
    return;
  }
  uint2 e[kSortMax];
  uint32_t m = n < (uint32_t)kBucket ? n : (uint32_t)kBucket;
  for (uint32_t u = 0; u < m; u++) e[u] = ldcg(bk + u);
  const bool spill = n > (uint32_t)kBucket;
  if (spill) {
    uint32_t r = ldcg(T->ovfHead + i);
    while (r != kNil && m < (uint32_t)kSortMax) {
      const OvfRec rec = a.ovf[gparity][r];
      e[m++] = make_uint2(rec.key, rec.bits);
      r = rec.next;
    }
    T->ovfHead[i] = kNil;
    if (r != kNil) atomicCAS(a.err, 0, FB_EOVERFLOW);  // more than kSortMax in one step
  }
  for (uint32_t u = 1; u < m; u++) {  // insertion sort by key
    const uint2 x = e[u];
    uint32_t w = u;
    while (w > 0 && e[w - 1].x > x.x) {
      e[w] = e[w - 1];
      w--;
    }
    e[w] = x;
  }
  for (uint32_t u = 0; u < m; u++) {
    if (e[u].x & 1u) gi = __fadd_rn(gi, __uint_as_float(e[u].y));
    else ge = __fadd_rn(ge, __uint_as_float(e[u].y));
  }
}

__device__ void update_tile(const StepArgs &a, Trial *T, int t, uint32_t gparity, uint32_t *scan) {
  const int tid = threadIdx.x;
  const int local = t - T->tileBase;
  const int i = local * kTile + tid;
  const int N = T->N;
  bool fired = false;
  uint32_t dg = 0;
  if (i < N) {
    float v = ldcg(T->v + i), r = ldcg(T->refr + i);
    float ge = ldcg(T->gE + i), gi = ldcg(T->gI + i);
    float tr = ldcg(T->trace + i), ad = ldcg(T->adapt + i), rs = ldcg(T->res + i);
    const float bias = ldcg(T->bias + i), thr = ldcg(T->thr + i);
    if (T->mode == FB_DELIVER_EXACT) {
      const uint32_t n = ldcg(T->cnt + i);
      if (n) {
        apply_contributions(a, T, i, n, gparity, ge, gi);
        T->cnt[i] = 0;
      }
    }
    if (T->flags & kHasBg) {  // lif.c:48, after every synaptic contribution
      const uint32_t h = ldcg(T->bgHits + i);
      if (h) {
        for (uint32_t u = 0; u < h; u++) ge = __fadd_rn(ge, T->bgAmp);
        T->bgHits[i] = 0;
      }
    }
    if ((T->flags & kHasDep) && T->mode != FB_DELIVER_SEQUENTIAL) {
      if (ldcg(T->arrived + i)) {  // lif.c:37-39: depressed at delivery unless sign*res == 0
        T->arrived[i] = 0;
        if (!(__fmul_rn(__ldg(T->sign + i), rs) == 0.f)) rs = __fsub_rn(rs, __fmul_rn(T->depU, rs));
      }
    }
    // lif.c:55-72, one IEEE f32 operation per C operation, in C order
    float acc = __fsub_rn(T->vRest, v);
    if (T->coba) {
      acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(ge, __fsub_rn(T->eExc, v)), T->cE));
      acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(gi, __fsub_rn(v, T->eInh)), T->cI));
    } else {
      acc = __fadd_rn(acc, ge);
      acc = __fadd_rn(acc, gi);
    }
    acc = __fadd_rn(acc, bias);
    const float dv = __fmul_rn(acc, T->kM);
    const bool refractory = r > 0;
    v = refractory ? T->vReset : __fadd_rn(v, dv);
    r = refractory ? __fsub_rn(r, T->dt) : r;
    ge = __fmul_rn(ge, T->dE);
    gi = __fmul_rn(gi, T->dE);
    tr = __fmul_rn(tr, T->dTr);
    ad = __fmul_rn(ad, T->dA);
    rs = __fadd_rn(rs, __fmul_rn(__fsub_rn(1.f, rs), T->kRec));
    // lif.c:74-75: threshold against the decayed adapt
    if (v >= __fadd_rn(__fadd_rn(T->vThresh, ad), thr) && r <= 0) {
      v = T->vReset;
      r = T->tRef;
      tr = 1.f;
      ad = __fadd_rn(ad, T->adaptInc);
      T->spikeCount[i] = ldcg(T->spikeCount + i) + 1u;
      fired = true;
      dg = __ldg(T->indptr + i + 1) - __ldg(T->indptr + i);
    }
    T->v[i] = v;
    T->refr[i] = r;
    T->gE[i] = ge;
    T->gI[i] = gi;
    T->trace[i] = tr;
    T->adapt[i] = ad;
    T->res[i] = rs;
  }
  // ascending compaction of the tile's spikes (and their out-degree prefix) into the staging area
  uint32_t nf, dsum;
  const uint32_t pos = block_exclusive_scan(fired ? 1u : 0u, &nf, scan);
  const uint32_t dpos = block_exclusive_scan(dg, &dsum, scan);
  if (fired) {
    T->stage[(int64_t)local * kTile + pos] = i;
    T->stageDeg[(int64_t)local * kTile + pos] = dpos;
  }
  if (tid == 0) {
    T->tileCnt[t] = (int32_t)nf;
    T->tileDeg[t] = dsum;
  }
}

// ---------------------------------------------------------------------------------------------
// The persistent kernel
// ---------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kBlock) step_kernel(StepArgs a) {
  extern __shared__ uint32_t sm[];
  // per-brain launch constants: start head, ring depth, steps of this launch; then the prefix of
  // this step's delivery work items over brains
  int32_t *sHead0 = (int32_t *)sm;
  int32_t *sNs = sHead0 + a.B;
  int32_t *sSteps = sNs + a.B;
  uint32_t *sPre = (uint32_t *)(sSteps + a.B);  // B + 1
  __shared__ uint32_t scan[33];
  __shared__ int64_t sStepsDone;
  const int tid = threadIdx.x;
  for (int b = tid; b < a.B; b += blockDim.x) {
    sHead0[b] = ldcg(&a.trials[b].head);
    sNs[b] = a.trials[b].nslots;
    sSteps[b] = a.steps[b];
  }
  __syncthreads();
  const int warpsPerBlock = blockDim.x >> 5;
  const uint32_t gwarp = blockIdx.x * warpsPerBlock + (tid >> 5);
  const uint32_t nwarps = gridDim.x * warpsPerBlock;

  for (int s = 0; s <= a.maxSteps; s++) {
    // ---------------- phase A: materialize step s-1, control + deliver step s ----------------
    for (int item = blockIdx.x; item < a.B + a.nTilesTotal; item += gridDim.x) {
      if (item < a.B) {
        const int b = item;
        if (s < sSteps[b]) {
          Trial *T = a.trials + b;
          if (tid == 0) sStepsDone = ldcg(&T->stepsDone);
          __syncthreads();
          const int ns = sNs[b];
          const int head = (sHead0[b] + s) % ns;
          brain_control(a, T, s, (uint64_t)(sStepsDone + s), head, (head + ns - 1) % ns, scan);
          __syncthreads();
        }
      } else {
        const int t = item - a.B;
        const int b = a.tileTrial[t];
        if (s >= 1 && s <= sSteps[b]) {
          Trial *T = a.trials + b;
          if (tid == 0) sStepsDone = ldcg(&T->stepsDone);
          __syncthreads();
          const int ns = sNs[b];
          const int head = (sHead0[b] + s - 1) % ns;
          const uint64_t g = (uint64_t)(sStepsDone + s - 1);
          materialize_tile(a, T, t, g, (head + ns - 1) % ns, (int64_t)g - ldcg(&T->logStart));
          __syncthreads();
        }
      }
    }
    if (s == a.maxSteps) break;
    // delivery work items of every brain still stepping, enumerated through a prefix over brains
    {
      uint32_t carry = 0;
      for (int b0 = 0; b0 < a.B; b0 += blockDim.x) {
        const int b = b0 + tid;
        uint32_t n = 0;
        if (b < a.B && s < sSteps[b]) {
          const Trial *T = a.trials + b;
          if (T->mode != FB_DELIVER_SEQUENTIAL) {
            const int head = (sHead0[b] + s) % sNs[b];
            n = (ldcg(T->slotEdges + head) + kChunk - 1) / kChunk;
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
    const uint32_t total = sPre[a.B];
    for (uint32_t w = gwarp; w < total; w += nwarps) {
      int lo = 0, hi = a.B;  // brain b with sPre[b] <= w < sPre[b+1]
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sPre[mid] <= w) lo = mid;
        else hi = mid;
      }
      Trial *T = a.trials + lo;
      const int head = (sHead0[lo] + s) % sNs[lo];
      deliver_chunk(a, T, head, ldcg(T->slotEdges + head), w - sPre[lo], (uint32_t)(s & 1));
    }
    if (!grid_sync(a)) return;

    // ---------------- phase B: update every neuron of every brain still stepping --------------
    // the overflow pool alternates with the launch-local step parity; the half used next step
    // was last read in the update phase of the step before this one
    if (blockIdx.x == 0 && tid == 0) a.ovfTop[(s + 1) & 1] = 0;
    for (int t = blockIdx.x; t < a.nTilesTotal; t += gridDim.x) {
      const int b = a.tileTrial[t];
      if (s < sSteps[b]) update_tile(a, a.trials + b, t, (uint32_t)(s & 1), scan);
    }
    if (!grid_sync(a)) return;
  }
  // per-brain scalars after the launch: ring head and step count
  __syncthreads();
  if (!grid_sync(a)) return;
  for (int b = blockIdx.x * blockDim.x + tid; b < a.B; b += gridDim.x * blockDim.x) {
    Trial *T = a.trials + b;
    T->head = (sHead0[b] + sSteps[b]) % sNs[b];
    T->stepsDone = T->stepsDone + sSteps[b];
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

}  // namespace fb

// ---------------------------------------------------------------------------------------------
// Host-side launch glue (internal; called from fb_api.cu)
// ---------------------------------------------------------------------------------------------
namespace fb {

int step_kernel_blocks_per_sm(size_t smem) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel, kBlock, smem) != cudaSuccess) return 0;
  return n;
}

cudaError_t launch_step(const StepArgs &a, int grid, size_t smem, cudaStream_t st) {
  void *args[] = {(void *)&a};
  return cudaLaunchCooperativeKernel((const void *)step_kernel, dim3(grid), dim3(kBlock), args, smem, st);
}

cudaError_t launch_deltas(Trial *trials, const Delta *d, const int32_t *gs, int32_t nGroups, cudaStream_t st) {
  if (nGroups <= 0) return cudaSuccess;
  apply_deltas_kernel<<<(nGroups + 255) / 256, 256, 0, st>>>(trials, d, gs, nGroups);
  return cudaGetLastError();
}

cudaError_t set_step_smem(size_t bytes) {
  return cudaFuncSetAttribute(step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t launch_reset(Trial *trials, int32_t b0, int32_t b1, cudaStream_t st) {
  reset_kernel<<<304, 256, 0, st>>>(trials, b0, b1);
  return cudaGetLastError();
}

}  // namespace fb
