// The differentiable brain step and its adjoint on sm_103a: the reference's LIFDiff
// (src/lifdiff.js:219-686). Forward with a spike tape and state checkpoints every K steps;
// backward replays one segment from its checkpoint (forced spikes from the tape, so the RNG is
// never redrawn), then sweeps the segment's steps in reverse.
//
// Arithmetic is LIFDiff's: every intermediate in double, every state word float32, operands in
// the JS order; per-target conductance sums run in the reference's arrival order (each
// contribution is pushed with its arrival rank into a per-target bucket and summed in rank order).
// The backward accumulates without float atomics: within one step every edge and every
// presynaptic neuron is touched by one arrival at most, so per-edge and per-neuron accumulators
// have a single writer per step and are summed in time order; scalars are reduced in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fb_internal.cuh"

namespace fb {
int set_error(int code, const char *msg);
void host_jump_tables(std::vector<uint32_t> &tab);

constexpr int kDB = 256;      // threads per block of the per-neuron kernels
constexpr int kDBucket = 8;   // bucket slots per target and step
constexpr int kDSortMax = 64; // contributions per target sorted in local memory

struct DOvf {
  uint32_t k, j, next, pad;
};

// Everything the kernels see: parameters (double), graph, derived arrays, state, tape, scratch.
struct DiffDev {
  int32_t N, nslots, K, coba, soft, nDriven, nro, pad;
  int64_t E;
  double dt, vRest, vThresh, vReset, tRef, wSyn, adaptInc, depU, eExc, eInh, inhGain;
  double kcThreshold, laminaBias, beta, adjClip, dE, dA, kRec, kM, dtS, cE, cI;
  // graph and per-neuron structure
  const uint32_t *indptr, *indices;
  const float *counts, *edgeGain, *sign, *logGain, *outScale, *thrOffset, *betaArr, *biasArr;
  const uint8_t *thrMask, *biasMask;
  const float *drive;
  const int32_t *driven;
  // derived per forward: inScale, gate, P[j] = (count * edgeGain) * inScale[q]
  const float *inScale;
  const uint8_t *gate;
  const double *P;
  const float *Pf;
  // state
  float *v, *gE, *gI, *adapt, *res, *refr, *spikeCount;
  uint8_t *isForced;
  uint32_t *rng;
  // tape: spike lists of every step (forced first, then threshold spikes ascending)
  int32_t *tIdx;
  float *tAmp;
  int64_t *tOff;
  int32_t *tForced;
  int64_t tapeCap;
  // delivery scratch
  uint32_t *cnt;
  uint2 *bucket;
  uint32_t *ovfHead, *ovfTop;
  DOvf *ovf;
  uint32_t ovfCap;
  double *effK;   // per arrival of the step
  // spike staging per tile
  int32_t *stage;
  float *stageAmp;
  int32_t *tileCnt;
  int32_t nTiles;
  // arena of a replayed segment (row r = step - segment start) and per-arrival res
  float *aV, *aGE, *aGI, *aAd, *aSp;
  uint8_t *aMode;
  float *resAt;
  int64_t maxArr;
  // adjoint state
  float *lv, *lgE, *lgI, *lad, *lres, *lsRing;
  // accumulators (double): per neuron A (adaptInc) V (vThresh) Kc La (laminaBias) EI (eInh)
  // W (wSyn) D (depU), per-neuron log-gain and bias gradients, per-edge weight gradients
  double *accA, *accV, *accKc, *accLa, *accEI, *accW, *accD, *gLog, *gBias, *gEdge;
  const float *dL;      // flat [N], or per step over the readout set [steps][nro]
  const int32_t *roMap; // neuron -> readout column, -1 elsewhere (per-step dL)
  int32_t *err;
  const uint32_t *jump;
};

// Model constants in the arithmetic type R of a pass: double reproduces the reference's
// arithmetic (JS numbers); float is the GB300 fast mode (the FP64 pipes are a small fraction of
// the FP32 ones). Built on the host from the double parameters, each rounded once.
template <typename R>
struct DP {
  R dt, vRest, vThresh, vReset, tRef, wSyn, adaptInc, depU, eExc, eInh, inhGain;
  R kcThreshold, laminaBias, beta, adjClip, dE, dA, kRec, kM, dtS, cE, cI;
};

template <typename R>
__device__ __forceinline__ R d_bias(const DiffDev &D, const DP<R> &P, int i, R *lam) {
  const R l = (D.biasMask && D.biasMask[i]) ? P.laminaBias : R(0);
  if (lam) *lam = l;
  return D.biasArr ? l + (R)D.biasArr[i] : l;
}
template <typename R>
__device__ __forceinline__ R d_kc(const DiffDev &D, const DP<R> &P, int i) {
  return (D.thrMask && D.thrMask[i]) ? P.kcThreshold : R(0);
}
template <typename R>
__device__ __forceinline__ R d_beta(const DiffDev &D, const DP<R> &P, int i) {
  return D.betaArr ? (R)D.betaArr[i] : P.beta;
}
template <typename R>
__device__ __forceinline__ R d_out(const DiffDev &D, int i) {
  return D.outScale ? (R)D.outScale[i] : R(1);
}
// u = v + (vRest - v + gE (eExc - v) cE + gI (v - eInh) cI + bias) kM   (src/lifdiff.js:327)
// current-based: u = v + (vRest - v + gE + gI + bias) kM              (src/wasm/lif.c:67)
template <typename R>
__device__ __forceinline__ R d_u(const DiffDev &D, const DP<R> &P, R vv, R ge, R gi, R bias) {
  if (D.coba) return vv + (P.vRest - vv + ge * (P.eExc - vv) * P.cE + gi * (vv - P.eInh) * P.cI + bias) * P.kM;
  return vv + (P.vRest - vv + ge + gi + bias) * P.kM;
}

// inScale (src/lifdiff.js:158-164).
__global__ void k_prepare(DiffDev D, float *inScale, uint8_t *gate, double *P, const float *sizeLog,
                          const float *inScaleSrc, const uint8_t *sensory, double sizeAlpha,
                          double maxSizeScale, double boostCap, double minSyn) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < D.N; i += nt) {
    if (inScaleSrc) inScale[i] = inScaleSrc[i];
    else {
      const double s = exp(-sizeAlpha * (double)sizeLog[i]);
      inScale[i] = (float)fmin(boostCap, fmax(1.0 / maxSizeScale, s));
    }
  }
}

// The gate (src/lifdiff.js:167-171) and P[j] = (count * edgeGain) * inScale[q], the first factors
// of the delivered amount (:281-282), in double and in float.
__global__ void k_prepare_edges(DiffDev D, const float *inScale, uint8_t *gate, double *P, float *Pf,
                                const uint8_t *sensory, double minSyn) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = tid; j < D.E; j += nt) {
    const uint32_t q = D.indices[j];
    const double c = (double)D.counts[j];
    gate[j] = (c >= minSyn && !(sensory && sensory[q])) ? 1 : 0;
    P[j] = c * (D.edgeGain ? (double)D.edgeGain[j] : 1.0) * (double)inScale[q];
    Pf[j] = D.counts[j] * (D.edgeGain ? D.edgeGain[j] : 1.f) * inScale[q];
  }
}

__global__ void k_reset(DiffDev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += gridDim.x * blockDim.x) {
    D.v[i] = (float)D.vRest;
    D.gE[i] = D.gI[i] = D.adapt[i] = D.refr[i] = D.spikeCount[i] = 0.f;
    D.res[i] = 1.f;
    D.isForced[i] = 0;
    D.cnt[i] = 0;
    D.ovfHead[i] = kNil;
  }
}

// Delivery of the arrivals at step t (the spikes of step t - (nslots-1)), warp per arrival
// (src/lifdiff.js:276-283): lane 0 forms eff and depresses res; lanes push (rank, edge) per
// gated edge into the target's bucket. resRow (replay) records res[pre] per arrival.
template <typename R>
__global__ void k_deliver(DiffDev D, DP<R> P, int32_t t, float *resRow) {
  const int e = t - (D.nslots - 1);
  if (e < 0) return;
  const int64_t a0 = D.tOff[e], na = D.tOff[e + 1] - a0;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = w0; k < na; k += nw) {
    const int32_t pre = D.tIdx[a0 + k];
    const float sg = D.sign[pre];
    if (lane == 0) {
      R eff = 0;
      if (sg != 0) {
        const R r = D.res[pre];
        if (resRow) resRow[k] = (float)r;
        eff = (R)sg * P.wSyn * d_out<R>(D, pre) * exp((R)D.logGain[pre]) * r * (R)D.tAmp[a0 + k];
        D.res[pre] = (float)(r - P.depU * r);
      }
      D.effK[k] = (double)eff;
    }
    if (sg == 0) continue;
    const uint32_t lo = D.indptr[pre], hi = D.indptr[pre + 1];
    for (uint32_t j = lo + lane; j < hi; j += 32) {
      if (!D.gate[j]) continue;
      const uint32_t q = D.indices[j];
      const uint32_t pos = atomicAdd(D.cnt + q, 1u);
      if (pos < (uint32_t)kDBucket) {
        D.bucket[(int64_t)q * kDBucket + pos] = make_uint2((uint32_t)k, j);
      } else {
        const uint32_t r = atomicAdd(D.ovfTop, 1u);
        if (r >= D.ovfCap) {
          atomicCAS(D.err, 0, FB_EOVERFLOW);
          continue;
        }
        DOvf o;
        o.k = (uint32_t)k;
        o.j = j;
        o.pad = q;
        o.next = atomicExch(D.ovfHead + q, r);
        D.ovf[r] = o;
      }
    }
  }
}

// Forced spikes of step t (src/lifdiff.js:290-297), one block. Forward: one draw per
// non-refractory driven neuron in drivenSet order, compared (in R) against drive * dt/1000; each
// spike goes to the head of step t's tape list. Replay: the tape's forced list.
template <typename R>
__global__ void k_forced(DiffDev D, DP<R> P, int32_t t, int32_t replay) {
  __shared__ uint32_t sJump[32 * 128];
  __shared__ uint32_t scan[33];
  __shared__ uint32_t sh_s0;
  const int tid = threadIdx.x;
  const int64_t base = D.tOff[t];
  if (replay) {
    const int32_t nf = D.tForced[t];
    for (int k = tid; k < nf; k += blockDim.x) {
      const int32_t i = D.tIdx[base + k];
      D.refr[i] = (float)(P.tRef + P.dt);
      D.adapt[i] = (float)((R)D.adapt[i] + P.adaptInc);
      D.isForced[i] = 1;
    }
    return;
  }
  for (int k = tid; k < 32 * 128; k += blockDim.x) sJump[k] = D.jump[k];
  if (tid == 0) sh_s0 = *D.rng;
  __syncthreads();
  const uint32_t s0 = sh_s0;
  uint32_t draws = 0, nf = 0;
  for (int32_t r0 = 0; r0 < D.nDriven; r0 += blockDim.x) {
    const int32_t k = r0 + tid;
    int32_t i = 0;
    uint32_t live = 0;
    float dr = 0.f;
    if (k < D.nDriven) {
      i = D.driven[k];
      live = D.refr[i] > 0 ? 0u : 1u;
      dr = D.drive[i];
    }
    uint32_t nlive;
    const uint32_t dpos = block_exclusive_scan(live, &nlive, scan);
    uint32_t fire = 0;
    if (live) {
      const uint32_t x = xs_jump(sJump, s0, draws + dpos + 1);
      const R u = (R)(x >> 8) * (R)(1.0 / 16777216.0);
      fire = u < (R)dr * P.dtS ? 1u : 0u;
    }
    uint32_t nfire;
    const uint32_t fpos = block_exclusive_scan(fire, &nfire, scan);
    if (fire) {
      const int64_t o = base + nf + fpos;
      if (o < D.tapeCap) {
        D.tIdx[o] = i;
        D.tAmp[o] = 1.f;
      } else {
        atomicCAS(D.err, 0, FB_EOVERFLOW);
      }
      D.refr[i] = (float)(P.tRef + P.dt);
      D.spikeCount[i] = (float)((R)D.spikeCount[i] + R(1));
      D.adapt[i] = (float)((R)D.adapt[i] + P.adaptInc);
      D.isForced[i] = 1;
    }
    draws += nlive;
    nf += nfire;
  }
  if (tid == 0) {
    *D.rng = xs_jump(sJump, s0, draws);
    D.tForced[t] = (int32_t)nf;
  }
}

// Adds target i's bucket in arrival-rank order: gE (or gI) = f32(g + P[j] (*inhGain) * eff) in R.
// Up to kDSortMax contributions are sorted in local memory; beyond that they are applied in
// successive windows of the kDSortMax smallest ranks above the last one applied (ranks are unique
// per target: one contribution per arrival).
template <typename R>
__device__ __forceinline__ void d_add(const DiffDev &D, const DP<R> &Pp, uint2 c, float &geF, float &giF) {
  const R eff = (R)D.effK[c.x];
  const R p = sizeof(R) == 8 ? (R)D.P[c.y] : (R)D.Pf[c.y];
  if (eff > 0) geF = (float)((R)geF + p * eff);
  else giF = (float)((R)giF + p * Pp.inhGain * eff);
}

template <typename R>
__device__ void d_apply(const DiffDev &D, const DP<R> &Pp, int i, uint32_t n, float &geF, float &giF) {
  uint2 e[kDSortMax];
  const uint2 *bk = D.bucket + (int64_t)i * kDBucket;
  const uint32_t nb = n < (uint32_t)kDBucket ? n : (uint32_t)kDBucket;
  bool any = false;
  uint32_t last = 0;
  for (uint32_t done = 0; done < n;) {
    uint32_t m = 0;
    auto offer = [&](uint2 x) {  // keep the kDSortMax smallest ranks above `last`, sorted
      if (any && x.x <= last) return;
      if (m == (uint32_t)kDSortMax && x.x >= e[m - 1].x) return;
      uint32_t w = m < (uint32_t)kDSortMax ? m++ : m - 1;
      while (w > 0 && e[w - 1].x > x.x) {
        e[w] = e[w - 1];
        w--;
      }
      e[w] = x;
    };
    for (uint32_t u = 0; u < nb; u++) offer(bk[u]);
    if (n > (uint32_t)kDBucket)
      for (uint32_t r = D.ovfHead[i], hops = 0; r != kNil && hops < n; hops++) {
        const DOvf o = D.ovf[r];
        offer(make_uint2(o.k, o.j));
        r = o.next;
      }
    if (m == 0) {  // fewer entries than counted: the overflow pool ran out
      atomicCAS(D.err, 0, FB_EOVERFLOW);
      break;
    }
    for (uint32_t u = 0; u < m; u++) d_add<R>(D, Pp, e[u], geF, giF);
    last = e[m - 1].x;
    any = true;
    done += m;
  }
  if (n > (uint32_t)kDBucket) D.ovfHead[i] = kNil;
}

// Integrate and spike (src/lifdiff.js:313-344), one thread per neuron; with `row` >= 0 it also
// records the replay arena (:439-456). Spikes above the tape threshold are staged per tile.
template <typename R>
__global__ void k_update(DiffDev D, DP<R> P, int32_t row) {
  __shared__ uint32_t scan[33];
  const int tid = threadIdx.x, i = blockIdx.x * blockDim.x + tid;
  bool emit = false;
  float amp = 0.f;
  if (i < D.N) {
    float geF = D.gE[i], giF = D.gI[i];
    const uint32_t n = D.cnt[i];
    if (n) {
      d_apply<R>(D, P, i, n, geF, giF);
      D.cnt[i] = 0;
    }
    const R ge = geF, gi = giF;
    const int64_t off = row >= 0 ? (int64_t)row * D.N + i : 0;
    R vi = D.v[i], s = 0;
    int md = 0;
    if (row >= 0) {
      D.aV[off] = D.v[i];
      D.aGE[off] = geF;
      D.aGI[off] = giF;
    }
    float refr = D.refr[i];
    const bool forced = D.isForced[i] != 0;
    if (forced) D.isForced[i] = 0;
    const bool wasRefr = refr > 0;
    if (wasRefr) {
      refr = (float)((R)refr - P.dt);
      vi = P.vReset;
      if (forced) {
        md = 2;
        s = 1;
      } else {
        md = 1;
      }
    } else {
      vi = d_u<R>(D, P, vi, ge, gi, d_bias<R>(D, P, i, nullptr));
    }
    geF = (float)(ge * P.dE);
    giF = (float)(gi * P.dE);
    float ad = (float)((R)D.adapt[i] * P.dA);
    const R rs = D.res[i];
    D.res[i] = (float)(rs + (R(1) - rs) * P.kRec);
    if (row >= 0) D.aAd[off] = ad;
    if (!wasRefr) {
      const R thr = P.vThresh + (R)ad + d_kc<R>(D, P, i) + (R)D.thrOffset[i];
      s = D.soft ? R(1) / (R(1) + exp(-(vi - thr) / d_beta<R>(D, P, i))) : (vi >= thr ? R(1) : R(0));
      if (s > 0) {
        vi = s * P.vReset + (R(1) - s) * vi;
        if (!D.soft) refr = (float)P.tRef;
        ad = (float)((R)ad + s * P.adaptInc);
      }
      D.spikeCount[i] = (float)((R)D.spikeCount[i] + s);
      if (s > (D.soft ? R(1e-4) : R(0.5))) {
        emit = true;
        amp = (float)s;
      }
    }
    if (row >= 0) {
      D.aMode[off] = (uint8_t)md;
      D.aSp[off] = (float)s;
    }
    D.gE[i] = geF;
    D.gI[i] = giF;
    D.adapt[i] = ad;
    D.refr[i] = refr;
    D.v[i] = (float)vi;
  }
  if (row >= 0) return;  // replay: the tape already holds the spikes
  uint32_t tot;
  const uint32_t pos = block_exclusive_scan(emit ? 1u : 0u, &tot, scan);
  if (emit) {
    D.stage[(int64_t)blockIdx.x * blockDim.x + pos] = i;
    D.stageAmp[(int64_t)blockIdx.x * blockDim.x + pos] = amp;
  }
  if (tid == 0) D.tileCnt[blockIdx.x] = (int32_t)tot;
}

// Appends step t's threshold spikes (tile order = ascending) after its forced ones.
__global__ void k_emit(DiffDev D, int32_t t) {
  __shared__ uint32_t scan[33];
  __shared__ int64_t sBase;
  const int tid = threadIdx.x;
  if (tid == 0) sBase = D.tOff[t] + D.tForced[t];
  __syncthreads();
  int64_t carry = sBase;
  for (int t0 = 0; t0 < D.nTiles; t0 += blockDim.x) {
    const int tl = t0 + tid;
    const uint32_t c = tl < D.nTiles ? (uint32_t)D.tileCnt[tl] : 0u;
    uint32_t tot;
    const uint32_t pre = block_exclusive_scan(c, &tot, scan);
    if (c) {
      const int64_t o = carry + pre;
      for (uint32_t p = 0; p < c; p++) {
        if (o + p < D.tapeCap) {
          D.tIdx[o + p] = D.stage[(int64_t)tl * kDB + p];
          D.tAmp[o + p] = D.stageAmp[(int64_t)tl * kDB + p];
        } else {
          atomicCAS(D.err, 0, FB_EOVERFLOW);
        }
      }
    }
    carry += tot;
  }
  if (tid == 0) {
    D.tOff[t + 1] = carry;
    *D.ovfTop = 0;
  }
}

// Reverse of integrate-and-spike at step t (src/lifdiff.js:555-617), with the adjoint clip
// (:623-629) fused: one thread per neuron. Scalar terms accumulate per neuron in double.
template <typename R>
__global__ void k_bneuron(DiffDev D, DP<R> P, int32_t t, int32_t row, int32_t scored) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= D.N) return;
  const int64_t off = (int64_t)row * D.N + i;
  float *ls = D.lsRing + (int64_t)(t % D.nslots) * D.N;
  const int md = D.aMode[off];
  const R lpA = D.lad[i];
  const R lE = (R)D.lgE[i] * P.dE, lI = (R)D.lgI[i] * P.dE, lA = lpA * P.dA;
  const R lR = (R)D.lres[i] * (R(1) - P.kRec);
  float lvF = D.lv[i], lgEF = (float)lE, lgIF = (float)lI, ladF = (float)lA, lresF = (float)lR;
  if (md == 1) {
    lvF = 0.f;
  } else if (md == 2) {
    D.accA[i] += (double)lA;
    lvF = 0.f;
    ls[i] = 0.f;
  } else {
    const R vv = D.aV[off], gEv = D.aGE[off], gIv = D.aGI[off];
    R lam;
    const R bias = d_bias<R>(D, P, i, &lam);
    const R u = d_u<R>(D, P, vv, gEv, gIv, bias);
    const R thr = P.vThresh + (R)D.aAd[off] + d_kc<R>(D, P, i) + (R)D.thrOffset[i];
    const R d = u - thr;
    const R s = D.aSp[off];
    const R beta = d_beta<R>(D, P, i);
    R sg;
    if (D.soft) sg = s * (R(1) - s) / beta;
    else {
      const R tt = R(1) + fabs(d) / beta;
      sg = R(1) / (beta * tt * tt);
    }
    R dl = 0;
    if (scored && D.dL) {
      if (D.roMap) {
        const int c = D.roMap[i];
        if (c >= 0) dl = D.dL[(int64_t)t * D.nro + c];
      } else {
        dl = D.dL[i];
      }
    }
    const R lspike = (R)ls[i] + dl;
    const R lvNew = lvF;
    const R lsTot = (P.vReset - u) * lvNew + lpA * P.adaptInc + lspike;
    const R lt = lsTot * R(1) * sg;
    const R lu = lvNew * (R(1) - s) + lt;
    const R lthr = -lt;
    D.accA[i] += (double)(lpA * s);
    D.accV[i] += (double)lthr;
    if (D.thrMask && D.thrMask[i]) D.accKc[i] += (double)lthr;
    ladF = (float)(lA + lthr * P.dA);
    if (D.coba) {
      lvF = (float)(lu * (R(1) + P.kM * (R(-1) - gEv * P.cE + gIv * P.cI)));
      lgEF = (float)(lE + lu * P.kM * (P.eExc - vv) * P.cE);
      lgIF = (float)(lI + lu * P.kM * (vv - P.eInh) * P.cI);
      D.accEI[i] += (double)(lu * P.kM * gIv * P.cI * (R(-1) + (vv - P.eInh) * P.cI));
    } else {
      lvF = (float)(lu * (R(1) - P.kM));
      lgEF = (float)(lE + lu * P.kM);
      lgIF = (float)(lI + lu * P.kM);
    }
    if (lam != 0) D.accLa[i] += (double)(lu * P.kM);
    D.gBias[i] += (double)(lu * P.kM);
    ls[i] = 0.f;
  }
  const R c = P.adjClip;
  if (c > 0) {
    auto cl = [c](float x) { return (float)((R)x > c ? c : ((R)x < -c ? -c : (R)x)); };
    lvF = cl(lvF); lgEF = cl(lgEF); lgIF = cl(lgIF); ladF = cl(ladF); lresF = cl(lresF);
  }
  D.lv[i] = lvF;
  D.lgE[i] = lgEF;
  D.lgI[i] = lgIF;
  D.lad[i] = ladF;
  D.lres[i] = lresF;
}

// Reverse of the delivery at step t (src/lifdiff.js:635-666), warp per arrival: lanes gather the
// fan-out's adjoint into lRaw (a fixed-order warp sum) and add each gated edge's
// dLoss/dW_j = lg[q] * eff to its accumulator; lane 0 updates the presynaptic neuron's terms.
template <typename R>
__global__ void k_barrival(DiffDev D, DP<R> P, int32_t t, const float *resRow) {
  const int e = t - (D.nslots - 1);
  if (e < 0) return;
  const int64_t a0 = D.tOff[e], na = D.tOff[e + 1] - a0;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float *target = D.lsRing + (int64_t)(e % D.nslots) * D.N;
  for (int64_t k = w0; k < na; k += nw) {
    const int32_t pre = D.tIdx[a0 + k];
    const R sgn = D.sign[pre];
    if (sgn == 0) continue;
    const R amp = D.tAmp[a0 + k];
    const R resAtv = resRow[k];
    const R gain = exp((R)D.logGain[pre]) * d_out<R>(D, pre);
    const R base = sgn * P.wSyn * gain * resAtv;
    const R eff = base * amp;
    const bool exc = eff > 0;
    const uint32_t lo = D.indptr[pre], hi = D.indptr[pre + 1];
    R lraw = 0;
    for (uint32_t j = lo + lane; j < hi; j += 32) {
      if (!D.gate[j]) continue;
      const uint32_t q = D.indices[j];
      const R lg = exc ? (R)D.lgE[q] : (R)D.lgI[q];
      const R cw = (R)D.counts[j] * (D.edgeGain ? (R)D.edgeGain[j] : R(1));
      lraw += exc ? lg * cw * (R)D.inScale[q] : lg * cw * (R)D.inScale[q] * P.inhGain;
      D.gEdge[j] += (double)(lg * eff);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) lraw += __shfl_xor_sync(0xffffffffu, lraw, o);
    if (lane == 0) {
      D.accW[pre] += (double)(lraw * sgn * gain * resAtv * amp);
      D.gLog[pre] += (double)(lraw * eff);
      float x = (float)((R)target[pre] + lraw * base);
      if (P.adjClip > 0) x = (float)fmin(P.adjClip, fmax(-P.adjClip, (R)x));
      target[pre] = x;
      const R lresAfter = D.lres[pre];
      D.accD[pre] += (double)(-lresAfter * resAtv);
      float y = (float)(lresAfter * (R(1) - P.depU) + lraw * sgn * P.wSyn * gain * amp);
      if (P.adjClip > 0) y = (float)fmin(P.adjClip, fmax(-P.adjClip, (R)y));
      D.lres[pre] = y;
    }
  }
}

// Sums the per-neuron accumulators in a fixed order: block partial sums, then one block.
__global__ void k_reduce(const double *const *src, int nsrc, int32_t N, double *partial) {
  __shared__ double sm[8][kDB];
  const int tid = threadIdx.x;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + tid; i < N; i += gridDim.x * blockDim.x)
    for (int k = 0; k < nsrc; k++) acc[k] += src[k][i];
  for (int k = 0; k < nsrc; k++) sm[k][tid] = acc[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s)
      for (int k = 0; k < nsrc; k++) sm[k][tid] += sm[k][tid + s];
    __syncthreads();
  }
  if (tid == 0)
    for (int k = 0; k < nsrc; k++) partial[(int64_t)blockIdx.x * 8 + k] = sm[k][0];
}

// The readout raster of the recorded forward: out[t * nro + c] = amplitude of readout c at t.
__global__ void k_raster(DiffDev D, int32_t steps, float *out) {
  for (int t = blockIdx.x; t < steps; t += gridDim.x) {
    const int64_t a = D.tOff[t], b = D.tOff[t + 1];
    for (int64_t k = a + threadIdx.x; k < b; k += blockDim.x) {
      const int c = D.roMap[D.tIdx[k]];
      if (c >= 0) out[(int64_t)t * D.nro + c] = D.tAmp[k];
    }
  }
}

}  // namespace fb

// =============================================================================================
// C ABI
// =============================================================================================
using namespace fb;

namespace {

int dfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return set_error(code, buf);
}

#define DCU(call)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return dfail(e_ == cudaErrorMemoryAllocation ? FB_ENOMEM : FB_ECUDA, "%s: %s", #call, \
                   cudaGetErrorString(e_));                                                  \
  } while (0)

}  // namespace

struct fb_diff {
  DiffDev D;
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  // inputs kept on the device
  float *sizeLog = nullptr, *inScaleSrc = nullptr;
  uint8_t *sensory = nullptr;
  float *inScale = nullptr;
  uint8_t *gate = nullptr;
  double *P = nullptr;
  float *Pf = nullptr;
  int32_t f32 = 0;  // FB_DIFF_F32 arithmetic
  DP<double> P64;
  DP<float> P32;
  float *ckpt = nullptr;
  uint32_t *ckptRng = nullptr;
  int64_t ckptCap = 0;     // checkpoints allocated
  int32_t recordedSteps = 0, recordedK = 0, tStepsCap = 0;
  uint32_t recordedSeed = 0;
  fb_diff_params lastP;
  int32_t *roMap = nullptr;
  int32_t nroCap = 0;
  float *dLbuf = nullptr;
  int64_t dLcap = 0;
  int64_t hostMaxArr = 0;
  float *resAt = nullptr;
  int64_t resAtCap = 0;
  float *arena = nullptr;  // aV aGE aGI aAd aSp for K rows
  uint8_t *aMode = nullptr;
  int32_t arenaK = 0;
  double *partial = nullptr;
};

template <typename T>
static int dalloc(fb_diff *d, T **p, size_t n) {
  void *q = nullptr;
  DCU(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
  d->allocs.push_back(q);
  *p = (T *)q;
  return FB_OK;
}

template <typename T>
static int dupload(fb_diff *d, T **p, const void *src, size_t n) {
  if (!src) {
    *p = nullptr;
    return FB_OK;
  }
  int rc = dalloc(d, p, n);
  if (rc) return rc;
  DCU(cudaMemcpy(*p, src, n * sizeof(T), cudaMemcpyDefault));
  return FB_OK;
}

extern "C" void fb_diff_default_params(fb_diff_params *p) {
  if (!p) return;
  memset(p, 0, sizeof *p);
  // src/lifdiff.js:86-109
  p->dt = 0.5; p->vRest = -52; p->vThresh = -45; p->vReset = -52; p->tauM = 20; p->tauSyn = 5;
  p->tRef = 2.2; p->delay = 1.8; p->wSyn = 0.3; p->adaptInc = 0; p->adaptTau = 100; p->depU = 0;
  p->depTau = 200; p->minSyn = 1; p->eExc = 0; p->eInh = -70; p->inhGain = 1; p->sizeAlpha = 0;
  p->maxSizeScale = 20; p->boostCap = 1; p->kcThreshold = 0; p->laminaBias = 0;
  p->surrogateBeta = 2.0; p->adjClip = 0; p->coba = 1; p->soft = 0; p->checkpoint = 16;
  p->precision = FB_DIFF_F64;
}

template <typename R>
static DP<R> typed_params(const DiffDev &D) {
  DP<R> q;
  q.dt = (R)D.dt; q.vRest = (R)D.vRest; q.vThresh = (R)D.vThresh; q.vReset = (R)D.vReset;
  q.tRef = (R)D.tRef; q.wSyn = (R)D.wSyn; q.adaptInc = (R)D.adaptInc; q.depU = (R)D.depU;
  q.eExc = (R)D.eExc; q.eInh = (R)D.eInh; q.inhGain = (R)D.inhGain; q.kcThreshold = (R)D.kcThreshold;
  q.laminaBias = (R)D.laminaBias; q.beta = (R)D.beta; q.adjClip = (R)D.adjClip; q.dE = (R)D.dE;
  q.dA = (R)D.dA; q.kRec = (R)D.kRec; q.kM = (R)D.kM; q.dtS = (R)D.dtS; q.cE = (R)D.cE; q.cI = (R)D.cI;
  return q;
}

extern "C" int fb_diff_create(const fb_diff_net *net, int64_t tape_cap, fb_diff **out) {
  if (!net || !out) return dfail(FB_EINVAL, "fb_diff_create: null argument");
  *out = nullptr;
  if (net->N <= 0 || net->E < 0 || !net->indptr || (net->E && (!net->indices || !net->counts)) || !net->sign ||
      net->nDriven < 0 || net->nDriven > net->N || (net->nDriven && (!net->driven || !net->drive)))
    return dfail(FB_EINVAL, "fb_diff_create: bad network description (N=%d E=%lld nDriven=%d)", net->N,
                 (long long)net->E, net->nDriven);
  fb_diff *d = new fb_diff;
  memset(&d->D, 0, sizeof d->D);
  DiffDev &D = d->D;
  const int64_t N = net->N, E = net->E;
  D.N = net->N;
  D.E = net->E;
  D.nDriven = net->nDriven;
  int rc = 0;
  auto up_u32 = [&](const uint32_t **dst, const uint32_t *src, size_t n) {
    uint32_t *p;
    int r = dupload(d, &p, src, n);
    *dst = p;
    return r;
  };
  auto up_f = [&](const float **dst, const float *src, size_t n) {
    float *p;
    int r = dupload(d, &p, src, n);
    *dst = p;
    return r;
  };
  auto up_u8 = [&](const uint8_t **dst, const uint8_t *src, size_t n) {
    uint8_t *p;
    int r = dupload(d, &p, src, n);
    *dst = p;
    return r;
  };
  if ((rc = up_u32(&D.indptr, net->indptr, N + 1)) || (rc = up_u32(&D.indices, net->indices, E)) ||
      (rc = up_f(&D.counts, net->counts, E)) || (rc = up_f(&D.edgeGain, net->edge_gain, E)) ||
      (rc = up_f(&D.sign, net->sign, N)) || (rc = up_f(&D.outScale, net->out_scale, N)) ||
      (rc = up_f(&D.betaArr, net->beta, N)) || (rc = up_f(&D.biasArr, net->bias, N)) ||
      (rc = up_u8(&D.thrMask, net->thr_mask, N)) || (rc = up_u8(&D.biasMask, net->bias_mask, N))) {
    fb_diff_destroy(d);
    return rc;
  }
  {
    float *p;
    std::vector<float> z(N, 0.f);
    if ((rc = dupload(d, &p, net->log_gain ? (const void *)net->log_gain : z.data(), N))) { fb_diff_destroy(d); return rc; }
    D.logGain = p;
    if ((rc = dupload(d, &p, net->thr_offset ? (const void *)net->thr_offset : z.data(), N))) { fb_diff_destroy(d); return rc; }
    D.thrOffset = p;
    if ((rc = dupload(d, &d->sizeLog, net->size_log ? (const void *)net->size_log : z.data(), N))) { fb_diff_destroy(d); return rc; }
    if ((rc = dupload(d, &d->inScaleSrc, net->in_scale, N)) || (rc = dupload(d, &d->sensory, net->sensory, N))) {
      fb_diff_destroy(d);
      return rc;
    }
    std::vector<float> dr(N, 0.f);
    std::vector<int32_t> dv(net->nDriven);
    if (net->nDriven) {
      std::vector<int32_t> hv(net->nDriven);
      std::vector<float> hd(N);
      if (cudaMemcpy(hv.data(), net->driven, 4 * net->nDriven, cudaMemcpyDefault) != cudaSuccess ||
          cudaMemcpy(hd.data(), net->drive, 4 * N, cudaMemcpyDefault) != cudaSuccess) {
        fb_diff_destroy(d);
        return dfail(FB_ECUDA, "fb_diff_create: reading the drive failed");
      }
      for (int32_t k = 0; k < net->nDriven; k++) {
        if (hv[k] < 0 || hv[k] >= N) { fb_diff_destroy(d); return dfail(FB_EINVAL, "fb_diff_create: driven[%d]=%d", k, hv[k]); }
        dv[k] = hv[k];
      }
      dr = hd;
    }
    if ((rc = dupload(d, &p, dr.data(), N))) { fb_diff_destroy(d); return rc; }
    D.drive = p;
    int32_t *q;
    if ((rc = dupload(d, &q, dv.data(), std::max<int32_t>(net->nDriven, 1)))) { fb_diff_destroy(d); return rc; }
    D.driven = q;
  }
  // derived arrays, state, scratch, tape, adjoint state
  D.nTiles = (int32_t)((N + kDB - 1) / kDB);
  int32_t *i32;
  float *f;
  if ((rc = dalloc(d, &d->inScale, N)) || (rc = dalloc(d, &d->gate, E)) || (rc = dalloc(d, &d->P, E)) ||
      (rc = dalloc(d, &d->Pf, E)) ||
      (rc = dalloc(d, &D.v, N)) || (rc = dalloc(d, &D.gE, N)) || (rc = dalloc(d, &D.gI, N)) ||
      (rc = dalloc(d, &D.adapt, N)) || (rc = dalloc(d, &D.res, N)) || (rc = dalloc(d, &D.refr, N)) ||
      (rc = dalloc(d, &D.spikeCount, N)) || (rc = dalloc(d, &D.isForced, N)) || (rc = dalloc(d, &D.rng, 1)) ||
      (rc = dalloc(d, &D.cnt, N)) || (rc = dalloc(d, &D.bucket, N * kDBucket)) || (rc = dalloc(d, &D.ovfHead, N)) ||
      (rc = dalloc(d, &D.ovfTop, 1)) || (rc = dalloc(d, &D.effK, N)) ||
      (rc = dalloc(d, &D.stage, (size_t)D.nTiles * kDB)) || (rc = dalloc(d, &D.stageAmp, (size_t)D.nTiles * kDB)) ||
      (rc = dalloc(d, &D.tileCnt, D.nTiles)) || (rc = dalloc(d, &D.err, 1)) ||
      (rc = dalloc(d, &D.lv, N)) || (rc = dalloc(d, &D.lgE, N)) || (rc = dalloc(d, &D.lgI, N)) ||
      (rc = dalloc(d, &D.lad, N)) || (rc = dalloc(d, &D.lres, N)) ||
      (rc = dalloc(d, &D.accA, N)) || (rc = dalloc(d, &D.accV, N)) || (rc = dalloc(d, &D.accKc, N)) ||
      (rc = dalloc(d, &D.accLa, N)) || (rc = dalloc(d, &D.accEI, N)) || (rc = dalloc(d, &D.accW, N)) ||
      (rc = dalloc(d, &D.accD, N)) || (rc = dalloc(d, &D.gLog, N)) || (rc = dalloc(d, &D.gBias, N)) ||
      (rc = dalloc(d, &D.gEdge, E)) || (rc = dalloc(d, &d->partial, 8 * 256))) {
    fb_diff_destroy(d);
    return rc;
  }
  D.inScale = d->inScale;
  D.gate = d->gate;
  D.P = d->P;
  D.Pf = d->Pf;
  D.ovfCap = (uint32_t)std::min<int64_t>((1 << 20) + E / 8, 0x7fffffff);
  DOvf *ov;
  if ((rc = dalloc(d, &ov, D.ovfCap))) { fb_diff_destroy(d); return rc; }
  D.ovf = ov;
  D.tapeCap = tape_cap > 0 ? tape_cap : std::max<int64_t>(1 << 20, 64 * N);
  if ((rc = dalloc(d, &i32, D.tapeCap)) || (rc = dalloc(d, &f, D.tapeCap))) { fb_diff_destroy(d); return rc; }
  D.tIdx = i32;
  D.tAmp = f;
  std::vector<uint32_t> tab;
  host_jump_tables(tab);
  uint32_t *jt;
  if ((rc = dupload(d, &jt, tab.data(), tab.size()))) { fb_diff_destroy(d); return rc; }
  D.jump = jt;
  cudaMemset(D.err, 0, 4);
  cudaMemset(D.ovfTop, 0, 4);
  if (cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking) != cudaSuccess) {
    fb_diff_destroy(d);
    return dfail(FB_ECUDA, "fb_diff_create: stream creation failed");
  }
  *out = d;
  return FB_OK;
}

extern "C" int fb_diff_destroy(fb_diff *d) {
  if (!d) return FB_OK;
  if (d->st) cudaStreamSynchronize(d->st);
  for (void *p : d->allocs) cudaFree(p);
  if (d->st) cudaStreamDestroy(d->st);
  delete d;
  return FB_OK;
}

extern "C" int fb_diff_set(fb_diff *d, int32_t field, const float *values) {
  if (!d || !values) return dfail(FB_EINVAL, "fb_diff_set: null argument");
  const float *dst;
  size_t n = (size_t)d->D.N;
  switch (field) {
    case FB_DIFF_LOG_GAIN: dst = d->D.logGain; break;
    case FB_DIFF_OUT_SCALE: dst = d->D.outScale; break;
    case FB_DIFF_THR_OFFSET: dst = d->D.thrOffset; break;
    case FB_DIFF_BIAS: dst = d->D.biasArr; break;
    case FB_DIFF_EDGE_GAIN: dst = d->D.edgeGain; n = (size_t)d->D.E; break;
    case FB_DIFF_DRIVE: dst = d->D.drive; break;
    default: return dfail(FB_EINVAL, "fb_diff_set: unknown field %d", field);
  }
  if (!dst) return dfail(FB_ESTATE, "fb_diff_set: field %d was not given at creation", field);
  DCU(cudaMemcpyAsync((void *)dst, values, n * 4, cudaMemcpyDefault, d->st));
  DCU(cudaStreamSynchronize(d->st));
  return FB_OK;
}

static int fill_params(fb_diff *d, const fb_diff_params *p) {
  DiffDev &D = d->D;
  if (!(p->dt > 0) || !(p->tauM > 0) || !(p->tauSyn > 0) || p->checkpoint <= 0)
    return dfail(FB_EINVAL, "fb_diff: dt, tauM, tauSyn and checkpoint must be positive");
  if (p->precision != FB_DIFF_F64 && p->precision != FB_DIFF_F32)
    return dfail(FB_EINVAL, "fb_diff: precision must be FB_DIFF_F64 or FB_DIFF_F32 (got %d)", p->precision);
  D.nslots = (int32_t)std::max(1.0, std::floor(p->delay / p->dt + 0.5)) + 1;
  D.K = p->checkpoint;
  D.coba = p->coba ? 1 : 0;
  D.soft = p->soft ? 1 : 0;
  D.dt = p->dt; D.vRest = p->vRest; D.vThresh = p->vThresh; D.vReset = p->vReset; D.tRef = p->tRef;
  D.wSyn = p->wSyn; D.adaptInc = p->adaptInc; D.depU = p->depU; D.eExc = p->eExc; D.eInh = p->eInh;
  D.inhGain = p->inhGain; D.kcThreshold = p->kcThreshold; D.laminaBias = p->laminaBias;
  D.beta = p->surrogateBeta; D.adjClip = p->adjClip;
  D.dE = std::exp(-p->dt / p->tauSyn);
  D.dA = std::exp(-p->dt / p->adaptTau);
  D.kRec = p->dt / p->depTau;
  D.kM = p->dt / p->tauM;
  D.dtS = p->dt / 1000;
  D.cE = 1 / (p->eExc - p->vRest);
  D.cI = 1 / (p->vRest - p->eInh);
  d->f32 = p->precision == FB_DIFF_F32;
  d->P64 = typed_params<double>(D);
  d->P32 = typed_params<float>(D);
  d->lastP = *p;
  return FB_OK;
}

static int prepare(fb_diff *d, const fb_diff_params *p) {
  DiffDev &D = d->D;
  k_prepare<<<256, kDB, 0, d->st>>>(D, d->inScale, d->gate, d->P, d->sizeLog, d->inScaleSrc, d->sensory,
                                     p->sizeAlpha, p->maxSizeScale, p->boostCap, p->minSyn);
  k_prepare_edges<<<1024, kDB, 0, d->st>>>(D, d->inScale, d->gate, d->P, d->Pf, d->sensory, p->minSyn);
  DCU(cudaGetLastError());
  return FB_OK;
}

static int check_err(fb_diff *d, const char *fn) {
  int32_t err = 0;
  DCU(cudaMemcpyAsync(&err, d->D.err, 4, cudaMemcpyDeviceToHost, d->st));
  DCU(cudaStreamSynchronize(d->st));
  if (err) {
    cudaMemset(d->D.err, 0, 4);
    return dfail(err, "%s: %s", fn, err == FB_EOVERFLOW ? "tape or delivery scratch overflow" : "device error");
  }
  return FB_OK;
}

template <typename R>
static void run_step_t(fb_diff *d, const DP<R> &P, int32_t t, int32_t replay, int32_t row, float *resRow) {
  DiffDev &D = d->D;
  const int nb = (int)((D.N + kDB - 1) / kDB);
  k_deliver<R><<<304, kDB, 0, d->st>>>(D, P, t, resRow);
  k_forced<R><<<1, 512, 0, d->st>>>(D, P, t, replay);
  k_update<R><<<nb, kDB, 0, d->st>>>(D, P, row);
  if (!replay) k_emit<<<1, 512, 0, d->st>>>(D, t);
  else cudaMemsetAsync(D.ovfTop, 0, 4, d->st);
}

static void run_step(fb_diff *d, int32_t t, int32_t replay, int32_t row, float *resRow) {
  if (d->f32) run_step_t<float>(d, d->P32, t, replay, row, resRow);
  else run_step_t<double>(d, d->P64, t, replay, row, resRow);
}

static void reverse_step(fb_diff *d, int32_t t, int32_t row, int32_t scored, const float *resRow) {
  DiffDev &D = d->D;
  const int nblk = (int)((D.N + kDB - 1) / kDB);
  if (d->f32) {
    k_bneuron<float><<<nblk, kDB, 0, d->st>>>(D, d->P32, t, row, scored);
    k_barrival<float><<<304, kDB, 0, d->st>>>(D, d->P32, t, resRow);
  } else {
    k_bneuron<double><<<nblk, kDB, 0, d->st>>>(D, d->P64, t, row, scored);
    k_barrival<double><<<304, kDB, 0, d->st>>>(D, d->P64, t, resRow);
  }
}

extern "C" int fb_diff_forward(fb_diff *d, const fb_diff_params *p, int32_t steps, uint32_t seed,
                               int32_t record, float *spike_count) {
  if (!d || !p || steps < 0) return dfail(FB_EINVAL, "fb_diff_forward: bad arguments");
  int rc = fill_params(d, p);
  if (rc) return rc;
  DiffDev &D = d->D;
  const int64_t N = D.N;
  if (record) {
    const int64_t nck = (steps + D.K - 1) / D.K;
    if (nck > d->ckptCap) {
      void *q = nullptr, *r = nullptr;
      if (cudaMalloc(&q, (size_t)std::max<int64_t>(nck, 1) * 6 * N * 4) != cudaSuccess ||
          cudaMalloc(&r, (size_t)std::max<int64_t>(nck, 1) * 4) != cudaSuccess) {
        cudaFree(q);
        return dfail(FB_ENOMEM, "fb_diff_forward: %lld checkpoints of %lld neurons", (long long)nck, (long long)N);
      }
      d->allocs.push_back(q);
      d->allocs.push_back(r);
      d->ckpt = (float *)q;
      d->ckptRng = (uint32_t *)r;
      d->ckptCap = nck;
    }
  }
  if (steps > d->tStepsCap || !D.tOff) {  // per-step tape offsets and forced counts
    int64_t *o;
    int32_t *fz;
    if ((rc = dalloc(d, &o, (size_t)steps + 1)) || (rc = dalloc(d, &fz, (size_t)std::max(steps, 1)))) return rc;
    D.tOff = o;
    D.tForced = fz;
    d->tStepsCap = steps;
  }
  if ((rc = prepare(d, p))) return rc;
  k_reset<<<256, kDB, 0, d->st>>>(D);
  // (seed * 2654435761) >>> 0 || 1, the product in double (src/lifdiff.js:221)
  uint32_t s0 = (uint32_t)std::fmod(std::floor((double)seed * 2654435761.0), 4294967296.0);
  if (!s0) s0 = 1;
  DCU(cudaMemcpyAsync(D.rng, &s0, 4, cudaMemcpyHostToDevice, d->st));
  DCU(cudaMemsetAsync(D.tOff, 0, 8, d->st));
  DCU(cudaMemsetAsync(D.ovfTop, 0, 4, d->st));
  const size_t nb = (size_t)N * 4;
  for (int32_t t = 0; t < steps; t++) {
    if (record && t % D.K == 0) {
      float *c = d->ckpt + (int64_t)(t / D.K) * 6 * N;
      cudaMemcpyAsync(c, D.v, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(c + N, D.gE, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(c + 2 * N, D.gI, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(c + 3 * N, D.adapt, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(c + 4 * N, D.res, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(c + 5 * N, D.refr, nb, cudaMemcpyDeviceToDevice, d->st);
      cudaMemcpyAsync(d->ckptRng + t / D.K, D.rng, 4, cudaMemcpyDeviceToDevice, d->st);
    }
    run_step(d, t, 0, -1, nullptr);
  }
  DCU(cudaGetLastError());
  if ((rc = check_err(d, "fb_diff_forward"))) return rc;
  if (spike_count) DCU(cudaMemcpy(spike_count, D.spikeCount, nb, cudaMemcpyDefault));
  if (record) {
    d->recordedSteps = steps;
    d->recordedK = D.K;
    d->recordedSeed = seed;
  } else {
    d->recordedSteps = 0;
  }
  return FB_OK;
}

extern "C" int fb_diff_tape(fb_diff *d, int64_t *offsets, int32_t *idx, float *amp, int64_t cap, int64_t *len) {
  if (!d || !d->recordedSteps) return dfail(FB_ESTATE, "fb_diff_tape: no recorded forward pass");
  const int32_t steps = d->recordedSteps;
  std::vector<int64_t> off(steps + 1);
  DCU(cudaMemcpy(off.data(), d->D.tOff, (steps + 1) * 8, cudaMemcpyDeviceToHost));
  if (len) *len = off[steps];
  if (offsets) memcpy(offsets, off.data(), (steps + 1) * 8);
  const int64_t n = std::min<int64_t>(cap, off[steps]);
  if (idx && n > 0) DCU(cudaMemcpy(idx, d->D.tIdx, n * 4, cudaMemcpyDefault));
  if (amp && n > 0) DCU(cudaMemcpy(amp, d->D.tAmp, n * 4, cudaMemcpyDefault));
  return FB_OK;
}

static int set_readout(fb_diff *d, int32_t nro, const int32_t *ro) {
  DiffDev &D = d->D;
  if (!d->roMap) {
    int rc = dalloc(d, &d->roMap, D.N);
    if (rc) return rc;
  }
  std::vector<int32_t> map(D.N, -1), h(nro);
  if (nro) DCU(cudaMemcpy(h.data(), ro, nro * 4, cudaMemcpyDefault));
  for (int32_t c = 0; c < nro; c++) {
    if (h[c] < 0 || h[c] >= D.N) return dfail(FB_EINVAL, "readout[%d]=%d out of range", c, h[c]);
    map[h[c]] = c;
  }
  DCU(cudaMemcpy(d->roMap, map.data(), D.N * 4, cudaMemcpyHostToDevice));
  D.nro = nro;
  return FB_OK;
}

extern "C" int fb_diff_raster(fb_diff *d, int32_t nro, const int32_t *readout, float *out) {
  if (!d || nro <= 0 || !readout || !out) return dfail(FB_EINVAL, "fb_diff_raster: bad arguments");
  if (!d->recordedSteps) return dfail(FB_ESTATE, "fb_diff_raster: no recorded forward pass");
  int rc = set_readout(d, nro, readout);
  if (rc) return rc;
  const int32_t steps = d->recordedSteps;
  float *dev = nullptr;
  cudaPointerAttributes at;
  const bool onDev = cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  if (onDev) dev = out;
  else DCU(cudaMalloc(&dev, (size_t)steps * nro * 4));
  DCU(cudaMemsetAsync(dev, 0, (size_t)steps * nro * 4, d->st));
  d->D.roMap = d->roMap;
  k_raster<<<std::min(steps, 4096), 256, 0, d->st>>>(d->D, steps, dev);
  DCU(cudaGetLastError());
  DCU(cudaStreamSynchronize(d->st));
  if (!onDev) {
    DCU(cudaMemcpy(out, dev, (size_t)steps * nro * 4, cudaMemcpyDeviceToHost));
    cudaFree(dev);
  }
  return FB_OK;
}

extern "C" int fb_diff_backward(fb_diff *d, const float *dL, int32_t nro, const int32_t *readout,
                                int32_t truncate, int32_t loss_from, fb_diff_grads *g) {
  if (!d || !dL || !g) return dfail(FB_EINVAL, "fb_diff_backward: null argument");
  if (!d->recordedSteps) return dfail(FB_ESTATE, "fb_diff_backward: no recorded forward pass (record=1)");
  DiffDev &D = d->D;
  const int32_t steps = d->recordedSteps, K = d->recordedK;
  const int64_t N = D.N, E = D.E;
  int rc = fill_params(d, &d->lastP);
  if (rc) return rc;
  // the loss gradient: flat over N, or per step over a readout set
  const int64_t dLn = nro > 0 ? (int64_t)steps * nro : N;
  if (dLn > d->dLcap) {
    float *q;
    if ((rc = dalloc(d, &q, dLn))) return rc;
    d->dLbuf = q;
    d->dLcap = dLn;
  }
  DCU(cudaMemcpyAsync(d->dLbuf, dL, dLn * 4, cudaMemcpyDefault, d->st));
  D.dL = d->dLbuf;
  if (nro > 0) {
    if (!readout) return dfail(FB_EINVAL, "fb_diff_backward: readout indices missing");
    if ((rc = set_readout(d, nro, readout))) return rc;
    D.roMap = d->roMap;
  } else {
    D.roMap = nullptr;
  }
  // arena and per-arrival res for one segment
  std::vector<int64_t> off(steps + 1);
  DCU(cudaMemcpy(off.data(), D.tOff, (steps + 1) * 8, cudaMemcpyDeviceToHost));
  int64_t maxArr = 1;
  for (int32_t t = 0; t < steps; t++) {
    const int e = t - (D.nslots - 1);
    if (e >= 0) maxArr = std::max<int64_t>(maxArr, off[e + 1] - off[e]);
  }
  if (K > d->arenaK) {
    float *a;
    uint8_t *m;
    if ((rc = dalloc(d, &a, (size_t)5 * K * N)) || (rc = dalloc(d, &m, (size_t)K * N))) return rc;
    d->arena = a;
    d->aMode = m;
    d->arenaK = K;
  }
  if (maxArr * K > d->resAtCap) {
    float *r;
    if ((rc = dalloc(d, &r, maxArr * K))) return rc;
    d->resAt = r;
    d->resAtCap = maxArr * K;
  }
  D.aV = d->arena;
  D.aGE = d->arena + (size_t)K * N;
  D.aGI = d->arena + (size_t)2 * K * N;
  D.aAd = d->arena + (size_t)3 * K * N;
  D.aSp = d->arena + (size_t)4 * K * N;
  D.aMode = d->aMode;
  D.resAt = d->resAt;
  D.maxArr = maxArr;
  // zero the adjoint state and accumulators
  for (float *p : {D.lv, D.lgE, D.lgI, D.lad, D.lres}) DCU(cudaMemsetAsync(p, 0, N * 4, d->st));
  for (double *p : {D.accA, D.accV, D.accKc, D.accLa, D.accEI, D.accW, D.accD, D.gLog, D.gBias})
    DCU(cudaMemsetAsync(p, 0, N * 8, d->st));
  DCU(cudaMemsetAsync(D.gEdge, 0, std::max<int64_t>(E, 1) * 8, d->st));
  float *lsRing;
  if (!D.lsRing) {
    if ((rc = dalloc(d, &lsRing, (size_t)D.nslots * N))) return rc;
    D.lsRing = lsRing;
  }
  DCU(cudaMemsetAsync(D.lsRing, 0, (size_t)D.nslots * N * 4, d->st));
  if ((rc = prepare(d, &d->lastP))) return rc;
  const size_t nb = (size_t)N * 4;
  const int nseg = (steps + K - 1) / K;
  for (int b = nseg - 1; b >= 0; b--) {
    const int32_t from = b * K, to = std::min(steps, from + K);
    // replay the segment from its checkpoint (src/lifdiff.js:390-464)
    const float *c = d->ckpt + (int64_t)b * 6 * N;
    cudaMemcpyAsync(D.v, c, nb, cudaMemcpyDeviceToDevice, d->st);
    cudaMemcpyAsync(D.gE, c + N, nb, cudaMemcpyDeviceToDevice, d->st);
    cudaMemcpyAsync(D.gI, c + 2 * N, nb, cudaMemcpyDeviceToDevice, d->st);
    cudaMemcpyAsync(D.adapt, c + 3 * N, nb, cudaMemcpyDeviceToDevice, d->st);
    cudaMemcpyAsync(D.res, c + 4 * N, nb, cudaMemcpyDeviceToDevice, d->st);
    cudaMemcpyAsync(D.refr, c + 5 * N, nb, cudaMemcpyDeviceToDevice, d->st);
    for (int32_t t = from; t < to; t++) run_step(d, t, 1, t - from, D.resAt + (int64_t)(t - from) * maxArr);
    // reverse sweep of the segment (src/lifdiff.js:540-667)
    for (int32_t t = to - 1; t >= from; t--) {
      if (truncate > 0 && (t + 1) % truncate == 0) {
        for (float *p : {D.lv, D.lgE, D.lgI, D.lad, D.lres}) cudaMemsetAsync(p, 0, nb, d->st);
        cudaMemsetAsync(D.lsRing, 0, (size_t)D.nslots * nb, d->st);
      }
      reverse_step(d, t, t - from, t >= loss_from ? 1 : 0, D.resAt + (int64_t)(t - from) * maxArr);
    }
  }
  DCU(cudaGetLastError());
  if ((rc = check_err(d, "fb_diff_backward"))) return rc;
  // fixed-order reductions of the scalar accumulators
  const double *srcs[7] = {D.accW, D.accEI, D.accV, D.accKc, D.accLa, D.accA, D.accD};
  const double **dsrc;
  DCU(cudaMalloc(&dsrc, sizeof srcs));
  DCU(cudaMemcpy(dsrc, srcs, sizeof srcs, cudaMemcpyHostToDevice));
  k_reduce<<<256, kDB, 0, d->st>>>(dsrc, 7, D.N, d->partial);
  std::vector<double> part(256 * 8);
  DCU(cudaMemcpyAsync(part.data(), d->partial, part.size() * 8, cudaMemcpyDeviceToHost, d->st));
  DCU(cudaStreamSynchronize(d->st));
  cudaFree(dsrc);
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int blk = 0; blk < 256; blk++)
    for (int k = 0; k < 7; k++) s[k] += part[blk * 8 + k];
  // per-edge gradient -> gInScale per target and the inhibitory-gain term, on the host in
  // edge order (the reference accumulates them per arrival, src/lifdiff.js:650-655)
  std::vector<double> gEdge(E), gIS(N, 0.0);
  std::vector<float> counts(E), eg(D.edgeGain ? E : 0), sign(N), inS(N), sizeLog(N), lg(N), outs(N);
  std::vector<uint32_t> ip(N + 1), ix(E);
  std::vector<uint8_t> gate(E);
  DCU(cudaMemcpy(gEdge.data(), D.gEdge, E * 8, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(counts.data(), D.counts, E * 4, cudaMemcpyDeviceToHost));
  if (D.edgeGain) DCU(cudaMemcpy(eg.data(), D.edgeGain, E * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(sign.data(), D.sign, N * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(inS.data(), D.inScale, N * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(sizeLog.data(), d->sizeLog, N * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(ip.data(), D.indptr, (N + 1) * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(ix.data(), D.indices, E * 4, cudaMemcpyDeviceToHost));
  DCU(cudaMemcpy(gate.data(), D.gate, E, cudaMemcpyDeviceToHost));
  double gInh = 0;
  const fb_diff_params &P = d->lastP;
  for (int64_t j0 = 0; j0 < N; j0++) {
    const bool inh = sign[j0] < 0;  // eff's sign follows the presynaptic sign (wSyn, gains > 0)
    for (uint32_t j = ip[j0]; j < ip[j0 + 1]; j++) {
      if (!gate[j]) continue;
      const double cw = (double)counts[j] * (D.edgeGain ? (double)eg[j] : 1.0);
      gIS[ix[j]] += cw * (inh ? P.inhGain : 1.0) * gEdge[j];
      if (inh) gInh += cw * (double)inS[ix[j]] * gEdge[j];
    }
  }
  double gSize = 0;
  for (int64_t i = 0; i < N; i++) {
    const double raw = std::exp(-P.sizeAlpha * (double)sizeLog[i]);
    if (raw < P.boostCap && raw > 1 / P.maxSizeScale) gSize += gIS[i] * (-(double)sizeLog[i]) * raw;
  }
  // src/lifdiff.js:75 order: wSyn sizeAlpha inhGain eInh vThresh kcThreshold laminaBias adaptInc depU
  double vals[9] = {s[0], gSize, gInh, s[1], s[2], s[3], s[4], s[5], s[6]};
  g->clamped_params = g->clamped_log_gain = 0;
  for (int k = 0; k < 9; k++) {
    if (!std::isfinite(vals[k])) { vals[k] = 0; g->clamped_params++; }
    g->params[k] = vals[k];
  }
  std::vector<double> glog(N);
  DCU(cudaMemcpy(glog.data(), D.gLog, N * 8, cudaMemcpyDeviceToHost));
  if (g->log_gain || g->out_scale) {
    std::vector<float> os(N, 1.f);
    if (D.outScale) DCU(cudaMemcpy(os.data(), D.outScale, N * 4, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < N; i++) {
      float x = (float)glog[i];
      if (!std::isfinite(x)) { x = 0; g->clamped_log_gain++; }
      if (g->log_gain) g->log_gain[i] = x;
      if (g->out_scale) g->out_scale[i] = (double)x / (double)os[i];
    }
  }
  if (g->edge) memcpy(g->edge, gEdge.data(), E * 8);
  if (g->bias) DCU(cudaMemcpy(g->bias, D.gBias, N * 8, cudaMemcpyDefault));
  return FB_OK;
}
