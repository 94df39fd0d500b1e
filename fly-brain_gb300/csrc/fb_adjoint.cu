// The differentiable brain step and its adjoint on sm_103a: the reference's LIFDiff
// (src/lifdiff.js:219-686), for a batch of independent instances (each its own network, drive,
// seed and length; one parameter set) advanced together: every kernel runs the whole batch, the
// instance in blockIdx.y. Forward with a spike tape and state checkpoints every K steps; backward
// replays one segment from its checkpoint (forced spikes from the tape, so the RNG is never
// redrawn), then sweeps the segment's steps in reverse. A single network is a batch of one.
//
// Arithmetic is LIFDiff's in FB_DIFF_F64 mode: every intermediate in double, every state word
// float32, operands in the JS order; per-target conductance sums run in the reference's arrival
// order (each contribution is pushed with its arrival rank into a per-target bucket and summed in
// rank order). FB_DIFF_F32 evaluates the same expressions with float intermediates.
// The backward accumulates without float atomics: within one step every edge and every
// presynaptic neuron is touched by one arrival at most, so per-edge and per-neuron accumulators
// have a single writer per step and are summed in time order; scalars are reduced in a fixed order.
//
// Inputs beyond the network: a drive schedule (driveIdx/driveEpoch, src/lifdiff.js:134-144) whose
// values are set at every epoch boundary with setDriveOne semantics -- the drivenSet keeps
// insertion order, so the host derives each boundary's edits (members removed, members appended)
// and a one-block kernel applies them to the live list the draws walk; driveSoft (:338), the
// drive's expected spike instead of a draw; a recorded spike train (:298-306) forced like driven
// spikes; and exact32 (:172-190, :256-275, :317-326), a forward in lif.c's f32 arithmetic with the
// two weight arrays writeGraph bakes.
#include <cuda_runtime.h>

#include <climits>
#include <cstddef>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "fb_internal.cuh"

namespace fb {
int set_error(int code, const char *msg);
void host_jump_tables(std::vector<uint32_t> &tab);

constexpr int kDB = 256;      // threads per block of the per-neuron kernels
constexpr int kDBucket = 8;   // bucket slots per target and step
constexpr int kDSortMax = 64; // contributions per target sorted in local memory
constexpr int kRB = 128;      // blocks per instance of the final reduction
constexpr int kNSums = 9;     // scalar sums per instance
constexpr int32_t kClaimFree = 0x7f7f7f7f;  // spike-train claim slots between steps
constexpr double kDriveMax = 0.999;         // a soft drive's largest expected spike (src/lifdiff.js:72)

struct DOvf {
  uint32_t k, j, next, pad;
};

// One instance as the kernels see it: sizes, graph, derived arrays, state, tape, scratch,
// adjoint state and accumulators. Kernels copy their instance's record into shared memory.
struct DiffDev {
  int32_t N, nslots, K, coba, soft, nDriven, nro, nTiles;
  int32_t steps;   // length of the current forward; the instance sits out steps t >= steps
  uint32_t seed0;  // xorshift state after seeding
  int32_t driveSoft, exact32;
  int32_t nDS, driveEpoch;  // schedule columns (0: no schedule) and steps per epoch
  int64_t E;
  // graph and per-neuron structure
  const uint32_t *indptr, *indices;
  const uint32_t *cscPtr, *cscEdge, *cscSrc;  // in-edges of each target, ascending edge id
  const float *counts, *edgeGain, *sign, *logGain, *outScale, *thrOffset, *betaArr, *biasArr, *sizeLog;
  const uint8_t *thrMask, *biasMask;
  const float *drive;     // the drive as set (Hz)
  const int32_t *driven;  // the drivenSet at reset, in insertion order
  // the drive schedule: neuron -> schedule column (-1: none), the values [epochs][nDS], the live
  // drivenSet, and per epoch the edits that keep it in insertion order ([removed | appended])
  const int32_t *dSlot;
  const float *driveAt;
  int32_t *drivenLive, *nLive;
  const int32_t *epOff, *epList;
  uint8_t *rmFlag;
  // a recorded spike train: step t forces trainIdx[trainOff[t] .. trainOff[t+1]); claim[i] picks
  // the first listing of a neuron within a step
  const int64_t *trainOff;
  const int32_t *trainIdx;
  int32_t *claim;
  // exact32: W32[j] = f32(count * edgeGain * inScale * inhibitory gain * outScale) (0 if gated
  // off) and signW32[i] = f32(sign * wSyn), lif.c's two weight arrays (src/lifdiff.js:177-189)
  float *W32, *signW32;
  // derived per forward: inScale, gate, P[j] = (count * edgeGain) * inScale[q] (double, float)
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
  // checkpoints: v gE gI adapt res refr every K steps, and the RNG state
  float *ckpt;
  uint32_t *ckptRng;
  // delivery scratch
  uint32_t *cnt;
  uint2 *bucket;
  uint32_t *ovfHead, *ovfTop;
  DOvf *ovf;
  double *effK;  // per arrival of the step
  // spike staging per tile
  int32_t *stage;
  float *stageAmp;
  int32_t *tileCnt;
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
  float *gLogF;  // log-gain gradient as returned (non-finite -> 0)
  double *gOut;  // outScale gradient
  float *gDrive; // [epochs][nDS] dLoss/d(scheduled drive), float as the reference accumulates it
  const float *dL;       // flat [N], or per step over the readout set [steps][nro]
  const int32_t *roMap;  // neuron -> readout column, -1 elsewhere (per-step dL)
  int32_t *nonfinite;    // counts of non-finite log-gain [0] and drive [1] gradients
  uint32_t ovfCap, pad0;
  int32_t *err;
  const uint32_t *jump;
};

static_assert(sizeof(DiffDev) % 4 == 0, "DiffDev is copied as 32-bit words");

// The block's instance record into shared memory.
__device__ __forceinline__ void load_dev(const DiffDev *Ds, DiffDev &s) {
  const uint32_t *src = reinterpret_cast<const uint32_t *>(Ds + blockIdx.y);
  uint32_t *dst = reinterpret_cast<uint32_t *>(&s);
  for (int k = threadIdx.x; k < (int)(sizeof(DiffDev) / 4); k += blockDim.x) dst[k] = src[k];
  __syncthreads();
}

// Model constants in the arithmetic type R of a pass: double reproduces the reference's
// arithmetic (JS numbers); float is the GB300 fast mode (the FP64 pipes are a small fraction of
// the FP32 ones). Built on the host from the double parameters, each rounded once.
template <typename R>
struct DP {
  R dt, vRest, vThresh, vReset, tRef, wSyn, adaptInc, depU, eExc, eInh, inhGain;
  R kcThreshold, laminaBias, beta, adjClip, dE, dA, kRec, kM, dtS, cE, cI;
  // exact32: the same scalars rounded to f32, as lif.c reads them from its header
  float xdt, xvRest, xvThresh, xvReset, xtRef, xadaptInc, xdepU, xeExc, xeInh, xlaminaBias;
  float xdE, xdA, xkRec, xkM, xdtS, xcE, xcI;
};

// The drive neuron i runs at in step t: the schedule's value for its column (the last driveIdx
// entry naming it), else the drive as set (src/lifdiff.js:242-251).
__device__ __forceinline__ float d_drive(const DiffDev &D, int i, int t) {
  if (D.driveAt) {
    const int k = D.dSlot[i];
    if (k >= 0) return D.driveAt[(int64_t)(t / D.driveEpoch) * D.nDS + k];
  }
  return D.drive[i];
}

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
__global__ void k_prepare(int32_t N, float *inScale, const float *sizeLog, const float *inScaleSrc,
                          double sizeAlpha, double maxSizeScale, double boostCap) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < N; i += nt) {
    if (inScaleSrc) inScale[i] = inScaleSrc[i];
    else {
      const double s = exp(-sizeAlpha * (double)sizeLog[i]);
      inScale[i] = (float)fmin(boostCap, fmax(1.0 / maxSizeScale, s));
    }
  }
}

// The gate (src/lifdiff.js:167-171) and P[j] = (count * edgeGain) * inScale[q], the first factors
// of the delivered amount (:281-282), in double and in float.
__global__ void k_prepare_edges(int64_t E, const uint32_t *indices, const float *counts, const float *edgeGain,
                                const float *inScale, const uint8_t *sensory, double minSyn, uint8_t *gate,
                                double *P, float *Pf) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = tid; j < E; j += nt) {
    const uint32_t q = indices[j];
    const double c = (double)counts[j];
    gate[j] = (c >= minSyn && !(sensory && sensory[q])) ? 1 : 0;
    P[j] = c * (edgeGain ? (double)edgeGain[j] : 1.0) * (double)inScale[q];
    Pf[j] = counts[j] * (edgeGain ? edgeGain[j] : 1.f) * inScale[q];
  }
}

// Reset (src/lifdiff.js:221-233): state, delivery scratch, RNG, tape offset 0.
__global__ void k_reset(const DiffDev *Ds, float vRest) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += (int64_t)gridDim.x * blockDim.x) {
    D.v[i] = vRest;
    D.gE[i] = D.gI[i] = D.adapt[i] = D.refr[i] = D.spikeCount[i] = 0.f;
    D.res[i] = 1.f;
    D.isForced[i] = 0;
    D.cnt[i] = 0;
    D.ovfHead[i] = kNil;
    if (i < D.nDriven) D.drivenLive[i] = D.driven[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *D.rng = D.seed0;
    D.tOff[0] = 0;
    *D.ovfTop = 0;
    *D.nLive = D.nDriven;
  }
}

// exact32's baked weights (src/lifdiff.js:177-189), warp per presynaptic row: every product in
// double, in the reference's operand order, stored once as f32.
__global__ void k_prepare_w32(const DiffDev *Ds, double wSyn, double inhGain) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  if (!D.W32) return;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w0; j < D.N; j += nw) {
    const double sg = D.sign[j];
    if (lane == 0) D.signW32[j] = (float)(sg * wSyn);
    const double ig = (sg < 0 ? inhGain : 1.0) * (D.outScale ? (double)D.outScale[j] : 1.0);
    for (uint32_t k = D.indptr[j] + lane; k < D.indptr[j + 1]; k += 32)
      D.W32[k] = D.gate[k] ? (float)((double)D.counts[k] * (D.edgeGain ? (double)D.edgeGain[k] : 1.0) *
                                     (double)D.inScale[D.indices[k]] * ig)
                           : 0.f;
  }
}

// An epoch boundary of the drive schedule (forward): the drivenSet loses the epoch's removed
// members (order kept) and gains its appended ones at the end, in the order setDriveOne calls in
// driveIdx order would leave them (src/lifdiff.js:207). One block per instance.
__global__ void __launch_bounds__(1024) k_epoch(const DiffDev *Ds, int32_t t) {
  __shared__ DiffDev D;
  __shared__ uint32_t scan[33];
  load_dev(Ds, D);
  if (t >= D.steps || !D.epOff || t % D.driveEpoch) return;
  const int tid = threadIdx.x, bd = blockDim.x;
  const int64_t e = t / D.driveEpoch;
  const int32_t r0 = D.epOff[2 * e], r1 = D.epOff[2 * e + 1], a1 = D.epOff[2 * e + 2];
  for (int32_t k = r0 + tid; k < r1; k += bd) D.rmFlag[D.epList[k]] = 1;
  __syncthreads();
  const int32_t n = *D.nLive;
  uint32_t kept = (uint32_t)n;
  if (r1 > r0) {
    // stable in-place compaction: every entry moves to a lower or equal index, and a chunk's reads
    // all precede (through the scan's barriers) its writes
    kept = 0;
    for (int32_t c0 = 0; c0 < n; c0 += bd) {
      const int32_t k = c0 + tid;
      int32_t i = 0;
      uint32_t keep = 0;
      if (k < n) {
        i = D.drivenLive[k];
        keep = D.rmFlag[i] ? 0u : 1u;
      }
      uint32_t tot;
      const uint32_t pos = block_exclusive_scan(keep, &tot, scan);
      if (keep) D.drivenLive[kept + pos] = i;
      kept += tot;
    }
    __syncthreads();
    for (int32_t k = r0 + tid; k < r1; k += bd) D.rmFlag[D.epList[k]] = 0;
  }
  for (int32_t k = r1 + tid; k < a1; k += bd) D.drivenLive[kept + (k - r1)] = D.epList[k];
  if (tid == 0) *D.nLive = (int32_t)kept + (a1 - r1);
}

// Saves (save=1, at t % K == 0) or restores (save=0) the checkpoint of step t.
__global__ void __launch_bounds__(kDB, 4) k_ckpt(const DiffDev *Ds, int32_t t, int32_t save) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  if (t >= D.steps || t % D.K) return;
  const int64_t N = D.N;
  float *c = D.ckpt + (int64_t)(t / D.K) * 6 * N;
  float *st[6] = {D.v, D.gE, D.gI, D.adapt, D.res, D.refr};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (save) c[a * N + i] = st[a][i];
      else st[a][i] = c[a * N + i];
    }
  }
  if (save && blockIdx.x == 0 && threadIdx.x == 0) D.ckptRng[t / D.K] = *D.rng;
}

// Delivery of the arrivals at step t (the spikes of step t - (nslots-1)), warp per arrival
// (src/lifdiff.js:276-283): lane 0 forms eff and depresses res; lanes push (rank, edge) per
// gated edge into the target's bucket. In a replay (row >= 0) the arrival's res is recorded.
// exact32 (forward): lane 0 forms lif.c's s = f32(signW32 * res) (times the amplitude when it is
// not 1) and skips a zero s before depressing res (src/lifdiff.js:256-272).
// Tape entries [a0, a0 + n) of an arrival step, cut at the tape's capacity: a forward that ran out
// of tape keeps counting offsets past it (and reports FB_EOVERFLOW when it ends), and the steps
// after the overflow must not read beyond the entries that exist.
__device__ __forceinline__ int64_t tape_count(const DiffDev &D, int64_t a0, int64_t a1) {
  if (a1 > D.tapeCap) a1 = D.tapeCap;
  return a1 > a0 ? a1 - a0 : 0;
}

// Edges of a row each lane of a warp-per-arrival kernel keeps in flight at once.
constexpr int kEdgeILP = 4;

template <typename R>
__global__ void __launch_bounds__(kDB, 4) k_deliver(const DiffDev *Ds, DP<R> P, int32_t t, int32_t row) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  const int e = t - (D.nslots - 1);
  if (t >= D.steps || e < 0) return;
  float *resRow = row >= 0 ? D.resAt + (int64_t)row * D.maxArr : nullptr;
  const bool ex = row < 0 && D.exact32;
  const int64_t a0 = D.tOff[e], na = tape_count(D, a0, D.tOff[e + 1]);
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = w0; k < na; k += nw) {
    const int32_t pre = D.tIdx[a0 + k];
    int go = 0;
    if (lane == 0) {
      if (ex) {
        const float r = D.res[pre], amp = D.tAmp[a0 + k];
        float sv = D.signW32[pre] * r;
        if (amp != 1.f) sv = sv * amp;
        if (sv != 0.f) {
          D.res[pre] = (float)((double)r - (double)P.xdepU * (double)r);
          go = 1;
        }
        D.effK[k] = (double)sv;
      } else {
        const float sg = D.sign[pre];
        R eff = 0;
        if (sg != 0) {
          const R r = D.res[pre];
          if (resRow) resRow[k] = (float)r;
          eff = (R)sg * P.wSyn * d_out<R>(D, pre) * exp((R)D.logGain[pre]) * r * (R)D.tAmp[a0 + k];
          D.res[pre] = (float)(r - P.depU * r);
          go = 1;
        }
        D.effK[k] = (double)eff;
      }
    }
    if (!__shfl_sync(0xffffffffu, go, 0)) continue;
    const uint32_t lo = D.indptr[pre], hi = D.indptr[pre + 1];
    // kEdgeILP edges per lane in flight (their loads, then their slot claims, then their
    // stores); the order of the pushes into a bucket does not matter, k_update orders a target's
    // contributions by (arrival, edge)
    for (uint32_t j0 = lo + lane; j0 < hi; j0 += 32 * kEdgeILP) {
      bool on[kEdgeILP];
      uint32_t q[kEdgeILP], pos[kEdgeILP];
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++) {
        const uint32_t j = j0 + 32u * u;
        on[u] = j < hi && D.gate[j];
        if (on[u]) q[u] = D.indices[j];
      }
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++)
        if (on[u]) pos[u] = atomicAdd(D.cnt + q[u], 1u);
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++) {
        if (!on[u]) continue;
        const uint32_t j = j0 + 32u * u;
        if (pos[u] < (uint32_t)kDBucket) {
          D.bucket[(int64_t)q[u] * kDBucket + pos[u]] = make_uint2((uint32_t)k, j);
        } else {
          const uint32_t r = atomicAdd(D.ovfTop, 1u);
          if (r >= D.ovfCap) {
            atomicCAS(D.err, 0, FB_EOVERFLOW);
            continue;
          }
          DOvf o;
          o.k = (uint32_t)k;
          o.j = j;
          o.pad = q[u];
          o.next = atomicExch(D.ovfHead + q[u], r);
          D.ovf[r] = o;
        }
      }
    }
  }
}

// Forced spikes of step t, one block per instance. Forward (src/lifdiff.js:290-306): unless
// driveSoft, one draw per non-refractory member of the live drivenSet in insertion order, compared
// (in R; exact32: in f32 as lif.c) against drive * dt/1000; then the spike train's neurons of step
// t that are not refractory, first listing only. Each spike goes to the head of step t's tape list.
// Replay: the tape's forced list. Shares no data with the step's delivery, beside which it runs.
constexpr int kForcedPer = 4;  // driven-list entries per thread and round in k_forced
template <typename R>
__global__ void k_forced(const DiffDev *Ds, DP<R> P, int32_t t, int32_t replay) {
  __shared__ DiffDev D;
  __shared__ uint32_t sJump[32 * 128];
  __shared__ uint32_t scan[33];
  __shared__ uint32_t sh_s0;
  load_dev(Ds, D);
  if (t >= D.steps) return;
  const int tid = threadIdx.x;
  const int64_t base = D.tOff[t];
  if (replay) {
    const int32_t nf = (int32_t)tape_count(D, base, base + D.tForced[t]);
    for (int k = tid; k < nf; k += blockDim.x) {
      const int32_t i = D.tIdx[base + k];
      D.refr[i] = (float)(P.tRef + P.dt);
      D.adapt[i] = (float)((R)D.adapt[i] + P.adaptInc);
      D.isForced[i] = 1;
    }
    return;
  }
  const bool ex = D.exact32 != 0;
  const float refrF = ex ? P.xtRef + P.xdt : (float)(P.tRef + P.dt);
  const R aInc = ex ? (R)P.xadaptInc : P.adaptInc;
  uint32_t nf = 0;
  auto fire_one = [&](int32_t i, int64_t o) {
    if (o < D.tapeCap) {
      D.tIdx[o] = i;
      D.tAmp[o] = 1.f;
    } else {
      atomicCAS(D.err, 0, FB_EOVERFLOW);
    }
    D.refr[i] = refrF;
    D.spikeCount[i] = (float)((R)D.spikeCount[i] + R(1));
    D.adapt[i] = (float)((R)D.adapt[i] + aInc);
    D.isForced[i] = 1;
  };
  if (!D.driveSoft) {
    for (int k = tid; k < 32 * 128; k += blockDim.x) sJump[k] = D.jump[k];
    if (tid == 0) sh_s0 = *D.rng;
    __syncthreads();
    const uint32_t s0 = sh_s0;
    const int32_t nLive = *D.nLive;
    uint32_t draws = 0;
    // rounds of kForcedPer entries per thread, each thread's a contiguous run of the list: one
    // block scan gives a thread's first draw (a jump); its later live entries take the next draws
    // (one generator step each)
    const int32_t span = (int32_t)blockDim.x * kForcedPer;
    for (int32_t r0 = 0; r0 < nLive; r0 += span) {
      int32_t ii[kForcedPer];
      float dr[kForcedPer];
      uint32_t liveMask = 0, nl = 0;
#pragma unroll
      for (int u = 0; u < kForcedPer; u++) {
        const int32_t k = r0 + tid * kForcedPer + u;
        ii[u] = 0;
        dr[u] = 0.f;
        if (k < nLive) {
          ii[u] = D.drivenLive[k];
          dr[u] = d_drive(D, ii[u], t);
          if (!(D.refr[ii[u]] > 0)) {
            liveMask |= 1u << u;
            nl++;
          }
        }
      }
      uint32_t nlive;
      const uint32_t dpos = block_exclusive_scan(nl, &nlive, scan);
      uint32_t fireMask = 0, nfr = 0;
      if (nl) {
        uint32_t x = xs_jump(sJump, s0, draws + dpos + 1);
        bool first = true;
#pragma unroll
        for (int u = 0; u < kForcedPer; u++) {
          if (!((liveMask >> u) & 1u)) continue;
          if (!first) x = xs_next(x);
          first = false;
          const R uu = (R)(x >> 8) * (R)(1.0 / 16777216.0);  // exact in f32 and f64
          if (ex ? uu < (R)(dr[u] * P.xdtS) : uu < (R)dr[u] * P.dtS) {
            fireMask |= 1u << u;
            nfr++;
          }
        }
      }
      uint32_t nfire;
      const uint32_t fpos = block_exclusive_scan(nfr, &nfire, scan);
      uint32_t o = 0;
#pragma unroll
      for (int u = 0; u < kForcedPer; u++)
        if ((fireMask >> u) & 1u) fire_one(ii[u], base + nf + fpos + o++);
      draws += nlive;
      nf += nfire;
    }
    if (tid == 0) *D.rng = xs_jump(sJump, s0, draws);
  }
  if (D.trainOff) {
    const int64_t q0 = D.trainOff[t], q1 = D.trainOff[t + 1];
    if (q1 > q0) {
      __syncthreads();  // the draws' refractory marks are visible
      for (int64_t q = q0 + tid; q < q1; q += blockDim.x) {
        const int32_t i = D.trainIdx[q];
        if (!(D.refr[i] > 0)) atomicMin(D.claim + i, (int32_t)(q - q0));
      }
      __syncthreads();
      for (int64_t c0 = q0; c0 < q1; c0 += blockDim.x) {
        const int64_t q = c0 + tid;
        int32_t i = 0;
        uint32_t fire = 0;
        if (q < q1) {
          i = D.trainIdx[q];
          fire = D.claim[i] == (int32_t)(q - q0) ? 1u : 0u;
        }
        uint32_t nfire;
        const uint32_t fpos = block_exclusive_scan(fire, &nfire, scan);
        if (fire) fire_one(i, base + nf + fpos);
        nf += nfire;
      }
      for (int64_t q = q0 + tid; q < q1; q += blockDim.x) D.claim[D.trainIdx[q]] = kClaimFree;
    }
  }
  if (tid == 0) D.tForced[t] = (int32_t)nf;
}

// Adds target i's bucket in arrival-rank order: gE (or gI) = f32(g + P[j] (*inhGain) * eff) in R.
// Up to kDSortMax contributions are sorted in local memory; beyond that they are applied in
// successive windows of the kDSortMax smallest ranks above the last one applied (ranks are unique
// per target: one contribution per arrival). exact32: lif.c's per-edge f32(W32 * s), skipped when
// zero, added in f32 (src/lifdiff.js:270).
template <typename R>
__device__ __forceinline__ void d_add(const DiffDev &D, const DP<R> &Pp, uint2 c, float &geF, float &giF, bool ex) {
  if (ex) {
    const float sv = (float)D.effK[c.x], dlt = D.W32[c.y] * sv;
    if (dlt != 0.f) {
      if (sv > 0.f) geF = geF + dlt;
      else giF = giF + dlt;
    }
    return;
  }
  const R eff = (R)D.effK[c.x];
  const R p = sizeof(R) == 8 ? (R)D.P[c.y] : (R)D.Pf[c.y];
  if (eff > 0) geF = (float)((R)geF + p * eff);
  else giF = (float)((R)giF + p * Pp.inhGain * eff);
}

template <typename R>
__device__ void d_apply(const DiffDev &D, const DP<R> &Pp, int i, uint32_t n, float &geF, float &giF, bool ex) {
  uint2 e[kDSortMax];
  const uint2 *bk = D.bucket + (int64_t)i * kDBucket;
  const uint32_t nb = n < (uint32_t)kDBucket ? n : (uint32_t)kDBucket;
  bool any = false;
  uint2 last = make_uint2(0u, 0u);
  // order: arrival rank, then edge id (a row naming the target more than once adds its edges
  // in row order, src/lifdiff.js as lif.c:40-42)
  auto before = [](uint2 p, uint2 q) { return p.x < q.x || (p.x == q.x && p.y < q.y); };
  for (uint32_t done = 0; done < n;) {
    uint32_t m = 0;
    auto offer = [&](uint2 x) {  // keep the kDSortMax smallest (rank, edge) pairs above `last`, sorted
      if (any && !before(last, x)) return;
      if (m == (uint32_t)kDSortMax && !before(x, e[m - 1])) return;
      uint32_t w = m < (uint32_t)kDSortMax ? m++ : m - 1;
      while (w > 0 && before(x, e[w - 1])) {
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
    for (uint32_t u = 0; u < m; u++) d_add<R>(D, Pp, e[u], geF, giF, ex);
    last = e[m - 1];
    any = true;
    done += m;
  }
  if (n > (uint32_t)kDBucket) D.ovfHead[i] = kNil;
}

// A neuron's inputs to its update, loaded for two neurons per lane before either is written.
struct UIn {
  float ge, gi, v, refr, ad, res, sc, thr;
  uint32_t n;
  uint8_t forced;
};
__device__ __forceinline__ void load_in(const DiffDev &D, int i, UIn &u) {
  u.ge = D.gE[i];
  u.gi = D.gI[i];
  u.n = D.cnt[i];
  u.v = D.v[i];
  u.refr = D.refr[i];
  u.forced = D.isForced[i];
  u.ad = D.adapt[i];
  u.res = D.res[i];
  u.sc = D.spikeCount[i];
  u.thr = D.thrOffset[i];
}

// One neuron's integrate and spike (src/lifdiff.js:313-344); with `row` >= 0 the replay arena
// (:439-456). Returns whether the spike goes on the tape (amplitude in *amp). exact32 (forward):
// lif.c's expression with one f32 rounding per C operation and the header's f32 scalars
// (:317-326). driveSoft: a driven neuron's spike is sd + (1 - sd) s, sd = min(0.999, drive
// dt/1000) (:338).
template <typename R>
__device__ __forceinline__ bool upd_neuron(const DiffDev &D, const DP<R> &P, int i, int t, int row, bool ex,
                                           const UIn &u, float &amp) {
  float geF = u.ge, giF = u.gi;
  if (u.n) {
    d_apply<R>(D, P, i, u.n, geF, giF, ex);
    D.cnt[i] = 0;
  }
  const R vReset = ex ? (R)P.xvReset : P.vReset, aInc = ex ? (R)P.xadaptInc : P.adaptInc;
  const R ge = geF, gi = giF;
  const int64_t off = row >= 0 ? (int64_t)row * D.N + i : 0;
  R vi = u.v, s = 0;
  int md = 0;
  if (row >= 0) {
    D.aV[off] = u.v;
    D.aGE[off] = geF;
    D.aGI[off] = giF;
  }
  float refr = u.refr;
  const bool forced = u.forced != 0;
  if (forced) D.isForced[i] = 0;
  const bool wasRefr = refr > 0;
  if (wasRefr) {
    refr = ex ? refr - P.xdt : (float)((R)refr - P.dt);
    vi = vReset;
    if (forced) {
      md = 2;
      s = 1;
    } else {
      md = 1;
    }
  } else if (ex) {
    const float vf = u.v;
    float acc = P.xvRest - vf;
    if (D.coba) {
      acc = acc + (geF * (P.xeExc - vf)) * P.xcE;
      acc = acc + (giF * (vf - P.xeInh)) * P.xcI;
    } else {
      acc = acc + geF;
      acc = acc + giF;
    }
    const float lam = (D.biasMask && D.biasMask[i]) ? P.xlaminaBias : 0.f;
    acc = D.biasArr ? (float)((double)acc + ((double)lam + (double)D.biasArr[i])) : acc + lam;
    vi = vf + acc * P.xkM;
  } else {
    vi = d_u<R>(D, P, vi, ge, gi, d_bias<R>(D, P, i, nullptr));
  }
  geF = ex ? geF * P.xdE : (float)(ge * P.dE);
  giF = ex ? giF * P.xdE : (float)(gi * P.dE);
  float ad = ex ? u.ad * P.xdA : (float)((R)u.ad * P.dA);
  const float rsF = u.res;
  D.res[i] = ex ? rsF + (1.f - rsF) * P.xkRec : (float)((R)rsF + (R(1) - (R)rsF) * P.kRec);
  if (row >= 0) D.aAd[off] = ad;
  bool emit = false;
  if (!wasRefr) {
    const R thr = ex ? (R)((P.xvThresh + ad) + u.thr) : P.vThresh + (R)ad + d_kc<R>(D, P, i) + (R)u.thr;
    s = D.soft ? R(1) / (R(1) + exp(-(vi - thr) / d_beta<R>(D, P, i))) : (vi >= thr ? R(1) : R(0));
    if (D.driveSoft) {
      const float dr = d_drive(D, i, t);
      if (dr > 0.f) {
        const R x = (R)dr * P.dtS, sd = x < (R)kDriveMax ? x : (R)kDriveMax;
        s = sd + (R(1) - sd) * s;
        md = 3;
      }
    }
    if (s > 0) {
      vi = s * vReset + (R(1) - s) * vi;
      if (!D.soft) refr = ex ? P.xtRef : (float)P.tRef;
      ad = (float)((R)ad + s * aInc);
    }
    D.spikeCount[i] = (float)((R)u.sc + s);
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
  return emit;
}

// Integrate and spike for every neuron, warp tiles of kWT = 64 neurons (two per lane, both
// loaded before either is written). In a forward pass the spikes above the tape threshold are
// staged per warp tile in ascending order (ballots; no block barrier).
constexpr int kWT = 64;
template <typename R>
__global__ void __launch_bounds__(kDB, 4) k_update(const DiffDev *Ds, DP<R> P, int32_t t, int32_t row) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  if (t >= D.steps) return;
  // the step's delivery is complete and the next one starts after this kernel: the overflow pool
  // is rewound here (its entries stay readable until the next delivery)
  if (blockIdx.x == 0 && threadIdx.x == 0) *D.ovfTop = 0;
  const bool ex = row < 0 && D.exact32;
  const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  const int nWT = (D.N + kWT - 1) / kWT;
  const int wpb = blockDim.x >> 5;
  for (int wt = blockIdx.x * wpb + (int)(threadIdx.x >> 5); wt < nWT; wt += gridDim.x * wpb) {
    const int i0 = wt * kWT + (int)lane, i1 = i0 + 32;
    UIn u0, u1;
    if (i0 < D.N) load_in(D, i0, u0);
    if (i1 < D.N) load_in(D, i1, u1);
    float a0 = 0.f, a1 = 0.f;
    const bool e0 = i0 < D.N && upd_neuron<R>(D, P, i0, t, row, ex, u0, a0);
    const bool e1 = i1 < D.N && upd_neuron<R>(D, P, i1, t, row, ex, u1, a1);
    if (row >= 0) continue;  // replay: the tape already holds the spikes
    const uint32_t b0 = __ballot_sync(0xffffffffu, e0), b1 = __ballot_sync(0xffffffffu, e1);
    const int64_t base = (int64_t)wt * kWT;
    if (e0) {
      const uint32_t p = __popc(b0 & lt);
      D.stage[base + p] = i0;
      D.stageAmp[base + p] = a0;
    }
    if (e1) {
      const uint32_t p = __popc(b0) + __popc(b1 & lt);
      D.stage[base + p] = i1;
      D.stageAmp[base + p] = a1;
    }
    if (lane == 0) D.tileCnt[wt] = (int32_t)(__popc(b0) + __popc(b1));
  }
}

// Appends step t's threshold spikes (tile order = ascending) after its forced ones; one block per
// instance.
__global__ void k_emit(const DiffDev *Ds, int32_t t) {
  __shared__ DiffDev D;
  __shared__ uint32_t scan[33];
  load_dev(Ds, D);
  if (t >= D.steps) return;
  const int tid = threadIdx.x;
  const int64_t carry = D.tOff[t] + D.tForced[t];
  // thread tid takes a contiguous run of tiles, so one block scan places every tile
  const int nWT = (D.N + kWT - 1) / kWT;
  const int per = (nWT + (int)blockDim.x - 1) / (int)blockDim.x;
  const int t0 = min(nWT, tid * per), t1 = min(nWT, t0 + per);
  uint32_t c = 0;
  for (int tl = t0; tl < t1; tl++) c += (uint32_t)D.tileCnt[tl];
  uint32_t tot;
  const uint32_t pre = block_exclusive_scan(c, &tot, scan);
  if (c) {
    int64_t o = carry + pre;
    for (int tl = t0; tl < t1; tl++) {
      const uint32_t n = (uint32_t)D.tileCnt[tl];
      for (uint32_t p = 0; p < n; p++) {
        if (o + p < D.tapeCap) {
          D.tIdx[o + p] = D.stage[(int64_t)tl * kWT + p];
          D.tAmp[o + p] = D.stageAmp[(int64_t)tl * kWT + p];
        } else {
          atomicCAS(D.err, 0, FB_EOVERFLOW);
        }
      }
      o += n;
    }
  }
  if (tid == 0) D.tOff[t + 1] = carry + tot;
}

// Zeroes the adjoint state and accumulators of every instance (before a backward pass).
__global__ void k_zero_adjoint(const DiffDev *Ds) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  const int64_t N = D.N, s0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, ns = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = s0; i < N; i += ns) {
    D.lv[i] = D.lgE[i] = D.lgI[i] = D.lad[i] = D.lres[i] = 0.f;
    D.accA[i] = D.accV[i] = D.accKc[i] = D.accLa[i] = D.accEI[i] = D.accW[i] = D.accD[i] = 0.0;
    D.gLog[i] = D.gBias[i] = 0.0;
  }
  for (int64_t i = s0; i < (int64_t)D.nslots * N; i += ns) D.lsRing[i] = 0.f;
  for (int64_t j = s0; j < D.E; j += ns) D.gEdge[j] = 0.0;
  if (D.gDrive) {
    const int64_t nd = (int64_t)((D.steps + D.driveEpoch - 1) / D.driveEpoch) * D.nDS;
    for (int64_t k = s0; k < nd; k += ns) D.gDrive[k] = 0.f;
  }
}

// Truncated BPTT (src/lifdiff.js:541-548): the adjoint state restarts at every multiple of
// `truncate` steps.
__global__ void __launch_bounds__(kDB, 4) k_truncate(const DiffDev *Ds, int32_t t, int32_t truncate) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  if (t >= D.steps || (t + 1) % truncate) return;
  const int64_t N = D.N, s0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, ns = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = s0; i < N; i += ns) D.lv[i] = D.lgE[i] = D.lgI[i] = D.lad[i] = D.lres[i] = 0.f;
  for (int64_t i = s0; i < (int64_t)D.nslots * N; i += ns) D.lsRing[i] = 0.f;
}

// A neuron's inputs to its reverse step, loaded for two neurons per lane before either is written.
struct BIn {
  float lad, lgE, lgI, lres, lv, ls, aV, aGE, aGI, aAd, aSp, thr, dl;
  double accA, accV, gBias;
  int md, ro;
};
__device__ __forceinline__ void load_bin(const DiffDev &D, const float *ls, int64_t off, int i, BIn &u) {
  u.md = D.aMode[off];
  u.lad = D.lad[i];
  u.lgE = D.lgE[i];
  u.lgI = D.lgI[i];
  u.lres = D.lres[i];
  u.lv = D.lv[i];
  if (u.md != 1) {
    u.ls = ls[i];
    u.accA = D.accA[i];
    if (u.md != 2) {
      u.aV = D.aV[off];
      u.aGE = D.aGE[off];
      u.aGI = D.aGI[off];
      u.aAd = D.aAd[off];
      u.aSp = D.aSp[off];
      u.thr = D.thrOffset[i];
      u.accV = D.accV[i];
      u.gBias = D.gBias[i];
    }
  }
  u.ro = (u.md != 1 && D.dL && D.roMap) ? D.roMap[i] : -1;  // the loss gradient's column, if read out
}

// The step's loss gradient for a neuron (second load phase: it depends on the readout column).
__device__ __forceinline__ void load_dl(const DiffDev &D, int i, int t, int32_t scored, BIn &u) {
  u.dl = 0.f;
  if (!scored || !D.dL || u.md == 1) return;
  if (D.roMap) {
    if (u.ro >= 0) u.dl = D.dL[(int64_t)t * D.nro + u.ro];
  } else {
    u.dl = D.dL[i];
  }
}

// Reverse of integrate-and-spike for neuron i at step t (src/lifdiff.js:555-617), with the adjoint
// clip (:623-629) fused. Scalar terms accumulate per neuron in double. The gradient of a scheduled
// drive (:565-573, :587-604) accumulates per neuron into its column of the step's epoch: a forced
// spike through ds/d(sd) = 1, a soft drive through ds/d(sd) = 1 - st, with d(sd)/d(rate) = dt/1000
// (the min's clamp is not differentiated, as in the reference).
template <typename R>
__device__ __forceinline__ void bneuron(const DiffDev &D, const DP<R> &P, int i, int t, int32_t scored, float *ls,
                                        float *gDrv, const BIn &u) {
  const int md = u.md;
  const R lpA = u.lad;
  const R lE = (R)u.lgE * P.dE, lI = (R)u.lgI * P.dE, lA = lpA * P.dA;
  const R lR = (R)u.lres * (R(1) - P.kRec);
  float lvF = u.lv, lgEF = (float)lE, lgIF = (float)lI, ladF = (float)lA, lresF = (float)lR;
  if (md == 1) {
    lvF = 0.f;
  } else {
    const R dl = u.dl;
    const int slot = gDrv ? D.dSlot[i] : -1;
    if (md == 2) {
      D.accA[i] = u.accA + (double)lA;
      if (slot >= 0) gDrv[slot] = (float)((R)gDrv[slot] + (lA * P.adaptInc + ((R)u.ls + dl)) * P.dtS);
      lvF = 0.f;
      ls[i] = 0.f;
    } else {
      const R vv = u.aV, gEv = u.aGE, gIv = u.aGI;
      R lam;
      const R bias = d_bias<R>(D, P, i, &lam);
      const R uu = d_u<R>(D, P, vv, gEv, gIv, bias);
      const R thr = P.vThresh + (R)u.aAd + d_kc<R>(D, P, i) + (R)u.thr;
      const R d = uu - thr;
      const R s = u.aSp;
      // a soft drive's composite spike split back into sd and the threshold's st
      R sd = 0, st = s;
      if (md == 3) {
        const R x = (R)d_drive(D, i, t) * P.dtS;
        sd = x < (R)kDriveMax ? x : (R)kDriveMax;
        st = (s - sd) / (R(1) - sd);
      }
      const R beta = d_beta<R>(D, P, i);
      R sg;
      if (D.soft) sg = st * (R(1) - st) / beta;
      else {
        const R tt = R(1) + fabs(d) / beta;
        sg = R(1) / (beta * tt * tt);
      }
      const R lspike = (R)u.ls + dl;
      const R lvNew = lvF;
      const R lsTot = (P.vReset - uu) * lvNew + lpA * P.adaptInc + lspike;
      const R lt = lsTot * (R(1) - sd) * sg;
      const R lu = lvNew * (R(1) - s) + lt;
      const R lthr = -lt;
      if (slot >= 0) gDrv[slot] = (float)((R)gDrv[slot] + lsTot * (R(1) - st) * P.dtS);
      D.accA[i] = u.accA + (double)(lpA * s);
      D.accV[i] = u.accV + (double)lthr;
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
      D.gBias[i] = u.gBias + (double)(lu * P.kM);
      ls[i] = 0.f;
    }
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

// The reverse neuron pass of step t over warp tiles of kWT neurons (two per lane).
template <typename R>
__global__ void __launch_bounds__(kDB, 3) k_bneuron(const DiffDev *Ds, DP<R> P, int32_t t, int32_t row, int32_t scored) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  if (t >= D.steps) return;
  float *ls = D.lsRing + (int64_t)(t % D.nslots) * D.N;
  float *gDrv = D.gDrive ? D.gDrive + (int64_t)(t / D.driveEpoch) * D.nDS : nullptr;
  const int lane = threadIdx.x & 31;
  const int nWT = (D.N + kWT - 1) / kWT;
  const int wpb = blockDim.x >> 5;
  const int64_t rowOff = (int64_t)row * D.N;
  for (int wt = blockIdx.x * wpb + (threadIdx.x >> 5); wt < nWT; wt += gridDim.x * wpb) {
    const int i0 = wt * kWT + lane, i1 = i0 + 32;
    BIn u0, u1;
    if (i0 < D.N) load_bin(D, ls, rowOff + i0, i0, u0);
    if (i1 < D.N) load_bin(D, ls, rowOff + i1, i1, u1);
    if (i0 < D.N) load_dl(D, i0, t, scored, u0);
    if (i1 < D.N) load_dl(D, i1, t, scored, u1);
    if (i0 < D.N) bneuron<R>(D, P, i0, t, scored, ls, gDrv, u0);
    if (i1 < D.N) bneuron<R>(D, P, i1, t, scored, ls, gDrv, u1);
  }
}

// Reverse of the delivery at step t (src/lifdiff.js:635-666), warp per arrival: lanes gather the
// fan-out's adjoint into lRaw (a fixed-order warp sum) and add each gated edge's
// dLoss/dW_j = lg[q] * eff to its accumulator; lane 0 updates the presynaptic neuron's terms.
template <typename R>
__global__ void __launch_bounds__(kDB, 2) k_barrival(const DiffDev *Ds, DP<R> P, int32_t t, int32_t row) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  const int e = t - (D.nslots - 1);
  if (t >= D.steps || e < 0) return;
  const float *resRow = D.resAt + (int64_t)row * D.maxArr;
  const int64_t a0 = D.tOff[e], na = tape_count(D, a0, D.tOff[e + 1]);
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
    // kEdgeILP edges per lane in flight: every load of a group is issued before any value is
    // used, so a long row costs one dependent round trip per group rather than per edge; each
    // lane still adds its edges in ascending order
    R lraw = 0;
    for (uint32_t j0 = lo + lane; j0 < hi; j0 += 32 * kEdgeILP) {
      bool on[kEdgeILP];
      uint32_t q[kEdgeILP];
      float cnt[kEdgeILP], eg[kEdgeILP], lgv[kEdgeILP], ins[kEdgeILP];
      double old[kEdgeILP];
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++) {
        const uint32_t j = j0 + 32u * u;
        on[u] = j < hi && D.gate[j];
        if (on[u]) {
          q[u] = D.indices[j];
          cnt[u] = D.counts[j];
          eg[u] = D.edgeGain ? D.edgeGain[j] : 1.f;
          old[u] = D.gEdge[j];
        }
      }
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++) {
        if (on[u]) {
          lgv[u] = exc ? D.lgE[q[u]] : D.lgI[q[u]];
          ins[u] = D.inScale[q[u]];
        }
      }
#pragma unroll
      for (int u = 0; u < kEdgeILP; u++) {
        if (on[u]) {
          const R lg = lgv[u];
          const R cw = (R)cnt[u] * (R)eg[u];
          lraw += exc ? lg * cw * (R)ins[u] : lg * cw * (R)ins[u] * P.inhGain;
          D.gEdge[j0 + 32u * u] = old[u] + (double)(lg * eff);
        }
      }
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

// Per instance, kRB blocks of fixed-order partial sums: the seven per-neuron accumulators
// (W EI V Kc La A D), the sizeAlpha term through inScale (src/lifdiff.js:650-655, 676-680:
// gInScale[q] summed over q's in-edges in edge order) and the inhibitory-gain term.
__global__ void k_reduce(const DiffDev *Ds, double inhGain, double sizeAlpha, double boostCap,
                         double maxSizeScale, double *partial) {
  __shared__ DiffDev D;
  __shared__ double sm[kNSums][kDB];
  load_dev(Ds, D);
  const int tid = threadIdx.x;
  double acc[kNSums];
#pragma unroll
  for (int k = 0; k < kNSums; k++) acc[k] = 0;
  for (int i = blockIdx.x * blockDim.x + tid; i < D.N; i += gridDim.x * blockDim.x) {
    acc[0] += D.accW[i];
    acc[1] += D.accEI[i];
    acc[2] += D.accV[i];
    acc[3] += D.accKc[i];
    acc[4] += D.accLa[i];
    acc[5] += D.accA[i];
    acc[6] += D.accD[i];
    double gis = 0, ginh = 0;
    for (uint32_t e = D.cscPtr[i]; e < D.cscPtr[i + 1]; e++) {
      const uint32_t j = D.cscEdge[e];
      if (!D.gate[j]) continue;
      const bool inh = D.sign[D.cscSrc[e]] < 0;  // eff's sign follows the presynaptic sign
      const double cw = (double)D.counts[j] * (D.edgeGain ? (double)D.edgeGain[j] : 1.0);
      gis += cw * (inh ? inhGain : 1.0) * D.gEdge[j];
      if (inh) ginh += cw * (double)D.inScale[i] * D.gEdge[j];
    }
    const double sl = (double)D.sizeLog[i];
    const double raw = exp(-sizeAlpha * sl);
    if (raw < boostCap && raw > 1 / maxSizeScale) acc[7] += gis * (-sl) * raw;
    acc[8] += ginh;
  }
#pragma unroll
  for (int k = 0; k < kNSums; k++) sm[k][tid] = acc[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s)
      for (int k = 0; k < kNSums; k++) sm[k][tid] += sm[k][tid + s];
    __syncthreads();
  }
  if (tid == 0)
    for (int k = 0; k < kNSums; k++) partial[((int64_t)blockIdx.y * kRB + blockIdx.x) * kNSums + k] = sm[k][0];
}

// Log-gain gradient as float with non-finite values zeroed and counted (src/lifdiff.js:681-684),
// and the outScale gradient dL/dlogGain / outScale.
__global__ void k_finalize(const DiffDev *Ds) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.N; i += gridDim.x * blockDim.x) {
    float x = (float)D.gLog[i];
    if (!isfinite(x)) {
      x = 0.f;
      atomicAdd(D.nonfinite, 1);
    }
    D.gLogF[i] = x;
    D.gOut[i] = (double)x / (D.outScale ? (double)D.outScale[i] : 1.0);
  }
  if (D.gDrive) {
    const int64_t nd = (int64_t)((D.steps + D.driveEpoch - 1) / D.driveEpoch) * D.nDS;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nd; k += (int64_t)gridDim.x * blockDim.x)
      if (!isfinite(D.gDrive[k])) {
        D.gDrive[k] = 0.f;
        atomicAdd(D.nonfinite + 1, 1);
      }
  }
}

// The readout raster of one instance's recorded forward: out[t * nro + c] = amplitude at t.
__global__ void k_raster(const DiffDev *Ds, int32_t steps, float *out) {
  __shared__ DiffDev D;
  load_dev(Ds, D);
  for (int t = blockIdx.x; t < steps; t += gridDim.x) {
    const int64_t a = D.tOff[t], b = a + tape_count(D, a, D.tOff[t + 1]);
    for (int64_t k = a + threadIdx.x; k < b; k += blockDim.x) {
      const int c = D.roMap[D.tIdx[k]];
      if (c >= 0) out[(int64_t)t * D.nro + c] = D.tAmp[k];
    }
  }
}

// out[j] = sum over the listed instances, in list order, of their per-edge gradients.
__global__ void k_edge_sum(const double *const *g, int32_t n, int64_t E, double *out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < E; j += (int64_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int k = 0; k < n; k++) s += g[k][j];
    out[j] = s;
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

// Arrays shared across instances: one device copy per (host pointer, field).
enum Field { F_INDPTR, F_INDICES, F_COUNTS, F_EDGE_GAIN, F_SIGN, F_OUT_SCALE, F_BETA, F_BIAS, F_THR_MASK,
             F_BIAS_MASK, F_LOG_GAIN, F_THR_OFFSET, F_SIZE_LOG, F_IN_SCALE, F_SENSORY };

// The derived per-edge arrays of instances with the same graph, edge gains and input scaling.
struct EdgeGroup {
  const void *key[5];
  int rep;  // instance whose arrays define the group
  float *inScale;
  uint8_t *gate;
  double *P;
  float *Pf;
};

struct Inst {
  DiffDev D;
  float *sizeLogSrc = nullptr, *inScaleSrc = nullptr;
  uint8_t *sensory = nullptr;
  int group = 0;
  int64_t ckptCap = 0, tStepsCap = 0, dLcap = 0, resAtCap = 0, arenaRows = 0;
  int32_t recordedSteps = 0;
  float *dLbuf = nullptr;
  int32_t *roMap = nullptr;
  std::vector<int32_t> roList;  // the readout set roMap holds
  // host copies for the drive schedule's set edits and the exact32 check
  std::vector<int32_t> driven0, driveIdx;
  bool thrMaskAny = false;
  // per-forward input buffers (grown on demand)
  float *sched = nullptr, *gDrive = nullptr;
  int32_t *epOff = nullptr, *epList = nullptr, *trainIdx = nullptr;
  int64_t *trainOff = nullptr;
  int64_t schedCap = 0, epOffCap = 0, epListCap = 0, trainOffCap = 0, trainIdxCap = 0, gDriveCap = 0;
};

}  // namespace

// One pass's launch sequence (a forward from reset, or a backward's replays and reverse steps)
// captured as a CUDA graph, and the key it was captured under.
struct PassGraph {
  std::vector<uint8_t> key;
  cudaGraphExec_t exec = nullptr;
  uint64_t used = 0;
};
constexpr size_t kPassGraphs = 4;  // graphs kept per batch

struct fb_diff_batch {
  int32_t B = 0;
  std::vector<Inst> in;
  std::vector<EdgeGroup> groups;
  std::map<std::pair<const void *, int>, std::pair<void *, size_t>> shared;
  std::map<std::pair<const void *, const void *>, std::vector<uint32_t *>> csc;  // (indptr, indices) -> CSC
  std::map<int64_t, float *> zeros;  // read-only zero arrays by length
  DiffDev *dDevs = nullptr;
  cudaStream_t st = nullptr;
  // the side branch of a step (the forced spikes and the tape), forked from and joined into `st`
  cudaStream_t side = nullptr;
  cudaEvent_t evFork = nullptr, evForced = nullptr, evUpdated = nullptr, evEmitted = nullptr;
  // a backward's reverse sweeps, beside the replay of the segment before (two arena halves)
  cudaStream_t rev = nullptr;
  cudaEvent_t evRep[2] = {nullptr, nullptr}, evRev[2] = {nullptr, nullptr}, evRevJoin = nullptr;
  int32_t arenaBufs = 1;
  cudaError_t orderErr = cudaSuccess;  // first failed event record or wait of the pass being issued
  std::vector<void *> allocs;
  fb_diff_params lastP;
  int32_t f32 = 0, recordedK = 0, recorded = 0, maxSteps = 0, maxTiles = 1, maxN = 1;
  int32_t tuneNeuron = 0, tuneArrival = 0;  // launch shape overrides (0: default)
  int32_t stepLaunches = 0;                   // 1: launch every step's kernels from the host
  std::vector<PassGraph> graphs;              // captured passes, least recently used evicted
  uint64_t graphTick = 0;
  DP<double> P64;
  DP<float> P32;
  int32_t *err = nullptr, *nonfinite = nullptr;
  uint32_t *jump = nullptr;
  double *partial = nullptr;
};

struct fb_diff {
  fb_diff_batch *b = nullptr;
};

namespace {

int balloc(fb_diff_batch *b, void **p, size_t bytes) {
  *p = nullptr;
  DCU(cudaMalloc(p, std::max<size_t>(bytes, 16)));
  b->allocs.push_back(*p);
  return FB_OK;
}

template <typename T>
int talloc(fb_diff_batch *b, T **p, size_t n) {
  void *q;
  int rc = balloc(b, &q, n * sizeof(T));
  *p = (T *)q;
  return rc;
}

// An allocation that may fail: out of memory is cleared and reported as false.
template <typename T>
bool try_talloc(fb_diff_batch *b, T **p, size_t n) {
  void *q = nullptr;
  *p = nullptr;
  if (cudaMalloc(&q, std::max<size_t>(n * sizeof(T), 16)) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b->allocs.push_back(q);
  *p = (T *)q;
  return true;
}

// Upload n elements of src (host or device), or reuse the copy made for the same pointer and field.
template <typename T>
int upload(fb_diff_batch *b, T **p, const void *src, size_t n, int field) {
  *p = nullptr;
  if (!src) return FB_OK;
  auto key = std::make_pair(src, field);
  auto it = b->shared.find(key);
  if (it != b->shared.end() && it->second.second == n * sizeof(T)) {
    *p = (T *)it->second.first;
    return FB_OK;
  }
  int rc = talloc(b, p, n);
  if (rc) return rc;
  DCU(cudaMemcpy(*p, src, n * sizeof(T), cudaMemcpyDefault));
  b->shared[key] = std::make_pair((void *)*p, n * sizeof(T));
  return FB_OK;
}

// Carves one allocation into aligned pieces.
struct Carver {
  size_t off = 0;
  std::vector<std::pair<void **, size_t>> items;
  template <typename T>
  void add(T **p, size_t n) {
    items.emplace_back((void **)p, off);
    off += (n * sizeof(T) + 255) / 256 * 256;
  }
  int commit(fb_diff_batch *b) {
    void *base;
    int rc = balloc(b, &base, off);
    if (rc) return rc;
    for (auto &it : items) *it.first = (char *)base + it.second;
    return FB_OK;
  }
};

// In-edges of every target in ascending edge id (a stable counting sort of the CSR by target).
int build_csc(fb_diff_batch *b, DiffDev &D) {
  auto it = b->csc.find(std::make_pair((const void *)D.indptr, (const void *)D.indices));
  if (it != b->csc.end()) {
    D.cscPtr = it->second[0];
    D.cscEdge = it->second[1];
    D.cscSrc = it->second[2];
    return FB_OK;
  }
  const int64_t N = D.N, E = D.E;
  std::vector<uint32_t> ip(N + 1), ix(E), cp(N + 1, 0), ce(E), cs(E);
  DCU(cudaMemcpy(ip.data(), D.indptr, (N + 1) * 4, cudaMemcpyDeviceToHost));
  if (E) DCU(cudaMemcpy(ix.data(), D.indices, E * 4, cudaMemcpyDeviceToHost));
  if (ip[0] != 0 || (int64_t)ip[N] != E)
    return dfail(FB_EINVAL, "fb_diff: indptr[0]=%u, indptr[N]=%u, E=%lld", ip[0], ip[N], (long long)E);
  for (int64_t i = 0; i < N; i++)
    if (ip[i + 1] < ip[i]) return dfail(FB_EINVAL, "fb_diff: indptr decreases at %lld", (long long)i);
  for (int64_t j = 0; j < E; j++)
    if (ix[j] >= (uint32_t)N) return dfail(FB_EINVAL, "fb_diff: indices[%lld]=%u >= N", (long long)j, ix[j]);
  for (int64_t j = 0; j < E; j++) cp[ix[j] + 1]++;
  for (int64_t q = 0; q < N; q++) cp[q + 1] += cp[q];
  std::vector<uint32_t> fill(cp.begin(), cp.end() - 1);
  for (int64_t s = 0; s < N; s++)
    for (uint32_t j = ip[s]; j < ip[s + 1]; j++) {
      const uint32_t o = fill[ix[j]]++;
      ce[o] = j;
      cs[o] = (uint32_t)s;
    }
  uint32_t *a, *e, *s;
  int rc;
  if ((rc = talloc(b, &a, N + 1)) || (rc = talloc(b, &e, E)) || (rc = talloc(b, &s, E))) return rc;
  DCU(cudaMemcpy(a, cp.data(), (N + 1) * 4, cudaMemcpyHostToDevice));
  if (E) {
    DCU(cudaMemcpy(e, ce.data(), E * 4, cudaMemcpyHostToDevice));
    DCU(cudaMemcpy(s, cs.data(), E * 4, cudaMemcpyHostToDevice));
  }
  b->csc[std::make_pair((const void *)D.indptr, (const void *)D.indices)] = {a, e, s};
  D.cscPtr = a;
  D.cscEdge = e;
  D.cscSrc = s;
  return FB_OK;
}

int create_instance(fb_diff_batch *b, Inst &I, const fb_diff_net *net, int64_t tape_cap) {
  DiffDev &D = I.D;
  memset(&D, 0, sizeof D);
  if (net->N <= 0 || net->E < 0 || !net->indptr || (net->E && (!net->indices || !net->counts)) || !net->sign ||
      net->nDriven < 0 || net->nDriven > net->N || (net->nDriven && (!net->driven || !net->drive)))
    return dfail(FB_EINVAL, "fb_diff: bad network description (N=%d E=%lld nDriven=%d)", net->N,
                 (long long)net->E, net->nDriven);
  const int64_t N = net->N, E = net->E;
  D.N = net->N;
  D.E = net->E;
  D.nDriven = net->nDriven;
  D.nTiles = (int32_t)((N + kDB - 1) / kDB);
  int rc;
  float *f;
#define UP(dst, src, n, fld, T)                           \
  do {                                                    \
    T *p_;                                                \
    if ((rc = upload(b, &p_, (src), (n), (fld)))) return rc; \
    dst = p_;                                             \
  } while (0)
  UP(D.indptr, net->indptr, N + 1, F_INDPTR, uint32_t);
  UP(D.indices, net->indices, E, F_INDICES, uint32_t);
  UP(D.counts, net->counts, E, F_COUNTS, float);
  UP(D.edgeGain, net->edge_gain, E, F_EDGE_GAIN, float);
  UP(D.sign, net->sign, N, F_SIGN, float);
  UP(D.outScale, net->out_scale, N, F_OUT_SCALE, float);
  UP(D.betaArr, net->beta, N, F_BETA, float);
  UP(D.biasArr, net->bias, N, F_BIAS, float);
  UP(D.thrMask, net->thr_mask, N, F_THR_MASK, uint8_t);
  UP(D.biasMask, net->bias_mask, N, F_BIAS_MASK, uint8_t);
  UP(I.inScaleSrc, net->in_scale, N, F_IN_SCALE, float);
  UP(I.sensory, net->sensory, N, F_SENSORY, uint8_t);
#undef UP
  if ((rc = build_csc(b, D))) return rc;
  // arrays that default to zeros get their own copy when not given (they can be set later)
  {
    std::vector<float> z(N, 0.f);
    auto own = [&](const float *src, int fld, const float **dst) -> int {
      float *p;
      int r = src ? upload(b, &p, src, N, fld) : talloc(b, &p, N);
      if (r) return r;
      if (!src) {
        DCU(cudaMemcpy(p, z.data(), N * 4, cudaMemcpyHostToDevice));
      }
      *dst = p;
      return FB_OK;
    };
    if ((rc = own(net->log_gain, F_LOG_GAIN, &D.logGain)) || (rc = own(net->thr_offset, F_THR_OFFSET, &D.thrOffset)))
      return rc;
    float *sl;
    if (net->size_log) {
      if ((rc = upload(b, &sl, net->size_log, N, F_SIZE_LOG))) return rc;
    } else if (b->zeros.count(N)) {
      sl = b->zeros[N];
    } else {  // sizeLog cannot be set later: instances of one size share a zero array
      if ((rc = talloc(b, &sl, N))) return rc;
      DCU(cudaMemcpy(sl, z.data(), N * 4, cudaMemcpyHostToDevice));
      b->zeros[N] = sl;
    }
    D.sizeLog = sl;
    I.sizeLogSrc = sl;
  }
  // the drive: validated on the host, one copy per instance
  {
    std::vector<float> dr(N, 0.f);
    std::vector<int32_t> dv(std::max<int32_t>(net->nDriven, 1), 0);
    if (net->nDriven) {
      DCU(cudaMemcpy(dv.data(), net->driven, 4 * (size_t)net->nDriven, cudaMemcpyDefault));
      DCU(cudaMemcpy(dr.data(), net->drive, 4 * (size_t)N, cudaMemcpyDefault));
      for (int32_t k = 0; k < net->nDriven; k++)
        if (dv[k] < 0 || dv[k] >= N) return dfail(FB_EINVAL, "fb_diff: driven[%d]=%d", k, dv[k]);
    }
    int32_t *dvD;
    if ((rc = talloc(b, &f, N)) || (rc = talloc(b, &dvD, dv.size()))) return rc;
    DCU(cudaMemcpy(f, dr.data(), N * 4, cudaMemcpyHostToDevice));
    DCU(cudaMemcpy(dvD, dv.data(), dv.size() * 4, cudaMemcpyHostToDevice));
    D.drive = f;
    D.driven = dvD;
    I.driven0.assign(dv.begin(), dv.begin() + net->nDriven);
  }
  // the schedule's columns (src/lifdiff.js:139-143): neuron -> the last driveIdx entry naming it
  if (net->nDriveIdx < 0 || (net->nDriveIdx > 0 && !net->drive_idx))
    return dfail(FB_EINVAL, "fb_diff: nDriveIdx=%d without drive_idx", net->nDriveIdx);
  if (net->nDriveIdx > 0) {
    I.driveIdx.resize(net->nDriveIdx);
    DCU(cudaMemcpy(I.driveIdx.data(), net->drive_idx, 4 * (size_t)net->nDriveIdx, cudaMemcpyDefault));
    std::vector<int32_t> slot(N, -1);
    for (int32_t k = 0; k < net->nDriveIdx; k++) {
      const int32_t i = I.driveIdx[k];
      if (i < 0 || i >= N) return dfail(FB_EINVAL, "fb_diff: drive_idx[%d]=%d", k, i);
      slot[i] = k;
    }
    int32_t *sl;
    if ((rc = talloc(b, &sl, N))) return rc;
    DCU(cudaMemcpy(sl, slot.data(), N * 4, cudaMemcpyHostToDevice));
    D.dSlot = sl;
  }
  if (net->thr_mask) {
    std::vector<uint8_t> m(N);
    DCU(cudaMemcpy(m.data(), net->thr_mask, N, cudaMemcpyDefault));
    for (int64_t i = 0; i < N && !I.thrMaskAny; i++) I.thrMaskAny = m[i] != 0;
  }
  // per-instance state, scratch, adjoint state and accumulators in one allocation
  D.ovfCap = (uint32_t)std::min<int64_t>(std::min<int64_t>(E + 1, (1 << 20) + E / 8), 0x7fffffff);
  D.tapeCap = tape_cap > 0 ? tape_cap : std::max<int64_t>(1 << 20, 64 * N);
  Carver c;
  c.add(&D.v, N); c.add(&D.gE, N); c.add(&D.gI, N); c.add(&D.adapt, N); c.add(&D.res, N);
  c.add(&D.refr, N); c.add(&D.spikeCount, N); c.add(&D.isForced, N); c.add(&D.rng, 1);
  c.add(&D.cnt, N); c.add(&D.bucket, N * kDBucket); c.add(&D.ovfHead, N); c.add(&D.ovfTop, 1);
  c.add(&D.ovf, D.ovfCap); c.add(&D.effK, N);
  c.add(&D.stage, (size_t)D.nTiles * kDB); c.add(&D.stageAmp, (size_t)D.nTiles * kDB);
  c.add(&D.tileCnt, (size_t)D.nTiles * (kDB / kWT));  // warp tiles of kWT neurons
  c.add(&D.lv, N); c.add(&D.lgE, N); c.add(&D.lgI, N); c.add(&D.lad, N); c.add(&D.lres, N);
  c.add(&D.accA, N); c.add(&D.accV, N); c.add(&D.accKc, N); c.add(&D.accLa, N); c.add(&D.accEI, N);
  c.add(&D.accW, N); c.add(&D.accD, N); c.add(&D.gLog, N); c.add(&D.gBias, N); c.add(&D.gEdge, E);
  c.add(&D.gLogF, N); c.add(&D.gOut, N); c.add(&D.nonfinite, 2);
  c.add(&D.tIdx, D.tapeCap); c.add(&D.tAmp, D.tapeCap);
  c.add(&D.drivenLive, N); c.add(&D.nLive, 1); c.add(&D.rmFlag, N); c.add(&D.claim, N);
  if ((rc = c.commit(b))) return rc;
  DCU(cudaMemset(D.rmFlag, 0, N));
  DCU(cudaMemset(D.claim, 0x7f, N * 4));  // kClaimFree in every word
  DCU(cudaMemset(D.ovfTop, 0, 4));
  DCU(cudaMemset(D.cnt, 0, N * 4));
  DCU(cudaMemset(D.ovfHead, 0xff, N * 4));
  D.err = b->err;
  D.jump = b->jump;
  return FB_OK;
}

// Edge groups: instances sharing graph, edge gains and input scaling share inScale/gate/P.
int build_groups(fb_diff_batch *b) {
  for (int k = 0; k < b->B; k++) {
    Inst &I = b->in[k];
    const void *key[5] = {I.D.indptr, I.D.edgeGain, I.sizeLogSrc, I.inScaleSrc, I.sensory};
    int g = -1;
    for (size_t q = 0; q < b->groups.size(); q++)
      if (!memcmp(b->groups[q].key, key, sizeof key)) g = (int)q;
    if (g < 0) {
      EdgeGroup G;
      memcpy(G.key, key, sizeof key);
      G.rep = k;
      const int64_t N = I.D.N, E = I.D.E;
      int rc;
      Carver c;
      c.add(&G.inScale, N); c.add(&G.gate, E); c.add(&G.P, E); c.add(&G.Pf, E);
      if ((rc = c.commit(b))) return rc;
      b->groups.push_back(G);
      g = (int)b->groups.size() - 1;
    }
    I.group = g;
    I.D.inScale = b->groups[g].inScale;
    I.D.gate = b->groups[g].gate;
    I.D.P = b->groups[g].P;
    I.D.Pf = b->groups[g].Pf;
  }
  return FB_OK;
}

template <typename R>
DP<R> typed_params(const fb_diff_params *p) {
  DP<R> q;
  q.dt = (R)p->dt; q.vRest = (R)p->vRest; q.vThresh = (R)p->vThresh; q.vReset = (R)p->vReset;
  q.tRef = (R)p->tRef; q.wSyn = (R)p->wSyn; q.adaptInc = (R)p->adaptInc; q.depU = (R)p->depU;
  q.eExc = (R)p->eExc; q.eInh = (R)p->eInh; q.inhGain = (R)p->inhGain; q.kcThreshold = (R)p->kcThreshold;
  q.laminaBias = (R)p->laminaBias; q.beta = (R)p->surrogateBeta; q.adjClip = (R)p->adjClip;
  q.dE = (R)std::exp(-p->dt / p->tauSyn);
  q.dA = (R)std::exp(-p->dt / p->adaptTau);
  q.kRec = (R)(p->dt / p->depTau);
  q.kM = (R)(p->dt / p->tauM);
  q.dtS = (R)(p->dt / 1000);
  q.cE = (R)(1 / (p->eExc - p->vRest));
  q.cI = (R)(1 / (p->vRest - p->eInh));
  q.xdt = (float)p->dt; q.xvRest = (float)p->vRest; q.xvThresh = (float)p->vThresh; q.xvReset = (float)p->vReset;
  q.xtRef = (float)p->tRef; q.xadaptInc = (float)p->adaptInc; q.xdepU = (float)p->depU; q.xeExc = (float)p->eExc;
  q.xeInh = (float)p->eInh; q.xlaminaBias = (float)p->laminaBias;
  q.xdE = (float)std::exp(-p->dt / p->tauSyn);
  q.xdA = (float)std::exp(-p->dt / p->adaptTau);
  q.xkRec = (float)(p->dt / p->depTau);
  q.xkM = (float)(p->dt / p->tauM);
  q.xdtS = (float)(p->dt / 1000);
  q.xcE = (float)(1 / (p->eExc - p->vRest));
  q.xcI = (float)(1 / (p->vRest - p->eInh));
  return q;
}

int fill_params(fb_diff_batch *b, const fb_diff_params *p) {
  if (!(p->dt > 0) || !(p->tauM > 0) || !(p->tauSyn > 0) || p->checkpoint <= 0)
    return dfail(FB_EINVAL, "fb_diff: dt, tauM, tauSyn and checkpoint must be positive");
  if (p->precision != FB_DIFF_F64 && p->precision != FB_DIFF_F32)
    return dfail(FB_EINVAL, "fb_diff: precision must be FB_DIFF_F64 or FB_DIFF_F32 (got %d)", p->precision);
  const int32_t nslots = (int32_t)std::max(1.0, std::floor(p->delay / p->dt + 0.5)) + 1;
  for (Inst &I : b->in) {
    if (I.D.nslots && I.D.nslots != nslots && I.D.lsRing) I.D.lsRing = nullptr;  // ring depth changed
    I.D.nslots = nslots;
    I.D.K = p->checkpoint;
    I.D.coba = p->coba ? 1 : 0;
    I.D.soft = p->soft ? 1 : 0;
    I.D.driveSoft = p->drive_soft ? 1 : 0;
    I.D.exact32 = p->exact32 ? 1 : 0;
    I.D.driveEpoch = std::max(1, p->drive_epoch);
    if (p->exact32 && I.thrMaskAny)
      return dfail(FB_EINVAL, "fb_diff: exact32 requires the full threshold field in thr_offset; thr_mask must be empty");
  }
  b->f32 = p->precision == FB_DIFF_F32;
  b->P64 = typed_params<double>(p);
  b->P32 = typed_params<float>(p);
  b->lastP = *p;
  return FB_OK;
}

int push_devs(fb_diff_batch *b) {
  std::vector<DiffDev> h(b->B);
  for (int k = 0; k < b->B; k++) h[k] = b->in[k].D;
  DCU(cudaMemcpyAsync(b->dDevs, h.data(), sizeof(DiffDev) * b->B, cudaMemcpyHostToDevice, b->st));
  DCU(cudaStreamSynchronize(b->st));
  return FB_OK;
}

int prepare(fb_diff_batch *b, const fb_diff_params *p) {
  for (const EdgeGroup &G : b->groups) {
    const Inst &I = b->in[G.rep];
    k_prepare<<<256, kDB, 0, b->st>>>(I.D.N, G.inScale, I.sizeLogSrc, I.inScaleSrc, p->sizeAlpha,
                                       p->maxSizeScale, p->boostCap);
    k_prepare_edges<<<1024, kDB, 0, b->st>>>(I.D.E, I.D.indices, I.D.counts, I.D.edgeGain, G.inScale, I.sensory,
                                              p->minSyn, G.gate, G.P, G.Pf);
  }
  DCU(cudaGetLastError());
  return FB_OK;
}

int check_err(fb_diff_batch *b, const char *fn) {
  int32_t err = 0;
  DCU(cudaMemcpyAsync(&err, b->err, 4, cudaMemcpyDeviceToHost, b->st));
  DCU(cudaStreamSynchronize(b->st));
  if (err) {
    cudaMemset(b->err, 0, 4);
    return dfail(err, "%s: %s", fn, err == FB_EOVERFLOW ? "tape or delivery scratch overflow" : "device error");
  }
  return FB_OK;
}

// Launch shapes: per-neuron kernels one tile per block for a single instance, about four waves of
// 256-thread blocks over the whole batch otherwise; warp-per-arrival kernels 304 blocks over the
// batch (at least two per instance).
dim3 neuron_grid(const fb_diff_batch *b) {
  if (b->tuneNeuron > 0) return dim3(std::min(b->maxTiles, b->tuneNeuron), b->B);
  const int gx = b->B == 1 ? b->maxTiles : std::max(1, std::min(b->maxTiles, 1216 / b->B));
  return dim3(gx, b->B);
}
dim3 arrival_grid(const fb_diff_batch *b) {
  if (b->tuneArrival > 0) return dim3(b->tuneArrival, b->B);
  return dim3(std::max(2, 304 / b->B), b->B);
}

// Stream ordering inside a pass: the first failure of an event record or wait is kept and
// reported by run_pass (the launches' own errors are read there too).
void order_note(fb_diff_batch *b, cudaError_t e) {
  if (e != cudaSuccess && b->orderErr == cudaSuccess) b->orderErr = e;
}
void ev_record(fb_diff_batch *b, cudaEvent_t ev, cudaStream_t st) { order_note(b, cudaEventRecord(ev, st)); }
void ev_wait(fb_diff_batch *b, cudaStream_t st, cudaEvent_t ev) { order_note(b, cudaStreamWaitEvent(st, ev, 0)); }

// One step on two streams. The side stream takes the step's forced spikes (after an epoch's drive
// edits) while the main stream delivers the step's arrivals: neither touches what the other
// reads or writes (the delivery reads the tape of step t - D and the presynaptic res and fills
// the buckets; the forced spikes write the refractory state, adaptation, spike counts and the
// head of step t's tape). The update waits for both. In a forward the side stream then writes
// the step's tape (k_emit) while the main stream goes on to the next step's delivery, which reads
// only older steps of the tape -- unless the delay is one step (two ring slots), when that
// delivery waits for the tape. The forced spikes of the next step wait for the tape (its offset).
template <typename R>
void run_step_t(fb_diff_batch *b, const DP<R> &P, int32_t t, int32_t replay, int32_t row, bool epoch) {
  ev_record(b, b->evFork, b->st);
  ev_wait(b, b->side, b->evFork);
  if (epoch) k_epoch<<<dim3(1, b->B), 1024, 0, b->side>>>(b->dDevs, t);
  k_forced<R><<<dim3(1, b->B), 1024, 0, b->side>>>(b->dDevs, P, t, replay);
  ev_record(b, b->evForced, b->side);
  if (!replay && t > 0 && b->in[0].D.nslots < 3) ev_wait(b, b->st, b->evEmitted);
  k_deliver<R><<<arrival_grid(b), kDB, 0, b->st>>>(b->dDevs, P, t, row);
  ev_wait(b, b->st, b->evForced);
  k_update<R><<<neuron_grid(b), kDB, 0, b->st>>>(b->dDevs, P, t, row);
  if (!replay) {
    ev_record(b, b->evUpdated, b->st);
    ev_wait(b, b->side, b->evUpdated);
    k_emit<<<dim3(1, b->B), 1024, 0, b->side>>>(b->dDevs, t);
    ev_record(b, b->evEmitted, b->side);
  }
}

// The side stream's work joins the main stream (the end of a pass that ran a step: the side
// stream takes part in a capture only once it has waited for the main stream).
void join_side(fb_diff_batch *b) {
  ev_record(b, b->evEmitted, b->side);
  ev_wait(b, b->st, b->evEmitted);
}

// Key of a captured pass: the pass kind and its integers, the launch shapes, the ring depth and
// the scalar parameters the kernels take by value. Every other input is in device memory, read
// when the graph runs.
struct PassKey {
  std::vector<uint8_t> v;
  template <typename T>
  PassKey &add(const T &x) {
    const uint8_t *q = (const uint8_t *)&x;
    v.insert(v.end(), q, q + sizeof(T));
    return *this;
  }
};
PassKey pass_key(const fb_diff_batch *b, char kind) {
  PassKey k;
  const dim3 ng = neuron_grid(b), ag = arrival_grid(b);
  // the ring depth shapes a forward's stream order (a one-step delay orders the tape before the
  // next delivery) and is not among the scalars below (it follows from delay / dt)
  k.add(kind).add(b->f32).add(ng.x).add(ng.y).add(ag.x).add(ag.y).add(b->in[0].D.nslots);
  // the typed parameters without the struct's trailing padding
  if (b->f32) {
    const uint8_t *q = (const uint8_t *)&b->P32;
    k.v.insert(k.v.end(), q, q + offsetof(DP<float>, xcI) + sizeof(float));
  } else {
    const uint8_t *q = (const uint8_t *)&b->P64;
    k.v.insert(k.v.end(), q, q + offsetof(DP<double>, xcI) + sizeof(float));
  }
  return k;
}

// Issues one pass's launch sequence on the batch's stream. By default the sequence is captured
// once into a CUDA graph under its key and every later pass with the same key replays it: one
// graph launch instead of several kernel launches per step. The graph holds kernel launches only
// (no copies, no host work), so a replay reads the members' current inputs. With step launches
// tuned on, the kernels are launched from the host step by step.
template <typename F>
int run_pass(fb_diff_batch *b, const PassKey &key, F issue, const char *fn) {
  b->orderErr = cudaSuccess;
  if (b->stepLaunches) {
    issue();
    DCU(cudaGetLastError());
    DCU(b->orderErr);
    return FB_OK;
  }
  for (PassGraph &g : b->graphs) {
    if (g.key == key.v) {
      g.used = ++b->graphTick;
      DCU(cudaGraphLaunch(g.exec, b->st));
      return FB_OK;
    }
  }
  cudaGraph_t graph = nullptr;
  DCU(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  issue();
  cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) le = b->orderErr;
  const cudaError_t ce = cudaStreamEndCapture(b->st, &graph);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return dfail(FB_ECUDA, "%s: capturing the pass failed: %s", fn, cudaGetErrorString(le != cudaSuccess ? le : ce));
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess)
    return dfail(ie == cudaErrorMemoryAllocation ? FB_ENOMEM : FB_ECUDA, "%s: instantiating the pass's graph failed: %s",
                 fn, cudaGetErrorString(ie));
  if (b->graphs.size() >= kPassGraphs) {
    auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                [](const PassGraph &x, const PassGraph &y) { return x.used < y.used; });
    cudaGraphExecDestroy(lru->exec);
    b->graphs.erase(lru);
  }
  b->graphs.push_back(PassGraph{key.v, exec, ++b->graphTick});
  DCU(cudaGraphLaunch(exec, b->st));
  return FB_OK;
}

void run_step(fb_diff_batch *b, int32_t t, int32_t replay, int32_t row, bool epoch = false) {
  if (b->f32) run_step_t<float>(b, b->P32, t, replay, row, epoch);
  else run_step_t<double>(b, b->P64, t, replay, row, epoch);
}

void reverse_step(fb_diff_batch *b, cudaStream_t st, int32_t t, int32_t row, int32_t scored) {
  if (b->f32) {
    k_bneuron<float><<<neuron_grid(b), kDB, 0, st>>>(b->dDevs, b->P32, t, row, scored);
    k_barrival<float><<<arrival_grid(b), kDB, 0, st>>>(b->dDevs, b->P32, t, row);
  } else {
    k_bneuron<double><<<neuron_grid(b), kDB, 0, st>>>(b->dDevs, b->P64, t, row, scored);
    k_barrival<double><<<arrival_grid(b), kDB, 0, st>>>(b->dDevs, b->P64, t, row);
  }
}

int set_readout(fb_diff_batch *b, Inst &I, int32_t nro, const int32_t *ro) {
  DiffDev &D = I.D;
  if (!I.roMap) {
    int rc = talloc(b, &I.roMap, D.N);
    if (rc) return rc;
  }
  std::vector<int32_t> h(nro);
  if (nro) DCU(cudaMemcpy(h.data(), ro, (size_t)nro * 4, cudaMemcpyDefault));
  if (D.roMap == I.roMap && h == I.roList) {  // the map already on the device
    D.nro = nro;
    return FB_OK;
  }
  std::vector<int32_t> map(D.N, -1);
  for (int32_t c = 0; c < nro; c++) {
    if (h[c] < 0 || h[c] >= D.N) return dfail(FB_EINVAL, "readout[%d]=%d out of range", c, h[c]);
    map[h[c]] = c;
  }
  DCU(cudaMemcpy(I.roMap, map.data(), (size_t)D.N * 4, cudaMemcpyHostToDevice));
  I.roList = std::move(h);
  D.roMap = I.roMap;
  D.nro = nro;
  return FB_OK;
}

// The drivenSet edits of every epoch boundary (src/lifdiff.js:207): setDriveOne(idx[k], at[e][k])
// in k order leaves the set it found minus the members it removed (the rest keep their order),
// plus the neurons it inserted, at the end in the order of their last insertion.
// list[off[2e] .. off[2e+1]) are epoch e's removals, list[off[2e+1] .. off[2e+2]) its appends.
int set_edits(int32_t N, const std::vector<int32_t> &driven0, const std::vector<int32_t> &idx, const float *at,
              int64_t nEp, std::vector<int32_t> &off, std::vector<int32_t> &list) {
  const int32_t nD = (int32_t)idx.size();
  std::vector<uint8_t> in(N, 0), startIn(N, 0), removed(N, 0);
  std::vector<int64_t> stamp(N, -1);
  std::vector<int32_t> key(N, -1), touched;
  std::vector<std::pair<int32_t, int32_t>> app;
  for (int32_t i : driven0) in[i] = 1;
  off.assign(2 * nEp + 1, 0);
  list.clear();
  for (int64_t e = 0; e < nEp; e++) {
    touched.clear();
    const float *row = at + e * nD;
    for (int32_t k = 0; k < nD; k++) {
      const int32_t i = idx[k];
      if (stamp[i] != e) {
        stamp[i] = e;
        startIn[i] = in[i];
        removed[i] = 0;
        key[i] = -1;
        touched.push_back(i);
      }
      if (row[k] > 0) {
        if (!in[i]) {
          in[i] = 1;
          key[i] = k;
        }
      } else if (in[i]) {
        in[i] = 0;
        key[i] = -1;
        if (startIn[i]) removed[i] = 1;
      }
    }
    for (int32_t i : touched)
      if (removed[i]) list.push_back(i);
    off[2 * e + 1] = (int32_t)list.size();
    app.clear();
    for (int32_t i : touched)
      if (in[i] && key[i] >= 0) app.emplace_back(key[i], i);
    std::sort(app.begin(), app.end());
    for (auto &a : app) list.push_back(a.second);
    if (list.size() > (size_t)INT32_MAX / 2)
      return dfail(FB_EINVAL, "fb_diff_forward: drive schedule edits exceed 2^30 entries");
    off[2 * e + 2] = (int32_t)list.size();
  }
  return FB_OK;
}

// Grows a per-instance device buffer to at least n elements.
template <typename T>
int grow(fb_diff_batch *b, T **p, int64_t *cap, int64_t n) {
  if (*p && *cap >= n) return FB_OK;
  int rc = talloc(b, p, (size_t)std::max<int64_t>(n, 1));
  if (rc) return rc;
  *cap = std::max<int64_t>(n, 1);
  return FB_OK;
}

// The schedule and spike train of one instance's forward (in may be null).
int set_inputs(fb_diff_batch *b, Inst &I, int32_t steps, const fb_diff_inputs *in) {
  DiffDev &D = I.D;
  const int64_t N = D.N;
  int rc;
  D.driveAt = nullptr;
  D.nDS = 0;
  D.epOff = D.epList = nullptr;
  D.trainOff = nullptr;
  D.trainIdx = nullptr;
  const int32_t nD = (int32_t)I.driveIdx.size();
  if (nD > 0) {
    // a drive schedule: the given one, else the drive as set held for every epoch (the values the
    // reference tapes when no onEpoch changes them), which only indexes the drive gradient
    const int32_t ep = D.driveEpoch;
    const int64_t nEp = std::max<int64_t>(1, ((int64_t)steps + ep - 1) / ep);
    std::vector<float> at((size_t)(nEp * nD));
    const bool given = in && in->drive_at;
    if (given) {
      DCU(cudaMemcpy(at.data(), in->drive_at, at.size() * 4, cudaMemcpyDefault));
    } else {
      std::vector<float> dr(N);
      DCU(cudaMemcpy(dr.data(), D.drive, N * 4, cudaMemcpyDeviceToHost));
      for (int64_t e = 0; e < nEp; e++)
        for (int32_t k = 0; k < nD; k++) at[e * nD + k] = dr[I.driveIdx[k]];
    }
    if ((rc = grow(b, &I.sched, &I.schedCap, nEp * nD))) return rc;
    DCU(cudaMemcpy(I.sched, at.data(), at.size() * 4, cudaMemcpyHostToDevice));
    D.driveAt = I.sched;
    D.nDS = nD;
    if (given) {
      std::vector<int32_t> off, list;
      if ((rc = set_edits(D.N, I.driven0, I.driveIdx, at.data(), nEp, off, list))) return rc;
      if ((rc = grow(b, &I.epOff, &I.epOffCap, (int64_t)off.size())) ||
          (rc = grow(b, &I.epList, &I.epListCap, (int64_t)list.size())))
        return rc;
      DCU(cudaMemcpy(I.epOff, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
      if (!list.empty()) DCU(cudaMemcpy(I.epList, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
      D.epOff = I.epOff;
      D.epList = I.epList;
    }
  } else if (in && in->drive_at) {
    return dfail(FB_EINVAL, "fb_diff_forward: a drive schedule needs drive_idx on the network");
  }
  if (in && in->train_off) {
    std::vector<int64_t> off(steps + 1);
    DCU(cudaMemcpy(off.data(), in->train_off, off.size() * 8, cudaMemcpyDefault));
    if (off[0] < 0) return dfail(FB_EINVAL, "fb_diff_forward: train_off[0]=%lld", (long long)off[0]);
    for (int32_t t = 0; t < steps; t++)
      if (off[t + 1] < off[t]) return dfail(FB_EINVAL, "fb_diff_forward: train_off decreases at step %d", t);
    const int64_t tot = off[steps];
    if (tot > 0 && !in->train_idx) return dfail(FB_EINVAL, "fb_diff_forward: train_off without train_idx");
    std::vector<int32_t> idx((size_t)std::max<int64_t>(tot, 1));
    if (tot > 0) DCU(cudaMemcpy(idx.data(), in->train_idx, tot * 4, cudaMemcpyDefault));
    for (int64_t q = off[0]; q < tot; q++)
      if (idx[q] < 0 || idx[q] >= N) return dfail(FB_EINVAL, "fb_diff_forward: train_idx[%lld]=%d", (long long)q, idx[q]);
    if ((rc = grow(b, &I.trainOff, &I.trainOffCap, steps + 1)) || (rc = grow(b, &I.trainIdx, &I.trainIdxCap, tot)))
      return rc;
    DCU(cudaMemcpy(I.trainOff, off.data(), off.size() * 8, cudaMemcpyHostToDevice));
    if (tot > 0) DCU(cudaMemcpy(I.trainIdx, idx.data(), tot * 4, cudaMemcpyHostToDevice));
    D.trainOff = I.trainOff;
    D.trainIdx = I.trainIdx;
  }
  if (D.exact32 && !D.W32) {
    if ((rc = talloc(b, &D.W32, std::max<int64_t>(D.E, 1))) || (rc = talloc(b, &D.signW32, N))) return rc;
  }
  return FB_OK;
}

uint32_t seed_state(uint32_t seed) {
  // (seed * 2654435761) >>> 0 || 1, the product in double (src/lifdiff.js:221)
  uint32_t s0 = (uint32_t)std::fmod(std::floor((double)seed * 2654435761.0), 4294967296.0);
  return s0 ? s0 : 1;
}

}  // namespace

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

extern "C" int fb_diff_batch_destroy(fb_diff_batch *b) {
  if (!b) return FB_OK;
  if (b->st) cudaStreamSynchronize(b->st);
  for (PassGraph &g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (void *p : b->allocs) cudaFree(p);
  if (b->side) cudaStreamSynchronize(b->side);
  if (b->rev) cudaStreamSynchronize(b->rev);
  for (cudaEvent_t e : {b->evFork, b->evForced, b->evUpdated, b->evEmitted, b->evRep[0], b->evRep[1], b->evRev[0],
                        b->evRev[1], b->evRevJoin})
    if (e) cudaEventDestroy(e);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->rev) cudaStreamDestroy(b->rev);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return FB_OK;
}

extern "C" int fb_diff_batch_create(const fb_diff_net *nets, int32_t B, int64_t tape_cap, fb_diff_batch **out) {
  if (!nets || !out || B <= 0) return dfail(FB_EINVAL, "fb_diff_batch_create: bad arguments (B=%d)", B);
  *out = nullptr;
  fb_diff_batch *b = new fb_diff_batch;
  b->B = B;
  b->in.resize(B);
  int rc;
  auto bail = [&](int r) {
    fb_diff_batch_destroy(b);
    return r;
  };
  std::vector<uint32_t> tab;
  host_jump_tables(tab);
  if ((rc = talloc(b, &b->err, 1)) || (rc = talloc(b, &b->jump, tab.size())) ||
      (rc = talloc(b, &b->partial, (size_t)B * kRB * kNSums)) || (rc = talloc(b, &b->dDevs, B)))
    return bail(rc);
  if (cudaMemcpy(b->jump, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(b->err, 0, 4) != cudaSuccess)
    return bail(dfail(FB_ECUDA, "fb_diff_batch_create: device setup failed"));
  for (int k = 0; k < B; k++) {
    if ((rc = create_instance(b, b->in[k], nets + k, tape_cap))) return bail(rc);
    b->maxTiles = std::max(b->maxTiles, b->in[k].D.nTiles);
    b->maxN = std::max(b->maxN, b->in[k].D.N);
  }
  if ((rc = build_groups(b))) return bail(rc);
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->rev, cudaStreamNonBlocking) != cudaSuccess)
    return bail(dfail(FB_ECUDA, "fb_diff_batch_create: stream creation failed"));
  for (cudaEvent_t *e : {&b->evFork, &b->evForced, &b->evUpdated, &b->evEmitted, &b->evRep[0], &b->evRep[1],
                         &b->evRev[0], &b->evRev[1], &b->evRevJoin})
    if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess)
      return bail(dfail(FB_ECUDA, "fb_diff_batch_create: event creation failed"));
  *out = b;
  return FB_OK;
}

extern "C" int fb_diff_batch_set_tuning(fb_diff_batch *b, const fb_diff_tuning *t) {
  if (!b || !t || t->neuron_blocks < 0 || t->arrival_blocks < 0 || t->arrival_blocks > 65535 ||
      (t->step_launches != 0 && t->step_launches != 1))
    return dfail(FB_EINVAL, "fb_diff_batch_set_tuning: bad arguments");
  b->tuneNeuron = t->neuron_blocks;
  b->tuneArrival = t->arrival_blocks;
  b->stepLaunches = t->step_launches;
  return FB_OK;
}

extern "C" int fb_diff_batch_set(fb_diff_batch *b, int32_t inst, int32_t field, const float *values) {
  if (!b || !values || inst < 0 || inst >= b->B) return dfail(FB_EINVAL, "fb_diff_set: bad arguments");
  const DiffDev &D = b->in[inst].D;
  const float *dst;
  size_t n = (size_t)D.N;
  switch (field) {
    case FB_DIFF_LOG_GAIN: dst = D.logGain; break;
    case FB_DIFF_OUT_SCALE: dst = D.outScale; break;
    case FB_DIFF_THR_OFFSET: dst = D.thrOffset; break;
    case FB_DIFF_BIAS: dst = D.biasArr; break;
    case FB_DIFF_EDGE_GAIN: dst = D.edgeGain; n = (size_t)D.E; break;
    case FB_DIFF_DRIVE: dst = D.drive; break;
    default: return dfail(FB_EINVAL, "fb_diff_set: unknown field %d", field);
  }
  if (!dst) return dfail(FB_ESTATE, "fb_diff_set: field %d was not given at creation", field);
  DCU(cudaMemcpyAsync((void *)dst, values, n * 4, cudaMemcpyDefault, b->st));
  DCU(cudaStreamSynchronize(b->st));
  return FB_OK;
}

extern "C" int fb_diff_batch_forward(fb_diff_batch *b, const fb_diff_params *p, const int32_t *steps,
                                     const uint32_t *seeds, int32_t record, float *spike_counts) {
  return fb_diff_batch_forward_ex(b, p, steps, seeds, record, spike_counts, nullptr);
}

extern "C" int fb_diff_batch_forward_ex(fb_diff_batch *b, const fb_diff_params *p, const int32_t *steps,
                                        const uint32_t *seeds, int32_t record, float *spike_counts,
                                        const fb_diff_inputs *in) {
  if (!b || !p || !steps || !seeds) return dfail(FB_EINVAL, "fb_diff_forward: bad arguments");
  int rc = fill_params(b, p);
  if (rc) return rc;
  int32_t maxSteps = 0;
  for (int k = 0; k < b->B; k++) {
    if (steps[k] < 0) return dfail(FB_EINVAL, "fb_diff_forward: steps[%d]=%d", k, steps[k]);
    maxSteps = std::max(maxSteps, steps[k]);
  }
  b->recorded = 0;  // the previous tape is gone once this forward starts writing
  for (int k = 0; k < b->B; k++) {
    Inst &I = b->in[k];
    DiffDev &D = I.D;
    const int64_t N = D.N;
    D.steps = steps[k];
    D.seed0 = seed_state(seeds[k]);
    if (record) {
      const int64_t nck = std::max<int64_t>(1, (steps[k] + D.K - 1) / D.K);
      if (nck > I.ckptCap) {
        if ((rc = talloc(b, &D.ckpt, (size_t)nck * 6 * N)) || (rc = talloc(b, &D.ckptRng, (size_t)nck))) return rc;
        I.ckptCap = nck;
      }
    }
    if (steps[k] + 1 > I.tStepsCap || !D.tOff) {
      const int64_t cap = std::max<int64_t>(steps[k] + 1, 2);
      if ((rc = talloc(b, &D.tOff, cap)) || (rc = talloc(b, &D.tForced, cap))) return rc;
      I.tStepsCap = cap;
    }
    if ((rc = set_inputs(b, I, steps[k], in ? in + k : nullptr))) return rc;
    // soft spikes (src/lifdiff.js:335-340) deliver every neuron above 1e-4 every step, so one step
    // can deliver a contribution over every edge: the overflow pool then needs E entries (a
    // neuron arrives at most once per step, so no step delivers more)
    if (p->soft && (int64_t)D.ovfCap < D.E + 1 && D.E + 1 <= 0x7fffffff) {
      DOvf *o = nullptr;
      if ((rc = talloc(b, &o, (size_t)(D.E + 1)))) return rc;
      D.ovf = o;
      D.ovfCap = (uint32_t)(D.E + 1);
    }
    // and record up to one entry per neuron and step (a neuron spikes at most once a step)
    if (p->soft && record && D.tapeCap < (int64_t)steps[k] * N) {
      int32_t *ti = nullptr;
      float *ta = nullptr;
      const int64_t cap = (int64_t)steps[k] * N;
      if ((rc = talloc(b, &ti, (size_t)cap)) || (rc = talloc(b, &ta, (size_t)cap))) return rc;
      D.tIdx = ti;
      D.tAmp = ta;
      D.tapeCap = cap;
    }
  }
  bool edits = false;
  for (int k = 0; k < b->B; k++) edits = edits || b->in[k].D.epOff;
  if ((rc = push_devs(b)) || (rc = prepare(b, p))) return rc;
  if (p->exact32) {
    k_prepare_w32<<<dim3(256, b->B), kDB, 0, b->st>>>(b->dDevs, p->wSyn, p->inhGain);
    DCU(cudaGetLastError());
  }
  const int32_t ep = std::max(1, p->drive_epoch);
  const float vRest = (float)p->vRest;
  const int32_t ck = p->checkpoint;
  PassKey key = pass_key(b, 'F');
  key.add(maxSteps).add(record).add(ck).add(edits).add(ep).add(vRest);
  rc = run_pass(b, key, [&] {
    k_reset<<<neuron_grid(b), kDB, 0, b->st>>>(b->dDevs, vRest);
    for (int32_t t = 0; t < maxSteps; t++) {
      if (record && t % ck == 0) k_ckpt<<<neuron_grid(b), kDB, 0, b->st>>>(b->dDevs, t, 1);
      run_step(b, t, 0, -1, edits && t % ep == 0);
    }
    if (maxSteps > 0) join_side(b);
  }, "fb_diff_forward");
  if (rc) return rc;
  if ((rc = check_err(b, "fb_diff_forward"))) return rc;
  if (spike_counts) {
    int64_t o = 0;
    for (int k = 0; k < b->B; k++) {
      DCU(cudaMemcpyAsync(spike_counts + o, b->in[k].D.spikeCount, (size_t)b->in[k].D.N * 4, cudaMemcpyDefault, b->st));
      o += b->in[k].D.N;
    }
    DCU(cudaStreamSynchronize(b->st));
  }
  b->recorded = record ? 1 : 0;
  b->recordedK = p->checkpoint;
  b->maxSteps = maxSteps;
  for (int k = 0; k < b->B; k++) b->in[k].recordedSteps = record ? steps[k] : 0;
  return FB_OK;
}

extern "C" int fb_diff_batch_tape(fb_diff_batch *b, int32_t inst, int64_t *offsets, int32_t *idx, float *amp,
                                  int64_t cap, int64_t *len) {
  if (!b || inst < 0 || inst >= b->B) return dfail(FB_EINVAL, "fb_diff_tape: bad arguments");
  if (!b->recorded) return dfail(FB_ESTATE, "fb_diff_tape: no recorded forward pass");
  const Inst &I = b->in[inst];
  const int32_t steps = I.recordedSteps;
  std::vector<int64_t> off(steps + 1);
  DCU(cudaMemcpy(off.data(), I.D.tOff, (size_t)(steps + 1) * 8, cudaMemcpyDeviceToHost));
  if (len) *len = off[steps];
  if (offsets) memcpy(offsets, off.data(), (size_t)(steps + 1) * 8);
  const int64_t n = std::min<int64_t>(cap, off[steps]);
  if (idx && n > 0) DCU(cudaMemcpy(idx, I.D.tIdx, n * 4, cudaMemcpyDefault));
  if (amp && n > 0) DCU(cudaMemcpy(amp, I.D.tAmp, n * 4, cudaMemcpyDefault));
  return FB_OK;
}

extern "C" int fb_diff_batch_raster(fb_diff_batch *b, int32_t inst, int32_t nro, const int32_t *readout, float *out) {
  if (!b || inst < 0 || inst >= b->B || nro <= 0 || !readout || !out)
    return dfail(FB_EINVAL, "fb_diff_raster: bad arguments");
  if (!b->recorded) return dfail(FB_ESTATE, "fb_diff_raster: no recorded forward pass");
  Inst &I = b->in[inst];
  int rc = set_readout(b, I, nro, readout);
  if (rc || (rc = push_devs(b))) return rc;
  const int32_t steps = I.recordedSteps;
  if (steps == 0) return FB_OK;
  float *dev = nullptr;
  cudaPointerAttributes at;
  const bool onDev = cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  if (onDev) dev = out;
  else DCU(cudaMalloc(&dev, (size_t)steps * nro * 4));
  DCU(cudaMemsetAsync(dev, 0, (size_t)steps * nro * 4, b->st));
  k_raster<<<std::min(steps, 4096), 256, 0, b->st>>>(b->dDevs + inst, steps, dev);
  DCU(cudaGetLastError());
  DCU(cudaStreamSynchronize(b->st));
  if (!onDev) {
    DCU(cudaMemcpy(out, dev, (size_t)steps * nro * 4, cudaMemcpyDeviceToHost));
    cudaFree(dev);
  }
  return FB_OK;
}

extern "C" int fb_diff_batch_rasters(fb_diff_batch *b, const int32_t *nro, const int32_t *const *readout,
                                     float *const *out) {
  if (!b || !nro || !readout || !out) return dfail(FB_EINVAL, "fb_diff_rasters: null argument");
  if (!b->recorded) return dfail(FB_ESTATE, "fb_diff_rasters: no recorded forward pass");
  int rc;
  for (int k = 0; k < b->B; k++) {
    if (nro[k] <= 0 || !readout[k] || !out[k]) return dfail(FB_EINVAL, "fb_diff_rasters: bad readout %d", k);
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, out[k]) != cudaSuccess || at.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return dfail(FB_EINVAL, "fb_diff_rasters: out[%d] is not device memory", k);
    }
    if ((rc = set_readout(b, b->in[k], nro[k], readout[k]))) return rc;
  }
  if ((rc = push_devs(b))) return rc;  // one upload of the member records for every raster
  for (int k = 0; k < b->B; k++) {
    const int32_t steps = b->in[k].recordedSteps;
    if (steps == 0) continue;
    DCU(cudaMemsetAsync(out[k], 0, (size_t)steps * nro[k] * 4, b->st));
    k_raster<<<std::min(steps, 4096), 256, 0, b->st>>>(b->dDevs + k, steps, out[k]);
  }
  DCU(cudaGetLastError());
  DCU(cudaStreamSynchronize(b->st));
  return FB_OK;
}

extern "C" int fb_diff_batch_backward(fb_diff_batch *b, const float *const *dL, const int32_t *nro,
                                      const int32_t *const *readout, int32_t truncate, int32_t loss_from,
                                      fb_diff_grads *g) {
  if (!b || !dL || !g) return dfail(FB_EINVAL, "fb_diff_backward: null argument");
  if (!b->recorded) return dfail(FB_ESTATE, "fb_diff_backward: no recorded forward pass (record=1)");
  const int32_t K = b->recordedK;
  int rc = fill_params(b, &b->lastP);
  if (rc) return rc;
  int32_t bufs = 2;  // arena halves every member has
  for (int k = 0; k < b->B; k++) {
    Inst &I = b->in[k];
    DiffDev &D = I.D;
    const int64_t N = D.N, steps = I.recordedSteps;
    const int32_t m = nro ? nro[k] : 0;
    if (!dL[k]) return dfail(FB_EINVAL, "fb_diff_backward: dL[%d] missing", k);
    // the loss gradient: flat over N, or per step over a readout set
    const int64_t dLn = m > 0 ? std::max<int64_t>(steps * m, 1) : N;
    if (dLn > I.dLcap) {
      if ((rc = talloc(b, &I.dLbuf, dLn))) return rc;
      I.dLcap = dLn;
    }
    if (m > 0 ? steps * m > 0 : true) DCU(cudaMemcpyAsync(I.dLbuf, dL[k], (m > 0 ? steps * m : N) * 4, cudaMemcpyDefault, b->st));
    D.dL = I.dLbuf;
    if (m > 0) {
      if (!readout || !readout[k]) return dfail(FB_EINVAL, "fb_diff_backward: readout indices missing");
      if ((rc = set_readout(b, I, m, readout[k]))) return rc;
    } else {
      D.roMap = nullptr;
    }
    // arena and per-arrival res for one segment
    std::vector<int64_t> off(steps + 1);
    DCU(cudaMemcpy(off.data(), D.tOff, (size_t)(steps + 1) * 8, cudaMemcpyDeviceToHost));
    int64_t maxArr = 1;
    for (int64_t t = 0; t < steps; t++) {
      const int64_t e = t - (D.nslots - 1);
      if (e >= 0) maxArr = std::max<int64_t>(maxArr, off[e + 1] - off[e]);
    }
    // rows for two segments when they fit (a segment's replay then runs beside the reverse
    // sweep of the segment after it, each in its own half), for one otherwise
    if (I.arenaRows < 2 * (int64_t)K) {
      int64_t rows = 2 * (int64_t)K;
      uint8_t *raw = nullptr;
      if (!try_talloc(b, &raw, (size_t)21 * rows * N)) {
        rows = K;
        if (I.arenaRows < rows && (rc = talloc(b, &raw, (size_t)21 * rows * N))) return rc;
      }
      if (raw) {  // 5 float planes (v, gE, gI, adapt, spike) and the byte plane of modes
        const size_t plane = (size_t)rows * N;
        float *a = (float *)raw;
        D.aV = a;
        D.aGE = a + plane;
        D.aGI = a + 2 * plane;
        D.aAd = a + 3 * plane;
        D.aSp = a + 4 * plane;
        D.aMode = raw + 20 * plane;
        I.arenaRows = rows;
      }
    }
    int64_t rows = I.arenaRows >= 2 * (int64_t)K ? 2 * (int64_t)K : K;
    if (maxArr * rows > I.resAtCap) {
      float *r = nullptr;
      if (!try_talloc(b, &r, (size_t)(maxArr * rows))) {
        rows = K;
        if (maxArr * rows > I.resAtCap && (rc = talloc(b, &r, (size_t)(maxArr * rows)))) return rc;
      }
      if (r) {
        D.resAt = r;
        I.resAtCap = maxArr * rows;
      }
    }
    bufs = std::min<int32_t>(bufs, rows >= 2 * (int64_t)K ? 2 : 1);
    D.maxArr = maxArr;
    D.gDrive = nullptr;
    if (D.driveAt) {
      const int64_t nd = ((steps + D.driveEpoch - 1) / D.driveEpoch) * D.nDS;
      if ((rc = grow(b, &I.gDrive, &I.gDriveCap, nd))) return rc;
      D.gDrive = I.gDrive;
    }
    if (!D.lsRing) {
      if ((rc = talloc(b, &D.lsRing, (size_t)D.nslots * N))) return rc;
    }
    D.steps = (int32_t)steps;
  }
  if ((rc = push_devs(b))) return rc;
  const dim3 ng = neuron_grid(b);
  k_zero_adjoint<<<ng, kDB, 0, b->st>>>(b->dDevs);
  for (int k = 0; k < b->B; k++) DCU(cudaMemsetAsync(b->in[k].D.nonfinite, 0, 8, b->st));
  if ((rc = prepare(b, &b->lastP))) return rc;
  const int32_t steps = b->maxSteps;
  const int nseg = (steps + K - 1) / K;
  b->arenaBufs = bufs;
  PassKey key = pass_key(b, 'B');
  key.add(steps).add(K).add(truncate).add(loss_from).add(bufs);
  // Segments are replayed on the main stream (one after another: they share the forward state)
  // and swept in reverse on the reverse stream (one after another: they share the adjoint
  // state). With two arena halves, segment sg's replay writes half sg & 1 and may run while the
  // segment after it (sg + 1, the other half) is swept; it waits for the sweep of sg + 2, the
  // last reader of its half. A sweep reads only its half, the tape and the adjoint state, and
  // a replay touches none of these, so the two overlap. With one half, everything runs in order
  // on the main stream.
  rc = run_pass(b, key, [&] {
    for (int sg = nseg - 1; sg >= 0; sg--) {
      const int32_t from = sg * K, to = std::min(steps, from + K);
      const int32_t half = bufs == 2 ? (sg & 1) * K : 0;
      // replay the segment from its checkpoint (src/lifdiff.js:390-464)
      if (bufs == 2 && sg + 2 < nseg) ev_wait(b, b->st, b->evRev[sg & 1]);
      k_ckpt<<<ng, kDB, 0, b->st>>>(b->dDevs, from, 0);
      for (int32_t t = from; t < to; t++) run_step(b, t, 1, half + t - from);
      cudaStream_t rs = b->st;
      if (bufs == 2) {
        ev_record(b, b->evRep[sg & 1], b->st);
        ev_wait(b, b->rev, b->evRep[sg & 1]);
        rs = b->rev;
      }
      // reverse sweep of the segment (src/lifdiff.js:540-667)
      for (int32_t t = to - 1; t >= from; t--) {
        if (truncate > 0) k_truncate<<<ng, kDB, 0, rs>>>(b->dDevs, t, truncate);
        reverse_step(b, rs, t, half + t - from, t >= loss_from ? 1 : 0);
      }
      if (bufs == 2) ev_record(b, b->evRev[sg & 1], b->rev);
    }
    if (steps > 0) {
      join_side(b);
      if (bufs == 2) {
        ev_record(b, b->evRevJoin, b->rev);
        ev_wait(b, b->st, b->evRevJoin);
      }
    }
  }, "fb_diff_backward");
  if (rc) return rc;
  if ((rc = check_err(b, "fb_diff_backward"))) return rc;
  // fixed-order reductions of the scalar terms
  const fb_diff_params &P = b->lastP;
  k_reduce<<<dim3(kRB, b->B), kDB, 0, b->st>>>(b->dDevs, P.inhGain, P.sizeAlpha, P.boostCap, P.maxSizeScale,
                                                b->partial);
  k_finalize<<<ng, kDB, 0, b->st>>>(b->dDevs);
  DCU(cudaGetLastError());
  std::vector<double> part((size_t)b->B * kRB * kNSums);
  std::vector<int32_t> nonfin(2 * b->B);
  DCU(cudaMemcpyAsync(part.data(), b->partial, part.size() * 8, cudaMemcpyDeviceToHost, b->st));
  for (int k = 0; k < b->B; k++)
    DCU(cudaMemcpyAsync(&nonfin[2 * k], b->in[k].D.nonfinite, 8, cudaMemcpyDeviceToHost, b->st));
  DCU(cudaStreamSynchronize(b->st));
  for (int k = 0; k < b->B; k++) {
    const DiffDev &D = b->in[k].D;
    double s[kNSums] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int blk = 0; blk < kRB; blk++)
      for (int q = 0; q < kNSums; q++) s[q] += part[((size_t)k * kRB + blk) * kNSums + q];
    // src/lifdiff.js:75 order: wSyn sizeAlpha inhGain eInh vThresh kcThreshold laminaBias adaptInc depU
    double vals[9] = {s[0], s[7], s[8], s[1], s[2], s[3], s[4], s[5], s[6]};
    fb_diff_grads &G = g[k];
    G.clamped_params = 0;
    for (int q = 0; q < 9; q++) {
      if (!std::isfinite(vals[q])) { vals[q] = 0; G.clamped_params++; }
      G.params[q] = vals[q];
    }
    G.clamped_log_gain = nonfin[2 * k];
    G.clamped_drive = nonfin[2 * k + 1];
    if (G.drive && D.gDrive) {
      const int64_t nd = ((int64_t)(D.steps + D.driveEpoch - 1) / D.driveEpoch) * D.nDS;
      if (nd > 0) DCU(cudaMemcpyAsync(G.drive, D.gDrive, (size_t)nd * 4, cudaMemcpyDefault, b->st));
    }
    if (G.log_gain) DCU(cudaMemcpyAsync(G.log_gain, D.gLogF, (size_t)D.N * 4, cudaMemcpyDefault, b->st));
    if (G.out_scale) DCU(cudaMemcpyAsync(G.out_scale, D.gOut, (size_t)D.N * 8, cudaMemcpyDefault, b->st));
    if (G.bias) DCU(cudaMemcpyAsync(G.bias, D.gBias, (size_t)D.N * 8, cudaMemcpyDefault, b->st));
    if (G.edge && D.E) DCU(cudaMemcpyAsync(G.edge, D.gEdge, (size_t)D.E * 8, cudaMemcpyDefault, b->st));
  }
  DCU(cudaStreamSynchronize(b->st));
  return FB_OK;
}

extern "C" int fb_diff_batch_edge_sum(fb_diff_batch *b, int32_t n, const int32_t *insts, double *out) {
  if (!b || n <= 0 || !insts || !out) return dfail(FB_EINVAL, "fb_diff_batch_edge_sum: bad arguments");
  std::vector<const double *> ptrs(n);
  int64_t E = -1;
  for (int k = 0; k < n; k++) {
    if (insts[k] < 0 || insts[k] >= b->B) return dfail(FB_EINVAL, "fb_diff_batch_edge_sum: instance %d", insts[k]);
    const DiffDev &D = b->in[insts[k]].D;
    if (E >= 0 && D.E != E) return dfail(FB_EINVAL, "fb_diff_batch_edge_sum: instances differ in edge count");
    E = D.E;
    ptrs[k] = D.gEdge;
  }
  const double **dp;
  DCU(cudaMalloc(&dp, n * sizeof(double *)));
  cudaMemcpy(dp, ptrs.data(), n * sizeof(double *), cudaMemcpyHostToDevice);
  cudaPointerAttributes at;
  const bool onDev = cudaPointerGetAttributes(&at, out) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  double *dev = out;
  if (!onDev && cudaMalloc(&dev, std::max<int64_t>(E, 1) * 8) != cudaSuccess) {
    cudaFree(dp);
    return dfail(FB_ENOMEM, "fb_diff_batch_edge_sum: %lld edges", (long long)E);
  }
  k_edge_sum<<<1024, kDB, 0, b->st>>>(dp, n, E, dev);
  cudaError_t e = cudaStreamSynchronize(b->st);
  if (e == cudaSuccess && !onDev) e = cudaMemcpy(out, dev, E * 8, cudaMemcpyDeviceToHost);
  if (!onDev) cudaFree(dev);
  cudaFree(dp);
  if (e != cudaSuccess) return dfail(FB_ECUDA, "fb_diff_batch_edge_sum: %s", cudaGetErrorString(e));
  return FB_OK;
}

// ---- the single-network API: a batch of one -------------------------------------------------

extern "C" int fb_diff_create(const fb_diff_net *net, int64_t tape_cap, fb_diff **out) {
  if (!net || !out) return dfail(FB_EINVAL, "fb_diff_create: null argument");
  *out = nullptr;
  fb_diff_batch *b = nullptr;
  int rc = fb_diff_batch_create(net, 1, tape_cap, &b);
  if (rc) return rc;
  *out = new fb_diff;
  (*out)->b = b;
  return FB_OK;
}

extern "C" int fb_diff_destroy(fb_diff *d) {
  if (!d) return FB_OK;
  fb_diff_batch_destroy(d->b);
  delete d;
  return FB_OK;
}

extern "C" int fb_diff_set(fb_diff *d, int32_t field, const float *values) {
  if (!d) return dfail(FB_EINVAL, "fb_diff_set: null argument");
  return fb_diff_batch_set(d->b, 0, field, values);
}

extern "C" int fb_diff_forward(fb_diff *d, const fb_diff_params *p, int32_t steps, uint32_t seed, int32_t record,
                               float *spike_count) {
  if (!d || !p || steps < 0) return dfail(FB_EINVAL, "fb_diff_forward: bad arguments");
  return fb_diff_batch_forward_ex(d->b, p, &steps, &seed, record, spike_count, nullptr);
}

extern "C" int fb_diff_forward_ex(fb_diff *d, const fb_diff_params *p, int32_t steps, uint32_t seed, int32_t record,
                                  float *spike_count, const fb_diff_inputs *in) {
  if (!d || !p || steps < 0) return dfail(FB_EINVAL, "fb_diff_forward: bad arguments");
  return fb_diff_batch_forward_ex(d->b, p, &steps, &seed, record, spike_count, in);
}

extern "C" int fb_diff_tape(fb_diff *d, int64_t *offsets, int32_t *idx, float *amp, int64_t cap, int64_t *len) {
  if (!d) return dfail(FB_EINVAL, "fb_diff_tape: null argument");
  return fb_diff_batch_tape(d->b, 0, offsets, idx, amp, cap, len);
}

extern "C" int fb_diff_raster(fb_diff *d, int32_t nro, const int32_t *readout, float *out) {
  if (!d) return dfail(FB_EINVAL, "fb_diff_raster: null argument");
  return fb_diff_batch_raster(d->b, 0, nro, readout, out);
}

extern "C" int fb_diff_backward(fb_diff *d, const float *dL, int32_t nro, const int32_t *readout, int32_t truncate,
                                int32_t loss_from, fb_diff_grads *g) {
  if (!d || !dL || !g) return dfail(FB_EINVAL, "fb_diff_backward: null argument");
  return fb_diff_batch_backward(d->b, &dL, &nro, &readout, truncate, loss_from, g);
}
