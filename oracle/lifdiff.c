/*
 * ORACLE -- test infrastructure only. Only the tests and the benchmark's CPU leg load it, as the
 * checker; no product path calls it.
 *
 * A C restatement of the reference's differentiable LIF, LIFDiff (src/lifdiff.js): forward with a
 * spike tape and checkpoints (:219-353), segment replay (:390-464) and the reverse sweep
 * (:494-686). Arithmetic follows the JS exactly: every intermediate in double, every state array
 * float32 (a Float32Array store rounds the double once), operands in the JS order.
 *
 * Parity status: the reference runs under Node, which is absent here, so this restatement is not
 * pinned against the reference's own outputs; it is pinned by central finite differences of its
 * own soft forward pass with the tolerance of scripts/grad_check.mjs:98, and its hard forward is
 * checked against the reference kernel lif.c where the two models coincide (tests).
 *
 * Covered: conductance-based dynamics (the reference's) and a current-based variant (flag),
 * hard or soft (logistic) spikes, scalar or per-neuron surrogate beta, adaptation, depression,
 * inScale from sizeAlpha/sizeLog (or given), outScale, thrOffset, thrMask/kcThreshold,
 * biasMask/laminaBias, edgeGain, the minSyn/sensory gate, logGain, the Poisson drive (xorshift32,
 * drivenSet order), adjClip, truncation, lossFrom, a per-step dLoss/dspike (dLdSpike per step
 * generalises dLdSpikePerEpoch), driveSoft (:338, :453, :588-604), driveIdx/driveEpoch with the
 * drive held per epoch and its gradient (:134-144, :242-251, :407-412, :523-528, :572, :604),
 * spikeTrain replay (:298-306, :430-436) and exact32 (:172-190, :231-240, :256-275, :317-326).
 * The drive schedule is given as the values the reference's onEpoch callback would set: at every
 * epoch boundary, driveAt[epoch][k] is set for driveIdx[k] in k order (setDriveOne semantics).
 *
 * Beyond the reference's outputs (which it also computes here), the sweep accumulates:
 *   gEdge[j]  = dLoss/dW_j for the effective weight W_j = count*edgeGain*inScale[q](*inhGain) of
 *               gated edges (the summand of gInScale, :650/:654, before the count factor);
 *   gBias[i]  = sum over integrating steps of lu_i * kM (dLoss / d per-neuron bias; :614 sums it
 *               over the laminaBias neurons only);
 *   gOut[i]   = gLogGain[i] / outScale[i] (dLoss / d outScale_i, since eff is linear in it).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  /* model parameters (src/lifdiff.js:85-110) */
  double dt, vRest, vThresh, vReset, tauM, tauSyn, tRef, delay;
  double wSyn, adaptInc, adaptTau, depU, depTau, minSyn;
  double eExc, eInh, inhGain, sizeAlpha, maxSizeScale, boostCap;
  double kcThreshold, laminaBias, surrogateBeta, adjClip;
  int32_t coba, soft, checkpoint, truncate, lossFrom, steps;
  uint32_t seed;
  int32_t nDriven;
  int32_t driveSoft, exact32, driveEpoch, nDriveIdx;
} ld_params;

typedef struct {
  int32_t N;
  int64_t E;
  const uint32_t *indptr, *indices;
  const float *counts, *edgeGain;      /* per edge (edgeGain may be null) */
  const float *sign;                   /* per neuron, before wSyn */
  const float *sizeLog, *inScaleSrc;   /* inScaleSrc overrides the sizeAlpha formula (may be null) */
  const float *logGain, *outScale, *thrOffset, *beta;  /* outScale/beta may be null */
  const uint8_t *thrMask, *biasMask, *sensory;         /* may be null */
  const float *drive;                  /* per neuron, Hz */
  const int32_t *driven;               /* driven set in insertion order, nDriven entries */
  const int32_t *driveIdx;             /* neurons whose drive is an input (nDriveIdx) or null */
  const float *driveAt;                /* [epochs][nDriveIdx] drive schedule, or null */
  const int64_t *trainOff;             /* spikeTrain: per step offsets (steps + 1) or null */
  const int32_t *trainIdx;
} ld_graph;

typedef struct {
  double params[9]; /* wSyn sizeAlpha inhGain eInh vThresh kcThreshold laminaBias adaptInc depU */
  int32_t clamped_params, clamped_logGain;
  float *logGain;   /* N */
  double *gEdge;    /* E (optional) */
  double *gBias;    /* N (optional) */
  double *gOut;     /* N (optional) */
  float *gDrive;    /* [epochs][nDriveIdx] (optional) */
  int32_t clamped_drive, pad;
} ld_grads;

/* ---- the tape -------------------------------------------------------------------------------- */
typedef struct {
  int32_t *idx;
  float *amp;
  int64_t *off;   /* per step start; off[t+1] - off[t] spikes at step t */
  int32_t *nForced;
  int64_t cap, len;
  float *ckpt;    /* per checkpoint: v gE gI adapt res refr (6 N floats) */
  uint32_t *ckptSeed;
  int32_t nCkpt;
} ld_tape;

typedef struct {
  int32_t N, nslots;
  double dE, dA, kRec, kM, dtS, cE, cI;
  float *v, *gE, *gI, *adapt, *res, *refr, *spikeCount, *inScale;
  uint8_t *gate;
  uint32_t rng;
  /* the live drive (setDriveOne changes it) and the driven set in insertion order */
  float *drive;
  int32_t *driven, nDriven;
  uint8_t *inSet;
  /* exact32: writeGraph's two baked arrays (src/lifdiff.js:177-189) */
  float *W32, *signW32;
} ld_state;

static const double DRIVE_MAX = 0.999; /* src/lifdiff.js:72 */
static inline float F(double x) { return (float)x; }

/* setDriveOne (src/lifdiff.js:207): a Set keeps insertion order; delete then re-add appends. */
static void ld_set_drive(ld_state *S, int32_t i, float rate) {
  S->drive[i] = rate;
  if (rate > 0) {
    if (!S->inSet[i]) { S->driven[S->nDriven++] = i; S->inSet[i] = 1; }
  } else if (S->inSet[i]) {
    int32_t n = 0;
    for (int32_t k = 0; k < S->nDriven; k++)
      if (S->driven[k] != i) S->driven[n++] = S->driven[k];
    S->nDriven = n;
    S->inSet[i] = 0;
  }
}

static void ld_drive_init(const ld_params *p, const ld_graph *g, ld_state *S) {
  memcpy(S->drive, g->drive, (size_t)S->N * 4);
  memset(S->inSet, 0, (size_t)S->N);
  S->nDriven = 0;
  for (int32_t k = 0; k < p->nDriven; k++) {
    S->driven[S->nDriven++] = g->driven[k];
    S->inSet[g->driven[k]] = 1;
  }
}

static uint32_t ld_rand_u32(uint32_t *s) {
  uint32_t x = *s;
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  *s = x;
  return x;
}
/* src/lifdiff.js:212: top 24 bits scaled by 2^-24, as a double */
static double ld_rand(uint32_t *s) { return (double)(ld_rand_u32(s) >> 8) * (1.0 / 16777216.0); }

/* src/lifdiff.js:158-172: inScale and the gate */
static void ld_prepare(const ld_params *p, const ld_graph *g, ld_state *S) {
  for (int32_t i = 0; i < g->N; i++) {
    if (g->inScaleSrc) S->inScale[i] = g->inScaleSrc[i];
    else {
      const double s = exp(-p->sizeAlpha * (double)g->sizeLog[i]);
      const double lo = fmax(1.0 / p->maxSizeScale, s);
      S->inScale[i] = (float)fmin(p->boostCap, lo);
    }
  }
  for (int64_t j = 0; j < g->E; j++)
    S->gate[j] = ((double)g->counts[j] >= p->minSyn && !(g->sensory && g->sensory[g->indices[j]])) ? 1 : 0;
  if (p->exact32 && S->W32) {
    for (int32_t j = 0; j < g->N; j++) {
      const double sg = g->sign[j];
      S->signW32[j] = F(sg * p->wSyn);
      const double og = g->outScale ? (double)g->outScale[j] : 1.0, ig = (sg < 0 ? p->inhGain : 1.0) * og;
      for (uint32_t k = g->indptr[j]; k < g->indptr[j + 1]; k++)
        S->W32[k] = S->gate[k] ? F((double)g->counts[k] * (g->edgeGain ? (double)g->edgeGain[k] : 1.0) *
                                   (double)S->inScale[g->indices[k]] * ig)
                               : 0.f;
    }
  }
}

static void ld_reset(const ld_params *p, ld_state *S) {
  for (int32_t i = 0; i < S->N; i++) {
    S->v[i] = (float)p->vRest;
    S->gE[i] = S->gI[i] = S->adapt[i] = S->refr[i] = S->spikeCount[i] = 0.f;
    S->res[i] = 1.f;
  }
}

static inline double outs(const ld_graph *g, int32_t i) { return g->outScale ? (double)g->outScale[i] : 1.0; }
static inline double betaOf(const ld_params *p, const ld_graph *g, int32_t i) {
  return g->beta ? (double)g->beta[i] : p->surrogateBeta;
}
static inline double biasOf(const ld_params *p, const ld_graph *g, int32_t i) {
  return (g->biasMask && g->biasMask[i]) ? p->laminaBias : 0.0;
}
static inline double kcOf(const ld_params *p, const ld_graph *g, int32_t i) {
  return (g->thrMask && g->thrMask[i]) ? p->kcThreshold : 0.0;
}

/* the integration expression u (src/lifdiff.js:327, :445, :578); current-based variant: lif.c:67 */
static inline double ld_u(const ld_params *p, double vv, double gEv, double gIv, double bias, double kM,
                          double cE, double cI) {
  if (p->coba) return vv + (p->vRest - vv + gEv * (p->eExc - vv) * cE + gIv * (vv - p->eInh) * cI + bias) * kM;
  return vv + (p->vRest - vv + gEv + gIv + bias) * kM;
}

/* Delivery of one step's arrivals (src/lifdiff.js:276-283). resAt (optional) records res[pre]. */
static void ld_deliver(const ld_params *p, const ld_graph *g, ld_state *S, const int32_t *idx,
                       const float *amp, int64_t na, float *resAt, int ex) {
  const float dU = F(p->depU);
  for (int64_t k = 0; k < na; k++) {
    const int32_t pre = idx[k];
    if (ex) {  /* lif.c's factorization (src/lifdiff.js:256-272) */
      float sv = F((double)S->signW32[pre] * (double)S->res[pre]);
      if (amp[k] != 1.f) sv = F((double)sv * (double)amp[k]);
      if (sv == 0) continue;
      S->res[pre] = F((double)S->res[pre] - (double)dU * (double)S->res[pre]);
      const uint32_t a = g->indptr[pre], b = g->indptr[pre + 1];
      float *gg = sv > 0 ? S->gE : S->gI;
      for (uint32_t j = a; j < b; j++) {
        const float dlt = F((double)S->W32[j] * (double)sv);
        if (dlt != 0) gg[g->indices[j]] = F((double)gg[g->indices[j]] + (double)dlt);
      }
      continue;
    }
    const double sg = g->sign[pre];
    if (sg == 0) continue;
    if (resAt) resAt[k] = S->res[pre];
    const double eff = sg * p->wSyn * outs(g, pre) * exp((double)g->logGain[pre]) * (double)S->res[pre] * (double)amp[k];
    S->res[pre] = (float)((double)S->res[pre] - p->depU * (double)S->res[pre]);
    const uint32_t a = g->indptr[pre], b = g->indptr[pre + 1];
    if (eff > 0) {
      for (uint32_t j = a; j < b; j++)
        if (S->gate[j]) {
          const uint32_t q = g->indices[j];
          const double eg = g->edgeGain ? (double)g->edgeGain[j] : 1.0;
          S->gE[q] = (float)((double)S->gE[q] + (double)g->counts[j] * eg * (double)S->inScale[q] * eff);
        }
    } else {
      for (uint32_t j = a; j < b; j++)
        if (S->gate[j]) {
          const uint32_t q = g->indices[j];
          const double eg = g->edgeGain ? (double)g->edgeGain[j] : 1.0;
          S->gI[q] = (float)((double)S->gI[q] + (double)g->counts[j] * eg * (double)S->inScale[q] * p->inhGain * eff);
        }
    }
  }
}

/* Arena of one replayed segment (src/lifdiff.js:358-370). */
typedef struct {
  float *vPre, *gE, *gI, *adapt, *sp;
  uint8_t *mode;
  float *resAt;
  int64_t *resOff;
} ld_arena;

/* One forward step; fills the tape's list for step t (and the arena row when A is given).
 * forced (optional): the step's forced spikes taken from the tape instead of drawn (the replay).
 * ex: exact32 arithmetic (forward only; the replay is not exact32 in the reference either). */
static void ld_step(const ld_params *p, const ld_graph *g, ld_state *S, int32_t t, const int32_t *arrIdx,
                    const float *arrAmp, int64_t na, ld_arena *A, int32_t r, const int32_t *forced,
                    int32_t nForced, int32_t *outIdx, float *outAmp, int64_t *outN, int32_t *outForced,
                    uint8_t *isForced, int ex) {
  const int32_t N = S->N;
  const double dtS = S->dtS;
  /* lif.c reads its scalars from the f32 header: exact32 uses the rounded values (:232-240) */
  const double vR = ex ? F(p->vRest) : p->vRest, eE = ex ? F(p->eExc) : p->eExc, eI = ex ? F(p->eInh) : p->eInh,
               vTh = ex ? F(p->vThresh) : p->vThresh, vRs = ex ? F(p->vReset) : p->vReset,
               tRf = ex ? F(p->tRef) : p->tRef, aI = ex ? F(p->adaptInc) : p->adaptInc, dT = ex ? F(p->dt) : p->dt,
               lB = ex ? F(p->laminaBias) : p->laminaBias, dEp = ex ? F(S->dE) : S->dE, dAp = ex ? F(S->dA) : S->dA,
               kRp = ex ? F(S->kRec) : S->kRec, kMp = ex ? F(S->kM) : S->kM, dtSp = ex ? F(dtS) : dtS,
               cEp = ex ? F(S->cE) : S->cE, cIp = ex ? F(S->cI) : S->cI;
  ld_deliver(p, g, S, arrIdx, arrAmp, na, A ? A->resAt + A->resOff[r] : NULL, ex);
  int64_t n = 0;
  if (forced) {
    for (int32_t k = 0; k < nForced; k++) {
      const int32_t i = forced[k];
      S->refr[i] = (float)(p->tRef + p->dt);
      S->spikeCount[i] = (float)((double)S->spikeCount[i] + 1);
      S->adapt[i] = (float)((double)S->adapt[i] + p->adaptInc);
      outIdx[n] = i;
      outAmp[n] = 1.f;
      n++;
      isForced[i] = 1;
    }
  } else {
    /* exogenous drive, in drivenSet order (:290-297); none under driveSoft */
    if (!p->driveSoft)
      for (int32_t k = 0; k < S->nDriven; k++) {
        const int32_t i = S->driven[k];
        if (S->refr[i] > 0) continue;
        const double thrP = ex ? (double)F((double)S->drive[i] * dtSp) : (double)S->drive[i] * dtS;
        if (ld_rand(&S->rng) < thrP) {
          S->refr[i] = ex ? F(tRf + dT) : (float)(p->tRef + p->dt);
          outIdx[n] = i;
          outAmp[n] = 1.f;
          n++;
          S->spikeCount[i] = (float)((double)S->spikeCount[i] + 1);
          S->adapt[i] = (float)((double)S->adapt[i] + aI);
          if (isForced) isForced[i] = 1;
        }
      }
    /* spikeTrain: recorded spikes forced at their steps, no draw (:298-306) */
    if (g->trainOff)
      for (int64_t q = g->trainOff[t]; q < g->trainOff[t + 1]; q++) {
        const int32_t i = g->trainIdx[q];
        if (S->refr[i] > 0) continue;
        S->refr[i] = ex ? F(tRf + dT) : (float)(p->tRef + p->dt);
        outIdx[n] = i;
        outAmp[n] = 1.f;
        n++;
        S->spikeCount[i] = (float)((double)S->spikeCount[i] + 1);
        S->adapt[i] = (float)((double)S->adapt[i] + aI);
        if (isForced) isForced[i] = 1;
      }
  }
  *outForced = (int32_t)n;
  /* integrate and spike (:313-344); replay's bookkeeping (:439-458) */
  const int64_t off = (int64_t)r * N;
  for (int32_t i = 0; i < N; i++) {
    double vi = S->v[i], s = 0;
    int md = 0;
    if (A) {
      A->vPre[off + i] = S->v[i];
      A->gE[off + i] = S->gE[i];
      A->gI[off + i] = S->gI[i];
    }
    const int wasRefr = S->refr[i] > 0;
    if (wasRefr) {
      S->refr[i] = (float)((double)S->refr[i] - dT);
      vi = vRs;
      if (isForced && isForced[i]) { md = 2; s = 1; } else md = 1;
    } else if (ex) {
      /* lif.c's expression, one f32 rounding per C operation (:317-326); current-based: lif.c:67 */
      const double bias = biasOf(p, g, i) != 0 ? lB : 0.0;
      float acc = F(vR - vi);
      if (p->coba) {
        acc = F((double)acc + (double)F((double)F((double)S->gE[i] * (double)F(eE - vi)) * cEp));
        acc = F((double)acc + (double)F((double)F((double)S->gI[i] * (double)F(vi - eI)) * cIp));
      } else {
        acc = F((double)acc + (double)S->gE[i]);
        acc = F((double)acc + (double)S->gI[i]);
      }
      vi = F(vi + (double)F((double)F((double)acc + bias) * kMp));
    } else {
      vi = ld_u(p, vi, S->gE[i], S->gI[i], biasOf(p, g, i), S->kM, S->cE, S->cI);
    }
    S->gE[i] = (float)((double)S->gE[i] * dEp);
    S->gI[i] = (float)((double)S->gI[i] * dEp);
    S->adapt[i] = (float)((double)S->adapt[i] * dAp);
    S->res[i] = ex ? F((double)S->res[i] + (double)F((double)F(1 - (double)S->res[i]) * kRp))
                   : (float)((double)S->res[i] + (1 - (double)S->res[i]) * kRp);
    if (A) A->adapt[off + i] = S->adapt[i];
    if (!wasRefr) {
      const double thr = ex ? (double)F((double)F(vTh + (double)S->adapt[i]) + (double)g->thrOffset[i])
                            : p->vThresh + (double)S->adapt[i] + kcOf(p, g, i) + (double)g->thrOffset[i];
      s = p->soft ? 1 / (1 + exp(-(vi - thr) / betaOf(p, g, i))) : (vi >= thr ? 1 : 0);
      /* driveSoft: the drive's expected spike (:338, :453) */
      if (p->driveSoft && S->drive[i] > 0) {
        const double sd = fmin(DRIVE_MAX, (double)S->drive[i] * dtS);
        s = sd + (1 - sd) * s;
        md = 3;
      }
      if (s > 0) {
        vi = s * vRs + (1 - s) * vi;
        if (!p->soft) S->refr[i] = (float)tRf;
        S->adapt[i] = (float)((double)S->adapt[i] + s * aI);
      }
      S->spikeCount[i] = (float)((double)S->spikeCount[i] + s);
      if (s > (p->soft ? 1e-4 : 0.5)) {
        outIdx[n] = i;
        outAmp[n] = (float)s;
        n++;
      }
    }
    if (A) {
      A->mode[off + i] = (uint8_t)md;
      A->sp[off + i] = (float)s;
    }
    S->v[i] = (float)vi;
  }
  if (isForced)
    for (int64_t k = 0; k < *outForced; k++) isForced[outIdx[k]] = 0;
  *outN = n;
}

/* The drive the forward pass used at step t (:242-251, :407-412): at each epoch boundary (and at
 * the first step of a replayed segment) the schedule's values for driveIdx, in k order. */
static void ld_drive_epoch(const ld_params *p, const ld_graph *g, ld_state *S, int32_t t, int32_t segStart) {
  if (!g->driveAt || !g->driveIdx) return;
  const int32_t ep = p->driveEpoch > 1 ? p->driveEpoch : 1;
  if (!(t % ep == 0 || t == segStart)) return;
  const float *row = g->driveAt + (int64_t)(t / ep) * p->nDriveIdx;
  for (int32_t k = 0; k < p->nDriveIdx; k++) ld_set_drive(S, g->driveIdx[k], row[k]);
}

static void ld_consts(const ld_params *p, ld_state *S) {
  S->dE = exp(-p->dt / p->tauSyn);
  S->dA = exp(-p->dt / p->adaptTau);
  S->kRec = p->dt / p->depTau;
  S->kM = p->dt / p->tauM;
  S->dtS = p->dt / 1000;
  S->cE = 1 / (p->eExc - p->vRest);
  S->cI = 1 / (p->vRest - p->eInh);
}

/* ---- public: forward ------------------------------------------------------------------------- */

/* Runs the forward pass (src/lifdiff.js:219-353) for p->steps steps from reset. Outputs:
 * spikeCount[N] (float, may include soft amplitudes), the tape (spike lists, per-step offsets,
 * forced counts; capacity tapeCap entries) and checkpoints every p->checkpoint steps
 * (ckpt: nCkpt * 6N floats, ckptSeed: nCkpt). Returns the tape length, or -1 on overflow. */
int64_t ld_forward(const ld_params *p, const ld_graph *g, float *spikeCount, int32_t *tIdx,
                   float *tAmp, int64_t *tOff, int32_t *tForced, int64_t tapeCap, float *ckpt,
                   uint32_t *ckptSeed) {
  const int32_t N = g->N;
  ld_state S;
  memset(&S, 0, sizeof S);
  S.N = N;
  S.nslots = (int32_t)fmax(1.0, floor(p->delay / p->dt + 0.5)) + 1;
  ld_consts(p, &S);
  float *buf = (float *)calloc((size_t)N * 7, sizeof(float));
  S.v = buf; S.gE = buf + N; S.gI = buf + 2 * N; S.adapt = buf + 3 * N; S.res = buf + 4 * N;
  S.refr = buf + 5 * N; S.inScale = buf + 6 * N;
  S.spikeCount = spikeCount;
  S.gate = (uint8_t *)malloc((size_t)(g->E > 0 ? g->E : 1));
  S.drive = (float *)malloc((size_t)N * 4);
  S.driven = (int32_t *)malloc((size_t)N * 4);
  S.inSet = (uint8_t *)malloc((size_t)N);
  if (p->exact32) {
    S.W32 = (float *)malloc((size_t)(g->E > 0 ? g->E : 1) * 4);
    S.signW32 = (float *)malloc((size_t)N * 4);
  }
  uint8_t *isForced = (uint8_t *)calloc((size_t)N, 1);
  int32_t *oIdx = (int32_t *)malloc((size_t)N * 2 * sizeof(int32_t));
  float *oAmp = (float *)malloc((size_t)N * 2 * sizeof(float));
  ld_prepare(p, g, &S);
  ld_reset(p, &S);
  ld_drive_init(p, g, &S);
  S.rng = (uint32_t)fmod(floor((double)p->seed * 2654435761.0), 4294967296.0);
  if (!S.rng) S.rng = 1;
  int64_t len = 0;
  tOff[0] = 0;
  int32_t ck = 0;
  for (int32_t t = 0; t < p->steps; t++) {
    if (t % p->checkpoint == 0) {
      float *c = ckpt + (int64_t)ck * 6 * N;
      memcpy(c, S.v, N * 4); memcpy(c + N, S.gE, N * 4); memcpy(c + 2 * N, S.gI, N * 4);
      memcpy(c + 3 * N, S.adapt, N * 4); memcpy(c + 4 * N, S.res, N * 4); memcpy(c + 5 * N, S.refr, N * 4);
      ckptSeed[ck] = S.rng;
      ck++;
    }
    const int32_t e = t - (S.nslots - 1);  /* arrivals now were emitted at step e */
    const int32_t *aI = NULL;
    const float *aA = NULL;
    int64_t na = 0;
    if (e >= 0) { aI = tIdx + tOff[e]; aA = tAmp + tOff[e]; na = tOff[e + 1] - tOff[e]; }
    int64_t n = 0;
    int32_t nf = 0;
    ld_drive_epoch(p, g, &S, t, -1);
    ld_step(p, g, &S, t, aI, aA, na, NULL, 0, NULL, 0, oIdx, oAmp, &n, &nf, isForced, p->exact32);
    if (len + n > tapeCap) { len = -1; break; }
    memcpy(tIdx + len, oIdx, n * 4);
    memcpy(tAmp + len, oAmp, n * 4);
    len += n;
    tOff[t + 1] = len;
    tForced[t] = nf;
  }
  free(buf); free(S.gate); free(isForced); free(oIdx); free(oAmp);
  free(S.drive); free(S.driven); free(S.inSet); free(S.W32); free(S.signW32);
  return len;
}

/* ---- public: backward ------------------------------------------------------------------------ */

static inline double clip(double x, double c) { return c > 0 ? (x > c ? c : (x < -c ? -c : x)) : x; }

/* The reverse sweep (src/lifdiff.js:494-686) over the tape of ld_forward. dL: per step x N
 * dLoss/dspike (dLPerStep != 0) or one N vector for every step. Returns 0, or -1 on allocation
 * failure. */
int32_t ld_backward(const ld_params *p, const ld_graph *g, const int32_t *tIdx, const float *tAmp,
                    const int64_t *tOff, const int32_t *tForced, const float *ckpt,
                    const uint32_t *ckptSeed, const float *dL, int32_t dLPerStep, ld_grads *out) {
  const int32_t N = g->N, steps = p->steps, K = p->checkpoint;
  ld_state S;
  memset(&S, 0, sizeof S);
  S.N = N;
  S.nslots = (int32_t)fmax(1.0, floor(p->delay / p->dt + 0.5)) + 1;
  ld_consts(p, &S);
  const int32_t ns = S.nslots;
  const double dE = S.dE, dA = S.dA, kRec = S.kRec, kM = S.kM, cE = S.cE, cI = S.cI;
  float *buf = (float *)calloc((size_t)N * 8, sizeof(float));
  S.v = buf; S.gE = buf + N; S.gI = buf + 2 * N; S.adapt = buf + 3 * N; S.res = buf + 4 * N;
  S.refr = buf + 5 * N; S.inScale = buf + 6 * N; S.spikeCount = buf + 7 * N;
  S.gate = (uint8_t *)malloc((size_t)(g->E > 0 ? g->E : 1));
  S.drive = (float *)malloc((size_t)N * 4);
  S.driven = (int32_t *)malloc((size_t)N * 4);
  S.inSet = (uint8_t *)malloc((size_t)N);
  ld_prepare(p, g, &S);
  ld_drive_init(p, g, &S);
  /* the drive adjoint, per epoch and driveIdx entry (:523-528) */
  const int32_t ep = p->driveEpoch > 1 ? p->driveEpoch : 1, nD = g->driveAt ? p->nDriveIdx : 0;
  int32_t *dSlot = NULL;
  if (nD) {
    dSlot = (int32_t *)malloc((size_t)N * 4);
    for (int32_t i = 0; i < N; i++) dSlot[i] = -1;
    for (int32_t k = 0; k < nD; k++) dSlot[g->driveIdx[k]] = k;
  }
  float *gDrive = out->gDrive;
  const int32_t nEpochs = (steps + ep - 1) / ep;
  if (gDrive) memset(gDrive, 0, (size_t)nEpochs * (nD ? nD : 0) * 4);
  /* adjoint state (Float32Array in the reference) */
  float *lv = (float *)calloc(N, 4), *lgE = (float *)calloc(N, 4), *lgI = (float *)calloc(N, 4);
  float *lad = (float *)calloc(N, 4), *lres = (float *)calloc(N, 4);
  float *gInScale = (float *)calloc(N, 4), *gLogGain = (float *)calloc(N, 4);
  float *lsRing = (float *)calloc((size_t)ns * N, 4);
  double gW = 0, gInh = 0, gDep = 0, sAdaptInc = 0, sVThresh = 0, sKc = 0, sLamin = 0, sEInh = 0;
  /* arena for one segment */
  ld_arena A;
  A.vPre = (float *)malloc((size_t)K * N * 4); A.gE = (float *)malloc((size_t)K * N * 4);
  A.gI = (float *)malloc((size_t)K * N * 4); A.adapt = (float *)malloc((size_t)K * N * 4);
  A.sp = (float *)malloc((size_t)K * N * 4); A.mode = (uint8_t *)malloc((size_t)K * N);
  A.resOff = (int64_t *)malloc((size_t)(K + 1) * 8);
  int64_t maxArr = 0;
  for (int32_t t = 0; t < steps; t++) {
    const int32_t e = t - (ns - 1);
    if (e >= 0 && tOff[e + 1] - tOff[e] > maxArr) maxArr = tOff[e + 1] - tOff[e];
  }
  A.resAt = (float *)malloc((size_t)(maxArr * K + 1) * 4);
  uint8_t *isForced = (uint8_t *)calloc(N, 1);
  int32_t *oIdx = (int32_t *)malloc((size_t)N * 2 * 4);
  float *oAmp = (float *)malloc((size_t)N * 2 * 4);
  if (out->gEdge) memset(out->gEdge, 0, (size_t)g->E * 8);
  if (out->gBias) memset(out->gBias, 0, (size_t)N * 8);
  const double aClip = p->adjClip;
  const int nseg = (steps + K - 1) / K;
  for (int b = nseg - 1; b >= 0; b--) {
    const int32_t from = b * K, to = from + K < steps ? from + K : steps;
    /* replay (src/lifdiff.js:390-464), forced spikes taken from the tape */
    const float *c = ckpt + (int64_t)b * 6 * N;
    memcpy(S.v, c, N * 4); memcpy(S.gE, c + N, N * 4); memcpy(S.gI, c + 2 * N, N * 4);
    memcpy(S.adapt, c + 3 * N, N * 4); memcpy(S.res, c + 4 * N, N * 4); memcpy(S.refr, c + 5 * N, N * 4);
    S.rng = ckptSeed[b];
    A.resOff[0] = 0;
    for (int32_t t = from; t < to; t++) {
      const int32_t r = t - from, e = t - (ns - 1);
      const int32_t *aI = NULL;
      const float *aA = NULL;
      int64_t na = 0;
      if (e >= 0) { aI = tIdx + tOff[e]; aA = tAmp + tOff[e]; na = tOff[e + 1] - tOff[e]; }
      A.resOff[r + 1] = A.resOff[r] + na;
      int64_t n = 0;
      int32_t nf = 0;
      ld_drive_epoch(p, g, &S, t, from);
      ld_step(p, g, &S, t, aI, aA, na, &A, r, tIdx + tOff[t], tForced[t], oIdx, oAmp, &n, &nf, isForced, 0);
    }
    /* reverse steps of the segment */
    for (int32_t t = to - 1; t >= from; t--) {
      const int32_t r = t - from;
      const int64_t off = (int64_t)r * N;
      const int scored = t >= p->lossFrom;
      if (p->truncate > 0 && (t + 1) % p->truncate == 0) {
        memset(lv, 0, N * 4); memset(lgE, 0, N * 4); memset(lgI, 0, N * 4);
        memset(lad, 0, N * 4); memset(lres, 0, N * 4); memset(lsRing, 0, (size_t)ns * N * 4);
      }
      float *ls = lsRing + (int64_t)(t % ns) * N;
      const float *dLt = dLPerStep ? dL + (int64_t)t * N : dL;
      const int64_t dOff = (int64_t)(t / ep) * nD;
      for (int32_t i = 0; i < N; i++) {
        const int md = A.mode[off + i];
        const double lpA = lad[i];
        const double lE = (double)lgE[i] * dE, lI = (double)lgI[i] * dE, lA = lpA * dA, lR = (double)lres[i] * (1 - kRec);
        lgE[i] = (float)lE; lgI[i] = (float)lI; lad[i] = (float)lA; lres[i] = (float)lR;
        if (md == 1) { lv[i] = 0; continue; }
        if (md == 2) {
          /* the drive fired: its gradient takes ds/d(sd) = 1 (:565-573) */
          const double lspike2 = (double)ls[i] + (scored ? (double)dLt[i] : 0);
          sAdaptInc += lA;
          if (gDrive && dSlot[i] >= 0)
            gDrive[dOff + dSlot[i]] = (float)((double)gDrive[dOff + dSlot[i]] + (lA * p->adaptInc + lspike2) * S.dtS);
          lv[i] = 0;
          ls[i] = 0;
          continue;
        }
        const double vv = A.vPre[off + i], gEv = A.gE[off + i], gIv = A.gI[off + i];
        const double bias = biasOf(p, g, i);
        const double u = ld_u(p, vv, gEv, gIv, bias, kM, cE, cI);
        const double thr = p->vThresh + (double)A.adapt[off + i] + kcOf(p, g, i) + (double)g->thrOffset[i];
        const double d = u - thr;
        const double s = A.sp[off + i];
        /* a soft drive's composite amplitude split back into sd and the threshold's st (:587-591) */
        double sd = 0, st = s;
        if (md == 3) {
          const double rate = (dSlot && dSlot[i] >= 0) ? (double)g->driveAt[dOff + dSlot[i]] : (double)g->drive[i];
          sd = fmin(DRIVE_MAX, rate * S.dtS);
          st = (s - sd) / (1 - sd);
        }
        const double beta = betaOf(p, g, i);
        double sgr;
        if (p->soft) sgr = st * (1 - st) / beta;
        else { const double tt = 1 + fabs(d) / beta; sgr = 1 / (beta * tt * tt); }
        const double lspike = (double)ls[i] + (scored ? (double)dLt[i] : 0);
        const double lvNew = lv[i];
        const double lsTot = (p->vReset - u) * lvNew + lpA * p->adaptInc + lspike;
        const double lt = lsTot * (1 - sd) * sgr;
        const double lu = lvNew * (1 - s) + lt;
        const double lthr = -lt;
        if (gDrive && dSlot[i] >= 0)  /* through sd: ds/d(sd) = 1 - st, d(sd)/d(rate) = dt/1000 (:604) */
          gDrive[dOff + dSlot[i]] = (float)((double)gDrive[dOff + dSlot[i]] + lsTot * (1 - st) * S.dtS);
        sAdaptInc += lpA * s;
        sVThresh += lthr;
        if (g->thrMask && g->thrMask[i]) sKc += lthr;
        lad[i] = (float)(lA + lthr * dA);
        /* u = v + (vRest - v + gE (eExc - v) cE + gI (v - eInh) cI + bias) kM (:610-613);
           current-based: u = v + (vRest - v + gE + gI + bias) kM */
        if (p->coba) {
          lv[i] = (float)(lu * (1 + kM * (-1 - gEv * cE + gIv * cI)));
          lgE[i] = (float)(lE + lu * kM * (p->eExc - vv) * cE);
          lgI[i] = (float)(lI + lu * kM * (vv - p->eInh) * cI);
        } else {
          lv[i] = (float)(lu * (1 - kM));
          lgE[i] = (float)(lE + lu * kM);
          lgI[i] = (float)(lI + lu * kM);
        }
        if (bias != 0) sLamin += lu * kM;
        if (out->gBias) out->gBias[i] += lu * kM;
        if (p->coba) sEInh += lu * kM * gIv * cI * (-1 + (vv - p->eInh) * cI);
        ls[i] = 0;
      }
      if (aClip > 0)
        for (int32_t i = 0; i < N; i++) {
          lv[i] = (float)clip(lv[i], aClip); lgE[i] = (float)clip(lgE[i], aClip); lgI[i] = (float)clip(lgI[i], aClip);
          lad[i] = (float)clip(lad[i], aClip); lres[i] = (float)clip(lres[i], aClip);
        }
      /* reverse delivery (src/lifdiff.js:635-666) */
      const int32_t e = t - (ns - 1);
      if (e >= 0) {
        const int64_t ro = A.resOff[r];
        float *target = e >= 0 ? lsRing + (int64_t)(e % ns) * N : NULL;
        for (int64_t k = 0; k < tOff[e + 1] - tOff[e]; k++) {
          const int32_t pre = tIdx[tOff[e] + k];
          const double sgn = g->sign[pre], amp = tAmp[tOff[e] + k];
          if (sgn == 0) continue;
          const double resAtv = A.resAt[ro + k];
          const double gain = exp((double)g->logGain[pre]) * outs(g, pre);
          const double base = sgn * p->wSyn * gain * resAtv;
          const double eff = base * amp;
          const uint32_t a = g->indptr[pre], b2 = g->indptr[pre + 1];
          double lRaw = 0;
          if (eff > 0) {
            for (uint32_t j = a; j < b2; j++) {
              if (!S.gate[j]) continue;
              const uint32_t q = g->indices[j];
              const double cw = (double)g->counts[j] * (g->edgeGain ? (double)g->edgeGain[j] : 1.0);
              lRaw += (double)lgE[q] * cw * (double)S.inScale[q];
              gInScale[q] = (float)((double)gInScale[q] + (double)lgE[q] * cw * eff);
              if (out->gEdge) out->gEdge[j] += (double)lgE[q] * eff;
            }
          } else {
            const double ig = p->inhGain;
            for (uint32_t j = a; j < b2; j++) {
              if (!S.gate[j]) continue;
              const uint32_t q = g->indices[j];
              const double cw = (double)g->counts[j] * (g->edgeGain ? (double)g->edgeGain[j] : 1.0);
              lRaw += (double)lgI[q] * cw * (double)S.inScale[q] * ig;
              gInScale[q] = (float)((double)gInScale[q] + (double)lgI[q] * cw * ig * eff);
              gInh += (double)lgI[q] * cw * (double)S.inScale[q] * eff;
              if (out->gEdge) out->gEdge[j] += (double)lgI[q] * eff;
            }
          }
          gW += lRaw * sgn * gain * resAtv * amp;
          gLogGain[pre] = (float)((double)gLogGain[pre] + lRaw * eff);
          if (target) {
            target[pre] = (float)((double)target[pre] + lRaw * base);
            if (aClip > 0) target[pre] = (float)clip(target[pre], aClip);
          }
          const double lresAfter = lres[pre];
          gDep += -lresAfter * resAtv;
          lres[pre] = (float)(lresAfter * (1 - p->depU) + lRaw * sgn * p->wSyn * gain * amp);
          if (aClip > 0) lres[pre] = (float)clip(lres[pre], aClip);
        }
      }
    }
  }
  /* finalize (src/lifdiff.js:669-686) */
  double gSize = 0;
  for (int32_t i = 0; i < N; i++) {
    const double raw = exp(-p->sizeAlpha * (double)g->sizeLog[i]);
    if (raw < p->boostCap && raw > 1 / p->maxSizeScale)
      gSize += (double)gInScale[i] * (-(double)g->sizeLog[i]) * raw;
  }
  double vals[9] = {gW, gSize, gInh, sEInh, sVThresh, sKc, sLamin, sAdaptInc, gDep};
  out->clamped_params = out->clamped_logGain = 0;
  for (int k = 0; k < 9; k++) {
    if (!isfinite(vals[k])) { vals[k] = 0; out->clamped_params++; }
    out->params[k] = vals[k];
  }
  for (int32_t i = 0; i < N; i++) {
    float x = gLogGain[i];
    if (!isfinite(x)) { x = 0; out->clamped_logGain++; }
    out->logGain[i] = x;
    if (out->gOut) out->gOut[i] = (double)x / outs(g, i);
  }
  out->clamped_drive = 0;
  if (gDrive)
    for (int64_t k = 0; k < (int64_t)nEpochs * nD; k++)
      if (!isfinite(gDrive[k])) { gDrive[k] = 0; out->clamped_drive++; }
  free(S.drive); free(S.driven); free(S.inSet); free(dSlot);
  free(buf); free(S.gate); free(lv); free(lgE); free(lgI); free(lad); free(lres); free(gInScale);
  free(gLogGain); free(lsRing); free(A.vPre); free(A.gE); free(A.gI); free(A.adapt); free(A.sp);
  free(A.mode); free(A.resOff); free(A.resAt); free(isForced); free(oIdx); free(oAmp);
  return 0;
}
