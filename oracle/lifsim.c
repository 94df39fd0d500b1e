/*
 * ORACLE -- test infrastructure only. Nothing in the product links or calls this file; only the
 * tests, the smoke check and bench.py's CPU-baseline leg load it (as the checker / the timed CPU
 * port). It is a CPU restatement of the reference brain step, src/wasm/lif.c:29-80, written from
 * that file's semantics, and it is pinned bit-for-bit against the reference lif.c itself (built by
 * oracle/Makefile into oracle/_ref/) on the golden cases under tests/golden/.
 *
 * Float semantics: every operation is a single IEEE binary32 operation in the reference's order.
 * Build with -ffp-contract=off -fno-fast-math (no FMA contraction, no reassociation).
 *
 * Interface (shared with oracle/ref_harness.c so the two are interchangeable from Python):
 *   ob_create(hdr, arrays...)  -> handle;   arrays are caller-owned, state is mutated in place
 *   ob_set(handle, hdr)  / ob_get(handle, hdr)   scalar header in / out
 *   ob_run(handle, nsteps, nfired[], raster[], cap, &len)   nsteps calls of the step
 *   ob_run_many(handles[], nb, steps[], nthreads)   independent brains over host threads (OpenMP)
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Scalar header. Field meaning follows the reference Brain header (src/wasm/lif.c:4-25) as
 * LIFWasm._writeHeader fills it (src/lifwasm.js:55-68). c[] holds the 17 f32 constants in the
 * header's order: dt vRest vThresh vReset tRef adaptInc depU dE dTr dA kRec kM dtS eExc eInh cE cI. */
typedef struct {
  int32_t N, nslots, head, coba;
  float c[17];
  uint32_t rng;
  int32_t nDriven, nFired, lastSlot;
  float bgEvents, bgAmp, bgAcc, preInh;
} ob_hdr;

enum { C_DT, C_VREST, C_VTH, C_VRESET, C_TREF, C_ADAPTINC, C_DEPU, C_DE, C_DTR, C_DA, C_KREC, C_KM,
       C_DTS, C_EEXC, C_EINH, C_CE, C_CI };

typedef struct {
  ob_hdr h;
  float *v, *gE, *gI, *refr, *trace, *adapt, *res, *bias, *thr, *drive, *sign;
  uint32_t *spikeCount;
  const uint32_t *indptr, *indices;
  const float *W;
  int32_t *ring, *ringCount, *driven;
} oracle_brain;

/* xorshift32 with shifts 13/17/5, as src/wasm/lif.c:27. */
static inline uint32_t rng_next(uint32_t *state) {
  uint32_t x = *state;
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  *state = x;
  return x;
}

/* Phase 1, src/wasm/lif.c:34-44: the arrival list of slot `head`, in list order; each arrival's
 * CSR row in CSR order; excitatory presynaptic amplitude into gE, inhibitory into gI. */
static void phase_deliver(oracle_brain *b) {
  ob_hdr *h = &b->h;
  const int32_t N = h->N;
  const int32_t *arr = b->ring + (int64_t)h->head * N;
  const int32_t na = b->ringCount[h->head];
  for (int32_t k = 0; k < na; k++) {
    const int32_t pre = arr[k];
    float amp = b->sign[pre] * b->res[pre];
    if (amp == 0.f) continue;
    if (h->preInh > 0.f && b->drive[pre] > 0.f) {
      const float inh = b->gI[pre] < 0.f ? -b->gI[pre] : 0.f;
      amp /= 1.f + h->preInh * inh;
    }
    b->res[pre] -= h->c[C_DEPU] * b->res[pre];
    const uint32_t lo = b->indptr[pre], hi = b->indptr[pre + 1];
    float *g = amp > 0 ? b->gE : b->gI;
    for (uint32_t j = lo; j < hi; j++) g[b->indices[j]] += b->W[j] * amp;
  }
  b->ringCount[h->head] = 0;
}

/* Phase 1b, src/wasm/lif.c:46-48: integer part of the accumulated background rate, one draw each. */
static void phase_background(oracle_brain *b) {
  ob_hdr *h = &b->h;
  h->bgAcc += h->bgEvents;
  const int32_t nbg = (int32_t)h->bgAcc;
  h->bgAcc -= nbg;
  for (int32_t k = 0; k < nbg; k++) {
    const uint32_t tgt = rng_next(&h->rng) % (uint32_t)h->N;
    b->gE[tgt] += h->bgAmp;
  }
}

/* Phase 2, src/wasm/lif.c:49-52: one uniform per non-refractory driven neuron, in list order. */
static int32_t phase_forced(oracle_brain *b, int32_t *out) {
  ob_hdr *h = &b->h;
  int32_t nf = 0;
  const float dtS = h->c[C_DTS];
  for (int32_t k = 0; k < h->nDriven; k++) {
    const int32_t i = b->driven[k];
    if (b->refr[i] > 0) continue;
    const float p = b->drive[i] * dtS;
    const float u = (float)(rng_next(&h->rng) >> 8) * (1.0f / 16777216.0f);
    if (u < p) {
      b->v[i] = h->c[C_VRESET];
      b->refr[i] = h->c[C_TREF] + h->c[C_DT];
      out[nf++] = i;
      b->spikeCount[i]++;
      b->trace[i] = 1.f;
      b->adapt[i] += h->c[C_ADAPTINC];
    }
  }
  return nf;
}

/* Phase 3, src/wasm/lif.c:53-72: membrane (current- or conductance-based) and all decays. */
static void phase_integrate(oracle_brain *b) {
  const ob_hdr *h = &b->h;
  const int32_t N = h->N;
  const float vRest = h->c[C_VREST], vReset = h->c[C_VRESET], kM = h->c[C_KM], dE = h->c[C_DE];
  const float dTr = h->c[C_DTR], dA = h->c[C_DA], kRec = h->c[C_KREC], dt = h->c[C_DT];
  const float eExc = h->c[C_EEXC], eInh = h->c[C_EINH], cE = h->c[C_CE], cI = h->c[C_CI];
  for (int32_t i = 0; i < N; i++) {
    float vi = b->v[i];
    const float r = b->refr[i];
    float acc = vRest - vi;
    if (h->coba) {
      acc = acc + b->gE[i] * (eExc - vi) * cE;
      acc = acc + b->gI[i] * (vi - eInh) * cI;
    } else {
      acc = acc + b->gE[i];
      acc = acc + b->gI[i];
    }
    acc = acc + b->bias[i];
    const float dv = acc * kM;
    vi = r > 0 ? vReset : vi + dv;
    b->refr[i] = r > 0 ? r - dt : r;
    b->v[i] = vi;
    b->gE[i] *= dE;
    b->gI[i] *= dE;
    b->trace[i] *= dTr;
    b->adapt[i] *= dA;
    b->res[i] += (1.f - b->res[i]) * kRec;
  }
}

/* Phase 4, src/wasm/lif.c:73-76: threshold against the decayed adapt, appended in ascending i. */
static int32_t phase_threshold(oracle_brain *b, int32_t *out, int32_t nf) {
  const ob_hdr *h = &b->h;
  const float vTh = h->c[C_VTH], vReset = h->c[C_VRESET], tRef = h->c[C_TREF];
  const float inc = h->c[C_ADAPTINC];
  for (int32_t i = 0; i < h->N; i++) {
    if (b->v[i] >= vTh + b->adapt[i] + b->thr[i] && b->refr[i] <= 0) {
      b->v[i] = vReset;
      b->refr[i] = tRef;
      out[nf++] = i;
      b->spikeCount[i]++;
      b->trace[i] = 1.f;
      b->adapt[i] += inc;
    }
  }
  return nf;
}

/* One step, src/wasm/lif.c:29-80, including the ring bookkeeping of :44-45 and :77-79. */
static int32_t brain_step(oracle_brain *b) {
  ob_hdr *h = &b->h;
  phase_deliver(b);
  const int32_t slot = (h->head + h->nslots - 1) % h->nslots;
  int32_t *out = b->ring + (int64_t)slot * h->N;
  phase_background(b);
  int32_t nf = phase_forced(b, out);
  phase_integrate(b);
  nf = phase_threshold(b, out, nf);
  b->ringCount[slot] = nf;
  h->lastSlot = slot;
  h->nFired = nf;
  h->head = (h->head + 1) % h->nslots;
  return nf;
}

void *ob_create(const ob_hdr *hdr, float *v, float *gE, float *gI, float *refr, float *trace,
                float *adapt, float *res, float *bias, float *thr, float *drive, float *sign,
                uint32_t *spikeCount, const uint32_t *indptr, const uint32_t *indices, const float *W,
                int32_t *ring, int32_t *ringCount, int32_t *driven) {
  oracle_brain *b = (oracle_brain *)calloc(1, sizeof(oracle_brain));
  if (!b) return NULL;
  b->h = *hdr;
  b->v = v; b->gE = gE; b->gI = gI; b->refr = refr; b->trace = trace; b->adapt = adapt;
  b->res = res; b->bias = bias; b->thr = thr; b->drive = drive; b->sign = sign;
  b->spikeCount = spikeCount; b->indptr = indptr; b->indices = indices; b->W = W;
  b->ring = ring; b->ringCount = ringCount; b->driven = driven;
  return b;
}

void ob_set(void *hb, const ob_hdr *hdr) { ((oracle_brain *)hb)->h = *hdr; }
void ob_get(void *hb, ob_hdr *hdr) { *hdr = ((oracle_brain *)hb)->h; }
void ob_destroy(void *hb) { free(hb); }

/* nsteps steps. nfired[t] (optional) receives each step's fired count; raster (optional) receives
 * the fired lists concatenated in ring order, up to cap entries (*len is the total needed). */
int32_t ob_run(void *hb, int32_t nsteps, int32_t *nfired, int32_t *raster, int64_t cap, int64_t *len) {
  oracle_brain *b = (oracle_brain *)hb;
  int64_t n = 0;
  int32_t nf = 0;
  for (int32_t t = 0; t < nsteps; t++) {
    nf = brain_step(b);
    if (nfired) nfired[t] = nf;
    if (raster) {
      const int32_t *out = b->ring + (int64_t)b->h.lastSlot * b->h.N;
      for (int32_t k = 0; k < nf; k++, n++)
        if (n < cap) raster[n] = out[k];
    } else {
      n += nf;
    }
  }
  if (len) *len = n;
  return nf;
}

/* Independent brains (one state block each, graphs may be shared read-only) over host threads:
 * the CPU counterpart of a batched ensemble, as brainsetup shares one graph across flies. */
int64_t ob_run_many(void **hbs, int32_t nb, const int32_t *steps, int32_t nthreads) {
  int64_t total = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
#endif
  for (int32_t k = 0; k < nb; k++) {
    int64_t n = 0;
    ob_run(hbs[k], steps[k], NULL, NULL, 0, &n);
    total += n;
  }
  return total;
}

int32_t ob_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- flyvis optic lobe (src/wasm/lif.c:82-93) ------------------------------------------------
 * The rate network lif.c's fv_step integrates: acc = sum over out-edges of the sources with
 * v > 0 of weight * v (sources in ascending order, each row in CSR order), then
 * v += kdt * (-v + bias + acc + x), every operation one f32 rounding in C order. */
static void fv_step_port(int32_t N, const float *bias, const float *kdt, const int32_t *indptr, const int32_t *target,
                         const float *weight, float *v, float *acc, const float *x) {
  for (int32_t i = 0; i < N; i++) acc[i] = 0.f;
  for (int32_t j = 0; j < N; j++) {
    const float r = v[j];
    if (r <= 0.f) continue;
    for (int32_t k = indptr[j]; k < indptr[j + 1]; k++) acc[target[k]] += weight[k] * r;
  }
  for (int32_t i = 0; i < N; i++) v[i] += kdt[i] * (-v[i] + bias[i] + acc[i] + x[i]);
}

/* B instances (eyes) sharing the model, each v[b*N ..], x[b*N ..], `steps` steps; instances run
 * in parallel over nthreads host threads (<= 0: the default). */
void ob_fv_run(int32_t N, const float *bias, const float *kdt, const int32_t *indptr, const int32_t *target,
               const float *weight, int32_t B, float *v, const float *x, int32_t steps, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int32_t b = 0; b < B; b++) {
    float *acc = (float *)malloc((size_t)(N > 0 ? N : 1) * sizeof(float));
    for (int32_t s = 0; s < steps; s++)
      fv_step_port(N, bias, kdt, indptr, target, weight, v + (int64_t)b * N, acc, x + (int64_t)b * N);
    free(acc);
  }
}
