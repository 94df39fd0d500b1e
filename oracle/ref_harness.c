/*
 * ORACLE -- test infrastructure only. Builds the reference kernel itself, src/wasm/lif.c, compiled
 * natively from where it lies in the reference tree (the include path is supplied by
 * oracle/Makefile; nothing of it is copied here) and exposes it through the same ob_* interface as
 * oracle/lifsim.c, so the tests can pin the restatement against the real thing and the CPU baseline
 * can time it. The header fill mirrors LIFWasm._writeHeader (src/lifwasm.js:55-68): the caller
 * passes the f32 constants already rounded from f64, and the arrays it lays out.
 */
#include "lif.c" /* the reference kernel: Brain, xs, lif_step */

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int32_t N, nslots, head, coba;
  float c[17];
  uint32_t rng;
  int32_t nDriven, nFired, lastSlot;
  float bgEvents, bgAmp, bgAcc, preInh;
} ob_hdr;

static void hdr_to_brain(const ob_hdr *h, Brain *b) {
  b->N = h->N; b->nslots = h->nslots; b->head = h->head; b->coba = h->coba;
  b->dt = h->c[0]; b->vRest = h->c[1]; b->vThresh = h->c[2]; b->vReset = h->c[3]; b->tRef = h->c[4];
  b->adaptInc = h->c[5]; b->depU = h->c[6]; b->dE = h->c[7]; b->dTr = h->c[8]; b->dA = h->c[9];
  b->kRec = h->c[10]; b->kM = h->c[11]; b->dtS = h->c[12]; b->eExc = h->c[13]; b->eInh = h->c[14];
  b->cE = h->c[15]; b->cI = h->c[16];
  b->rng = h->rng; b->nDriven = h->nDriven; b->nFired = h->nFired; b->lastSlot = h->lastSlot;
  b->bgEvents = h->bgEvents; b->bgAmp = h->bgAmp; b->bgAcc = h->bgAcc; b->preInh = h->preInh;
}

static void brain_to_hdr(const Brain *b, ob_hdr *h) {
  h->N = b->N; h->nslots = b->nslots; h->head = b->head; h->coba = b->coba;
  h->c[0] = b->dt; h->c[1] = b->vRest; h->c[2] = b->vThresh; h->c[3] = b->vReset; h->c[4] = b->tRef;
  h->c[5] = b->adaptInc; h->c[6] = b->depU; h->c[7] = b->dE; h->c[8] = b->dTr; h->c[9] = b->dA;
  h->c[10] = b->kRec; h->c[11] = b->kM; h->c[12] = b->dtS; h->c[13] = b->eExc; h->c[14] = b->eInh;
  h->c[15] = b->cE; h->c[16] = b->cI;
  h->rng = b->rng; h->nDriven = b->nDriven; h->nFired = b->nFired; h->lastSlot = b->lastSlot;
  h->bgEvents = b->bgEvents; h->bgAmp = b->bgAmp; h->bgAcc = b->bgAcc; h->preInh = b->preInh;
}

void *ob_create(const ob_hdr *hdr, float *v, float *gE, float *gI, float *refr, float *trace,
                float *adapt, float *res, float *bias, float *thr, float *drive, float *sign,
                uint32_t *spikeCount, const uint32_t *indptr, const uint32_t *indices, const float *W,
                int32_t *ring, int32_t *ringCount, int32_t *driven) {
  Brain *b = (Brain *)calloc(1, sizeof(Brain));
  if (!b) return NULL;
  hdr_to_brain(hdr, b);
  b->v = v; b->gE = gE; b->gI = gI; b->refr = refr; b->trace = trace; b->adapt = adapt;
  b->res = res; b->bias = bias; b->thr = thr; b->drive = drive; b->sign = sign;
  b->spikeCount = spikeCount; b->indptr = indptr; b->indices = indices; b->weights = W;
  b->ring = ring; b->ringCount = ringCount; b->driven = driven;
  return b;
}

void ob_set(void *hb, const ob_hdr *hdr) { hdr_to_brain(hdr, (Brain *)hb); }
void ob_get(void *hb, ob_hdr *hdr) { brain_to_hdr((const Brain *)hb, hdr); }
void ob_destroy(void *hb) { free(hb); }

int32_t ob_run(void *hb, int32_t nsteps, int32_t *nfired, int32_t *raster, int64_t cap, int64_t *len) {
  Brain *b = (Brain *)hb;
  int64_t n = 0;
  int32_t nf = 0;
  for (int32_t t = 0; t < nsteps; t++) {
    nf = lif_step(b);
    if (nfired) nfired[t] = nf;
    if (raster) {
      const int32_t *out = b->ring + (int64_t)b->lastSlot * b->N;
      for (int32_t k = 0; k < nf; k++, n++)
        if (n < cap) raster[n] = out[k];
    } else {
      n += nf;
    }
  }
  if (len) *len = n;
  return nf;
}

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

/* B flyvis instances sharing the model, run by the reference's own fv_step (lif.c:86-93). */
void ob_fv_run(int32_t N, const float *bias, const float *kdt, const int32_t *indptr, const int32_t *target,
               const float *weight, int32_t B, float *v, const float *x, int32_t steps, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int32_t b = 0; b < B; b++) {
    float *acc = (float *)malloc((size_t)(N > 0 ? N : 1) * sizeof(float));
    for (int32_t s = 0; s < steps; s++)
      fv_step(N, bias, kdt, indptr, target, weight, v + (int64_t)b * N, acc, x + (int64_t)b * N);
    free(acc);
  }
}
