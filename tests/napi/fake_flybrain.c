/* A stand-in for libflybrain's C ABI in the addon's host tests (no GPU): each call prints its
 * arguments, one line per call, and returns fixed results (a three-spike fired list, patterned
 * state fields); an index out of [0, N) makes the list setters fail with FB_EINVAL and a message.
 * Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "flybrain.h"

static char g_err[256] = "";
static int32_t g_N = 0;

const char *fb_last_error(void) { return g_err; }

void fb_default_params(fb_params *p) {
  memset(p, 0, sizeof *p);
  p->dt = 0.1;
  p->vRest = -52;
  p->vThresh = -45;
  p->vReset = -52;
  p->tauM = 20;
  p->tauSyn = 5;
  p->tRef = 2.2;
  p->delay = 1.8;
}

int fb_graph_create(int32_t N, int64_t E, const uint32_t *indptr, const uint32_t *indices, const float *weights,
                    const float *sign, fb_graph **out) {
  printf("graph_create N=%d E=%lld indptr_last=%u indices0=%u w0=%g sign0=%g\n", N, (long long)E, indptr[N],
         E ? indices[0] : 0u, E ? weights[0] : 0.f, sign[0]);
  g_N = N;
  *out = (fb_graph *)malloc(16);
  return FB_OK;
}

int fb_graph_destroy(fb_graph *g) {
  printf("graph_destroy\n");
  free(g);
  return FB_OK;
}

int fb_brains_create(const fb_graph *const *graphs, int32_t B, const fb_params *params, int32_t params_stride,
                     const uint32_t *seeds, fb_brains **out) {
  (void)graphs;
  printf("brains_create B=%d stride=%d dt=%g vThresh=%g tauM=%g bgRate=%g coba=%d seed=%u\n", B, params_stride,
         params->dt, params->vThresh, params->tauM, params->bgRate, params->coba, seeds[0]);
  *out = (fb_brains *)malloc(16);
  return FB_OK;
}

int fb_brains_destroy(fb_brains *br) {
  printf("brains_destroy\n");
  free(br);
  return FB_OK;
}

int fb_step(fb_brains *br, int32_t nsteps, int32_t *out_nfired) {
  (void)br;
  printf("step n=%d\n", nsteps);
  if (out_nfired) *out_nfired = 3;
  return FB_OK;
}

int fb_fired(fb_brains *br, int32_t b, int32_t *dst, int32_t cap, int32_t *n) {
  (void)br;
  static const int32_t list[3] = {7, 3, 5};
  printf("fired b=%d cap=%d\n", b, cap);
  for (int k = 0; k < 3 && k < cap; k++) dst[k] = list[k];
  *n = 3;
  return FB_OK;
}

static int list_call(const char *name, int32_t b, const int32_t *idx, const double *v, int32_t n) {
  printf("%s b=%d n=%d", name, b, n);
  for (int32_t k = 0; k < n; k++) printf(" %d:%g", idx[k], v[k]);
  printf("\n");
  for (int32_t k = 0; k < n; k++)
    if (idx[k] < 0 || idx[k] >= g_N) {
      snprintf(g_err, sizeof g_err, "%s: neuron %d out of range", name, idx[k]);
      return FB_EINVAL;
    }
  return FB_OK;
}

int fb_set_drive(fb_brains *br, int32_t b, const int32_t *idx, const double *hz, int32_t n) {
  (void)br;
  return list_call("set_drive", b, idx, hz, n);
}

int fb_set_bias(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  (void)br;
  return list_call("set_bias", b, idx, mv, n);
}

int fb_set_thr(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  (void)br;
  return list_call("set_thr", b, idx, mv, n);
}

int fb_pulse(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  (void)br;
  return list_call("pulse", b, idx, mv, n);
}

int fb_add_g(fb_brains *br, int32_t b, const int32_t *idx, const double *e, const double *i, int32_t n) {
  (void)br;
  printf("add_g b=%d n=%d %d:%g:%g\n", b, n, idx[0], e[0], i ? i[0] : 0.0);
  return FB_OK;
}

int fb_set_background(fb_brains *br, int32_t b, double rate_hz, double amp_mv) {
  (void)br;
  printf("set_background b=%d %g %g\n", b, rate_hz, amp_mv);
  return FB_OK;
}

int fb_set_params(fb_brains *br, int32_t b, const fb_params *params) {
  (void)br;
  printf("set_params b=%d dt=%g vThresh=%g tauM=%g bgRate=%g bgAmp=%g coba=%d\n", b, params->dt, params->vThresh,
         params->tauM, params->bgRate, params->bgAmp, params->coba);
  if (params->dt != 0.1) {
    snprintf(g_err, sizeof g_err, "fb_set_params: the ring depth would change");
    return FB_EINVAL;
  }
  return FB_OK;
}

int fb_reset(fb_brains *br, int32_t b) {
  (void)br;
  printf("reset b=%d\n", b);
  return FB_OK;
}

int fb_read(fb_brains *br, int32_t field, int32_t b, void *dst) {
  (void)br;
  printf("read field=%d b=%d\n", field, b);
  for (int32_t k = 0; k < g_N; k++) {
    if (field == FB_FIELD_SPIKECOUNT) ((uint32_t *)dst)[k] = (uint32_t)(100 * field + k);
    else ((float *)dst)[k] = (float)field + 0.5f * (float)k;
  }
  return FB_OK;
}
