/* Drives the LIFNative addon (fly-brain_gb300/napi/flybrain_napi.c) through the test Node-API
 * runtime, as JavaScript would.
 *
 *   driver marshal        scripted calls against the stand-in C ABI (fake_flybrain.c): every
 *                         method, getter and error path; prints what the addon returns or throws
 *   driver run IN OUT     a brain on the real libflybrain: the operations below on the graph and
 *                         inputs of IN, the fired lists and state written to OUT (the test
 *                         replays the same operations on the oracle)
 *
 * Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "flybrain.h"
#include "napi_runtime.h"

napi_value flybrain_napi_init(napi_env env, napi_value exports);

static napi_value load_class(void) {
  napi_value exports = rt_object();
  if (!flybrain_napi_init(rt_env(), exports)) {
    fprintf(stderr, "init failed\n");
    exit(2);
  }
  return rt_get(exports, "LIFNative");
}

/* ---- marshal ------------------------------------------------------------------------------ */

static void show(const char *what, napi_value r) {
  if (!r) {
    const char *m = rt_take_exception();
    printf("%s -> throws: %s\n", what, m ? m : "(no message)");
    return;
  }
  const int t = rt_typed_type(r);
  if (rt_is_object(r)) {
    printf("%s -> object\n", what);
    return;
  }
  if (t < 0) {
    const double x = rt_num(r);
    if (x == x) printf("%s -> %g\n", what, x);
    else printf("%s -> undefined\n", what);
    return;
  }
  const size_t n = rt_typed_len(r);
  printf("%s -> %s[%zu]", what, t == napi_int32_array ? "Int32Array" : t == napi_uint32_array ? "Uint32Array" : "Float32Array", n);
  for (size_t k = 0; k < n; k++) {
    if (t == napi_float32_array) printf(" %g", ((const float *)rt_typed_data(r))[k]);
    else if (t == napi_uint32_array) printf(" %u", ((const uint32_t *)rt_typed_data(r))[k]);
    else printf(" %d", ((const int32_t *)rt_typed_data(r))[k]);
  }
  printf("\n");
}

static int marshal(void) {
  napi_value cls = load_class();
  const uint32_t ip[5] = {0, 2, 3, 3, 4}, ix[4] = {1, 2, 3, 0};
  const float w[4] = {0.5f, 1.f, 2.f, -1.f}, sg[4] = {1.f, 1.f, -1.f, 1.f};
  napi_value opts = rt_object();
  show("new LIFNative()", rt_new(cls, 0, NULL));
  show("new LIFNative({})", rt_new(cls, 1, &opts));
  rt_set(opts, "N", rt_number(4));
  rt_set(opts, "indptr", rt_typed(napi_float32_array, w, 4));
  show("new LIFNative({N, indptr: Float32Array})", rt_new(cls, 1, &opts));
  rt_set(opts, "indptr", rt_typed(napi_uint32_array, ip, 5));
  rt_set(opts, "indices", rt_typed(napi_uint32_array, ix, 4));
  rt_set(opts, "weights", rt_typed(napi_float32_array, w, 4));
  rt_set(opts, "sign", rt_typed(napi_float32_array, sg, 4));
  napi_value params = rt_object();
  rt_set(params, "vThresh", rt_number(-40));
  rt_set(params, "tauM", rt_number(10));
  rt_set(params, "bgRate", rt_number(3));
  rt_set(params, "coba", rt_bool(true));
  rt_set(opts, "params", params);
  rt_set(opts, "seed", rt_number(1.5));
  show("new LIFNative({..., seed: 1.5})", rt_new(cls, 1, &opts));
  rt_set(opts, "seed", rt_number(7));
  napi_value b = rt_new(cls, 1, &opts);
  show("new LIFNative({...})", b);
  if (!b) return 1;
  show("N", rt_prop(b, "N"));
  show("nAwake", rt_prop(b, "nAwake"));
  show("step()", rt_call(b, "step", 0, NULL));
  napi_value a2[3];
  a2[0] = rt_number(2);
  a2[1] = rt_number(150);
  show("setDriveOne(2, 150)", rt_call(b, "setDriveOne", 2, a2));
  const int32_t l13[2] = {1, 3};
  a2[0] = rt_typed(napi_int32_array, l13, 2);
  a2[1] = rt_number(80);
  show("setDrive(Int32Array [1, 3], 80)", rt_call(b, "setDrive", 2, a2));
  const double l02[2] = {0, 2};
  a2[0] = rt_array(l02, 2);
  a2[1] = rt_number(0);
  show("setDrive([0, 2], 0)", rt_call(b, "setDrive", 2, a2));
  a2[0] = rt_number(3);
  a2[1] = rt_number(-1.5);
  show("setBias(3, -1.5)", rt_call(b, "setBias", 2, a2));
  a2[0] = rt_number(1);
  a2[1] = rt_number(2);
  show("setThr(1, 2)", rt_call(b, "setThr", 2, a2));
  a2[0] = rt_number(0);
  a2[1] = rt_number(0.25);
  show("addG(0, 0.25)", rt_call(b, "addG", 2, a2));
  a2[0] = rt_number(1);
  a2[1] = rt_number(0.5);
  a2[2] = rt_number(0.75);
  show("addG(1, 0.5, 0.75)", rt_call(b, "addG", 3, a2));
  const uint32_t l2[1] = {2};
  a2[0] = rt_typed(napi_uint32_array, l2, 1);
  a2[1] = rt_number(1);
  show("pulse(Uint32Array [2], 1)", rt_call(b, "pulse", 2, a2));
  a2[0] = rt_number(20);
  a2[1] = rt_number(1.5);
  show("setBackground(20, 1.5)", rt_call(b, "setBackground", 2, a2));
  a2[0] = rt_number(10);
  show("run(10)", rt_call(b, "run", 1, a2));
  show("t", rt_prop(b, "t"));
  show("v", rt_prop(b, "v"));
  show("spikeCount", rt_prop(b, "spikeCount"));
  napi_value q = rt_object();
  rt_set(q, "tauM", rt_number(12));
  rt_set(q, "coba", rt_bool(false));
  show("setParams({tauM: 12, coba: false})", rt_call(b, "setParams", 1, &q));
  rt_set(q, "dt", rt_number(0.5));
  show("setParams({dt: 0.5, ...})", rt_call(b, "setParams", 1, &q));
  a2[0] = rt_number(3);
  show("setParams(3)", rt_call(b, "setParams", 1, a2));
  show("wake()", rt_call(b, "wake", 0, NULL));
  show("flush()", rt_call(b, "flush", 0, NULL));
  show("reset()", rt_call(b, "reset", 0, NULL));
  show("t", rt_prop(b, "t"));
  const int32_t l9[1] = {9};
  a2[0] = rt_typed(napi_int32_array, l9, 1);
  a2[1] = rt_number(10);
  show("setDrive(Int32Array [9], 10)", rt_call(b, "setDrive", 2, a2));
  a2[0] = rt_bool(true);
  a2[1] = rt_number(10);
  show("setDriveOne(true, 10)", rt_call(b, "setDriveOne", 2, a2));
  const float lf[1] = {1.f};
  a2[0] = rt_typed(napi_float32_array, lf, 1);
  a2[1] = rt_number(1);
  show("setBias(Float32Array [1], 1)", rt_call(b, "setBias", 2, a2));
  show("run()", rt_call(b, "run", 0, NULL));
  show("destroy()", rt_call(b, "destroy", 0, NULL));
  show("dispose()", rt_call(b, "dispose", 0, NULL));
  show("step()", rt_call(b, "step", 0, NULL));
  show("v", rt_prop(b, "v"));
  rt_collect(b);
  printf("collected\n");
  return 0;
}

/* ---- run ---------------------------------------------------------------------------------- */

static FILE *g_in, *g_out;

static void rd(void *p, size_t n) {
  if (n && fread(p, 1, n, g_in) != n) {
    fprintf(stderr, "short input\n");
    exit(2);
  }
}

static void *rd_alloc(size_t n) {
  void *p = malloc(n ? n : 1);
  rd(p, n);
  return p;
}

static void wr(const void *p, size_t n) {
  if (n) fwrite(p, 1, n, g_out);
}

static napi_value must(napi_value r, const char *what) {
  if (!r) {
    const char *m = rt_take_exception();
    fprintf(stderr, "%s threw: %s\n", what, m ? m : "?");
    exit(3);
  }
  return r;
}

static void record_step(napi_value b) {
  napi_value r = must(rt_call(b, "step", 0, NULL), "step");
  const int32_t n = (int32_t)rt_typed_len(r);
  wr(&n, 4);
  wr(rt_typed_data(r), (size_t)n * 4);
}

static int run(const char *in, const char *out) {
  static const char *names[18] = {"dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "traceTau",
                                  "adaptInc", "adaptTau", "depU", "depTau", "eExc", "eInh", "bgRate", "bgAmp", "preInh"};
  g_in = fopen(in, "rb");
  g_out = fopen(out, "wb");
  if (!g_in || !g_out) return 2;
  int32_t N, seed, nD, nB, s1, s2, s3, s4, nP, addgI, thrI;
  int64_t E;
  double pv[19], biasMv, bgRate, bgAmp, pulseMv, addgE, thrMv;
  rd(&N, 4);
  rd(&E, 8);
  rd(&seed, 4);
  rd(pv, sizeof pv);
  uint32_t *ip = (uint32_t *)rd_alloc((size_t)(N + 1) * 4), *ix = (uint32_t *)rd_alloc((size_t)E * 4);
  float *w = (float *)rd_alloc((size_t)E * 4), *sg = (float *)rd_alloc((size_t)N * 4);
  rd(&nD, 4);
  int32_t *dIdx = (int32_t *)rd_alloc((size_t)nD * 4);
  double *dHz = (double *)rd_alloc((size_t)nD * 8);
  rd(&nB, 4);
  int32_t *bIdx = (int32_t *)rd_alloc((size_t)nB * 4);
  rd(&biasMv, 8);
  rd(&bgRate, 8);
  rd(&bgAmp, 8);
  rd(&s1, 4);
  rd(&s2, 4);
  rd(&s3, 4);
  rd(&s4, 4);
  rd(&nP, 4);
  int32_t *pIdx = (int32_t *)rd_alloc((size_t)nP * 4);
  rd(&pulseMv, 8);
  rd(&addgI, 4);
  rd(&addgE, 8);
  rd(&thrI, 4);
  rd(&thrMv, 8);

  napi_value cls = load_class(), opts = rt_object(), params = rt_object();
  rt_set(opts, "N", rt_number(N));
  rt_set(opts, "indptr", rt_typed(napi_uint32_array, ip, (size_t)N + 1));
  rt_set(opts, "indices", rt_typed(napi_uint32_array, ix, (size_t)E));
  rt_set(opts, "weights", rt_typed(napi_float32_array, w, (size_t)E));
  rt_set(opts, "sign", rt_typed(napi_float32_array, sg, (size_t)N));
  for (int k = 0; k < 18; k++) rt_set(params, names[k], rt_number(pv[k]));
  rt_set(params, "coba", rt_bool(pv[18] != 0));
  rt_set(opts, "params", params);
  rt_set(opts, "seed", rt_number(seed));
  napi_value b = must(rt_new(cls, 1, &opts), "new LIFNative");
  napi_value a[2];
  for (int32_t k = 0; k < nD; k++) {
    a[0] = rt_number(dIdx[k]);
    a[1] = rt_number(dHz[k]);
    must(rt_call(b, "setDriveOne", 2, a), "setDriveOne");
  }
  double *bl = (double *)malloc((size_t)(nB ? nB : 1) * 8);
  for (int32_t k = 0; k < nB; k++) bl[k] = bIdx[k];
  a[0] = rt_array(bl, (uint32_t)nB);
  a[1] = rt_number(biasMv);
  must(rt_call(b, "setBias", 2, a), "setBias");
  if (bgRate > 0) {
    a[0] = rt_number(bgRate);
    a[1] = rt_number(bgAmp);
    must(rt_call(b, "setBackground", 2, a), "setBackground");
  }
  for (int32_t s = 0; s < s1; s++) record_step(b);
  a[0] = rt_typed(napi_int32_array, pIdx, (size_t)nP);
  a[1] = rt_number(pulseMv);
  must(rt_call(b, "pulse", 2, a), "pulse");
  a[0] = rt_number(addgI);
  a[1] = rt_number(addgE);
  must(rt_call(b, "addG", 2, a), "addG");
  a[0] = rt_number(thrI);
  a[1] = rt_number(thrMv);
  must(rt_call(b, "setThr", 2, a), "setThr");
  for (int32_t s = 0; s < s2; s++) record_step(b);
  a[0] = rt_number(s3);
  const double nf = rt_num(must(rt_call(b, "run", 1, a), "run"));
  wr(&nf, 8);
  record_step(b);
  const double t = rt_num(must(rt_prop(b, "t"), "t"));
  wr(&t, 8);
  napi_value v = must(rt_prop(b, "v"), "v"), sc = must(rt_prop(b, "spikeCount"), "spikeCount");
  wr(rt_typed_data(v), (size_t)N * 4);
  wr(rt_typed_data(sc), (size_t)N * 4);
  must(rt_call(b, "reset", 0, NULL), "reset");
  for (int32_t s = 0; s < s4; s++) record_step(b);
  rt_collect(b);
  fclose(g_out);
  fclose(g_in);
  return 0;
}

int main(int argc, char **argv) {
  if (argc >= 2 && !strcmp(argv[1], "marshal")) return marshal();
  if (argc >= 4 && !strcmp(argv[1], "run")) return run(argv[2], argv[3]);
  fprintf(stderr, "usage: driver marshal | driver run IN OUT\n");
  return 2;
}
