/* The LIFWasm brain object (src/lifwasm.js:36-87) as a Node-API addon over libflybrain's C ABI
 * (include/flybrain.h): the native backend src/brainsetup.js:63-79 can pick before its WASM
 * fallback, for the loop that steps a brain once per simulated millisecond
 * (src/sim/fly.js:151,191-196).
 *
 *   const { LIFNative } = require('./flybrain_napi.node');
 *   const b = new LIFNative({ N, indptr, indices, weights, sign, params, seed });
 *
 * indptr (Uint32Array N+1), indices (Uint32Array E), weights (Float32Array E) and sign
 * (Float32Array N) are the arrays writeGraph lays out (src/lifwasm.js:14-34): effective weights,
 * sign already multiplied by wSyn. params takes the DEFAULTS names of src/lif.js:6-15 (missing
 * ones keep the defaults); seed is LIFWasm's (the RNG starts at (seed * 2654435761) >>> 0 || 1).
 *
 * The methods are LIFWasm's: step() returns the fired list of the step in ring order (driven
 * spikes in driven-list order, then threshold spikes ascending) as an Int32Array the caller owns;
 * setDriveOne, setDrive, setBias, setThr, addG, pulse, setBackground, reset and wake act as
 * LIFWasm's do; the state arrays v, gE, gI, refr, trace, adapt, res, bias, thr, drive (Float32Array)
 * and spikeCount (Uint32Array) read as copies of the device state; N, nAwake and t (simulated ms
 * since reset) are numbers. LIFGpu's extras (src/lifgpu.js:349-351): setParams(q) merges q into
 * the parameters (the ring depth round(delay / dt) + 1 must stay), flush() has nothing to submit,
 * destroy() frees the device state. Beyond both: run(n) takes n steps in one launch and returns
 * the last step's fired count; dispose() is destroy() under another name.
 * A failing call throws an Error with the library's message (attachBrain falls back on any
 * exception, src/brainsetup.js:66-75).
 *
 * Build: node-gyp with binding.gyp beside this file, linked against libflybrain.so. */
#include <node_api.h>

#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "flybrain.h"

typedef struct {
  fb_graph *graph;
  fb_brains *brains;
  fb_params p; /* the parameters in force */
  int32_t N;
  double dt; /* ms per step */
  double t;  /* simulated ms since reset */
  int32_t *fired;
} Brain;

static void brain_free(Brain *b) {
  if (b->brains) fb_brains_destroy(b->brains);
  if (b->graph) fb_graph_destroy(b->graph);
  free(b->fired);
  b->brains = NULL;
  b->graph = NULL;
  b->fired = NULL;
}

static void brain_finalize(napi_env env, void *data, void *hint) {
  (void)env;
  (void)hint;
  brain_free((Brain *)data);
  free(data);
}

static napi_value throw_msg(napi_env env, const char *msg) {
  napi_throw_error(env, NULL, msg);
  return NULL;
}

static napi_value throw_fb(napi_env env) {
  const char *m = fb_last_error();
  return throw_msg(env, m && m[0] ? m : "flybrain: call failed");
}

static napi_value undefined_value(napi_env env) {
  napi_value u = NULL;
  napi_get_undefined(env, &u);
  return u;
}

/* The brain behind `this` and up to n arguments (missing ones read as undefined); NULL when
 * `this` is not a live brain. */
static Brain *this_brain(napi_env env, napi_callback_info info, size_t n, napi_value *argv, void **data) {
  napi_value self = NULL;
  void *p = NULL;
  size_t argc = n;
  if (napi_get_cb_info(env, info, &argc, argv, &self, data) != napi_ok) return NULL;
  if (napi_unwrap(env, self, &p) != napi_ok || !p) return NULL;
  Brain *b = (Brain *)p;
  return b->brains ? b : NULL;
}

static bool is_undefined(napi_env env, napi_value v) {
  napi_valuetype t;
  return !v || (napi_typeof(env, v, &t) == napi_ok && t == napi_undefined);
}

static bool get_f64(napi_env env, napi_value v, double *out) {
  return v && napi_get_value_double(env, v, out) == napi_ok;
}

static bool get_i32(napi_env env, napi_value v, int32_t *out) {
  return v && napi_get_value_int32(env, v, out) == napi_ok;
}

/* An index list as LIFWasm's methods take one: an Int32Array / Uint32Array, an array of numbers,
 * or one number. *idx is allocated here (free() it). */
static bool get_index_list(napi_env env, napi_value v, int32_t **idx, uint32_t *n) {
  bool typed = false, array = false;
  *idx = NULL;
  *n = 0;
  if (!v) return false;
  napi_is_typedarray(env, v, &typed);
  if (typed) {
    napi_typedarray_type t;
    size_t len = 0;
    void *data = NULL;
    if (napi_get_typedarray_info(env, v, &t, &len, &data, NULL, NULL) != napi_ok) return false;
    if (t != napi_int32_array && t != napi_uint32_array) return false;
    *idx = (int32_t *)malloc((len ? len : 1) * sizeof(int32_t));
    if (!*idx) return false;
    if (len) memcpy(*idx, data, len * sizeof(int32_t));
    *n = (uint32_t)len;
    return true;
  }
  napi_is_array(env, v, &array);
  if (!array) {
    int32_t i;
    if (!get_i32(env, v, &i)) return false;
    *idx = (int32_t *)malloc(sizeof(int32_t));
    if (!*idx) return false;
    **idx = i;
    *n = 1;
    return true;
  }
  uint32_t len = 0;
  if (napi_get_array_length(env, v, &len) != napi_ok) return false;
  *idx = (int32_t *)malloc((len ? len : 1) * sizeof(int32_t));
  if (!*idx) return false;
  for (uint32_t k = 0; k < len; k++) {
    napi_value e = NULL;
    if (napi_get_element(env, v, k, &e) != napi_ok || !get_i32(env, e, &(*idx)[k])) {
      free(*idx);
      *idx = NULL;
      return false;
    }
  }
  *n = len;
  return true;
}

/* A typed array of the given type, its element count and data; false otherwise. */
static bool get_typed(napi_env env, napi_value v, napi_typedarray_type want, size_t *len, void **data) {
  bool typed = false;
  napi_typedarray_type t;
  if (!v || napi_is_typedarray(env, v, &typed) != napi_ok || !typed) return false;
  if (napi_get_typedarray_info(env, v, &t, len, data, NULL, NULL) != napi_ok) return false;
  return t == want;
}

static napi_value new_typed(napi_env env, napi_typedarray_type t, size_t n, size_t esz, void **data) {
  napi_value ab = NULL, out = NULL;
  if (napi_create_arraybuffer(env, n * esz, data, &ab) != napi_ok) return NULL;
  if (napi_create_typedarray(env, t, n, ab, 0, &out) != napi_ok) return NULL;
  return out;
}

static bool merge_params(napi_env env, napi_value obj, fb_params *p);

/* ---- methods ----------------------------------------------------------------------------- */

static napi_value m_step(napi_env env, napi_callback_info info) {
  Brain *b = this_brain(env, info, 0, NULL, NULL);
  if (!b) return throw_msg(env, "LIFNative.step: not a live brain");
  int32_t nf = 0, n = 0;
  if (fb_step(b->brains, 1, &nf) || fb_fired(b->brains, 0, b->fired, b->N, &n)) return throw_fb(env);
  b->t += b->dt;
  void *data = NULL;
  napi_value out = new_typed(env, napi_int32_array, (size_t)n, sizeof(int32_t), &data);
  if (out && n) memcpy(data, b->fired, (size_t)n * sizeof(int32_t));
  return out;
}

static napi_value m_run(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  Brain *b = this_brain(env, info, 1, argv, NULL);
  int32_t steps = 0, nf = 0;
  if (!b) return throw_msg(env, "LIFNative.run: not a live brain");
  if (!get_i32(env, argv[0], &steps) || steps < 0) return throw_msg(env, "LIFNative.run(n): a step count >= 0");
  if (steps && fb_step(b->brains, steps, &nf)) return throw_fb(env);
  b->t += steps * b->dt;
  napi_value out = NULL;
  napi_create_double(env, (double)nf, &out);
  return out;
}

static napi_value m_set_drive_one(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  Brain *b = this_brain(env, info, 2, argv, NULL);
  int32_t i;
  double hz;
  if (!b) return throw_msg(env, "LIFNative.setDriveOne: not a live brain");
  if (!get_i32(env, argv[0], &i) || !get_f64(env, argv[1], &hz))
    return throw_msg(env, "LIFNative.setDriveOne(i, rate): numbers expected");
  if (fb_set_drive(b->brains, 0, &i, &hz, 1)) return throw_fb(env);
  return undefined_value(env);
}

typedef int (*list_setter)(fb_brains *, int32_t, const int32_t *, const double *, int32_t);

/* setDrive / setBias / pulse: one value for every index of a list, applied in list order as
 * LIFWasm's loops over the list do. */
static napi_value list_call(napi_env env, napi_callback_info info, list_setter fn, const char *usage) {
  napi_value argv[2];
  Brain *b = this_brain(env, info, 2, argv, NULL);
  int32_t *idx = NULL;
  uint32_t n = 0;
  double value;
  if (!b) return throw_msg(env, "LIFNative: not a live brain");
  if (!get_index_list(env, argv[0], &idx, &n) || !get_f64(env, argv[1], &value)) {
    free(idx);
    return throw_msg(env, usage);
  }
  double *v = (double *)malloc((n ? n : 1) * sizeof(double));
  if (!v) {
    free(idx);
    return throw_msg(env, "LIFNative: out of host memory");
  }
  for (uint32_t k = 0; k < n; k++) v[k] = value;
  const int rc = n ? fn(b->brains, 0, idx, v, (int32_t)n) : FB_OK;
  free(idx);
  free(v);
  return rc ? throw_fb(env) : undefined_value(env);
}

static napi_value m_set_drive(napi_env env, napi_callback_info info) {
  return list_call(env, info, fb_set_drive, "LIFNative.setDrive(ix, rate): an index list and a number");
}

static napi_value m_set_bias(napi_env env, napi_callback_info info) {
  return list_call(env, info, fb_set_bias, "LIFNative.setBias(ix, mv): an index list and a number");
}

static napi_value m_pulse(napi_env env, napi_callback_info info) {
  return list_call(env, info, fb_pulse, "LIFNative.pulse(ix, mv): an index list and a number");
}

static napi_value m_set_thr(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  Brain *b = this_brain(env, info, 2, argv, NULL);
  int32_t i;
  double mv;
  if (!b) return throw_msg(env, "LIFNative.setThr: not a live brain");
  if (!get_i32(env, argv[0], &i) || !get_f64(env, argv[1], &mv))
    return throw_msg(env, "LIFNative.setThr(i, mv): numbers expected");
  if (fb_set_thr(b->brains, 0, &i, &mv, 1)) return throw_fb(env);
  return undefined_value(env);
}

static napi_value m_add_g(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  Brain *b = this_brain(env, info, 3, argv, NULL);
  int32_t i;
  double e, ii = 0.0;
  if (!b) return throw_msg(env, "LIFNative.addG: not a live brain");
  /* ii || 0: a missing inhibitory increment adds nothing */
  if (!get_i32(env, argv[0], &i) || !get_f64(env, argv[1], &e) ||
      (!is_undefined(env, argv[2]) && !get_f64(env, argv[2], &ii)))
    return throw_msg(env, "LIFNative.addG(i, e, ii): numbers expected");
  if (fb_add_g(b->brains, 0, &i, &e, &ii, 1)) return throw_fb(env);
  return undefined_value(env);
}

static napi_value m_set_background(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  Brain *b = this_brain(env, info, 2, argv, NULL);
  double rate, amp;
  if (!b) return throw_msg(env, "LIFNative.setBackground: not a live brain");
  if (!get_f64(env, argv[0], &rate) || !get_f64(env, argv[1], &amp))
    return throw_msg(env, "LIFNative.setBackground(rateHz, ampMv): numbers expected");
  if (fb_set_background(b->brains, 0, rate, amp)) return throw_fb(env);
  b->p.bgRate = rate;
  b->p.bgAmp = amp;
  return undefined_value(env);
}

static napi_value m_set_params(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  Brain *b = this_brain(env, info, 1, argv, NULL);
  if (!b) return throw_msg(env, "LIFNative.setParams: not a live brain");
  fb_params p = b->p;
  napi_valuetype t;
  if (napi_typeof(env, argv[0], &t) != napi_ok || t != napi_object || !merge_params(env, argv[0], &p))
    return throw_msg(env, "LIFNative.setParams(q): an object of numbers");
  if (fb_set_params(b->brains, 0, &p)) return throw_fb(env);
  b->p = p;
  b->dt = p.dt;
  return undefined_value(env);
}

static napi_value m_reset(napi_env env, napi_callback_info info) {
  Brain *b = this_brain(env, info, 0, NULL, NULL);
  if (!b) return throw_msg(env, "LIFNative.reset: not a live brain");
  if (fb_reset(b->brains, 0)) return throw_fb(env);
  b->t = 0.0;
  return undefined_value(env);
}

/* wake (LIFWasm) and flush (LIFGpu): nothing to do, host writes apply before the next step */
static napi_value m_nothing(napi_env env, napi_callback_info info) {
  (void)info;
  return undefined_value(env);
}

static napi_value m_dispose(napi_env env, napi_callback_info info) {
  napi_value self = NULL;
  void *p = NULL;
  size_t argc = 0;
  if (napi_get_cb_info(env, info, &argc, NULL, &self, NULL) == napi_ok && napi_unwrap(env, self, &p) == napi_ok && p)
    brain_free((Brain *)p);
  return undefined_value(env);
}

/* ---- getters ----------------------------------------------------------------------------- */

/* A state field (data = FB_FIELD_* + 1) as a fresh typed array. */
static napi_value g_field(napi_env env, napi_callback_info info) {
  void *data = NULL;
  Brain *b = this_brain(env, info, 0, NULL, &data);
  if (!b) return throw_msg(env, "LIFNative: not a live brain");
  const int32_t field = (int32_t)(intptr_t)data - 1;
  void *dst = NULL;
  napi_value out = new_typed(env, field == FB_FIELD_SPIKECOUNT ? napi_uint32_array : napi_float32_array,
                             (size_t)b->N, 4, &dst);
  if (!out) return NULL;
  if (fb_read(b->brains, field, 0, dst)) return throw_fb(env);
  return out;
}

static napi_value g_number(napi_env env, napi_callback_info info) {
  void *data = NULL;
  Brain *b = this_brain(env, info, 0, NULL, &data);
  if (!b) return throw_msg(env, "LIFNative: not a live brain");
  napi_value out = NULL;
  napi_create_double(env, (intptr_t)data == 1 ? b->t : (double)b->N, &out);
  return out;
}

/* ---- construction ------------------------------------------------------------------------ */

static bool named(napi_env env, napi_value obj, const char *name, napi_value *out) {
  bool has = false;
  *out = NULL;
  if (!obj || napi_has_named_property(env, obj, name, &has) != napi_ok || !has) return false;
  return napi_get_named_property(env, obj, name, out) == napi_ok && !is_undefined(env, *out);
}

/* params named as DEFAULTS names them (src/lif.js:6-15), merged over *p; coba as a boolean or a
 * number. */
static bool merge_params(napi_env env, napi_value obj, fb_params *p) {
  static const char *names[] = {"dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "traceTau",
                                "adaptInc", "adaptTau", "depU", "depTau", "eExc", "eInh", "bgRate", "bgAmp", "preInh"};
  double *slot[] = {&p->dt, &p->vRest, &p->vThresh, &p->vReset, &p->tauM, &p->tauSyn, &p->tRef, &p->delay,
                    &p->traceTau, &p->adaptInc, &p->adaptTau, &p->depU, &p->depTau, &p->eExc, &p->eInh,
                    &p->bgRate, &p->bgAmp, &p->preInh};
  if (!obj) return true;
  for (size_t k = 0; k < sizeof(names) / sizeof(names[0]); k++) {
    napi_value v;
    if (named(env, obj, names[k], &v) && !get_f64(env, v, slot[k])) return false;
  }
  napi_value c;
  if (named(env, obj, "coba", &c)) {
    bool flag = false;
    double x = 0;
    if (napi_get_value_bool(env, c, &flag) == napi_ok) p->coba = flag ? 1 : 0;
    else if (get_f64(env, c, &x)) p->coba = x != 0 ? 1 : 0;
    else return false;
  }
  return true;
}

static napi_value ctor(napi_env env, napi_callback_info info) {
  napi_value argv[1], self = NULL;
  size_t argc = 1;
  if (napi_get_cb_info(env, info, &argc, argv, &self, NULL) != napi_ok || argc < 1)
    return throw_msg(env, "new LIFNative({N, indptr, indices, weights, sign, params, seed})");
  napi_value o = argv[0], v;
  int32_t N = 0;
  size_t nIp = 0, E = 0, nW = 0, nS = 0;
  void *ip = NULL, *ix = NULL, *w = NULL, *sg = NULL;
  if (!named(env, o, "N", &v) || !get_i32(env, v, &N) || N <= 0) return throw_msg(env, "LIFNative: N > 0 expected");
  if (!named(env, o, "indptr", &v) || !get_typed(env, v, napi_uint32_array, &nIp, &ip) || nIp != (size_t)N + 1)
    return throw_msg(env, "LIFNative: indptr must be a Uint32Array of N + 1");
  if (!named(env, o, "indices", &v) || !get_typed(env, v, napi_uint32_array, &E, &ix))
    return throw_msg(env, "LIFNative: indices must be a Uint32Array");
  if (!named(env, o, "weights", &v) || !get_typed(env, v, napi_float32_array, &nW, &w) || nW != E)
    return throw_msg(env, "LIFNative: weights must be a Float32Array as long as indices");
  if (!named(env, o, "sign", &v) || !get_typed(env, v, napi_float32_array, &nS, &sg) || nS != (size_t)N)
    return throw_msg(env, "LIFNative: sign must be a Float32Array of N");
  fb_params p;
  napi_value po = NULL;
  fb_default_params(&p);
  named(env, o, "params", &po);
  if (!merge_params(env, po, &p)) return throw_msg(env, "LIFNative: params values must be numbers");
  double seedv = 1;
  if (named(env, o, "seed", &v) && !get_f64(env, v, &seedv)) return throw_msg(env, "LIFNative: seed must be a number");
  if (!(seedv >= 0 && seedv < 4294967296.0) || seedv != (double)(uint32_t)seedv)
    return throw_msg(env, "LIFNative: seed must be an integer in [0, 2^32)");
  const uint32_t seed = (uint32_t)seedv;

  Brain *b = (Brain *)calloc(1, sizeof(Brain));
  if (!b) return throw_msg(env, "LIFNative: out of host memory");
  b->N = N;
  b->p = p;
  b->dt = p.dt;
  b->fired = (int32_t *)malloc((size_t)N * sizeof(int32_t));
  if (!b->fired || fb_graph_create(N, (int64_t)E, (const uint32_t *)ip, (const uint32_t *)ix, (const float *)w,
                                   (const float *)sg, &b->graph) ||
      fb_brains_create((const fb_graph *const *)&b->graph, 1, &p, 0, &seed, &b->brains)) {
    napi_value err = throw_fb(env);
    brain_free(b);
    free(b);
    return err;
  }
  if (napi_wrap(env, self, b, brain_finalize, NULL, NULL) != napi_ok) {
    brain_free(b);
    free(b);
    return throw_msg(env, "LIFNative: could not attach the brain");
  }
  return self;
}

/* The module's exports: { LIFNative }. */
napi_value flybrain_napi_init(napi_env env, napi_value exports) {
#define METHOD(name, fn) {name, NULL, fn, NULL, NULL, NULL, napi_default, NULL}
#define FIELD(name, id) {name, NULL, NULL, g_field, NULL, NULL, napi_default, (void *)(intptr_t)((id) + 1)}
  const napi_property_descriptor props[] = {
      METHOD("step", m_step),
      METHOD("run", m_run),
      METHOD("setDriveOne", m_set_drive_one),
      METHOD("setDrive", m_set_drive),
      METHOD("setBias", m_set_bias),
      METHOD("setThr", m_set_thr),
      METHOD("addG", m_add_g),
      METHOD("pulse", m_pulse),
      METHOD("setBackground", m_set_background),
      METHOD("reset", m_reset),
      METHOD("setParams", m_set_params),
      METHOD("wake", m_nothing),
      METHOD("flush", m_nothing),
      METHOD("destroy", m_dispose),
      METHOD("dispose", m_dispose),
      FIELD("v", FB_FIELD_V),
      FIELD("gE", FB_FIELD_GE),
      FIELD("gI", FB_FIELD_GI),
      FIELD("refr", FB_FIELD_REFR),
      FIELD("trace", FB_FIELD_TRACE),
      FIELD("adapt", FB_FIELD_ADAPT),
      FIELD("res", FB_FIELD_RES),
      FIELD("bias", FB_FIELD_BIAS),
      FIELD("thr", FB_FIELD_THR),
      FIELD("drive", FB_FIELD_DRIVE),
      FIELD("spikeCount", FB_FIELD_SPIKECOUNT),
      {"N", NULL, NULL, g_number, NULL, NULL, napi_default, (void *)(intptr_t)0},
      {"nAwake", NULL, NULL, g_number, NULL, NULL, napi_default, (void *)(intptr_t)0},
      {"t", NULL, NULL, g_number, NULL, NULL, napi_default, (void *)(intptr_t)1},
  };
#undef METHOD
#undef FIELD
  napi_value cls = NULL;
  if (napi_define_class(env, "LIFNative", NAPI_AUTO_LENGTH, ctor, NULL, sizeof(props) / sizeof(props[0]), props,
                        &cls) != napi_ok ||
      napi_set_named_property(env, exports, "LIFNative", cls) != napi_ok)
    return NULL;
  return exports;
}

#ifndef FLYBRAIN_NAPI_NO_MODULE
NAPI_MODULE(NODE_GYP_MODULE_NAME, flybrain_napi_init)
#endif
