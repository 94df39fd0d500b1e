/* A minimal Node-API runtime for tests: values (undefined, numbers, booleans, objects with named
 * properties, arrays, array buffers, typed arrays, classes), wrapped native objects, callback
 * info and one pending exception, enough to construct an addon's class and call its methods and
 * getters from C with the semantics Node documents for these calls (argc in/out with missing
 * arguments as undefined; int32 conversion by truncation to the low 32 bits). Nothing is garbage
 * collected. Test infrastructure only. */
#include "napi_runtime.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { K_UNDEF, K_NUM, K_BOOL, K_OBJECT, K_ARRAY, K_BUFFER, K_TYPED, K_CLASS };

struct prop {
  char *name;
  napi_value v;
  struct prop *next;
};

struct napi_value__ {
  int kind;
  double num;
  bool b;
  struct prop *props;  /* object */
  napi_value cls;      /* object: the class it was constructed from */
  void *native;        /* object: the wrapped native pointer */
  napi_finalize fin;
  void *fin_hint;
  napi_value *elems;   /* array */
  uint32_t nelems;
  unsigned char *bytes;  /* array buffer */
  size_t nbytes;
  napi_typedarray_type ta;  /* typed array */
  size_t len, off;
  napi_value buffer;
  napi_callback ctor;  /* class */
  void *cdata;
  napi_property_descriptor *descs;
  size_t ndesc;
};

struct napi_env__ {
  int pending;
  char msg[1024];
};

struct napi_callback_info__ {
  napi_value self;
  size_t argc;
  napi_value *argv;
  void *data;
};

static struct napi_env__ g_env;
static struct napi_value__ g_undef = {K_UNDEF};

static napi_value new_value(int kind) {
  napi_value v = (napi_value)calloc(1, sizeof(struct napi_value__));
  if (!v) abort();
  v->kind = kind;
  return v;
}

static size_t elem_size(napi_typedarray_type t) {
  switch (t) {
    case napi_int8_array:
    case napi_uint8_array:
    case napi_uint8_clamped_array: return 1;
    case napi_int16_array:
    case napi_uint16_array: return 2;
    case napi_float64_array:
    case napi_bigint64_array:
    case napi_biguint64_array: return 8;
    default: return 4;
  }
}

/* ---- the Node-API calls -------------------------------------------------------------------- */

napi_status napi_define_class(napi_env env, const char *utf8name, size_t length, napi_callback constructor, void *data,
                              size_t property_count, const napi_property_descriptor *properties, napi_value *result) {
  (void)env;
  (void)utf8name;
  (void)length;
  if (!constructor || !result || (property_count && !properties)) return napi_invalid_arg;
  napi_value c = new_value(K_CLASS);
  c->ctor = constructor;
  c->cdata = data;
  c->ndesc = property_count;
  c->descs = (napi_property_descriptor *)calloc(property_count ? property_count : 1, sizeof(napi_property_descriptor));
  if (property_count) memcpy(c->descs, properties, property_count * sizeof(napi_property_descriptor));
  *result = c;
  return napi_ok;
}

napi_status napi_wrap(napi_env env, napi_value js_object, void *native_object, napi_finalize finalize_cb,
                      void *finalize_hint, napi_ref *result) {
  (void)env;
  if (!js_object || js_object->kind != K_OBJECT || js_object->native) return napi_invalid_arg;
  js_object->native = native_object;
  js_object->fin = finalize_cb;
  js_object->fin_hint = finalize_hint;
  if (result) *result = NULL;
  return napi_ok;
}

napi_status napi_unwrap(napi_env env, napi_value js_object, void **result) {
  (void)env;
  if (!js_object || js_object->kind != K_OBJECT || !js_object->native || !result) return napi_invalid_arg;
  *result = js_object->native;
  return napi_ok;
}

napi_status napi_get_cb_info(napi_env env, napi_callback_info cbinfo, size_t *argc, napi_value *argv,
                             napi_value *this_arg, void **data) {
  (void)env;
  if (!cbinfo) return napi_invalid_arg;
  if (argc) {
    if (argv)
      for (size_t k = 0; k < *argc; k++) argv[k] = k < cbinfo->argc ? cbinfo->argv[k] : &g_undef;
    *argc = cbinfo->argc;
  }
  if (this_arg) *this_arg = cbinfo->self;
  if (data) *data = cbinfo->data;
  return napi_ok;
}

napi_status napi_get_undefined(napi_env env, napi_value *result) {
  (void)env;
  *result = &g_undef;
  return napi_ok;
}

napi_status napi_typeof(napi_env env, napi_value value, napi_valuetype *result) {
  (void)env;
  if (!value || !result) return napi_invalid_arg;
  switch (value->kind) {
    case K_UNDEF: *result = napi_undefined; break;
    case K_NUM: *result = napi_number; break;
    case K_BOOL: *result = napi_boolean; break;
    case K_CLASS: *result = napi_function; break;
    default: *result = napi_object; break;
  }
  return napi_ok;
}

napi_status napi_get_value_double(napi_env env, napi_value value, double *result) {
  (void)env;
  if (!value || value->kind != K_NUM) return napi_number_expected;
  *result = value->num;
  return napi_ok;
}

napi_status napi_get_value_int32(napi_env env, napi_value value, int32_t *result) {
  (void)env;
  if (!value || value->kind != K_NUM) return napi_number_expected;
  const double x = value->num;
  if (!isfinite(x)) {
    *result = 0;
  } else {
    const double t = trunc(x);
    const double m = fmod(t, 4294967296.0);
    *result = (int32_t)(uint32_t)(int64_t)(m < 0 ? m + 4294967296.0 : m);
  }
  return napi_ok;
}

napi_status napi_get_value_bool(napi_env env, napi_value value, bool *result) {
  (void)env;
  if (!value || value->kind != K_BOOL) return napi_boolean_expected;
  *result = value->b;
  return napi_ok;
}

napi_status napi_create_double(napi_env env, double value, napi_value *result) {
  (void)env;
  *result = rt_number(value);
  return napi_ok;
}

static struct prop *find_prop(napi_value obj, const char *name) {
  for (struct prop *p = obj->props; p; p = p->next)
    if (!strcmp(p->name, name)) return p;
  return NULL;
}

napi_status napi_has_named_property(napi_env env, napi_value object, const char *utf8name, bool *result) {
  (void)env;
  if (!object || object->kind != K_OBJECT) return napi_object_expected;
  *result = find_prop(object, utf8name) != NULL;
  return napi_ok;
}

napi_status napi_get_named_property(napi_env env, napi_value object, const char *utf8name, napi_value *result) {
  (void)env;
  if (!object || object->kind != K_OBJECT) return napi_object_expected;
  struct prop *p = find_prop(object, utf8name);
  *result = p ? p->v : &g_undef;
  return napi_ok;
}

napi_status napi_set_named_property(napi_env env, napi_value object, const char *utf8name, napi_value value) {
  (void)env;
  if (!object || object->kind != K_OBJECT) return napi_object_expected;
  rt_set(object, utf8name, value);
  return napi_ok;
}

napi_status napi_is_array(napi_env env, napi_value value, bool *result) {
  (void)env;
  *result = value && value->kind == K_ARRAY;
  return napi_ok;
}

napi_status napi_get_array_length(napi_env env, napi_value value, uint32_t *result) {
  (void)env;
  if (!value || value->kind != K_ARRAY) return napi_array_expected;
  *result = value->nelems;
  return napi_ok;
}

napi_status napi_get_element(napi_env env, napi_value object, uint32_t index, napi_value *result) {
  (void)env;
  if (!object || object->kind != K_ARRAY) return napi_array_expected;
  *result = index < object->nelems ? object->elems[index] : &g_undef;
  return napi_ok;
}

napi_status napi_is_typedarray(napi_env env, napi_value value, bool *result) {
  (void)env;
  *result = value && value->kind == K_TYPED;
  return napi_ok;
}

napi_status napi_get_typedarray_info(napi_env env, napi_value typedarray, napi_typedarray_type *type, size_t *length,
                                     void **data, napi_value *arraybuffer, size_t *byte_offset) {
  (void)env;
  if (!typedarray || typedarray->kind != K_TYPED) return napi_invalid_arg;
  if (type) *type = typedarray->ta;
  if (length) *length = typedarray->len;
  if (data) *data = typedarray->buffer->bytes + typedarray->off;
  if (arraybuffer) *arraybuffer = typedarray->buffer;
  if (byte_offset) *byte_offset = typedarray->off;
  return napi_ok;
}

napi_status napi_create_arraybuffer(napi_env env, size_t byte_length, void **data, napi_value *result) {
  (void)env;
  napi_value b = new_value(K_BUFFER);
  b->bytes = (unsigned char *)calloc(byte_length ? byte_length : 1, 1);
  if (!b->bytes) return napi_generic_failure;
  b->nbytes = byte_length;
  if (data) *data = b->bytes;
  *result = b;
  return napi_ok;
}

napi_status napi_create_typedarray(napi_env env, napi_typedarray_type type, size_t length, napi_value arraybuffer,
                                   size_t byte_offset, napi_value *result) {
  (void)env;
  if (!arraybuffer || arraybuffer->kind != K_BUFFER || byte_offset + length * elem_size(type) > arraybuffer->nbytes)
    return napi_invalid_arg;
  napi_value t = new_value(K_TYPED);
  t->ta = type;
  t->len = length;
  t->off = byte_offset;
  t->buffer = arraybuffer;
  *result = t;
  return napi_ok;
}

napi_status napi_throw_error(napi_env env, const char *code, const char *msg) {
  (void)code;
  if (!env->pending) {
    env->pending = 1;
    snprintf(env->msg, sizeof env->msg, "%s", msg ? msg : "");
  }
  return napi_ok;
}

/* ---- the driver's side ---------------------------------------------------------------------- */

napi_env rt_env(void) { return &g_env; }
napi_value rt_undefined(void) { return &g_undef; }

napi_value rt_number(double v) {
  napi_value x = new_value(K_NUM);
  x->num = v;
  return x;
}

napi_value rt_bool(bool v) {
  napi_value x = new_value(K_BOOL);
  x->b = v;
  return x;
}

napi_value rt_object(void) { return new_value(K_OBJECT); }

napi_value rt_array(const double *v, uint32_t n) {
  napi_value a = new_value(K_ARRAY);
  a->elems = (napi_value *)calloc(n ? n : 1, sizeof(napi_value));
  a->nelems = n;
  for (uint32_t k = 0; k < n; k++) a->elems[k] = rt_number(v[k]);
  return a;
}

napi_value rt_typed(napi_typedarray_type t, const void *data, size_t n) {
  void *dst = NULL;
  napi_value ab = NULL, out = NULL;
  napi_create_arraybuffer(&g_env, n * elem_size(t), &dst, &ab);
  if (n) memcpy(dst, data, n * elem_size(t));
  napi_create_typedarray(&g_env, t, n, ab, 0, &out);
  return out;
}

void rt_set(napi_value obj, const char *name, napi_value v) {
  struct prop *p = find_prop(obj, name);
  if (!p) {
    p = (struct prop *)calloc(1, sizeof(struct prop));
    const size_t len = strlen(name) + 1;
    p->name = (char *)malloc(len);
    memcpy(p->name, name, len);
    p->next = obj->props;
    obj->props = p;
  }
  p->v = v;
}

napi_value rt_get(napi_value obj, const char *name) {
  struct prop *p = obj && obj->kind == K_OBJECT ? find_prop(obj, name) : NULL;
  return p ? p->v : NULL;
}

static napi_value invoke(napi_callback cb, napi_value self, size_t argc, napi_value *argv, void *data) {
  struct napi_callback_info__ info = {self, argc, argv, data};
  napi_value r = cb(&g_env, &info);
  return g_env.pending ? NULL : (r ? r : &g_undef);
}

napi_value rt_new(napi_value cls, size_t argc, napi_value *argv) {
  if (!cls || cls->kind != K_CLASS) return NULL;
  napi_value obj = new_value(K_OBJECT);
  obj->cls = cls;
  return invoke(cls->ctor, obj, argc, argv, cls->cdata) ? obj : NULL;
}

static const napi_property_descriptor *find_desc(napi_value obj, const char *name) {
  if (!obj || obj->kind != K_OBJECT || !obj->cls) return NULL;
  for (size_t k = 0; k < obj->cls->ndesc; k++)
    if (!strcmp(obj->cls->descs[k].utf8name, name)) return &obj->cls->descs[k];
  return NULL;
}

napi_value rt_call(napi_value obj, const char *method, size_t argc, napi_value *argv) {
  const napi_property_descriptor *d = find_desc(obj, method);
  if (!d || !d->method) {
    napi_throw_error(&g_env, NULL, "not a method");
    return NULL;
  }
  return invoke(d->method, obj, argc, argv, d->data);
}

napi_value rt_prop(napi_value obj, const char *getter) {
  const napi_property_descriptor *d = find_desc(obj, getter);
  if (!d || !d->getter) {
    napi_throw_error(&g_env, NULL, "not a getter");
    return NULL;
  }
  return invoke(d->getter, obj, 0, NULL, d->data);
}

void rt_collect(napi_value obj) {
  if (obj && obj->fin) obj->fin(&g_env, obj->native, obj->fin_hint);
  if (obj) {
    obj->native = NULL;
    obj->fin = NULL;
  }
}

const char *rt_take_exception(void) {
  static char msg[1024];
  if (!g_env.pending) return NULL;
  g_env.pending = 0;
  snprintf(msg, sizeof msg, "%s", g_env.msg);
  return msg;
}

double rt_num(napi_value v) { return v && v->kind == K_NUM ? v->num : NAN; }
int rt_is_object(napi_value v) { return v && v->kind == K_OBJECT; }
int rt_typed_type(napi_value v) { return v && v->kind == K_TYPED ? (int)v->ta : -1; }
size_t rt_typed_len(napi_value v) { return v && v->kind == K_TYPED ? v->len : 0; }
const void *rt_typed_data(napi_value v) { return v && v->kind == K_TYPED ? v->buffer->bytes + v->off : NULL; }
