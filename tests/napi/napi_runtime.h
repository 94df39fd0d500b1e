/* Driving a Node-API addon from C in tests: build argument values, construct the addon's class,
 * call its methods and getters, read results, take the pending exception. The value model is
 * napi_runtime.c's. Test infrastructure only. */
#ifndef FLYBRAIN_TEST_NAPI_RUNTIME_H
#define FLYBRAIN_TEST_NAPI_RUNTIME_H

#include "node_api.h"

napi_env rt_env(void);
napi_value rt_undefined(void);
napi_value rt_number(double v);
napi_value rt_bool(bool v);
napi_value rt_object(void);
napi_value rt_array(const double *v, uint32_t n);              /* an array of numbers */
napi_value rt_typed(napi_typedarray_type t, const void *data, size_t n);  /* a copy of n elements */
void rt_set(napi_value obj, const char *name, napi_value v);
napi_value rt_get(napi_value obj, const char *name);           /* a plain property, NULL if absent */

napi_value rt_new(napi_value cls, size_t argc, napi_value *argv);                   /* NULL if it threw */
napi_value rt_call(napi_value obj, const char *method, size_t argc, napi_value *argv);  /* NULL if it threw */
napi_value rt_prop(napi_value obj, const char *getter);                             /* NULL if it threw */
void rt_collect(napi_value obj);  /* the object is collected: its finalizer runs */

const char *rt_take_exception(void);  /* the pending exception's message (cleared), or NULL */
double rt_num(napi_value v);
int rt_is_object(napi_value v);  /* an object (not an array, buffer or typed array) */
int rt_typed_type(napi_value v);
size_t rt_typed_len(napi_value v);
const void *rt_typed_data(napi_value v);

#endif
