// The flyvis optic-lobe rate network (src/wasm/lif.c:82-93, src/flyvis.js, src/flyvisgpu.js) on
// sm_103a: B instances (the eyes of one or many flies) sharing one model, advanced together.
//
//   acc[i] = sum over edges (j -> i) with v[j] > 0 of weight * v[j]
//   v[i]  += kdt[i] * (-v[i] + bias[i] + acc[i] + x[i])
//
// lif.c scatters by source (acc[target[k]] += weight[k] * v[j], sources ascending, each row in
// CSR order); per target that is its in-edges in ascending edge id. Here every (target, instance)
// pair gathers its in-edges in that order from a transposed copy of the graph built once, so the
// sums are lif.c's bit for bit with no atomics (the WGSL port rounds to 1/65536 fixed point
// instead). State is instance-minor ([N][B]): the B threads of one target read one edge record
// and B adjacent words of the source's state, so a batch of eyes streams the edge list once per
// step. v is double-buffered: a step reads the previous step's v everywhere, as lif.c's separate
// scatter and update passes do.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fb_internal.cuh"

namespace fb {
int set_error(int code, const char *msg);
}
using namespace fb;

namespace {

int fvfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return set_error(code, buf);
}

#define FVCU(call)                                                                            \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fvfail(e_ == cudaErrorMemoryAllocation ? FB_ENOMEM : FB_ECUDA, "%s: %s", #call, \
                    cudaGetErrorString(e_));                                                  \
  } while (0)

constexpr int kFvThreads = 256;

// One step for every (target i, instance b), thread per pair, b fastest.
__global__ void __launch_bounds__(kFvThreads) fv_step_kernel(int32_t N, int32_t B, const int32_t *__restrict__ cscPtr,
                                                              const int32_t *__restrict__ cscSrc,
                                                              const float *__restrict__ cscW,
                                                              const float *__restrict__ bias,
                                                              const float *__restrict__ kdt,
                                                              const float *__restrict__ vin, float *__restrict__ vout,
                                                              const float *__restrict__ x) {
  const int64_t total = (int64_t)N * B;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = (int32_t)(t / B);
    const int32_t b = (int32_t)(t - (int64_t)i * B);
    const int32_t lo = __ldg(cscPtr + i), hi = __ldg(cscPtr + i + 1);
    float acc = 0.f;
    int32_t e = lo;
    // eight in-edges per round: their loads are issued together, the sum stays in edge order
    for (; e + 8 <= hi; e += 8) {
      int32_t j[8];
      float w[8], r[8];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        j[u] = __ldg(cscSrc + e + u);
        w[u] = __ldg(cscW + e + u);
      }
#pragma unroll
      for (int u = 0; u < 8; u++) r[u] = vin[(int64_t)j[u] * B + b];
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (!(r[u] <= 0.f)) acc = __fadd_rn(acc, __fmul_rn(w[u], r[u]));  // lif.c:90-91
    }
    for (; e < hi; e++) {
      const float r = vin[(int64_t)__ldg(cscSrc + e) * B + b];
      if (!(r <= 0.f)) acc = __fadd_rn(acc, __fmul_rn(__ldg(cscW + e), r));
    }
    const int64_t o = (int64_t)i * B + b;
    const float v = vin[o];
    // lif.c:92: v += kdt * (-v + bias + acc + x), one rounding per operation in C order
    const float s = __fadd_rn(__fadd_rn(__fadd_rn(-v, __ldg(bias + i)), acc), x[o]);
    vout[o] = __fadd_rn(v, __fmul_rn(__ldg(kdt + i), s));
  }
}

// v[b] = bias (src/flyvis.js:24), every instance when b < 0.
__global__ void fv_reset_kernel(int32_t N, int32_t B, int32_t b, const float *bias, float *v) {
  const int64_t total = (int64_t)N * B;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = (int32_t)(t / B), c = (int32_t)(t - (int64_t)i * B);
    if (b < 0 || c == b) v[t] = bias[i];
  }
}

// x[idx[k]] of instance b = values[k] (src/flyvis.js:21). The reference loop leaves a repeated
// index at its last value: each index's last list position is claimed first (win[], reset to -1
// by the writes).
__global__ void fv_claim_kernel(int32_t N, int32_t n, const int32_t *idx, int32_t *win, int32_t *err) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int32_t i = idx[k];
    if (i < 0 || i >= N) atomicCAS(err, 0, FB_EINVAL);
    else atomicMax(win + i, k);
  }
}
__global__ void fv_input_kernel(int32_t N, int32_t B, int32_t b, int32_t n, const int32_t *idx, const float *values,
                                float *x, int32_t *win) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int32_t i = idx[k];
    if (i < 0 || i >= N || win[i] != k) continue;
    x[(int64_t)i * B + b] = values[k];
    win[i] = -1;  // ready for the next list (only the winner of i gets here)
  }
}

// Instance b's N values out of (or into) the instance-minor layout.
__global__ void fv_gather_kernel(int32_t N, int32_t B, int32_t b, const float *src, float *dst) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) dst[i] = src[(int64_t)i * B + b];
}
__global__ void fv_scatter_kernel(int32_t N, int32_t B, int32_t b, const float *src, float *dst) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) dst[(int64_t)i * B + b] = src[i];
}

}  // namespace

struct fb_flyvis {
  int32_t N = 0, B = 0;
  int64_t E = 0;
  int32_t *cscPtr = nullptr, *cscSrc = nullptr;
  float *cscW = nullptr, *bias = nullptr, *kdt = nullptr;
  float *v[2] = {nullptr, nullptr};
  float *x = nullptr, *scratch = nullptr;
  int32_t *idxBuf = nullptr, *err = nullptr, *win = nullptr;
  int64_t idxCap = 0;
  int cur = 0, grid = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float lastMs = 0.f;
};

extern "C" int fb_flyvis_destroy(fb_flyvis *f) {
  if (!f) return FB_OK;
  if (f->st) cudaStreamSynchronize(f->st);
  for (void *p : {(void *)f->cscPtr, (void *)f->cscSrc, (void *)f->cscW, (void *)f->bias, (void *)f->kdt, (void *)f->v[0],
                  (void *)f->v[1], (void *)f->x, (void *)f->scratch, (void *)f->idxBuf, (void *)f->err, (void *)f->win})
    if (p) cudaFree(p);
  if (f->ev0) cudaEventDestroy(f->ev0);
  if (f->ev1) cudaEventDestroy(f->ev1);
  if (f->st) cudaStreamDestroy(f->st);
  delete f;
  return FB_OK;
}

extern "C" int fb_flyvis_create(int32_t N, int64_t E, const int32_t *indptr, const int32_t *target, const float *weight,
                                const float *bias, const float *kdt, int32_t B, fb_flyvis **out) {
  if (!out || N <= 0 || E < 0 || B <= 0 || !indptr || (E && (!target || !weight)) || !bias || !kdt)
    return fvfail(FB_EINVAL, "fb_flyvis_create: bad arguments (N=%d E=%lld B=%d)", N, (long long)E, B);
  if (E > INT32_MAX) return fvfail(FB_EINVAL, "fb_flyvis_create: %lld edges (at most 2^31 - 1)", (long long)E);
  *out = nullptr;
  // the transposed graph, in-edges of each target in ascending edge id (lif.c's summation order)
  std::vector<int32_t> ip(N + 1), tg((size_t)std::max<int64_t>(E, 1)), cp(N + 1, 0), cs((size_t)std::max<int64_t>(E, 1));
  std::vector<float> w((size_t)std::max<int64_t>(E, 1)), cw((size_t)std::max<int64_t>(E, 1));
  auto copy_in = [](void *dst, const void *src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDefault) == cudaSuccess;
  };
  if (!copy_in(ip.data(), indptr, (size_t)(N + 1) * 4) || (E && (!copy_in(tg.data(), target, (size_t)E * 4) ||
                                                                 !copy_in(w.data(), weight, (size_t)E * 4))))
    return fvfail(FB_ECUDA, "fb_flyvis_create: reading the model failed");
  if (ip[0] != 0 || ip[N] != E) return fvfail(FB_EINVAL, "fb_flyvis_create: indptr[0]=%d indptr[N]=%d E=%lld", ip[0], ip[N], (long long)E);
  for (int32_t j = 0; j < N; j++)
    if (ip[j + 1] < ip[j]) return fvfail(FB_EINVAL, "fb_flyvis_create: indptr decreases at %d", j);
  for (int64_t k = 0; k < E; k++) {
    if (tg[k] < 0 || tg[k] >= N) return fvfail(FB_EINVAL, "fb_flyvis_create: target[%lld]=%d", (long long)k, tg[k]);
    cp[tg[k] + 1]++;
  }
  for (int32_t i = 0; i < N; i++) cp[i + 1] += cp[i];
  {
    std::vector<int32_t> fill(cp.begin(), cp.end() - 1);
    for (int32_t j = 0; j < N; j++)
      for (int32_t k = ip[j]; k < ip[j + 1]; k++) {
        const int32_t o = fill[tg[k]]++;
        cs[o] = j;
        cw[o] = w[k];
      }
  }
  fb_flyvis *f = new fb_flyvis;
  f->N = N;
  f->B = B;
  f->E = E;
  auto bail = [&](int rc) {
    fb_flyvis_destroy(f);
    return rc;
  };
  const size_t nb = (size_t)N * B;
  if (cudaMalloc(&f->cscPtr, (size_t)(N + 1) * 4) != cudaSuccess || cudaMalloc(&f->cscSrc, cs.size() * 4) != cudaSuccess ||
      cudaMalloc(&f->cscW, cw.size() * 4) != cudaSuccess || cudaMalloc(&f->bias, (size_t)N * 4) != cudaSuccess ||
      cudaMalloc(&f->kdt, (size_t)N * 4) != cudaSuccess || cudaMalloc(&f->v[0], nb * 4) != cudaSuccess ||
      cudaMalloc(&f->v[1], nb * 4) != cudaSuccess || cudaMalloc(&f->x, nb * 4) != cudaSuccess ||
      cudaMalloc(&f->scratch, (size_t)N * 4) != cudaSuccess || cudaMalloc(&f->err, 4) != cudaSuccess ||
      cudaMalloc(&f->win, (size_t)N * 4) != cudaSuccess)
    return bail(fvfail(FB_ENOMEM, "fb_flyvis_create: device allocation failed (N=%d E=%lld B=%d)", N, (long long)E, B));
  if (cudaMemcpy(f->cscPtr, cp.data(), (size_t)(N + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(f->cscSrc, cs.data(), cs.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(f->cscW, cw.data(), cw.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(f->bias, bias, (size_t)N * 4, cudaMemcpyDefault) != cudaSuccess ||
      cudaMemcpy(f->kdt, kdt, (size_t)N * 4, cudaMemcpyDefault) != cudaSuccess || cudaMemset(f->x, 0, nb * 4) != cudaSuccess ||
      cudaMemset(f->win, 0xff, (size_t)N * 4) != cudaSuccess ||
      cudaMemset(f->err, 0, 4) != cudaSuccess)
    return bail(fvfail(FB_ECUDA, "fb_flyvis_create: upload failed"));
  if (cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&f->ev0) != cudaSuccess ||
      cudaEventCreate(&f->ev1) != cudaSuccess)
    return bail(fvfail(FB_ECUDA, "fb_flyvis_create: stream setup failed"));
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t blocks = ((int64_t)nb + kFvThreads - 1) / kFvThreads;
  f->grid = (int)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)sms * 8));
  fv_reset_kernel<<<f->grid, kFvThreads, 0, f->st>>>(N, B, -1, f->bias, f->v[0]);
  if (cudaStreamSynchronize(f->st) != cudaSuccess) return bail(fvfail(FB_ECUDA, "fb_flyvis_create: reset failed"));
  *out = f;
  return FB_OK;
}

static int fv_check(fb_flyvis *f, int32_t b, const char *fn, bool allowAll = false) {
  if (!f) return fvfail(FB_EINVAL, "%s: null handle", fn);
  if (b >= f->B || (b < 0 && !allowAll)) return fvfail(FB_EINVAL, "%s: instance %d out of range [0, %d)", fn, b, f->B);
  return FB_OK;
}

static int fv_sync_err(fb_flyvis *f, const char *fn) {
  int32_t err = 0;
  FVCU(cudaMemcpyAsync(&err, f->err, 4, cudaMemcpyDeviceToHost, f->st));
  FVCU(cudaStreamSynchronize(f->st));
  if (err) {
    cudaMemset(f->err, 0, 4);
    return fvfail(err, "%s: an index out of range was skipped", fn);
  }
  return FB_OK;
}

extern "C" int fb_flyvis_reset(fb_flyvis *f, int32_t b) {
  int rc = fv_check(f, b, "fb_flyvis_reset", true);
  if (rc) return rc;
  fv_reset_kernel<<<f->grid, kFvThreads, 0, f->st>>>(f->N, f->B, b, f->bias, f->v[f->cur]);
  FVCU(cudaGetLastError());
  FVCU(cudaStreamSynchronize(f->st));
  return FB_OK;
}

extern "C" int fb_flyvis_set_input(fb_flyvis *f, int32_t b, int32_t n, const int32_t *idx, const float *values) {
  int rc = fv_check(f, b, "fb_flyvis_set_input");
  if (rc) return rc;
  if (n < 0 || (n && (!idx || !values))) return fvfail(FB_EINVAL, "fb_flyvis_set_input: bad list");
  if (n == 0) return FB_OK;
  if (n > f->idxCap) {
    if (f->idxBuf) cudaFree(f->idxBuf);
    f->idxBuf = nullptr;
    FVCU(cudaMalloc(&f->idxBuf, (size_t)n * 8));
    f->idxCap = n;
  }
  float *vals = (float *)(f->idxBuf + n);
  FVCU(cudaMemcpyAsync(f->idxBuf, idx, (size_t)n * 4, cudaMemcpyDefault, f->st));
  FVCU(cudaMemcpyAsync(vals, values, (size_t)n * 4, cudaMemcpyDefault, f->st));
  const int g = std::max(1, std::min(f->grid, (n + 255) / 256));
  fv_claim_kernel<<<g, 256, 0, f->st>>>(f->N, n, f->idxBuf, f->win, f->err);
  fv_input_kernel<<<g, 256, 0, f->st>>>(f->N, f->B, b, n, f->idxBuf, vals, f->x, f->win);
  FVCU(cudaGetLastError());
  return fv_sync_err(f, "fb_flyvis_set_input");
}

extern "C" int fb_flyvis_write(fb_flyvis *f, int32_t field, int32_t b, const float *values) {
  int rc = fv_check(f, b, "fb_flyvis_write");
  if (rc) return rc;
  if (!values || (field != FB_FV_V && field != FB_FV_X)) return fvfail(FB_EINVAL, "fb_flyvis_write: bad field %d", field);
  FVCU(cudaMemcpyAsync(f->scratch, values, (size_t)f->N * 4, cudaMemcpyDefault, f->st));
  fv_scatter_kernel<<<std::min(f->grid, (f->N + 255) / 256), 256, 0, f->st>>>(f->N, f->B, b, f->scratch,
                                                                            field == FB_FV_V ? f->v[f->cur] : f->x);
  FVCU(cudaGetLastError());
  FVCU(cudaStreamSynchronize(f->st));
  return FB_OK;
}

extern "C" int fb_flyvis_read(fb_flyvis *f, int32_t field, int32_t b, float *out) {
  int rc = fv_check(f, b, "fb_flyvis_read");
  if (rc) return rc;
  if (!out || (field != FB_FV_V && field != FB_FV_X)) return fvfail(FB_EINVAL, "fb_flyvis_read: bad field %d", field);
  fv_gather_kernel<<<std::min(f->grid, (f->N + 255) / 256), 256, 0, f->st>>>(f->N, f->B, b,
                                                                           field == FB_FV_V ? f->v[f->cur] : f->x, f->scratch);
  FVCU(cudaGetLastError());
  FVCU(cudaMemcpyAsync(out, f->scratch, (size_t)f->N * 4, cudaMemcpyDefault, f->st));
  FVCU(cudaStreamSynchronize(f->st));
  return FB_OK;
}

extern "C" int fb_flyvis_step(fb_flyvis *f, int32_t nsteps) {
  int rc = fv_check(f, 0, "fb_flyvis_step");
  if (rc) return rc;
  if (nsteps < 0) return fvfail(FB_EINVAL, "fb_flyvis_step: nsteps=%d", nsteps);
  FVCU(cudaEventRecord(f->ev0, f->st));
  for (int32_t s = 0; s < nsteps; s++) {
    fv_step_kernel<<<f->grid, kFvThreads, 0, f->st>>>(f->N, f->B, f->cscPtr, f->cscSrc, f->cscW, f->bias, f->kdt,
                                                       f->v[f->cur], f->v[f->cur ^ 1], f->x);
    f->cur ^= 1;
  }
  FVCU(cudaEventRecord(f->ev1, f->st));
  FVCU(cudaGetLastError());
  FVCU(cudaStreamSynchronize(f->st));
  cudaEventElapsedTime(&f->lastMs, f->ev0, f->ev1);
  return FB_OK;
}

extern "C" int fb_flyvis_last_ms(fb_flyvis *f, float *ms) {
  if (!f || !ms) return fvfail(FB_EINVAL, "fb_flyvis_last_ms: null argument");
  *ms = f->lastMs;
  return FB_OK;
}

extern "C" int fb_flyvis_state(fb_flyvis *f, float **v, float **x, int32_t *layout_b) {
  if (!f) return fvfail(FB_EINVAL, "fb_flyvis_state: null handle");
  if (v) *v = f->v[f->cur];
  if (x) *x = f->x;
  if (layout_b) *layout_b = f->B;
  return FB_OK;
}
