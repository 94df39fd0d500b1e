// C ABI of the brain step (include/flybrain.h): graphs, brain batches, the LIFWasm-shaped
// injection/readout surface, and the persistent step launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "fb_internal.cuh"
#include "fb_lagged.cuh"

namespace fb {
cudaError_t launch_rebuild_slots(Trial *Td, int nslots, int32_t *err, cudaStream_t st);
int step_kernel_blocks_per_sm(size_t smem);
size_t step_smem_bytes(int B);
cudaError_t launch_step(const StepArgs &a, int grid, size_t smem, cudaStream_t st);
struct Delta {
  int32_t brain, field, idx, pad;
  double val;
};
cudaError_t launch_deltas(Trial *trials, const Delta *d, const int32_t *gs, int32_t nGroups, cudaStream_t st);
cudaError_t launch_reset(Trial *trials, int32_t b0, int32_t b1, cudaStream_t st);
cudaError_t set_step_smem(size_t bytes);
struct CompileArgs {
  int32_t N;
  const uint32_t *indptr, *indices;
  const float *counts, *edgeGain, *preSign, *inScale, *outScale;
  const uint8_t *sensory;
  double wSyn, inhGain, minSyn, preInh;
  float *W, *sign;
};
cudaError_t launch_compile(const CompileArgs &a, cudaStream_t st);
}  // namespace fb

using namespace fb;

// ---------------------------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------------------------
static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CU(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      return fail(e_ == cudaErrorMemoryAllocation ? FB_ENOMEM : FB_ECUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                 \
    }                                                                                  \
  } while (0)

// Constant-state flags of a brain whose state was just reset (adapt 0, res 1).
static int32_t rest_flags(const Trial &T) {
  return (T.adaptInc == 0.f ? kAdaptZero : 0) | (T.depU == 0.f ? kResRest : 0);
}

extern "C" const char *fb_last_error(void) { return g_err.c_str(); }
extern "C" int fb_version(void) { return 100; }

extern "C" int fb_device_info(int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  cudaDeviceProp p;
  CU(cudaGetDeviceProperties(&p, dev));
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return FB_OK;
}

extern "C" void fb_default_params(fb_params *p) {
  if (!p) return;
  memset(p, 0, sizeof *p);
  p->dt = 0.5; p->vRest = -52; p->vThresh = -45; p->vReset = -52; p->tauM = 20; p->tauSyn = 5;
  p->tRef = 2.2; p->delay = 1.8; p->traceTau = 30; p->adaptInc = 2.0; p->adaptTau = 100;
  p->depU = 0.2; p->depTau = 200; p->eExc = 0; p->eInh = -70; p->bgRate = 0; p->bgAmp = 0;
  p->preInh = 0; p->coba = 0;
}

// ---------------------------------------------------------------------------------------------
// per-device constants: xorshift32 jump tables
// ---------------------------------------------------------------------------------------------

// Columns of M^(2^j) for the xorshift32 map M (x ^= x<<13; x ^= x>>17; x ^= x<<5), expanded to 8
// nibble tables of 16 words each: table[j][n][v] = M^(2^j) applied to (v << 4n).
static void build_jump_tables(std::vector<uint32_t> &tab) {
  auto step = [](uint32_t x) { x ^= x << 13; x ^= x >> 17; x ^= x << 5; return x; };
  uint32_t col[32][32];  // col[j][b] = M^(2^j) e_b
  for (int b = 0; b < 32; b++) col[0][b] = step(1u << b);
  auto apply = [&](int j, uint32_t x) {
    uint32_t y = 0;
    for (int b = 0; b < 32; b++)
      if (x >> b & 1u) y ^= col[j][b];
    return y;
  };
  for (int j = 1; j < 32; j++)
    for (int b = 0; b < 32; b++) col[j][b] = apply(j - 1, col[j - 1][b]);
  tab.assign(32 * 128, 0);
  for (int j = 0; j < 32; j++)
    for (int n = 0; n < 8; n++)
      for (uint32_t v = 0; v < 16; v++) {
        uint32_t y = 0;
        for (int b = 0; b < 4; b++)
          if (v >> b & 1u) y ^= col[j][4 * n + b];
        tab[j * 128 + n * 16 + v] = y;
      }
}

namespace fb {
// The jump tables and the error slot, for the allocation-free entry point.
void host_jump_tables(std::vector<uint32_t> &tab) { build_jump_tables(tab); }
int set_error(int code, const char *msg) {
  g_err = msg;
  return code;
}
}  // namespace fb

static std::mutex g_dev_mu;
static uint32_t *g_jump[64];

static int device_jump(uint32_t **out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FB_ENODEV, "device ordinal %d unsupported", dev);
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (!g_jump[dev]) {
    cudaDeviceProp p;
    CU(cudaGetDeviceProperties(&p, dev));
    if (p.major != 10 || p.minor != 3)
      return fail(FB_ENODEV, "device %d is sm_%d%d; this library is built for sm_103a", dev, p.major, p.minor);
    std::vector<uint32_t> tab;
    build_jump_tables(tab);
    uint32_t *d = nullptr;
    CU(cudaMalloc(&d, tab.size() * 4));
    CU(cudaMemcpy(d, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
    g_jump[dev] = d;
  }
  *out = g_jump[dev];
  return FB_OK;
}

// ---------------------------------------------------------------------------------------------
// graphs
// ---------------------------------------------------------------------------------------------
struct Topology {
  int32_t N = 0;
  int64_t E = 0;
  uint32_t *indptr = nullptr, *indices = nullptr;
  // per edge, how many earlier edges of its row have the same target (0 .. kMaxRepeat); null
  // when no row repeats a target
  uint8_t *dup = nullptr;
  int refs = 0;
};

struct fb_graph {
  Topology *topo = nullptr;
  float *W = nullptr, *sign = nullptr;
};

static void topo_release(Topology *t) {
  if (t && --t->refs == 0) {
    cudaFree(t->indptr);
    cudaFree(t->indices);
    cudaFree(t->dup);
    delete t;
  }
}

extern "C" int fb_graph_create(int32_t N, int64_t E, const uint32_t *indptr, const uint32_t *indices,
                               const float *weights, const float *sign, fb_graph **out) {
  if (!out) return fail(FB_EINVAL, "fb_graph_create: out is null");
  *out = nullptr;
  if (N <= 0 || E < 0 || !indptr || (E > 0 && (!indices || !weights)) || !sign)
    return fail(FB_EINVAL, "fb_graph_create: bad sizes or null arrays (N=%d E=%lld)", N, (long long)E);
  if (E > 0xfffffff0LL) return fail(FB_EINVAL, "fb_graph_create: E=%lld exceeds 32-bit edge offsets", (long long)E);
  uint32_t *jt;
  int rc = device_jump(&jt);
  if (rc) return rc;
  // validate the CSR on the host (arrays may live on either side)
  std::vector<uint32_t> ip(N + 1), ix(E);
  CU(cudaMemcpy(ip.data(), indptr, (size_t)(N + 1) * 4, cudaMemcpyDefault));
  if (E) CU(cudaMemcpy(ix.data(), indices, (size_t)E * 4, cudaMemcpyDefault));
  if (ip[0] != 0 || ip[N] != (uint64_t)E) return fail(FB_EINVAL, "fb_graph_create: indptr[0]=%u indptr[N]=%u, E=%lld", ip[0], ip[N], (long long)E);
  if (N >= (1 << 29) - kLagPer * kLagThreads * kLagMaxDB)
    return fail(FB_EINVAL, "fb_graph_create: N=%d exceeds the delivery keys' %d", N, (1 << 29) - kLagPer * kLagThreads * kLagMaxDB);
  // a row may name a target more than once (lif.c:40-42 adds each edge in row order): each edge
  // gets its repeat index, which orders a presynaptic neuron's contributions to one target
  std::vector<int32_t> stamp(N, -1);
  std::vector<uint8_t> rep, seen(N, 0);
  bool anyRep = false;
  for (int32_t r = 0; r < N; r++) {
    if (ip[r + 1] < ip[r]) return fail(FB_EINVAL, "fb_graph_create: indptr decreases at row %d", r);
    for (uint32_t j = ip[r]; j < ip[r + 1]; j++) {
      const uint32_t q = ix[j];
      if (q >= (uint32_t)N) return fail(FB_EINVAL, "fb_graph_create: indices[%u]=%u out of range", j, q);
      if (stamp[q] == r) {
        if (seen[q] >= kMaxRepeat)
          return fail(FB_EINVAL, "fb_graph_create: row %d names target %u more than %d times", r, q, kMaxRepeat + 1);
        if (!anyRep) {
          rep.assign((size_t)E, 0);
          anyRep = true;
        }
        rep[j] = ++seen[q];
      } else {
        stamp[q] = r;
        seen[q] = 0;
      }
    }
  }
  Topology *t = new (std::nothrow) Topology;
  fb_graph *g = new (std::nothrow) fb_graph;
  if (!t || !g) { delete t; delete g; return fail(FB_ENOMEM, "host allocation"); }
  t->N = N; t->E = E; t->refs = 1;
  g->topo = t;
  auto cleanup = [&]() { cudaFree(g->W); cudaFree(g->sign); topo_release(t); delete g; };
  if (cudaMalloc(&t->indptr, (size_t)(N + 1) * 4) != cudaSuccess ||
      cudaMalloc(&t->indices, (size_t)std::max<int64_t>(E, 1) * 4) != cudaSuccess ||
      cudaMalloc(&g->W, (size_t)std::max<int64_t>(E, 1) * 4) != cudaSuccess ||
      cudaMalloc(&g->sign, (size_t)N * 4) != cudaSuccess) {
    cleanup();
    return fail(FB_ENOMEM, "fb_graph_create: device allocation of %lld edges failed", (long long)E);
  }
  if (cudaMemcpy(t->indptr, ip.data(), (size_t)(N + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      (E && cudaMemcpy(t->indices, ix.data(), (size_t)E * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
      (E && cudaMemcpy(g->W, weights, (size_t)E * 4, cudaMemcpyDefault) != cudaSuccess) ||
      cudaMemcpy(g->sign, sign, (size_t)N * 4, cudaMemcpyDefault) != cudaSuccess) {
    cleanup();
    return fail(FB_ECUDA, "fb_graph_create: upload failed");
  }
  if (anyRep && (cudaMalloc(&t->dup, (size_t)E) != cudaSuccess ||
                 cudaMemcpy(t->dup, rep.data(), (size_t)E, cudaMemcpyHostToDevice) != cudaSuccess)) {
    cleanup();
    return fail(FB_ECUDA, "fb_graph_create: upload of the repeat indices failed");
  }
  *out = g;
  return FB_OK;
}

extern "C" int fb_graph_create_shared(const fb_graph *topology, const float *weights, const float *sign,
                                      fb_graph **out) {
  if (!topology || !out || !weights || !sign) return fail(FB_EINVAL, "fb_graph_create_shared: null argument");
  *out = nullptr;
  Topology *t = topology->topo;
  fb_graph *g = new (std::nothrow) fb_graph;
  if (!g) return fail(FB_ENOMEM, "host allocation");
  if (cudaMalloc(&g->W, (size_t)std::max<int64_t>(t->E, 1) * 4) != cudaSuccess ||
      cudaMalloc(&g->sign, (size_t)t->N * 4) != cudaSuccess) {
    cudaFree(g->W); cudaFree(g->sign); delete g;
    return fail(FB_ENOMEM, "fb_graph_create_shared: device allocation failed");
  }
  if ((t->E && cudaMemcpy(g->W, weights, (size_t)t->E * 4, cudaMemcpyDefault) != cudaSuccess) ||
      cudaMemcpy(g->sign, sign, (size_t)t->N * 4, cudaMemcpyDefault) != cudaSuccess) {
    cudaFree(g->W); cudaFree(g->sign); delete g;
    return fail(FB_ECUDA, "fb_graph_create_shared: upload failed");
  }
  t->refs++;
  g->topo = t;
  *out = g;
  return FB_OK;
}

// A device-resident view of an argument array: the array itself when it already lives on the
// device, else a temporary device copy (released by the caller through `tmp`).
static int device_view(const void *src, size_t bytes, const void **dst, std::vector<void *> &tmp) {
  *dst = nullptr;
  if (!src) return FB_OK;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, src) == cudaSuccess && at.type == cudaMemoryTypeDevice) {
    *dst = src;
    return FB_OK;
  }
  cudaGetLastError();
  void *d = nullptr;
  CU(cudaMalloc(&d, bytes ? bytes : 1));
  tmp.push_back(d);
  CU(cudaMemcpy(d, src, bytes, cudaMemcpyDefault));
  *dst = d;
  return FB_OK;
}

extern "C" int fb_graph_compile(const fb_graph *topology, const float *counts, const float *pre_sign,
                                const float *in_scale, const float *out_scale,
                                const uint8_t *sensory_mask, const float *edge_gain,
                                const fb_compile_params *p, fb_graph **out) {
  if (!topology || !counts || !pre_sign || !p || !out) return fail(FB_EINVAL, "fb_graph_compile: null argument");
  *out = nullptr;
  Topology *t = topology->topo;
  const size_t N = (size_t)t->N, E = (size_t)t->E;
  std::vector<void *> tmp;
  auto release = [&]() { for (void *q : tmp) cudaFree(q); };
  CompileArgs a;
  memset(&a, 0, sizeof a);
  const void *v;
  int rc;
#define VIEW(ptr, bytes, field, type)                          \
  rc = device_view(ptr, bytes, &v, tmp);                       \
  if (rc) { release(); return rc; }                            \
  a.field = (const type *)v;
  VIEW(counts, E * 4, counts, float)
  VIEW(edge_gain, E * 4, edgeGain, float)
  VIEW(pre_sign, N * 4, preSign, float)
  VIEW(in_scale, N * 4, inScale, float)
  VIEW(out_scale, N * 4, outScale, float)
  VIEW(sensory_mask, N, sensory, uint8_t)
#undef VIEW
  fb_graph *g = new (std::nothrow) fb_graph;
  if (!g) { release(); return fail(FB_ENOMEM, "host allocation"); }
  if (cudaMalloc(&g->W, std::max<size_t>(E, 1) * 4) != cudaSuccess || cudaMalloc(&g->sign, N * 4) != cudaSuccess) {
    cudaFree(g->W); cudaFree(g->sign); delete g; release();
    return fail(FB_ENOMEM, "fb_graph_compile: device allocation failed");
  }
  a.N = t->N;
  a.indptr = t->indptr;
  a.indices = t->indices;
  a.wSyn = p->wSyn;
  a.inhGain = p->inhGain;
  a.minSyn = p->minSyn;
  a.preInh = p->preInh;
  a.W = g->W;
  a.sign = g->sign;
  cudaError_t e = launch_compile(a, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  release();
  if (e != cudaSuccess) {
    cudaFree(g->W); cudaFree(g->sign); delete g;
    return fail(FB_ECUDA, "fb_graph_compile: %s", cudaGetErrorString(e));
  }
  t->refs++;
  g->topo = t;
  *out = g;
  return FB_OK;
}

extern "C" int fb_graph_read(const fb_graph *g, float *weights, float *sign) {
  if (!g) return fail(FB_EINVAL, "fb_graph_read: null graph");
  if (weights && g->topo->E) CU(cudaMemcpy(weights, g->W, (size_t)g->topo->E * 4, cudaMemcpyDefault));
  if (sign) CU(cudaMemcpy(sign, g->sign, (size_t)g->topo->N * 4, cudaMemcpyDefault));
  return FB_OK;
}

extern "C" int fb_graph_set_sign(fb_graph *g, const float *sign) {
  if (!g || !sign) return fail(FB_EINVAL, "fb_graph_set_sign: null argument");
  CU(cudaDeviceSynchronize());  // no step may be reading the old vector
  CU(cudaMemcpy(g->sign, sign, (size_t)g->topo->N * 4, cudaMemcpyDefault));
  return FB_OK;
}

extern "C" int fb_graph_info(const fb_graph *g, int32_t *N, int64_t *E) {
  if (!g) return fail(FB_EINVAL, "fb_graph_info: null graph");
  if (N) *N = g->topo->N;
  if (E) *E = g->topo->E;
  return FB_OK;
}

extern "C" int fb_graph_destroy(fb_graph *g) {
  if (!g) return FB_OK;
  cudaFree(g->W);
  cudaFree(g->sign);
  topo_release(g->topo);
  delete g;
  return FB_OK;
}

// ---------------------------------------------------------------------------------------------
// brain batches
// ---------------------------------------------------------------------------------------------

// Insertion-ordered set of driven neurons (a JS Set: deletion keeps the others' order, re-adding
// appends). Deleted entries are tombstones until the next sync compacts the list.
struct DrivenSet {
  std::vector<int32_t> order;  // neuron or -1
  std::vector<int32_t> pos;    // index in order, or -1
  bool dirty = true;
  uint64_t version = 0;  // changes with the set (ownership of the delay-scheduled kernel)
  void init(int N) { order.clear(); pos.assign(N, -1); dirty = true; version++; }
  void add(int32_t i) {
    if (pos[i] >= 0) return;
    pos[i] = (int32_t)order.size();
    order.push_back(i);
    dirty = true;
    version++;
  }
  void remove(int32_t i) {
    if (pos[i] < 0) return;
    order[pos[i]] = -1;
    pos[i] = -1;
    dirty = true;
    version++;
  }
  void compact() {
    size_t n = 0;
    for (size_t k = 0; k < order.size(); k++)
      if (order[k] >= 0) {
        order[n] = order[k];
        pos[order[n]] = (int32_t)n;
        n++;
      }
    order.resize(n);
  }
};

// Device resources of the delay-scheduled kernel (fb_lagged.cu) for a single brain, allocated
// at its first use at the largest sizes the brain can need.
struct LagRes {
  bool ready = false;
  int D = 0, S = 0, nTB = 0, capMax = 0, nDmax = 0, bgCap = 0, grid = 0;
  uint64_t drivenVersion = ~0ull;
  std::vector<void *> allocs;
  uint32_t *inOff = nullptr, *cnt = nullptr, *pend0 = nullptr, *sync = nullptr, *bgList = nullptr;
  uint32_t *jumpHex = nullptr;
  uint4 *edgeRec = nullptr;
  uint2 *buf = nullptr;
  uint4 *dbList = nullptr;
  int32_t *bgCount = nullptr, *dbCnt = nullptr, *dbNF = nullptr, *tStage = nullptr, *tCnt = nullptr;
  int32_t *ndIds = nullptr, *ndLo = nullptr, *drvPosOf = nullptr;
  int cap = 1, nD = 0;
  int nDB = 1, nDcap = 32, nDall = 32, dLo[kLagMaxDB + 1] = {0, 0, 0};
  unsigned long long *liveTag = nullptr;
  size_t smem = 0;
};

struct fb_brains {
  int B = 0;
  int dev = 0;
  cudaStream_t stream = nullptr;
  std::vector<Trial> host;   // host mirror: constants and device pointers
  Trial *trials = nullptr;   // device array
  std::vector<void *> arenas;
  std::vector<DrivenSet> driven;
  std::vector<Delta> deltas;
  std::vector<int32_t> tileTrial;
  int32_t *d_tileTrial = nullptr, *d_steps = nullptr, *d_err = nullptr, *d_groups = nullptr;
  Delta *d_deltas = nullptr;
  size_t deltaCap = 0, groupCap = 0;
  // pinned staging of a call's small transfers: queued writes and their group starts, the step
  // counts, the error flag and fired counts read back. A flush's copies leave the staging before
  // the next flush refills it (flushDone); the step counts are copied only when they change.
  Delta *h_deltas = nullptr;
  int32_t *h_groups = nullptr;
  size_t hDeltaCap = 0, hGroupCap = 0;
  int32_t *h_small = nullptr;  // [2 + B]: error flag, unused, fired count of each brain
  int32_t *h_steps = nullptr;  // [B]
  std::vector<int32_t> stepsUploaded, groupStarts;
  cudaEvent_t flushDone = nullptr;
  bool flushPending = false;
  uint32_t *d_bar = nullptr;   // the grid barrier's counter word (own 128-byte line)
  static constexpr size_t kBarWords = 32;
  unsigned long long *d_phase = nullptr;  // per-phase ns accumulators when profiling
  uint32_t *d_dbg = nullptr;              // index-check record of checked builds
  int profiling = 0;
  OvfRec *d_ovf[2] = {nullptr, nullptr};
  uint32_t *d_ovfTop = nullptr;
  uint32_t ovfCap = 0;
  uint32_t *jump = nullptr;
  std::vector<int32_t> stepsHost;
  std::vector<double> dts;   // each brain's dt as given (double), for setBackground
  int grid = 0;
  size_t smem = 0;
  int blocksPerSm = 0, maxBlocksPerSm = 0, sms = 0;  // the persistent grid: sms x blocksPerSm
  int32_t itemChunks = 1;
  int32_t subGrab = 4;
  int64_t timeoutNs = 5000000000LL;  // bound of every device-side wait (fb_tuning.timeout_us)
  int32_t tripStep = -1;             // test hook (fb_debug_trip_wait): armed for one launch
  int32_t lagDB = 0;                 // driven blocks of the delay-scheduled kernel (0: automatic)
  int logging = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float lastMs = 0.f;
  int32_t schedule = FB_SCHEDULE_AUTO, lastSchedule = FB_SCHEDULE_GRID;
  LagRes lag;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static int brains_fail_cleanup(fb_brains *br, int rc) {
  std::string keep = g_err;
  fb_brains_destroy(br);
  g_err = keep;
  return rc;
}

// Per-brain header constants: each computed in double and rounded once to f32, in the
// expressions of LIFWasm._writeHeader (src/lifwasm.js:58-67).
static void fill_constants(Trial &T, const fb_params &p, int32_t N) {
  T.coba = p.coba ? 1 : 0;
  T.dt = (float)p.dt; T.vRest = (float)p.vRest; T.vThresh = (float)p.vThresh; T.vReset = (float)p.vReset;
  T.tRef = (float)p.tRef; T.adaptInc = (float)p.adaptInc; T.depU = (float)p.depU;
  T.dE = (float)std::exp(-p.dt / p.tauSyn);
  T.dTr = (float)std::exp(-p.dt / p.traceTau);
  T.dA = (float)std::exp(-p.dt / p.adaptTau);
  T.kRec = (float)(p.dt / p.depTau);
  T.kM = (float)(p.dt / p.tauM);
  T.dtS = (float)(p.dt / 1000);
  T.eExc = (float)p.eExc; T.eInh = (float)p.eInh;
  T.cE = (float)(1 / (p.eExc - p.vRest));
  T.cI = (float)(1 / (p.vRest - p.eInh));
  T.bgEvents = (float)((double)N * p.bgRate * p.dt / 1000);
  T.bgAmp = (float)p.bgAmp;
  T.preInh = (float)p.preInh;
  T.flags = (T.bgEvents > 0 ? kHasBg : 0) | (T.depU != 0.f ? kHasDep : 0) | (T.preInh > 0.f ? kHasPreInh : 0) |
            rest_flags(T) | kBiasZero | kThrZero;  // the state starts at rest (launch_reset below)
}

// JS: (seed * 2654435761) >>> 0 || 1, the product formed in double (src/lifwasm.js:52).
static uint32_t seed_state(uint32_t seed) {
  const double prod = (double)seed * 2654435761.0;
  const double m = std::fmod(std::floor(prod), 4294967296.0);
  const uint32_t s = (uint32_t)m;
  return s ? s : 1u;
}

extern "C" int fb_brains_create(const fb_graph *const *graphs, int32_t B, const fb_params *params,
                                int32_t params_stride, const uint32_t *seeds, fb_brains **out) {
  if (!out) return fail(FB_EINVAL, "fb_brains_create: out is null");
  *out = nullptr;
  if (!graphs || B <= 0 || !params || !seeds) return fail(FB_EINVAL, "fb_brains_create: bad arguments (B=%d)", B);
  if (B > 8192) return fail(FB_EINVAL, "fb_brains_create: B=%d exceeds 8192 brains per batch", B);
  fb_brains *br = new (std::nothrow) fb_brains;
  if (!br) return fail(FB_ENOMEM, "host allocation");
  int rc = device_jump(&br->jump);
  if (rc) { delete br; return rc; }
  if (cudaGetDevice(&br->dev) != cudaSuccess || cudaStreamCreateWithFlags(&br->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete br;
    return fail(FB_ECUDA, "stream creation failed");
  }
  br->B = B;
  br->host.assign(B, Trial{});
  br->dts.assign(B, 0.0);
  br->driven.resize(B);
  int tileBase = 0;
  for (int b = 0; b < B; b++) {
    const fb_graph *g = graphs[b];
    const fb_params &p = *(const fb_params *)((const char *)params + (size_t)b * params_stride);
    if (!g) return brains_fail_cleanup(br, fail(FB_EINVAL, "fb_brains_create: graphs[%d] is null", b));
    if (!(p.dt > 0) || !(p.delay >= 0) || !(p.tauM > 0) || !(p.tauSyn > 0))
      return brains_fail_cleanup(br, fail(FB_EINVAL, "fb_brains_create: brain %d: dt, tauM, tauSyn must be > 0", b));
    const int32_t N = g->topo->N;
    const int64_t E = g->topo->E;
    // ring depth, src/lifwasm.js:39: max(1, Math.round(delay / dt)) + 1
    const int ns = (int)std::max(1.0, std::floor(p.delay / p.dt + 0.5)) + 1;
    if (ns < 3)
      return brains_fail_cleanup(br, fail(FB_EINVAL, "fb_brains_create: brain %d: delay/dt rounds to %d step; at least 2 are required", b, ns - 1));
    Trial &T = br->host[b];
    br->dts[b] = p.dt;
    T.N = N;
    T.E = E;
    T.nslots = ns;
    T.mode = FB_DELIVER_EXACT;
    fill_constants(T, p, N);
    if (T.flags & kHasPreInh) T.mode = FB_DELIVER_SEQUENTIAL;
    T.nTiles = (N + kTile - 1) / kTile;
    T.tileBase = tileBase;
    tileBase += T.nTiles;
    for (int u = 0; u < T.nTiles; u++) br->tileTrial.push_back(b);
    T.chunkCap = (E + kChunk - 1) / kChunk + 1;
    T.indptr = g->topo->indptr;
    T.indices = g->topo->indices;
    T.dup = g->topo->dup;
    T.W = g->W;
    T.sign = g->sign;
    T.rngP[0] = seed_state(seeds[b]);
    T.maxDch = std::max(1, (N + kBlock - 1) / kBlock);
    // arena layout
    const size_t n4 = align256((size_t)N * 4);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    size_t o_state = take(n4 * 11);
    size_t o_ring = take((size_t)ns * N * 4), o_ringCount = take((size_t)ns * 4);
    size_t o_ringOff = take((size_t)ns * (N + 1) * 4), o_chunkK = take((size_t)ns * T.chunkCap * 16);
    size_t o_ringRow = take((size_t)ns * N * 4);
    size_t o_slotEdges = take((size_t)ns * 4), o_driven = take((size_t)N * 4);
    size_t o_cnt = take((size_t)N * 4), o_bucket = take((size_t)N * kBucket * 8);
    size_t o_ovfHead = take((size_t)N * 4), o_bg = take((size_t)N * 4), o_arr = take((size_t)N);
    size_t o_stage = take((size_t)T.nTiles * kTile * 4), o_stageDeg = take((size_t)T.nTiles * kTile * 4);
    size_t o_tileCnt = take((size_t)T.nTiles * kSubPerTile * 4), o_tileDeg = take((size_t)T.nTiles * kSubPerTile * 4);
    size_t o_dStage = take((size_t)2 * T.maxDch * kBlock * 4), o_dStageDeg = take((size_t)2 * T.maxDch * kBlock * 4);
    size_t o_dCnt = take((size_t)2 * T.maxDch * 4), o_dDeg = take((size_t)2 * T.maxDch * 4);
    size_t o_live = take((size_t)T.maxDch * 8);
    char *base = nullptr;
    if (cudaMalloc(&base, off) != cudaSuccess)
      return brains_fail_cleanup(br, fail(FB_ENOMEM, "fb_brains_create: brain %d: %zu bytes of device memory", b, off));
    br->arenas.push_back(base);
    if (cudaMemsetAsync(base, 0, off, br->stream) != cudaSuccess ||
        cudaMemsetAsync(base + o_ovfHead, 0xff, (size_t)N * 4, br->stream) != cudaSuccess)
      return brains_fail_cleanup(br, fail(FB_ECUDA, "fb_brains_create: clearing state failed"));
    float *st = (float *)(base + o_state);
    T.v = st; T.gE = (float *)((char *)st + n4); T.gI = (float *)((char *)st + 2 * n4);
    T.refr = (float *)((char *)st + 3 * n4); T.trace = (float *)((char *)st + 4 * n4);
    T.adapt = (float *)((char *)st + 5 * n4); T.res = (float *)((char *)st + 6 * n4);
    T.bias = (float *)((char *)st + 7 * n4); T.thr = (float *)((char *)st + 8 * n4);
    T.drive = (float *)((char *)st + 9 * n4); T.spikeCount = (uint32_t *)((char *)st + 10 * n4);
    T.ring = (int32_t *)(base + o_ring); T.ringCount = (int32_t *)(base + o_ringCount);
    T.ringOff = (uint32_t *)(base + o_ringOff); T.chunkK = (uint4 *)(base + o_chunkK);
    T.ringRow = (uint32_t *)(base + o_ringRow);
    T.slotEdges = (uint32_t *)(base + o_slotEdges); T.driven = (int32_t *)(base + o_driven);
    T.cnt = (uint32_t *)(base + o_cnt); T.bucket = (uint2 *)(base + o_bucket);
    T.ovfHead = (uint32_t *)(base + o_ovfHead); T.bgHits = (uint32_t *)(base + o_bg);
    T.arrived = (uint8_t *)(base + o_arr);
    T.stage = (int32_t *)(base + o_stage); T.stageDeg = (uint32_t *)(base + o_stageDeg);
    T.tileCnt = (int32_t *)(base + o_tileCnt); T.tileDeg = (uint32_t *)(base + o_tileDeg);
    T.dStage = (int32_t *)(base + o_dStage); T.dStageDeg = (uint32_t *)(base + o_dStageDeg);
    T.dCnt = (int32_t *)(base + o_dCnt); T.dDeg = (uint32_t *)(base + o_dDeg);
    T.liveTag = (unsigned long long *)(base + o_live);
    br->driven[b].init(N);
  }
  // batch-wide buffers
  const int nTiles = (int)br->tileTrial.size();
  if (cudaMalloc(&br->trials, sizeof(Trial) * B) != cudaSuccess ||
      cudaMalloc(&br->d_tileTrial, sizeof(int32_t) * nTiles) != cudaSuccess ||
      cudaMalloc(&br->d_steps, sizeof(int32_t) * B) != cudaSuccess ||
      cudaMalloc(&br->d_err, sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&br->d_dbg, sizeof(uint32_t) * 4) != cudaSuccess ||
      cudaMalloc(&br->d_bar, sizeof(uint32_t) * fb_brains::kBarWords) != cudaSuccess ||
      cudaMalloc(&br->d_ovfTop, sizeof(uint32_t) * 4) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ENOMEM, "fb_brains_create: batch buffers"));
  // overflow pool: 1M records per parity plus one per 16 edges of the largest graph
  int64_t maxE = 0;
  for (int b = 0; b < B; b++) maxE = std::max<int64_t>(maxE, graphs[b]->topo->E);
  br->ovfCap = (uint32_t)std::min<int64_t>((1 << 20) + maxE / 16, 0x7fffffff);
  for (int k = 0; k < 2; k++)
    if (cudaMalloc(&br->d_ovf[k], sizeof(OvfRec) * (size_t)br->ovfCap) != cudaSuccess)
      return brains_fail_cleanup(br, fail(FB_ENOMEM, "fb_brains_create: overflow pool"));
  if (cudaMemsetAsync(br->d_err, 0, 4, br->stream) != cudaSuccess ||
      cudaMemsetAsync(br->d_dbg, 0, 16, br->stream) != cudaSuccess ||
      cudaMemsetAsync(br->d_bar, 0, sizeof(uint32_t) * fb_brains::kBarWords, br->stream) != cudaSuccess ||
      cudaMemsetAsync(br->d_ovfTop, 0, 16, br->stream) != cudaSuccess ||
      cudaMemcpyAsync(br->d_tileTrial, br->tileTrial.data(), sizeof(int32_t) * nTiles, cudaMemcpyHostToDevice, br->stream) != cudaSuccess ||
      cudaMemcpyAsync(br->trials, br->host.data(), sizeof(Trial) * B, cudaMemcpyHostToDevice, br->stream) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ECUDA, "fb_brains_create: upload failed"));
  if (launch_reset(br->trials, 0, B, br->stream) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ECUDA, "fb_brains_create: reset launch failed"));
  // persistent grid: every SM, as many blocks as stay co-resident
  br->smem = step_smem_bytes(B);
  if (set_step_smem(br->smem) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ECUDA, "step kernel: %zu bytes of shared memory refused", br->smem));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, br->dev);
  const int per = step_kernel_blocks_per_sm(br->smem);
  if (per <= 0) return brains_fail_cleanup(br, fail(FB_ECUDA, "step kernel does not fit on an SM (smem %zu)", br->smem));
  br->grid = sms * per;
  br->sms = sms;
  br->blocksPerSm = br->maxBlocksPerSm = per;
  cudaEventCreate(&br->ev0);
  cudaEventCreate(&br->ev1);
  cudaEventCreateWithFlags(&br->flushDone, cudaEventDisableTiming);
  if (cudaMallocHost(&br->h_small, sizeof(int32_t) * (2 + (size_t)B)) != cudaSuccess ||
      cudaMallocHost(&br->h_steps, sizeof(int32_t) * (size_t)B) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ENOMEM, "fb_brains_create: pinned host staging"));
  if (cudaStreamSynchronize(br->stream) != cudaSuccess)
    return brains_fail_cleanup(br, fail(FB_ECUDA, "fb_brains_create: %s", cudaGetErrorString(cudaGetLastError())));
  *out = br;
  return FB_OK;
}

extern "C" int fb_brains_destroy(fb_brains *br) {
  if (!br) return FB_OK;
  if (br->stream) cudaStreamSynchronize(br->stream);
  for (int b = 0; b < (int)br->host.size(); b++) {
    cudaFree(br->host[b].logCount);
    cudaFree(br->host[b].logRaster);
  }
  for (void *p : br->arenas) cudaFree(p);
  cudaFree(br->trials); cudaFree(br->d_tileTrial); cudaFree(br->d_steps); cudaFree(br->d_err);
  cudaFree(br->d_groups); cudaFree(br->d_deltas); cudaFree(br->d_bar); cudaFree(br->d_ovfTop);
  cudaFree(br->d_phase);
  cudaFree(br->d_dbg);
  cudaFree(br->d_ovf[0]); cudaFree(br->d_ovf[1]);
  for (void *p : br->lag.allocs) cudaFree(p);
  if (br->ev0) cudaEventDestroy(br->ev0);
  if (br->ev1) cudaEventDestroy(br->ev1);
  if (br->flushDone) cudaEventDestroy(br->flushDone);
  cudaFreeHost(br->h_deltas);
  cudaFreeHost(br->h_groups);
  cudaFreeHost(br->h_small);
  cudaFreeHost(br->h_steps);
  if (br->stream) cudaStreamDestroy(br->stream);
  delete br;
  return FB_OK;
}

extern "C" int fb_brains_set_schedule(fb_brains *br, int32_t schedule) {
  if (!br || schedule < FB_SCHEDULE_AUTO || schedule > FB_SCHEDULE_LAGGED)
    return fail(FB_EINVAL, "fb_brains_set_schedule: bad schedule %d", schedule);
  br->schedule = schedule;
  return FB_OK;
}

extern "C" int fb_brains_set_tuning(fb_brains *br, const fb_tuning *t) {
  if (!br || !t) return fail(FB_EINVAL, "fb_brains_set_tuning: null argument");
  if (t->blocks_per_sm < 0 || t->blocks_per_sm > br->maxBlocksPerSm || t->item_chunks < 0 || t->item_chunks > 64 ||
      t->sub_grab < -1 || t->sub_grab > 256 || t->timeout_us < 0)
    return fail(FB_EINVAL, "fb_brains_set_tuning: blocks_per_sm %d (1..%d), item_chunks %d (1..64), sub_grab %d (-1, 1..256), "
                "timeout_us %d (>= 1)", t->blocks_per_sm, br->maxBlocksPerSm, t->item_chunks, t->sub_grab, t->timeout_us);
  if (t->timeout_us) br->timeoutNs = (int64_t)t->timeout_us * 1000;
  if (t->lag_driven_blocks < 0 || t->lag_driven_blocks > kLagMaxDB)
    return fail(FB_EINVAL, "fb_brains_set_tuning: lag_driven_blocks %d (0 automatic, 1..%d)", t->lag_driven_blocks, kLagMaxDB);
  if (t->lag_driven_blocks != br->lagDB) {
    br->lagDB = t->lag_driven_blocks;
    br->lag.drivenVersion = ~0ull;  // the ownership is recomputed at the next launch
  }
  if (t->blocks_per_sm) {
    br->blocksPerSm = t->blocks_per_sm;
    br->grid = br->sms * br->blocksPerSm;
  }
  if (t->item_chunks) br->itemChunks = t->item_chunks;
  if (t->sub_grab) br->subGrab = t->sub_grab < 0 ? 0 : t->sub_grab;
  return FB_OK;
}

extern "C" int fb_brains_tuning(fb_brains *br, fb_tuning *t) {
  if (!br || !t) return fail(FB_EINVAL, "fb_brains_tuning: null argument");
  t->blocks_per_sm = br->blocksPerSm;
  t->item_chunks = br->itemChunks;
  t->sub_grab = br->subGrab ? br->subGrab : -1;
  t->timeout_us = (int32_t)std::min<int64_t>(br->timeoutNs / 1000, 0x7fffffff);
  t->lag_driven_blocks = br->lagDB;
  t->pad = 0;
  t->max_blocks_per_sm = br->maxBlocksPerSm;
  t->sms = br->sms;
  return FB_OK;
}

extern "C" int fb_debug_trip_wait(fb_brains *br, int32_t step) {
  if (!br || step < -1) return fail(FB_EINVAL, "fb_debug_trip_wait: bad arguments");
  br->tripStep = step;
  return FB_OK;
}

extern "C" int fb_last_schedule(fb_brains *br, int32_t *schedule) {
  if (!br || !schedule) return fail(FB_EINVAL, "fb_last_schedule: null argument");
  *schedule = br->lastSchedule;
  return FB_OK;
}

extern "C" int fb_brains_set_mode(fb_brains *br, int32_t mode) {
  if (!br || mode < FB_DELIVER_EXACT || mode > FB_DELIVER_FAST) return fail(FB_EINVAL, "fb_brains_set_mode: bad mode %d", mode);
  for (int b = 0; b < br->B; b++) {
    Trial &T = br->host[b];
    T.mode = (T.flags & kHasPreInh) && mode == FB_DELIVER_EXACT ? FB_DELIVER_SEQUENTIAL : mode;
    if (T.mode == FB_DELIVER_FAST && (T.flags & kHasPreInh)) T.mode = FB_DELIVER_SEQUENTIAL;
    CU(cudaMemcpyAsync(&br->trials[b].mode, &T.mode, 4, cudaMemcpyHostToDevice, br->stream));
  }
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

static int check_brain(fb_brains *br, int32_t b, const char *fn) {
  if (!br) return fail(FB_EINVAL, "%s: null handle", fn);
  if (b < 0 || b >= br->B) return fail(FB_EINVAL, "%s: brain %d out of range [0, %d)", fn, b, br->B);
  return FB_OK;
}

// Applies queued injections (in call order) and re-uploads changed driven lists.
// Applies the queued host writes and the driven set. sync: wait for the writes to land (callers
// that go on with copies outside the brains' stream); the step path leaves them in stream order.
static int flush(fb_brains *br, bool sync = true) {
  if (!br->deltas.empty()) {
    std::vector<Delta> &d = br->deltas;
    auto before = [](const Delta &x, const Delta &y) {
      if (x.brain != y.brain) return x.brain < y.brain;
      if (x.field != y.field) return x.field < y.field;
      return x.idx < y.idx;
    };
    // groups of one (brain, field, index) in call order; lists written in ascending index order
    // (the usual case) need no sort
    if (!std::is_sorted(d.begin(), d.end(), before)) std::stable_sort(d.begin(), d.end(), before);
    std::vector<int32_t> &gs = br->groupStarts;
    gs.clear();
    for (size_t k = 0; k < d.size(); k++)
      if (k == 0 || d[k].brain != d[k - 1].brain || d[k].field != d[k - 1].field || d[k].idx != d[k - 1].idx)
        gs.push_back((int32_t)k);
    const int32_t ng = (int32_t)gs.size();
    gs.push_back((int32_t)d.size());
    if (br->flushPending) {  // the last flush's copies have left the staging (and its kernel ran)
      CU(cudaEventSynchronize(br->flushDone));
      br->flushPending = false;
    }
    if (d.size() > br->deltaCap) {
      cudaFree(br->d_deltas);
      br->deltaCap = std::max<size_t>(d.size(), 1024);
      CU(cudaMalloc(&br->d_deltas, sizeof(Delta) * br->deltaCap));
    }
    if (gs.size() > br->groupCap) {
      cudaFree(br->d_groups);
      br->groupCap = std::max<size_t>(gs.size(), 1025);
      CU(cudaMalloc(&br->d_groups, sizeof(int32_t) * br->groupCap));
    }
    if (d.size() > br->hDeltaCap) {
      cudaFreeHost(br->h_deltas);
      br->h_deltas = nullptr;
      br->hDeltaCap = std::max<size_t>(d.size(), 1024);
      CU(cudaMallocHost(&br->h_deltas, sizeof(Delta) * br->hDeltaCap));
    }
    if (gs.size() > br->hGroupCap) {
      cudaFreeHost(br->h_groups);
      br->h_groups = nullptr;
      br->hGroupCap = std::max<size_t>(gs.size(), 1025);
      CU(cudaMallocHost(&br->h_groups, sizeof(int32_t) * br->hGroupCap));
    }
    std::memcpy(br->h_deltas, d.data(), sizeof(Delta) * d.size());
    std::memcpy(br->h_groups, gs.data(), sizeof(int32_t) * gs.size());
    CU(cudaMemcpyAsync(br->d_deltas, br->h_deltas, sizeof(Delta) * d.size(), cudaMemcpyHostToDevice, br->stream));
    CU(cudaMemcpyAsync(br->d_groups, br->h_groups, sizeof(int32_t) * gs.size(), cudaMemcpyHostToDevice, br->stream));
    CU(launch_deltas(br->trials, br->d_deltas, br->d_groups, ng, br->stream));
    CU(cudaEventRecord(br->flushDone, br->stream));
    br->flushPending = true;
    d.clear();
  }
  for (int b = 0; b < br->B; b++) {
    DrivenSet &ds = br->driven[b];
    if (!ds.dirty) continue;
    ds.compact();
    Trial &T = br->host[b];
    T.nDriven = (int32_t)ds.order.size();
    if (T.nDriven)
      CU(cudaMemcpyAsync(T.driven, ds.order.data(), sizeof(int32_t) * T.nDriven, cudaMemcpyHostToDevice, br->stream));
    CU(cudaMemcpyAsync(&br->trials[b].nDriven, &T.nDriven, 4, cudaMemcpyHostToDevice, br->stream));
    CU(cudaStreamSynchronize(br->stream));
    ds.dirty = false;
  }
  if (sync && br->flushPending) {
    CU(cudaEventSynchronize(br->flushDone));
    br->flushPending = false;
  }
  return FB_OK;
}

static int queue(fb_brains *br, int32_t b, int32_t field, const int32_t *idx, const double *val,
                 int32_t n, const char *fn) {
  int rc = check_brain(br, b, fn);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!idx || !val))) return fail(FB_EINVAL, "%s: bad list (n=%d)", fn, n);
  const int32_t N = br->host[b].N;
  for (int32_t k = 0; k < n; k++) {
    if (idx[k] < 0 || idx[k] >= N) return fail(FB_EINVAL, "%s: index %d out of range [0, %d)", fn, idx[k], N);
    if (!std::isfinite(val[k]) && field != FB_FIELD_THR && field != FB_FIELD_BIAS)
      return fail(FB_EINVAL, "%s: value %g is not finite", fn, val[k]);
  }
  for (int32_t k = 0; k < n; k++) br->deltas.push_back(Delta{b, field, idx[k], 0, val[k]});
  if (field == FB_FIELD_BIAS || field == FB_FIELD_THR) {  // a word other than +0: the update reads the field
    const int32_t zf = field == FB_FIELD_BIAS ? kBiasZero : kThrZero;
    Trial &T = br->host[b];
    for (int32_t k = 0; k < n && (T.flags & zf); k++) {
      const float f = (float)val[k];
      uint32_t bits;
      std::memcpy(&bits, &f, 4);
      if (bits != 0u) {
        T.flags &= ~zf;
        CU(cudaMemcpyAsync(&br->trials[b].flags, &T.flags, 4, cudaMemcpyHostToDevice, br->stream));
      }
    }
  }
  return FB_OK;
}

extern "C" int fb_set_drive(fb_brains *br, int32_t b, const int32_t *idx, const double *hz, int32_t n) {
  int rc = queue(br, b, FB_FIELD_DRIVE, idx, hz, n, "fb_set_drive");
  if (rc) return rc;
  DrivenSet &ds = br->driven[b];
  for (int32_t k = 0; k < n; k++) {
    if (hz[k] > 0) ds.add(idx[k]);
    else ds.remove(idx[k]);
  }
  return FB_OK;
}

extern "C" int fb_set_bias(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  return queue(br, b, FB_FIELD_BIAS, idx, mv, n, "fb_set_bias");
}

extern "C" int fb_set_thr(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  return queue(br, b, FB_FIELD_THR, idx, mv, n, "fb_set_thr");
}

extern "C" int fb_add_g(fb_brains *br, int32_t b, const int32_t *idx, const double *e, const double *i, int32_t n) {
  int rc = queue(br, b, FB_FIELD_GE, idx, e, n, "fb_add_g");
  if (rc) return rc;
  if (i) {
    // addG(i, e, ii) always adds ii || 0 to gI (src/lifwasm.js:75)
    return queue(br, b, FB_FIELD_GI, idx, i, n, "fb_add_g");
  }
  std::vector<double> z(n, 0.0);
  return queue(br, b, FB_FIELD_GI, idx, z.data(), n, "fb_add_g");
}

extern "C" int fb_pulse(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n) {
  return queue(br, b, FB_FIELD_GE, idx, mv, n, "fb_pulse");
}

extern "C" int fb_reset(fb_brains *br, int32_t b) {
  if (!br) return fail(FB_EINVAL, "fb_reset: null handle");
  if (b != -1) {
    int rc = check_brain(br, b, "fb_reset");
    if (rc) return rc;
  }
  int rc = flush(br);
  if (rc) return rc;
  CU(launch_reset(br->trials, b < 0 ? 0 : b, b < 0 ? br->B : b + 1, br->stream));
  for (int32_t k = b < 0 ? 0 : b; k < (b < 0 ? br->B : b + 1); k++) {  // adapt 0 and res 1 again
    Trial &T = br->host[k];
    T.flags = (T.flags & ~(kAdaptZero | kResRest)) | rest_flags(T);
    CU(cudaMemcpyAsync(&br->trials[k].flags, &T.flags, 4, cudaMemcpyHostToDevice, br->stream));
  }
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

extern "C" int fb_set_background(fb_brains *br, int32_t b, double rate_hz, double amp_mv) {
  int rc = check_brain(br, b, "fb_set_background");
  if (rc) return rc;
  Trial &T = br->host[b];
  // src/lifwasm.js:69: header f32 at byte 172 <- N * rate * p.dt / 1000 (double dt), 176 <- amp
  T.bgEvents = (float)((double)T.N * rate_hz * br->dts[b] / 1000);
  T.bgAmp = (float)amp_mv;
  T.flags = (T.flags & ~kHasBg) | (T.bgEvents > 0 ? kHasBg : 0);
  CU(cudaMemcpyAsync(&br->trials[b].bgEvents, &T.bgEvents, 8, cudaMemcpyHostToDevice, br->stream));
  CU(cudaMemcpyAsync(&br->trials[b].flags, &T.flags, 4, cudaMemcpyHostToDevice, br->stream));
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

// LIFGpu.setParams (src/lifgpu.js:349): new parameters for brain b's header constants, taking
// effect at the next step. The ring depth round(delay/dt)+1 must not change (the ring and the
// delay-scheduled buffers are sized by it). Constant-state flags stay only while their condition
// holds (adapt 0 needs adaptInc 0, res 1 needs depU 0); presynaptic inhibition switches the
// delivery to the sequential mode and back.
extern "C" int fb_set_params(fb_brains *br, int32_t b, const fb_params *p) {
  int rc = check_brain(br, b, "fb_set_params");
  if (rc) return rc;
  if (!p) return fail(FB_EINVAL, "fb_set_params: params is null");
  if (!(p->dt > 0) || !(p->delay >= 0) || !(p->tauM > 0) || !(p->tauSyn > 0))
    return fail(FB_EINVAL, "fb_set_params: dt, tauM, tauSyn must be > 0");
  Trial &T = br->host[b];
  const int ns = (int)std::max(1.0, std::floor(p->delay / p->dt + 0.5)) + 1;
  if (ns != T.nslots)
    return fail(FB_EINVAL, "fb_set_params: delay/dt gives a ring of %d slots; the brain was created with %d", ns, T.nslots);
  if ((rc = flush(br))) return rc;
  Trial nt = T;
  fill_constants(nt, *p, T.N);
  int32_t f = nt.flags & (kHasBg | kHasDep | kHasPreInh);
  if ((T.flags & kAdaptZero) && nt.adaptInc == 0.f) f |= kAdaptZero;
  if ((T.flags & kResRest) && nt.depU == 0.f) f |= kResRest;
  f |= T.flags & (kBiasZero | kThrZero);
  int32_t mode = T.mode;
  if (f & kHasPreInh) mode = FB_DELIVER_SEQUENTIAL;
  else if ((T.flags & kHasPreInh) && mode == FB_DELIVER_SEQUENTIAL) mode = FB_DELIVER_EXACT;
  T.coba = nt.coba;
  T.mode = mode;
  T.flags = f;
  T.dt = nt.dt; T.vRest = nt.vRest; T.vThresh = nt.vThresh; T.vReset = nt.vReset; T.tRef = nt.tRef;
  T.adaptInc = nt.adaptInc; T.depU = nt.depU; T.dE = nt.dE; T.dTr = nt.dTr; T.dA = nt.dA; T.kRec = nt.kRec;
  T.kM = nt.kM; T.dtS = nt.dtS; T.eExc = nt.eExc; T.eInh = nt.eInh; T.cE = nt.cE; T.cI = nt.cI;
  T.bgEvents = nt.bgEvents; T.bgAmp = nt.bgAmp; T.preInh = nt.preInh;
  br->dts[b] = p->dt;
  // the constants, coba, mode and flags only: the device owns the header's dynamic scalars
  Trial *D = br->trials + b;
  const size_t c0 = offsetof(Trial, dt), c1 = offsetof(Trial, preInh) + sizeof(float);
  CU(cudaMemcpyAsync((char *)D + c0, (const char *)&T + c0, c1 - c0, cudaMemcpyHostToDevice, br->stream));
  CU(cudaMemcpyAsync(&D->coba, &T.coba, 8, cudaMemcpyHostToDevice, br->stream));  // coba, mode
  CU(cudaMemcpyAsync(&D->flags, &T.flags, 4, cudaMemcpyHostToDevice, br->stream));
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

// ---- the delay-scheduled kernel ----------------------------------------------------------------

// AUTO: shorter launches take the grid kernel. The delay-scheduled launch carries a fixed ~110 us
// (clearing its buffers, loading every block's state into shared memory and writing it back, the
// ring bookkeeping) against the grid kernel's ~15 us; at the full graph they break even near 6
// steps (grid 20-26 us per step, delay-scheduled 4-7).
constexpr int kLagMinSteps = 8;

// Whether the delay-scheduled kernel applies to this launch (why not, in *why).
static bool lag_applies(fb_brains *br, int32_t steps, const char **why) {
  const Trial &T = br->host[0];
  *why = nullptr;
  if (br->B != 1) *why = "a batch of more than one brain";
  else if (T.mode != FB_DELIVER_EXACT || (T.flags & kHasPreInh)) *why = "a delivery mode other than exact without presynaptic inhibition";
  else if (br->profiling && br->schedule != FB_SCHEDULE_LAGGED) *why = "phase profiling";
  else if (br->logging && steps > kLagRing) *why = "per-step logging of a launch longer than 64 steps";
  // a block's wait at step s (for step s - L, L = D - help) must not need its own completion of
  // that step, which it publishes at step s - L + 1: L >= 2
  else if (T.nslots - 1 < 4 || T.nslots - 1 > 32) *why = "a ring depth outside 5..33 slots";
  else if (T.bgEvents > (float)(1 << 20)) *why = "more than 2^20 background events per step";
  return *why == nullptr;
}

template <typename X>
static int lag_alloc(fb_brains *br, X **p, size_t n) {
  void *q = nullptr;
  if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(X)) != cudaSuccess) {
    cudaGetLastError();
    return fail(FB_ENOMEM, "fb_step: %zu bytes for the delay-scheduled kernel", n * sizeof(X));
  }
  br->lag.allocs.push_back(q);
  *p = (X *)q;
  return FB_OK;
}

// Allocates the kernel's resources and (when the driven set changed) the neuron ownership.
static int lag_setup(fb_brains *br) {
  LagRes &R = br->lag;
  Trial &T = br->host[0];
  const int N = T.N;
  const int64_t E = T.E;
  int rc;
  if (!R.ready) {
    int sms = 0, optin = 0;
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, br->dev));
    CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, br->dev));
    R.grid = sms;
    R.nTB = sms - 1;
    R.D = T.nslots - 1;
    R.S = 2 * R.D;
    // tile blocks hold at most ceil(N / (sms - kLagMaxDB)) neurons (the fewest tile blocks)
    R.capMax = std::max(1, (N + sms - kLagMaxDB - 1) / (sms - kLagMaxDB));
    int perDB = 0;  // driven entries one driven block holds at most
    for (int nd = 32; nd <= kLagPer * kLagThreads; nd += 32)
      if (lagged_smem_bytes(R.capMax, nd, kLagMaxDB * nd) <= (size_t)optin) perDB = nd;
    if (perDB == 0) return fail(FB_EINVAL, "fb_step: the delay-scheduled kernel does not fit in shared memory");
    R.nDmax = kLagMaxDB * perDB;
    // in-degree prefix: each target's bucket entries start at inOff[q]
    std::vector<uint32_t> ix(E), off(N + 1, 0);
    if (E) CU(cudaMemcpy(ix.data(), T.indices, E * 4, cudaMemcpyDeviceToHost));
    for (int64_t j = 0; j < E; j++) off[ix[j] + 1]++;
    for (int q = 0; q < N; q++) off[q + 1] += off[q];
    if ((rc = lag_alloc(br, &R.inOff, N + 1)) || (rc = lag_alloc(br, &R.cnt, (size_t)R.S * (N + R.nDmax))) ||
        (rc = lag_alloc(br, &R.buf, (size_t)R.S * std::max<int64_t>(E, 1))) || (rc = lag_alloc(br, &R.pend0, N)) ||
        (rc = lag_alloc(br, &R.sync, 256)) || (rc = lag_alloc(br, &R.bgCount, kLagRing)) ||
        (rc = lag_alloc(br, &R.dbList, (size_t)kLagRing * R.nDmax * 2)) ||
        (rc = lag_alloc(br, &R.dbCnt, (size_t)kLagRing * kLagMaxDB)) ||
        (rc = lag_alloc(br, &R.liveTag, (size_t)kLagRing * kLagMaxDB)) ||
        (rc = lag_alloc(br, &R.dbNF, kLagRing)) || (rc = lag_alloc(br, &R.tStage, (size_t)kLagRing * R.grid * R.capMax)) ||
        (rc = lag_alloc(br, &R.tCnt, (size_t)kLagRing * R.grid)) || (rc = lag_alloc(br, &R.ndIds, N)) ||
        (rc = lag_alloc(br, &R.ndLo, R.grid + 1)) || (rc = lag_alloc(br, &R.drvPosOf, N)) || (rc = lag_alloc(br, &R.edgeRec, std::max<int64_t>(E, 1))))
      return rc;
    CU(cudaMemcpy(R.inOff, off.data(), (N + 1) * 4, cudaMemcpyHostToDevice));
    std::vector<uint32_t> tab;
    lagged_jump_tables(tab);
    if ((rc = lag_alloc(br, &R.jumpHex, tab.size()))) return rc;
    CU(cudaMemcpyAsync(R.jumpHex, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, br->stream));
    CU(cudaStreamSynchronize(br->stream));
    R.ready = true;
  }
  const int bgNeed = T.bgEvents > 0 ? (int)std::ceil((double)T.bgEvents) + 1 : 1;
  if (bgNeed > R.bgCap) {
    if ((rc = lag_alloc(br, &R.bgList, (size_t)kLagRing * bgNeed))) return rc;
    R.bgCap = bgNeed;
  }
  const DrivenSet &ds = br->driven[0];
  if (ds.version != R.drivenVersion) {
    const int nD = (int)ds.order.size();
    if (nD > R.nDmax) return fail(FB_EINVAL, "fb_step: %d driven neurons exceed the delay-scheduled kernel's %d", nD, R.nDmax);
    if ((int64_t)nD + R.bgCap + 64 >= 65536)
      return fail(FB_EINVAL, "fb_step: %d draws per step exceed the delay-scheduled kernel's jump tables", nD + R.bgCap);
    std::vector<uint8_t> isD(N, 0);
    for (int32_t i : ds.order) isD[i] = 1;
    std::vector<int32_t> nd;
    nd.reserve(N - nD);
    for (int i = 0; i < N; i++)
      if (!isD[i]) nd.push_back(i);
    const int64_t Nnd = (int64_t)nd.size();
    // a long driven list is split over two driven blocks in list order (their draws stay in
    // lif.c's order: each offsets its own by the other's share); the other SMs are tile blocks
    R.nDB = br->lagDB ? br->lagDB : nD >= kLagSplit ? 2 : 1;
    if (R.nDB > 1 && nD < R.nDB) R.nDB = 1;  // every driven block owns at least one entry
    R.nTB = R.grid - R.nDB;
    for (int d = 0; d <= R.nDB; d++) R.dLo[d] = (int)((int64_t)nD * d / R.nDB);
    int part = 0;
    for (int d = 0; d < R.nDB; d++) part = std::max(part, R.dLo[d + 1] - R.dLo[d]);
    std::vector<int32_t> lo(R.nTB + 1);
    for (int t = 0; t <= R.nTB; t++) lo[t] = (int32_t)(Nnd * t / R.nTB);
    std::vector<int32_t> posOf(N, -1);
    for (int k = 0; k < nD; k++) posOf[ds.order[k]] = k;
    if (Nnd) CU(cudaMemcpyAsync(R.ndIds, nd.data(), Nnd * 4, cudaMemcpyHostToDevice, br->stream));
    CU(cudaMemcpyAsync(R.ndLo, lo.data(), (R.nTB + 1) * 4, cudaMemcpyHostToDevice, br->stream));
    CU(cudaMemcpyAsync(R.drvPosOf, posOf.data(), (size_t)N * 4, cudaMemcpyHostToDevice, br->stream));
    CU(launch_edge_records(T.indices, T.dup, R.inOff, R.drvPosOf, N, E, R.edgeRec, br->stream));
    CU(cudaStreamSynchronize(br->stream));
    R.nD = nD;
    R.cap = std::max<int>(1, (int)((Nnd + R.nTB - 1) / R.nTB));
    if (R.cap > std::min(R.capMax, kLagPer * kLagTileWorkers) || part > kLagPer * kLagThreads ||
        (nD + R.nTB - 1) / R.nTB > kLagHelpMax)
      return fail(FB_EINVAL, "fb_step: %d neurons per tile block (at most %d) or %d driven neurons per driven block "
                  "(at most %d) exceed the delay-scheduled kernel", R.cap, std::min(R.capMax, kLagPer * kLagTileWorkers),
                  part, kLagPer * kLagThreads);
    R.nDcap = std::max(32, (part + 31) / 32 * 32);
    R.nDall = std::max(32, (nD + 31) / 32 * 32);
    R.smem = lagged_smem_bytes(R.cap, R.nDcap, R.nDall);
    if (lagged_blocks_per_sm(R.smem) < 1)
      return fail(FB_EINVAL, "fb_step: the delay-scheduled kernel does not fit on an SM (%zu bytes)", R.smem);
    R.drivenVersion = ds.version;
  }
  return FB_OK;
}

static int run_lagged(fb_brains *br, int32_t steps) {
  LagRes &R = br->lag;
  Trial &T = br->host[0];
  const int N = T.N;
  CU(cudaEventRecord(br->ev0, br->stream));  // the launch's clearing is part of its time
  CU(cudaMemsetAsync(R.sync, 0, 256 * 4, br->stream));
  CU(cudaMemsetAsync(R.cnt, 0, (size_t)R.S * (N + R.nDmax) * 4, br->stream));
  CU(cudaMemsetAsync(R.pend0, 0, (size_t)N * 4, br->stream));
  CU(cudaMemsetAsync(R.liveTag, 0, sizeof(unsigned long long) * kLagRing * kLagMaxDB, br->stream));
  LagArgs a;
  memset(&a, 0, sizeof a);
  a.G = br->trials;
  a.N = N;
  a.E = T.E;
  a.T = steps;
  a.D = R.D;
  a.S = R.S;
  a.help = lag_help(R.D);
  a.dbPub = a.help - 1;
  a.L = R.D - a.help;
  a.nTB = R.nTB;
  a.cap = R.cap;
  a.nD = R.nD;
  a.nDcap = R.nDcap;
  a.nDall = R.nDall;
  a.nDB = R.nDB;
  for (int d = 0; d <= kLagMaxDB; d++) a.dLo[d] = R.dLo[std::min(d, R.nDB)];
  a.hasBg = T.bgEvents > 0 ? 1 : 0;
  a.bgCap = R.bgCap;
  a.dt = T.dt; a.vRest = T.vRest; a.vThresh = T.vThresh; a.vReset = T.vReset; a.tRef = T.tRef;
  a.adaptInc = T.adaptInc; a.depU = T.depU; a.dE = T.dE; a.dTr = T.dTr; a.dA = T.dA; a.kRec = T.kRec;
  a.kM = T.kM; a.dtS = T.dtS; a.eExc = T.eExc; a.eInh = T.eInh; a.cE = T.cE; a.cI = T.cI;
  a.bgEvents = T.bgEvents; a.bgAmp = T.bgAmp; a.coba = T.coba;
  a.indptr = T.indptr; a.indices = T.indices; a.W = T.W; a.sign = T.sign; a.inOff = R.inOff;
  a.v = T.v; a.gE = T.gE; a.gI = T.gI; a.refr = T.refr; a.trace = T.trace; a.adapt = T.adapt; a.res = T.res;
  a.bias = T.bias; a.thr = T.thr; a.drive = T.drive; a.spikeCount = T.spikeCount;
  a.ring = T.ring; a.ringCount = T.ringCount; a.driven = T.driven;
  a.ndIds = R.ndIds; a.ndLo = R.ndLo; a.drvPosOf = R.drvPosOf;
  a.cnt = R.cnt; a.cntStride = N + R.nDmax; a.buf = R.buf; a.pend0 = R.pend0;
  a.done = R.sync; a.dbDone = R.sync + 64; a.bgReady = R.sync + 72; a.barCount = R.sync + 128;
  a.liveTag = R.liveTag;
  a.stepTot = (int32_t *)(R.sync + 192);
  a.bgList = R.bgList; a.bgCount = R.bgCount; a.dbList = R.dbList; a.dbCnt = R.dbCnt;
  a.tStage = R.tStage; a.tCnt = R.tCnt;
  a.log = br->logging;
  a.logCount = T.logCount; a.logRaster = T.logRaster; a.logCap = T.logCap; a.logRasterCap = T.logRasterCap;
  a.prof = br->profiling ? br->d_phase : nullptr;
  a.jumpHex = R.jumpHex;
  a.edgeRec = R.edgeRec;
  a.err = br->d_err;
  a.timeoutNs = br->timeoutNs;
  a.tripStep = br->tripStep;
  br->tripStep = -1;  // one launch only
  CU(launch_lagged(a, R.grid, R.smem, br->stream));
  CU(launch_rebuild_slots(br->trials, T.nslots, br->d_err, br->stream));
  CU(cudaEventRecord(br->ev1, br->stream));
  br->lastSchedule = FB_SCHEDULE_LAGGED;
  return FB_OK;
}

static int run_steps(fb_brains *br, int32_t maxSteps, int32_t *out_nfired) {
  int rc = flush(br, false);
  if (rc) return rc;
  bool lagged = false;
  if (maxSteps > 0 && br->schedule != FB_SCHEDULE_GRID) {
    const char *why = nullptr;
    const bool applies = lag_applies(br, maxSteps, &why);
    if (br->schedule == FB_SCHEDULE_LAGGED) {
      if (!applies) return fail(FB_EINVAL, "fb_step: the delay-scheduled kernel does not apply to %s", why);
      if ((rc = lag_setup(br))) return rc;
      lagged = true;
    } else if (applies && maxSteps >= kLagMinSteps) {
      lagged = lag_setup(br) == FB_OK;
      if (!lagged) g_err.clear();
    }
  }
  // the error flag and the fired counts come back in one synchronisation
  auto read_back = [&]() -> int {
    CU(cudaMemcpyAsync(br->h_small, br->d_err, 4, cudaMemcpyDeviceToHost, br->stream));
    if (out_nfired)
      for (int b = 0; b < br->B; b++)
        CU(cudaMemcpyAsync(br->h_small + 2 + b, &br->trials[b].nFired, 4, cudaMemcpyDeviceToHost, br->stream));
    CU(cudaStreamSynchronize(br->stream));
    br->flushPending = false;
    return FB_OK;
  };
  if (lagged) {
    if ((rc = run_lagged(br, maxSteps))) return rc;
    if ((rc = read_back())) return rc;
    const int32_t err = br->h_small[0];
    cudaEventElapsedTime(&br->lastMs, br->ev0, br->ev1);
    if (err) {
      cudaMemsetAsync(br->d_err, 0, 4, br->stream);
      cudaStreamSynchronize(br->stream);
      return fail(err, err == FB_ETIMEOUT ? "fb_step: a device-side wait timed out; the step was abandoned"
                                          : "fb_step: delay-scheduled kernel error %d", err);
    }
  } else if (maxSteps > 0) {
    br->lastSchedule = FB_SCHEDULE_GRID;
    if (br->stepsUploaded != br->stepsHost) {  // the last launch's counts stay on the device otherwise
      std::memcpy(br->h_steps, br->stepsHost.data(), sizeof(int32_t) * br->B);
      CU(cudaMemcpyAsync(br->d_steps, br->h_steps, sizeof(int32_t) * br->B, cudaMemcpyHostToDevice, br->stream));
      br->stepsUploaded = br->stepsHost;
    }
    StepArgs a;
    memset(&a, 0, sizeof a);
    a.trials = br->trials;
    a.B = br->B;
    a.maxSteps = maxSteps;
    a.steps = br->d_steps;
    a.tileTrial = br->d_tileTrial;
    a.nTilesTotal = (int32_t)br->tileTrial.size();
    a.jump = br->jump;
    a.barCount = br->d_bar;
    a.phaseNs = br->profiling ? br->d_phase : nullptr;
    a.err = br->d_err;
    a.ovf[0] = br->d_ovf[0];
    a.ovf[1] = br->d_ovf[1];
    a.ovfTop = br->d_ovfTop;
    a.ovfCap = br->ovfCap;
    a.log = br->logging;
    a.itemChunks = br->itemChunks;
    a.subGrab = br->subGrab;
    a.subNext = br->d_ovfTop + 2;
    a.timeoutNs = br->timeoutNs;
    a.dbg = br->d_dbg;
    CU(cudaEventRecord(br->ev0, br->stream));
    CU(launch_step(a, br->grid, br->smem, br->stream));
    CU(cudaEventRecord(br->ev1, br->stream));
    if ((rc = read_back())) return rc;
    const int32_t err = br->h_small[0];
    cudaEventElapsedTime(&br->lastMs, br->ev0, br->ev1);
    if (err) {
      // leave the handle launchable: clear the flag, the barrier and the overflow pool
      cudaMemsetAsync(br->d_err, 0, 4, br->stream);
      cudaMemsetAsync(br->d_bar, 0, sizeof(uint32_t) * fb_brains::kBarWords, br->stream);
      cudaMemsetAsync(br->d_ovfTop, 0, 16, br->stream);
      cudaStreamSynchronize(br->stream);
      uint32_t dbg[4] = {0, 0, 0, 0};
      cudaMemcpy(dbg, br->d_dbg, 16, cudaMemcpyDeviceToHost);
      cudaMemset(br->d_dbg, 0, 16);
      if (err == FB_EINVAL)
        return fail(err, "fb_step: index check failed at site %u (values %u, %u; %u failures)", dbg[0], dbg[1], dbg[2], dbg[3]);
      return fail(err, err == FB_ETIMEOUT ? "fb_step: a device-side wait timed out; the step was abandoned"
                                          : "fb_step: delivery overflow (the pool of %u overflow records for one step is full)",
                  br->ovfCap);
    }
  }
  if (out_nfired) {
    if (maxSteps > 0) {
      std::memcpy(out_nfired, br->h_small + 2, sizeof(int32_t) * br->B);
    } else {  // nothing ran: the counts of the last step before
      if ((rc = read_back())) return rc;
      std::memcpy(out_nfired, br->h_small + 2, sizeof(int32_t) * br->B);
    }
  }
  return FB_OK;
}

extern "C" int fb_step(fb_brains *br, int32_t nsteps, int32_t *out_nfired) {
  if (!br) return fail(FB_EINVAL, "fb_step: null handle");
  if (nsteps < 0) return fail(FB_EINVAL, "fb_step: nsteps=%d", nsteps);
  br->stepsHost.assign(br->B, nsteps);
  return run_steps(br, nsteps, out_nfired);
}

extern "C" int fb_step_uneven(fb_brains *br, const int32_t *steps, int32_t *out_nfired) {
  if (!br || !steps) return fail(FB_EINVAL, "fb_step_uneven: null argument");
  br->stepsHost.assign(steps, steps + br->B);
  int32_t mx = 0;
  for (int b = 0; b < br->B; b++) {
    if (steps[b] < 0) return fail(FB_EINVAL, "fb_step_uneven: steps[%d]=%d", b, steps[b]);
    mx = std::max(mx, steps[b]);
  }
  return run_steps(br, mx, out_nfired);
}

extern "C" int fb_last_step_ms(fb_brains *br, float *ms) {
  if (!br || !ms) return fail(FB_EINVAL, "fb_last_step_ms: null argument");
  *ms = br->lastMs;
  return FB_OK;
}

extern "C" int fb_record(fb_brains *br, int32_t cap_steps, int64_t cap_spikes) {
  if (!br || cap_steps < 0 || cap_spikes < 0) return fail(FB_EINVAL, "fb_record: bad arguments");
  CU(cudaStreamSynchronize(br->stream));
  for (int b = 0; b < br->B; b++) {
    Trial &T = br->host[b];
    cudaFree(T.logCount);
    cudaFree(T.logRaster);
    T.logCount = nullptr;
    T.logRaster = nullptr;
    T.logCap = T.logRasterCap = 0;
    if (cap_steps > 0) {
      CU(cudaMalloc(&T.logCount, sizeof(int32_t) * (size_t)cap_steps));
      CU(cudaMemsetAsync(T.logCount, 0, sizeof(int32_t) * (size_t)cap_steps, br->stream));
      T.logCap = cap_steps;
      if (cap_spikes > 0) {
        CU(cudaMalloc(&T.logRaster, sizeof(int32_t) * (size_t)cap_spikes));
        T.logRasterCap = cap_spikes;
      }
    }
    // the device owns stepsDone: read it, start the log at the next step
    int64_t done = 0;
    CU(cudaMemcpy(&done, &br->trials[b].stepsDone, 8, cudaMemcpyDeviceToHost));
    T.stepsDone = done;
    T.logStart = done;
    T.logRasterLen[0] = T.logRasterLen[1] = 0;
    CU(cudaMemcpyAsync(&br->trials[b].logCount, &T.logCount, sizeof(void *) * 2 + sizeof(int64_t) * 2, cudaMemcpyHostToDevice, br->stream));
    CU(cudaMemcpyAsync(&br->trials[b].logStart, &T.logStart, sizeof(int64_t) * 3, cudaMemcpyHostToDevice, br->stream));
  }
  br->logging = cap_steps > 0 ? 1 : 0;
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

extern "C" int fb_spike_log(fb_brains *br, int32_t b, int32_t *counts, int32_t cap_steps, int32_t *raster,
                            int64_t cap_spikes, int64_t *n_steps, int64_t *n_spikes) {
  int rc = check_brain(br, b, "fb_spike_log");
  if (rc) return rc;
  CU(cudaStreamSynchronize(br->stream));
  Trial dev;
  CU(cudaMemcpy(&dev, &br->trials[b], sizeof(Trial), cudaMemcpyDeviceToHost));
  const int64_t steps = dev.stepsDone - dev.logStart;
  const int64_t spikes = dev.logRasterLen[dev.stepsDone & 1];
  if (n_steps) *n_steps = steps;
  if (n_spikes) *n_spikes = dev.logRaster ? spikes : 0;
  if (counts && dev.logCount) {
    const int64_t n = std::min<int64_t>({(int64_t)cap_steps, steps, dev.logCap});
    if (n > 0) CU(cudaMemcpy(counts, dev.logCount, sizeof(int32_t) * n, cudaMemcpyDefault));
  }
  if (raster && dev.logRaster) {
    const int64_t n = std::min<int64_t>({cap_spikes, spikes, dev.logRasterCap});
    if (n > 0) CU(cudaMemcpy(raster, dev.logRaster, sizeof(int32_t) * n, cudaMemcpyDefault));
  }
  return FB_OK;
}

extern "C" int fb_fired(fb_brains *br, int32_t b, int32_t *dst, int32_t cap, int32_t *n) {
  int rc = check_brain(br, b, "fb_fired");
  if (rc) return rc;
  CU(cudaStreamSynchronize(br->stream));
  int32_t nf_slot[2];
  CU(cudaMemcpy(nf_slot, &br->trials[b].nFired, 8, cudaMemcpyDeviceToHost));
  if (n) *n = nf_slot[0];
  const int32_t m = std::min(nf_slot[0], cap);
  if (dst && m > 0) {
    const Trial &T = br->host[b];
    CU(cudaMemcpy(dst, T.ring + (int64_t)nf_slot[1] * T.N, sizeof(int32_t) * m, cudaMemcpyDefault));
  }
  return FB_OK;
}

extern "C" int fb_ring_read(fb_brains *br, int32_t b, int32_t *ring, int32_t *counts, int32_t *head) {
  int rc = check_brain(br, b, "fb_ring_read");
  if (rc) return rc;
  rc = flush(br);
  if (rc) return rc;
  CU(cudaStreamSynchronize(br->stream));
  const Trial &T = br->host[b];
  if (ring) CU(cudaMemcpy(ring, T.ring, sizeof(int32_t) * (size_t)T.nslots * T.N, cudaMemcpyDefault));
  if (counts) CU(cudaMemcpy(counts, T.ringCount, sizeof(int32_t) * T.nslots, cudaMemcpyDefault));
  if (head) CU(cudaMemcpy(head, &br->trials[b].head, sizeof(int32_t), cudaMemcpyDeviceToHost));
  return FB_OK;
}

static void *field_ptr(Trial &T, int32_t field) {
  switch (field) {
    case FB_FIELD_V: return T.v;
    case FB_FIELD_GE: return T.gE;
    case FB_FIELD_GI: return T.gI;
    case FB_FIELD_REFR: return T.refr;
    case FB_FIELD_TRACE: return T.trace;
    case FB_FIELD_ADAPT: return T.adapt;
    case FB_FIELD_RES: return T.res;
    case FB_FIELD_BIAS: return T.bias;
    case FB_FIELD_THR: return T.thr;
    case FB_FIELD_DRIVE: return T.drive;
    case FB_FIELD_SPIKECOUNT: return T.spikeCount;
    default: return nullptr;
  }
}

extern "C" int fb_read(fb_brains *br, int32_t field, int32_t b, void *dst) {
  int rc = check_brain(br, b, "fb_read");
  if (rc) return rc;
  void *src = field_ptr(br->host[b], field);
  if (!src || !dst) return fail(FB_EINVAL, "fb_read: bad field %d or null dst", field);
  rc = flush(br);
  if (rc) return rc;
  CU(cudaMemcpyAsync(dst, src, (size_t)br->host[b].N * 4, cudaMemcpyDefault, br->stream));
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

extern "C" int fb_write(fb_brains *br, int32_t field, int32_t b, const void *src) {
  int rc = check_brain(br, b, "fb_write");
  if (rc) return rc;
  void *dst = field_ptr(br->host[b], field);
  if (!dst || !src) return fail(FB_EINVAL, "fb_write: bad field %d or null src", field);
  if (field == FB_FIELD_DRIVE) return fail(FB_EINVAL, "fb_write: the drive field is written through fb_set_drive, which keeps the driven set");
  rc = flush(br);
  if (rc) return rc;
  const int32_t clear = field == FB_FIELD_ADAPT ? kAdaptZero : field == FB_FIELD_RES ? kResRest
                        : field == FB_FIELD_BIAS ? kBiasZero : field == FB_FIELD_THR ? kThrZero : 0;
  if (br->host[b].flags & clear) {  // the field may no longer be at rest: the update reads it again
    br->host[b].flags &= ~clear;
    CU(cudaMemcpyAsync(&br->trials[b].flags, &br->host[b].flags, 4, cudaMemcpyHostToDevice, br->stream));
  }
  CU(cudaMemcpyAsync(dst, src, (size_t)br->host[b].N * 4, cudaMemcpyDefault, br->stream));
  CU(cudaStreamSynchronize(br->stream));
  return FB_OK;
}

extern "C" int fb_scalars(fb_brains *br, int32_t b, int32_t *head, uint32_t *rng, int32_t *nfired,
                          int32_t *last_slot, int32_t *n_driven, int64_t *steps_done) {
  int rc = check_brain(br, b, "fb_scalars");
  if (rc) return rc;
  rc = flush(br);
  if (rc) return rc;
  Trial dev;
  CU(cudaMemcpy(&dev, &br->trials[b], sizeof(Trial), cudaMemcpyDeviceToHost));
  if (head) *head = dev.head;
  if (rng) *rng = dev.rngP[dev.stepsDone & 1];
  if (nfired) *nfired = dev.nFired;
  if (last_slot) *last_slot = dev.lastSlot;
  if (n_driven) *n_driven = dev.nDriven;
  if (steps_done) *steps_done = dev.stepsDone;
  return FB_OK;
}

extern "C" int fb_profile(fb_brains *br, int32_t on) {
  if (!br) return fail(FB_EINVAL, "fb_profile: null handle");
  if (!br->d_phase) CU(cudaMalloc(&br->d_phase, sizeof(unsigned long long) * FB_NPHASES));
  CU(cudaMemsetAsync(br->d_phase, 0, sizeof(unsigned long long) * FB_NPHASES, br->stream));
  CU(cudaStreamSynchronize(br->stream));
  br->profiling = on ? 1 : 0;
  return FB_OK;
}

extern "C" int fb_phase_times(fb_brains *br, double *ms, int32_t n) {
  if (!br || !ms) return fail(FB_EINVAL, "fb_phase_times: null argument");
  unsigned long long ns[FB_NPHASES] = {0};
  if (br->d_phase) {
    CU(cudaStreamSynchronize(br->stream));
    CU(cudaMemcpy(ns, br->d_phase, sizeof ns, cudaMemcpyDeviceToHost));
  }
  for (int k = 0; k < n && k < FB_NPHASES; k++) ms[k] = ns[k] * 1e-6;
  return FB_OK;
}
