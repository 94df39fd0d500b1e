// fb_lif_step_noalloc: the brain step for callers that cannot allocate device memory.
//
// Some callers of the brain step may not call cudaMalloc or cudaFree: a host application that
// hands every byte of device memory out of its own pool (a physics or rendering engine with a
// fixed device budget, where an allocation behind its back breaks the budget), or a real-time
// control loop such as the embodied fly, which steps the brain twice per simulated millisecond
// and cannot take the implicit device-wide synchronisation that cudaMalloc/cudaFree may perform.
// This entry point takes a view shaped like the reference's Brain header (every array a
// caller-owned device pointer) and allocates nothing: the step's scratch (delivery buckets, ring
// bookkeeping, spike staging, overflow records, barrier words, xorshift jump tables) lives in one
// file-scope __device__ array of a fixed 64 MiB, which every GPU that loads this library holds
// until the process exits.
//
// The array is shared by every call on a device and keeps the last call's contents, so each call
// first clears what must start at zero and rebuilds the ring's delivery bookkeeping from the
// caller's own ring lists. Calls whose work overlaps on the GPU (two streams, two threads) race on
// the array and corrupt each other: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fb_internal.cuh"

namespace fb {
int step_kernel_blocks_per_sm(size_t smem);
size_t step_smem_bytes(int B);
cudaError_t launch_step(const StepArgs &a, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_rebuild_slots(Trial *Td, int nslots, int32_t *err, cudaStream_t st);
void host_jump_tables(std::vector<uint32_t> &tab);
int set_error(int code, const char *msg);
}  // namespace fb

using namespace fb;

// The static scratch: 64 MiB, enough for a brain of N = 20,000 neurons and 1.2M edges with a
// 19-slot ring (the dt = 0.1 ms, 1.8 ms delay model); the bound a call must fit is computed by
// noalloc_layout below. Its overflow records (contributions beyond a target's in-place bucket)
// are sized by E per step parity: a presynaptic neuron arrives at most once per step, so one step
// never delivers more than E contributions, and no burst can overflow them.
static constexpr size_t kNoAllocBytes = 64u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

struct Layout {
  size_t jump, trial, bar, err, dbg, ovfTop, steps, ovf0, ovf1, ringOff, ringRow, chunkK, slotEdges,
      cnt, bucket, ovfHead, bgHits, arrived, stage, stageDeg, tileCnt, tileDeg, dStage, dStageDeg,
      dCnt, dDeg, liveTag, total;
};

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout noalloc_layout(int64_t N, int64_t E, int64_t ns) {
  Layout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += up256(bytes); return r; };
  const int64_t nTiles = (N + kTile - 1) / kTile;
  const int64_t maxDch = std::max<int64_t>(1, (N + kBlock - 1) / kBlock);
  const int64_t chunkCap = (E + kChunk - 1) / kChunk + 1;
  L.jump = take(32 * 128 * 4);  // persistent: written once per device at set-up
  L.trial = take(sizeof(Trial));
  L.bar = take(128);
  L.err = take(4);
  L.dbg = take(16);
  L.ovfTop = take(8);
  L.steps = take(4);
  L.ovf0 = take(sizeof(OvfRec) * (size_t)(E + 1));
  L.ovf1 = take(sizeof(OvfRec) * (size_t)(E + 1));
  L.ringOff = take((size_t)ns * (N + 1) * 4);
  L.ringRow = take((size_t)ns * N * 4);
  L.chunkK = take((size_t)ns * chunkCap * 16);
  L.slotEdges = take((size_t)ns * 4);
  L.cnt = take((size_t)N * 4);
  L.bucket = take((size_t)N * kBucket * 8);
  L.ovfHead = take((size_t)N * 4);
  L.bgHits = take((size_t)N * 4);
  L.arrived = take((size_t)N);
  L.stage = take((size_t)nTiles * kTile * 4);
  L.stageDeg = take((size_t)nTiles * kTile * 4);
  L.tileCnt = take((size_t)nTiles * kSubPerTile * 4);
  L.tileDeg = take((size_t)nTiles * kSubPerTile * 4);
  L.dStage = take((size_t)2 * maxDch * kBlock * 4);
  L.dStageDeg = take((size_t)2 * maxDch * kBlock * 4);
  L.dCnt = take((size_t)2 * maxDch * 4);
  L.dDeg = take((size_t)2 * maxDch * 4);
  L.liveTag = take((size_t)maxDch * 8);
  L.total = o;
  return L;
}

// The caller's arrays are not checked by anyone else (fb_graph_create checks its CSR on the host;
// here the CSR, the driven list and the ring lists are device memory the caller filled). Every
// index the step dereferences is checked once per call before anything is written: indptr
// starts at 0, never decreases and ends at E; every target is in [0, N); every driven entry and
// every ring entry (of its slot's count, itself in [0, N]) is in [0, N). A violation records
// FB_EINVAL; nothing else is written.
__global__ void validate_view_kernel(const uint32_t *indptr, const uint32_t *indices, const int32_t *driven,
                                     const int32_t *ring, const int32_t *ringCount, int32_t N, int64_t E,
                                     int32_t nDriven, int32_t nslots, int32_t *err) {
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  bool bad = false;
  if (t0 == 0) bad = indptr[0] != 0u || (int64_t)indptr[N] != E;
  for (int64_t i = t0; i < N; i += nt) bad |= indptr[i + 1] < indptr[i];
  for (int64_t j = t0; j < E; j += nt) bad |= indices[j] >= (uint32_t)N;
  for (int64_t k = t0; k < nDriven; k += nt) bad |= driven[k] < 0 || driven[k] >= N;
  for (int32_t sl = 0; sl < nslots; sl++) {
    const int32_t na = ringCount[sl];
    if (na < 0 || na > N) {
      bad = true;
      continue;
    }
    for (int64_t k = t0; k < na; k += nt) {
      const int32_t x = ring[(int64_t)sl * N + k];
      bad |= x < 0 || x >= N;
    }
  }
  if (bad) atomicCAS(err, 0, FB_EINVAL);
}

struct DeviceSetup {
  bool ready = false;
  unsigned char *base = nullptr;
  int grid = 0;
};
std::mutex g_mu;
DeviceSetup g_dev[64];

int fail_na(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return set_error(code, buf);
}

#define NA_CU(call)                                                                   \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail_na(FB_ECUDA, "fb_lif_step_noalloc: %s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Once per device, with that device current: the scratch array's device address (a host-side
// reference to the array is only a stand-in), the persistent grid size, and the jump tables.
int setup_device(int dev, DeviceSetup **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceSetup &d = g_dev[dev];
  if (!d.ready) {
    cudaDeviceProp p;
    NA_CU(cudaGetDeviceProperties(&p, dev));
    if (p.major != 10 || p.minor != 3)
      return fail_na(FB_ENODEV, "fb_lif_step_noalloc: device %d is sm_%d%d; built for sm_103a", dev, p.major, p.minor);
    void *ptr = nullptr;
    NA_CU(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    const int per = step_kernel_blocks_per_sm(step_smem_bytes(1));
    if (per <= 0) return fail_na(FB_ECUDA, "fb_lif_step_noalloc: step kernel does not fit on an SM");
    std::vector<uint32_t> tab;
    host_jump_tables(tab);
    NA_CU(cudaMemcpy(ptr, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
    // a copy from pageable memory may return before the data has reached the device; a step on a
    // non-blocking stream would not be ordered after it
    NA_CU(cudaDeviceSynchronize());
    d.base = (unsigned char *)ptr;
    d.grid = p.multiProcessorCount * per;
    d.ready = true;
  }
  *out = &d;
  return FB_OK;
}

}  // namespace

extern "C" int fb_lif_step_noalloc(fb_brain_view *v, int32_t nsteps, void *stream) {
  if (!v) return fail_na(FB_EINVAL, "fb_lif_step_noalloc: null view");
  if (nsteps < 0) return fail_na(FB_EINVAL, "fb_lif_step_noalloc: nsteps=%d", nsteps);
  if (v->N <= 0 || v->E < 0 || v->nslots < 3 || v->head < 0 || v->head >= v->nslots ||
      v->nDriven < 0 || v->nDriven > v->N)
    return fail_na(FB_EINVAL, "fb_lif_step_noalloc: bad header (N=%d E=%lld nslots=%d head=%d nDriven=%d); "
                   "the ring needs at least 3 slots", v->N, (long long)v->E, v->nslots, v->head, v->nDriven);
  const void *arrays[] = {v->v, v->gE, v->gI, v->refr, v->trace, v->adapt, v->res, v->bias, v->thr,
                          v->drive, v->sign, v->spikeCount, v->indptr, v->indices, v->weights,
                          v->ring, v->ringCount, v->driven};
  for (const void *p : arrays)
    if (!p) return fail_na(FB_EINVAL, "fb_lif_step_noalloc: a state, graph or ring array is null");
  if (v->E > 0xfffffff0LL) return fail_na(FB_EINVAL, "fb_lif_step_noalloc: E=%lld exceeds 32-bit edge offsets", (long long)v->E);
  const Layout L = noalloc_layout(v->N, v->E, v->nslots);
  if (L.total > kNoAllocBytes)
    return fail_na(FB_EINVAL, "fb_lif_step_noalloc: a brain of N=%d, E=%lld and %d ring slots needs %zu bytes of "
                   "scratch; the static scratch holds %zu bytes (use fb_brains_create for larger brains)",
                   v->N, (long long)v->E, v->nslots, L.total, kNoAllocBytes);
  if (nsteps == 0) return FB_OK;
  int dev = 0;
  NA_CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail_na(FB_ENODEV, "fb_lif_step_noalloc: device ordinal %d unsupported", dev);
  DeviceSetup *d = nullptr;
  int rc = setup_device(dev, &d);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char *B = d->base;

  // the brain's header: the view's f32 constants and pointers, plus scratch pointers
  Trial T;
  memset(&T, 0, sizeof T);
  T.N = v->N;
  T.E = v->E;
  T.nslots = v->nslots;
  T.coba = v->coba ? 1 : 0;
  T.dt = v->dt; T.vRest = v->vRest; T.vThresh = v->vThresh; T.vReset = v->vReset; T.tRef = v->tRef;
  T.adaptInc = v->adaptInc; T.depU = v->depU; T.dE = v->dE; T.dTr = v->dTr; T.dA = v->dA;
  T.kRec = v->kRec; T.kM = v->kM; T.dtS = v->dtS; T.eExc = v->eExc; T.eInh = v->eInh;
  T.cE = v->cE; T.cI = v->cI; T.bgEvents = v->bgEvents; T.bgAmp = v->bgAmp; T.preInh = v->preInh;
  T.flags = (T.bgEvents > 0 ? kHasBg : 0) | (T.depU != 0.f ? kHasDep : 0) | (T.preInh > 0.f ? kHasPreInh : 0);
  T.mode = (T.flags & kHasPreInh) ? FB_DELIVER_SEQUENTIAL : FB_DELIVER_EXACT;
  T.nTiles = (v->N + kTile - 1) / kTile;
  T.tileBase = 0;
  T.chunkCap = (v->E + kChunk - 1) / kChunk + 1;
  T.maxDch = std::max(1, (v->N + kBlock - 1) / kBlock);
  T.indptr = v->indptr; T.indices = v->indices; T.W = v->weights; T.sign = v->sign;
  T.v = v->v; T.gE = v->gE; T.gI = v->gI; T.refr = v->refr; T.trace = v->trace; T.adapt = v->adapt;
  T.res = v->res; T.bias = v->bias; T.thr = v->thr; T.drive = v->drive; T.spikeCount = v->spikeCount;
  T.ring = v->ring; T.ringCount = v->ringCount; T.driven = v->driven;
  T.ringOff = (uint32_t *)(B + L.ringOff); T.ringRow = (uint32_t *)(B + L.ringRow);
  T.chunkK = (uint4 *)(B + L.chunkK); T.slotEdges = (uint32_t *)(B + L.slotEdges);
  T.cnt = (uint32_t *)(B + L.cnt); T.bucket = (uint2 *)(B + L.bucket);
  T.ovfHead = (uint32_t *)(B + L.ovfHead); T.bgHits = (uint32_t *)(B + L.bgHits);
  T.arrived = (uint8_t *)(B + L.arrived);
  T.stage = (int32_t *)(B + L.stage); T.stageDeg = (uint32_t *)(B + L.stageDeg);
  T.tileCnt = (int32_t *)(B + L.tileCnt); T.tileDeg = (uint32_t *)(B + L.tileDeg);
  T.dStage = (int32_t *)(B + L.dStage); T.dStageDeg = (uint32_t *)(B + L.dStageDeg);
  T.dCnt = (int32_t *)(B + L.dCnt); T.dDeg = (uint32_t *)(B + L.dDeg);
  T.liveTag = (unsigned long long *)(B + L.liveTag);
  T.rngP[0] = v->rng;
  T.bgAccP[0] = v->bgAcc;
  T.head = v->head;
  T.nDriven = v->nDriven;
  T.nFired = v->nFired;
  T.lastSlot = v->lastSlot;
  Trial *Td = (Trial *)(B + L.trial);
  int32_t *errd = (int32_t *)(B + L.err);

  // what must start at zero (the array keeps the previous call's contents), then the header
  NA_CU(cudaMemsetAsync(B + L.cnt, 0, (size_t)v->N * 4, st));
  NA_CU(cudaMemsetAsync(B + L.bgHits, 0, (size_t)v->N * 4, st));
  NA_CU(cudaMemsetAsync(B + L.arrived, 0, (size_t)v->N, st));
  NA_CU(cudaMemsetAsync(B + L.ovfHead, 0xff, (size_t)v->N * 4, st));
  NA_CU(cudaMemsetAsync(B + L.bar, 0, 128, st));
  NA_CU(cudaMemsetAsync(B + L.err, 0, 4, st));
  NA_CU(cudaMemsetAsync(B + L.dbg, 0, 16, st));
  NA_CU(cudaMemsetAsync(B + L.ovfTop, 0, 8, st));
  NA_CU(cudaMemsetAsync(B + L.liveTag, 0, (size_t)T.maxDch * 8, st));
  NA_CU(cudaMemcpyAsync(Td, &T, sizeof T, cudaMemcpyHostToDevice, st));
  NA_CU(cudaMemcpyAsync(B + L.steps, &nsteps, 4, cudaMemcpyHostToDevice, st));
  // the caller's indices, checked before anything of the brain is written
  validate_view_kernel<<<d->grid, 256, 0, st>>>(v->indptr, v->indices, v->driven, v->ring, v->ringCount, v->N,
                                               v->E, v->nDriven, v->nslots, errd);
  NA_CU(cudaGetLastError());
  int32_t verr = 0;
  NA_CU(cudaMemcpyAsync(&verr, errd, 4, cudaMemcpyDeviceToHost, st));
  NA_CU(cudaStreamSynchronize(st));
  if (verr)
    return fail_na(FB_EINVAL, "fb_lif_step_noalloc: the view's indptr, indices, driven list or ring lists hold an "
                   "index outside [0, N) (or indptr does not run from 0 to E); nothing was changed");
  NA_CU(launch_rebuild_slots(Td, v->nslots, errd, st));

  StepArgs a;
  memset(&a, 0, sizeof a);
  a.itemChunks = 1;
  a.trials = Td;
  a.B = 1;
  a.maxSteps = nsteps;
  a.steps = (const int32_t *)(B + L.steps);
  a.tileTrial = nullptr;
  a.nTilesTotal = T.nTiles;
  a.jump = (const uint32_t *)(B + L.jump);
  a.barCount = (uint32_t *)(B + L.bar);
  a.phaseNs = nullptr;
  a.err = errd;
  a.ovf[0] = (OvfRec *)(B + L.ovf0);
  a.ovf[1] = (OvfRec *)(B + L.ovf1);
  a.ovfTop = (uint32_t *)(B + L.ovfTop);
  a.ovfCap = (uint32_t)(v->E + 1);
  a.log = 0;
  a.timeoutNs = 5000000000LL;
  a.dbg = (uint32_t *)(B + L.dbg);
  NA_CU(launch_step(a, d->grid, step_smem_bytes(1), st));

  // the view's scalars after the call
  Trial out;
  int32_t err = 0;
  NA_CU(cudaMemcpyAsync(&out, Td, sizeof out, cudaMemcpyDeviceToHost, st));
  NA_CU(cudaMemcpyAsync(&err, errd, 4, cudaMemcpyDeviceToHost, st));
  NA_CU(cudaStreamSynchronize(st));
  if (err)
    return fail_na(err, err == FB_ETIMEOUT ? "fb_lif_step_noalloc: a device-side wait timed out; the brain's arrays "
                                             "may be partly advanced and the view was not updated: rebuild the brain"
                   : err == FB_EOVERFLOW ? "fb_lif_step_noalloc: delivery overflow; the brain's arrays may be partly "
                                           "advanced and the view was not updated: rebuild the brain"
                                         : "fb_lif_step_noalloc: device error %d; the brain's arrays may be partly "
                                           "advanced and the view was not updated: rebuild the brain", err);
  v->head = out.head;
  v->rng = out.rngP[nsteps & 1];
  v->bgAcc = out.bgAccP[nsteps & 1];
  v->nFired = out.nFired;
  v->lastSlot = out.lastSlot;
  return FB_OK;
}
