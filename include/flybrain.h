/*
 * flybrain.h -- C ABI of the GB300 brain step (connectome LIF network + its adjoint).
 *
 * This is the drop-in boundary for the reference's brain-model API: the LIFWasm object of
 * src/lifwasm.js:36-87 (and its WebGPU twin LIFGpu, src/lifgpu.js:183-370), which wraps the native
 * kernel `int32_t lif_step(Brain*)` of src/wasm/lif.c:29-80, plus the LIFDiff adjoint of
 * src/lifdiff.js:219-686. Every entry point takes plain pointers and sizes; no C++ or torch types
 * cross it. Array arguments may be host or device pointers (copies use unified addressing).
 *
 * Conventions
 *   - Every function returns an int status: FB_OK (0) or a negative FB_E* code. The message of the
 *     last failure on the calling thread is fb_last_error(). Nothing throws across the ABI.
 *   - A graph is read-only and may be shared by many brain batches (src/brainsetup.js:10-28 shares
 *     one connectome across flies), except for its sign vector (fb_graph_set_sign).
 *   - A brain batch holds B independent brains (trials), each with its own state block, seed,
 *     drive set and graph. Brain b of a batch is what one LIFWasm instance is in the reference.
 *   - Setters (drive, bias, thr, addG, pulse) are queued and applied in call order before the next
 *     step or read, so a read always observes every earlier write, as with LIFWasm's shared memory.
 *   - Handles are not thread-safe: use one handle per host thread (the reference runs one brain per
 *     worker thread).
 */
#ifndef FLYBRAIN_H
#define FLYBRAIN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FB_OK 0
#define FB_EINVAL -1     /* bad argument (size, index, null pointer, malformed CSR) */
#define FB_ECUDA -2      /* a CUDA runtime call failed (message names it) */
#define FB_ENOMEM -3     /* device allocation failed */
#define FB_ETIMEOUT -4   /* a device-side wait exceeded its limit; the step was abandoned */
#define FB_EOVERFLOW -5  /* per-step delivery scratch overflowed; state of that step is invalid */
#define FB_ESTATE -6     /* call not valid in the handle's current state */
#define FB_ENODEV -7     /* no CUDA device, or not an sm_103 device */

typedef struct fb_graph fb_graph;   /* opaque: one compiled connectome on the device */
typedef struct fb_brains fb_brains; /* opaque: a batch of B brains on the device */

/* Model parameters of one brain. Field meaning and units follow DEFAULTS of src/lif.js:6-15 (times
 * in ms, potentials in mV, rates in Hz). The derived f32 header constants (decays, kM, dtS, cE, cI,
 * background events per step) are computed from these in double and rounded once, as
 * LIFWasm._writeHeader does (src/lifwasm.js:55-68). */
typedef struct fb_params {
  double dt, vRest, vThresh, vReset, tauM, tauSyn, tRef, delay;
  double traceTau, adaptInc, adaptTau, depU, depTau;
  double eExc, eInh, bgRate, bgAmp, preInh;
  int32_t coba; /* 0: current-based (lif.c:65-71), 1: conductance-based (lif.c:55-63) */
  int32_t reserved;
} fb_params;

/* Fills *p with DEFAULTS of src/lif.js:6-15. */
void fb_default_params(fb_params *p);

/* Delivery modes of fb_brains_set_mode. */
#define FB_DELIVER_EXACT 0      /* default: per-target sums in the reference's order (bit-exact) */
#define FB_DELIVER_SEQUENTIAL 1 /* arrivals one by one; exact also with preInh > 0 (slow) */
#define FB_DELIVER_FAST 2       /* float atomics: statistical parity only */

/* Readable / writable per-neuron fields of fb_read / fb_write. */
#define FB_FIELD_V 0
#define FB_FIELD_GE 1
#define FB_FIELD_GI 2
#define FB_FIELD_REFR 3
#define FB_FIELD_TRACE 4
#define FB_FIELD_ADAPT 5
#define FB_FIELD_RES 6
#define FB_FIELD_BIAS 7
#define FB_FIELD_THR 8
#define FB_FIELD_DRIVE 9
#define FB_FIELD_SPIKECOUNT 10 /* uint32 */
#define FB_NFIELDS 11

/* Library and error reporting. */
int fb_version(void);             /* 10000 * major + 100 * minor + patch */
const char *fb_last_error(void);  /* thread-local message of the last failure ("" if none) */
int fb_device_info(int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor);

/* ---- graphs ------------------------------------------------------------------------------- */

/* Uploads a compiled CSR connectome: the arrays writeGraph lays out (src/lifwasm.js:14-34):
 * indptr u32[N+1], indices u32[E], weights f32[E], sign f32[N] (sign already carries wSyn).
 * A row may name a target up to four times (lif.c:40-42 adds every edge in row order, and so do
 * the kernels); more is refused with FB_EINVAL, as is N >= 2^29 - 4096 (the delivery keys). */
int fb_graph_create(int32_t N, int64_t E, const uint32_t *indptr, const uint32_t *indices,
                    const float *weights, const float *sign, fb_graph **out);

/* A second graph over the same topology (indptr/indices shared on the device, not copied) with its
 * own weights and sign: per-trial type gains bake into weights as writeGraph's outScale does
 * (src/lifwasm.js:23,31). */
int fb_graph_create_shared(const fb_graph *topology, const float *weights, const float *sign,
                           fb_graph **out);

/* writeGraph (src/lifwasm.js:14-34) on the device: a new graph over topology's CSR whose sign and
 * weights are compiled from raw per-edge synapse counts:
 *   sign[j] = f32(pre_sign[j] * wSyn)
 *   W[k] = (counts[k] >= minSyn && keep) ? f32(counts[k] * edge_gain[k] * in_scale[q] * ig) : 0
 *   ig = (pre_sign[j] < 0 ? inhGain : 1) * out_scale[j]
 *   keep = !sensory_mask[q] || (preInh > 0 && pre_sign[j] < 0)
 * each product formed in double in that order and rounded once, as the reference's Float32Array
 * stores round. in_scale, out_scale, sensory_mask and edge_gain may be null (factor 1 / no mask).
 * Arrays may be host or device pointers: f32 counts[E], edge_gain[E], pre_sign[N], in_scale[N],
 * out_scale[N] (outScale, the per-presynaptic type gain), u8 sensory_mask[N]. */
typedef struct fb_compile_params {
  double wSyn, inhGain, minSyn, preInh;
} fb_compile_params;
int fb_graph_compile(const fb_graph *topology, const float *counts, const float *pre_sign,
                     const float *in_scale, const float *out_scale, const uint8_t *sensory_mask,
                     const float *edge_gain, const fb_compile_params *p, fb_graph **out);

/* Copies a graph's weights f32[E] and/or sign f32[N] out (either may be null). */
int fb_graph_read(const fb_graph *g, float *weights, float *sign);

/* Replaces the sign vector, f32[N]. Replaces the direct write into graph.sign that
 * src/sim/neuromod.js:107 performs through brain.mem; every brain on this graph sees it. */
int fb_graph_set_sign(fb_graph *g, const float *sign);

/* N and E of a graph. */
int fb_graph_info(const fb_graph *g, int32_t *N, int64_t *E);

int fb_graph_destroy(fb_graph *g);

/* ---- brain batches (the LIFWasm surface) -------------------------------------------------- */

/* Creates B brains. graphs[b], params[b], seeds[b] per brain (params may be a single struct when
 * params_stride == 0). Each brain starts as `new LIFWasm(...)` leaves it (src/lifwasm.js:37-53):
 * state at rest, bias/thr/drive zero, head 0, RNG state (seed * 2654435761) >>> 0 || 1. */
int fb_brains_create(const fb_graph *const *graphs, int32_t B, const fb_params *params,
                     int32_t params_stride, const uint32_t *seeds, fb_brains **out);
int fb_brains_destroy(fb_brains *br);

/* Delivery mode for all brains of the batch (FB_DELIVER_*). */
int fb_brains_set_mode(fb_brains *br, int32_t mode);

/* Kernel schedules of fb_step (both exact). No counterpart in the reference, whose lif_step is a
 * serial loop. GRID: the persistent two-phase kernel with two grid barriers per step (any batch,
 * mode and logging). LAGGED: for one brain in exact mode without presynaptic inhibition, blocks
 * synchronise only at the synaptic delay (4 <= nslots - 1 <= 32 steps; per-step logging only in
 * launches of at most 64 steps). AUTO (default) takes LAGGED where it applies and the launch has
 * at least 8 steps, GRID otherwise; forcing LAGGED where it does not apply fails with
 * FB_EINVAL at fb_step. */
#define FB_SCHEDULE_AUTO 0
#define FB_SCHEDULE_GRID 1
#define FB_SCHEDULE_LAGGED 2
int fb_brains_set_schedule(fb_brains *br, int32_t schedule);
/* The schedule the last fb_step / fb_step_uneven launch ran (FB_SCHEDULE_GRID or _LAGGED). */
int fb_last_schedule(fb_brains *br, int32_t *schedule);

/* Launch shape of the grid schedule's persistent kernel, the knobs the autotuner
 * (flybrain.autotune) searches: resident CTAs per SM (1 .. max_blocks_per_sm; the grid is
 * sms x blocks_per_sm, 512 threads each) and kChunk = 32-edge delivery chunks per warp work item
 * (edges per warp item = 32 x item_chunks, 1 .. 64), and how the update phase's 64-neuron warp
 * sub-tiles reach the warps when each warp has many (a batch): 5/8 dealt round-robin, the rest
 * taken sub_grab at a time from a counter, or all dealt (-1). fb_brains_set_tuning ignores
 * max_blocks_per_sm and sms; 0 in a field keeps its current value. Results do not depend on the
 * shape. */
typedef struct fb_tuning {
  int32_t blocks_per_sm, item_chunks;
  int32_t max_blocks_per_sm, sms; /* read only */
  int32_t sub_grab;               /* update sub-tiles per dynamic grab, 1 .. 256; -1: all dealt statically */
  int32_t timeout_us;             /* bound of every device-side wait of both schedules, microseconds
                                     (default 5,000,000); a wait that runs out ends the launch with
                                     FB_ETIMEOUT */
  int32_t lag_driven_blocks;      /* delay-scheduled kernel: blocks the driven list is split over
                                     (1 or 2; 0 = automatic: 2 from 512 driven neurons) */
  int32_t pad;
} fb_tuning;
int fb_brains_set_tuning(fb_brains *br, const fb_tuning *t);
int fb_brains_tuning(fb_brains *br, fb_tuning *t);

/* Test hook for the timeout path, no counterpart in the reference (whose kernel has no waits; its
 * GPU path falls back on a failure, src/brainsetup.js:66-75). Arms the next launch of the
 * delay-scheduled kernel so that one tile block, at step `step` of that launch, waits on a flag
 * nothing sets: the wait runs out after timeout_us, every other block leaves its own bounded wait,
 * and the call returns FB_ETIMEOUT. A failed launch of that kernel leaves the brain as it was
 * before the call (state lives in shared memory until the launch completes), so the handle steps
 * on from there. Consumed by that one launch; -1 disarms. */
int fb_debug_trip_wait(fb_brains *br, int32_t step);

/* Advances every brain by nsteps steps in one persistent launch (lif_step, src/wasm/lif.c:29-80,
 * nsteps times). out_nfired (optional, int32[B]) receives each brain's fired count of its last
 * step: the value lif_step returns. */
int fb_step(fb_brains *br, int32_t nsteps, int32_t *out_nfired);

/* Uneven batch: brain b advances steps[b] steps (0 leaves it untouched), all in one launch. */
int fb_step_uneven(fb_brains *br, const int32_t *steps, int32_t *out_nfired);

/* Records, from the next step on, every step's fired count and fired list (ring order) of every
 * brain into device logs of cap_steps counts and cap_spikes indices per brain; fb_spike_log reads
 * brain b's log back (*n_steps, *n_spikes: totals recorded, which may exceed the caps given to
 * either call). fb_record(br, 0, 0) stops recording and frees the logs. */
int fb_record(fb_brains *br, int32_t cap_steps, int64_t cap_spikes);
int fb_spike_log(fb_brains *br, int32_t b, int32_t *counts, int32_t cap_steps, int32_t *raster,
                 int64_t cap_spikes, int64_t *n_steps, int64_t *n_spikes);

/* Fired list of brain b's last step, in ring order (driven spikes first, in driven-list order,
 * then threshold spikes in ascending index): the view LIFWasm.step returns
 * (src/lifwasm.js:83-84). *n receives the count; at most cap indices are copied. */
int fb_fired(fb_brains *br, int32_t b, int32_t *dst, int32_t cap, int32_t *n);

/* Brain b's delay ring as lif.c keeps it (src/wasm/lif.c:35,44-45,77-79; the ring LIFWasm lays
 * out in its memory, src/lifwasm.js:39-49): ring[nslots * N] receives the fired lists, of which
 * only the first counts[s] entries of slot s are meaningful; counts[nslots] the list lengths; *head
 * the slot the next step delivers. Slots head .. head + nslots - 2 (mod nslots) hold the spikes
 * still in flight. Any output may be NULL. */
int fb_ring_read(fb_brains *br, int32_t b, int32_t *ring, int32_t *counts, int32_t *head);

/* Injections, queued in call order and applied before the next step or read.
 * fb_set_drive: drive[idx[k]] = hz[k]; a positive rate appends the neuron to the driven set if
 *   absent, zero or negative removes it -- the insertion-ordered set of src/lifwasm.js:70-72,
 *   which fixes the RNG draw order. (setDriveOne / setDrive)
 * fb_set_bias: bias[idx[k]] = mv[k] (setBias, src/lifwasm.js:73)
 * fb_set_thr:  thr[idx[k]] = mv[k]  (setThr, :74)
 * fb_add_g:    gE[idx[k]] += e[k]; gI[idx[k]] += i[k], each sum formed in double and rounded once
 *              as a JS Float32Array store rounds (addG, :75)
 * fb_pulse:    gE[idx[k]] += mv[k], same rounding (pulse, :76) */
int fb_set_drive(fb_brains *br, int32_t b, const int32_t *idx, const double *hz, int32_t n);
int fb_set_bias(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n);
int fb_set_thr(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n);
int fb_add_g(fb_brains *br, int32_t b, const int32_t *idx, const double *e, const double *i,
             int32_t n);
int fb_pulse(fb_brains *br, int32_t b, const int32_t *idx, const double *mv, int32_t n);

/* State back to rest (src/lifwasm.js:78): v = vRest, gE = gI = refr = trace = adapt = 0, res = 1,
 * spikeCount = 0, ring counts 0. The ring head, RNG and background accumulator are kept, and
 * bias/thr/drive untouched, exactly as the reference. b == -1 resets every brain. */
int fb_reset(fb_brains *br, int32_t b);

/* Background synaptic events (setBackground, src/lifwasm.js:69). */
int fb_set_background(fb_brains *br, int32_t b, double rate_hz, double amp_mv);
/* LIFGpu.setParams (src/lifgpu.js:349): brain b's header constants recomputed from *params for
 * the next step (as at creation, src/lifwasm.js:55-68). The ring depth round(delay/dt)+1 must be
 * unchanged (FB_EINVAL otherwise); the state is kept. */
int fb_set_params(fb_brains *br, int32_t b, const fb_params *params);

/* Copies field (FB_FIELD_*) of brain b, N elements of 4 bytes, into dst / from src. */
int fb_read(fb_brains *br, int32_t field, int32_t b, void *dst);
int fb_write(fb_brains *br, int32_t field, int32_t b, const void *src);

/* Scalars of brain b: head, RNG state, last fired count, last slot, driven-set size, t in steps. */
int fb_scalars(fb_brains *br, int32_t b, int32_t *head, uint32_t *rng, int32_t *nfired,
               int32_t *last_slot, int32_t *n_driven, int64_t *steps_done);

/* Device-side timing of the last fb_step launch (ms, CUDA events on the launch stream). */
int fb_last_step_ms(fb_brains *br, float *ms);

/* In-library phase timer (no counterpart in the reference, which times stages from JS with
 * performance.now, scripts/profile_fly.mjs:13-27). fb_profile(br, 1) zeroes and enables it; each
 * step then adds, as seen by the first block of the grid, the time of: [0] the per-brain serial
 * part and ring bookkeeping, [1] the delivery work items, [2] the wait at the first barrier,
 * [3] the neuron update, [4] the wait at the second barrier; within [0], for the brain block 0
 * serves: [5] the header and background draws, [6] the driven-list gathers, [7] the draws,
 * [8] the forced spikes' emission, [9] the RNG advance. fb_phase_times copies up to n
 * accumulated totals in ms. With the schedule forced to FB_SCHEDULE_LAGGED the delay-scheduled
 * kernel runs instead (AUTO takes the grid kernel while profiling) and the slots hold: the first
 * driven block's [0] lag wait and completion signal, [1] background and delivery, [2] draws,
 * [3] update and spike list, [4] the next step's live entries; the first tile block's [5] wait at
 * the step barrier for its service warps, [6] compaction, [7] own spikes' pushes, [8] the driven
 * spikes' pushes, [9] delivery and update, [10] its publisher warp's work per step (completion
 * signal, the next step's lag check), [11] its helper warp's work per step (the next step's
 * driven spikes). */
#define FB_NPHASES 12
int fb_profile(fb_brains *br, int32_t on);
int fb_phase_times(fb_brains *br, double *ms, int32_t n);

/* ---- the differentiable brain (LIFDiff) and its adjoint ------------------------------------ */

/* Model parameters of LIFDiff (src/lifdiff.js:85-110): the brain step's parameters plus the nine
 * differentiable globals and the gradient options. coba 1 is the reference's conductance-based
 * model; 0 a current-based variant (lif.c's current-based membrane, src/wasm/lif.c:67). soft 1
 * replaces the hard threshold by a logistic in the forward pass too (src/lifdiff.js:101). */
typedef struct fb_diff_params {
  double dt, vRest, vThresh, vReset, tauM, tauSyn, tRef, delay;
  double wSyn, adaptInc, adaptTau, depU, depTau, minSyn;
  double eExc, eInh, inhGain, sizeAlpha, maxSizeScale, boostCap;
  double kcThreshold, laminaBias, surrogateBeta, adjClip;
  int32_t coba, soft, checkpoint;
  int32_t precision;  /* FB_DIFF_F64 (the reference's double intermediates) or FB_DIFF_F32 */
  int32_t drive_soft; /* driveSoft (src/lifdiff.js:102-104, :338): the drive's expected spike */
  int32_t exact32;    /* exact32 (:105-109): the forward in lif.c's f32 arithmetic */
  int32_t drive_epoch;/* driveEpoch (:134-144): steps a scheduled drive value is held */
  int32_t pad;
} fb_diff_params;

/* Arithmetic of the differentiable step's intermediates. FB_DIFF_F64 is LIFDiff's (JS numbers:
 * every intermediate in double, state in float32). FB_DIFF_F32 computes the same expressions in
 * float32 (state, tape and gradient accumulators are unchanged); it exists because GB300's FP64
 * rate is a small fraction of its FP32 rate. Not bit-identical to the reference. */
#define FB_DIFF_F64 0
#define FB_DIFF_F32 1

/* Fills *p with the defaults of src/lifdiff.js:86-109 (checkpoint 16, conductance-based). */
void fb_diff_default_params(fb_diff_params *p);

/* The network of a differentiable brain (src/lifdiff.js:84-145), host or device arrays:
 * CSR over raw synapse counts (indptr u32[N+1], indices u32[E], counts f32[E]); sign f32[N]
 * (before wSyn); optional: edge_gain f32[E], size_log / in_scale / log_gain / out_scale /
 * thr_offset / beta / bias f32[N], thr_mask / bias_mask / sensory u8[N]; the drive (drive f32[N]
 * in Hz and the driven set in insertion order, nDriven entries). bias is an additive per-neuron
 * current (mV) on top of bias_mask * laminaBias; it has no counterpart in LIFDiff, whose only bias
 * is laminaBias, and defaults to none. Fields given as null cannot be set later. */
typedef struct fb_diff_net {
  int32_t N, nDriven;
  int64_t E;
  const uint32_t *indptr, *indices;
  const float *counts, *edge_gain, *sign, *size_log, *in_scale, *log_gain, *out_scale;
  const float *thr_offset, *beta, *bias;
  const uint8_t *thr_mask, *bias_mask, *sensory;
  const float *drive;
  const int32_t *driven;
  int32_t nDriveIdx, pad;
  const int32_t *drive_idx; /* driveIdx (src/lifdiff.js:134-144): neurons whose drive is an input */
} fb_diff_net;

/* Gradients returned by fb_diff_backward (host arrays; each pointer may be null):
 * params[9] in the reference's order wSyn sizeAlpha inhGain eInh vThresh kcThreshold laminaBias
 * adaptInc depU (src/lifdiff.js:75); log_gain f32[N] (:658); edge f64[E]: dLoss/dW_j of each gated
 * edge's effective weight W_j = count * edge_gain * in_scale[post] (* inhGain); bias f64[N]:
 * dLoss/d per-neuron bias; out_scale f64[N]: dLoss/d out_scale (= log_gain / out_scale).
 * Non-finite values are zeroed and counted (src/lifdiff.js:681-684). */
typedef struct fb_diff_grads {
  double params[9];
  int32_t clamped_params, clamped_log_gain;
  float *log_gain;
  double *edge, *bias, *out_scale;
  float *drive;          /* [epochs][nDriveIdx]: dLoss/d(scheduled drive) (src/lifdiff.js:685) */
  int32_t clamped_drive, pad;
} fb_diff_grads;

/* Per-forward inputs beyond the network: the drive schedule drive_at[epochs][nDriveIdx] (the
 * values the reference's onEpoch callback sets, applied at every epoch boundary in driveIdx order
 * with setDriveOne semantics), and a recorded spike train (spikeTrain, src/lifdiff.js:298-306):
 * step t forces neurons train_idx[train_off[t] .. train_off[t+1]). Any pointer may be null. */
typedef struct fb_diff_inputs {
  const float *drive_at;
  const int64_t *train_off;
  const int32_t *train_idx;
} fb_diff_inputs;

typedef struct fb_diff fb_diff; /* opaque */

#define FB_DIFF_LOG_GAIN 0
#define FB_DIFF_OUT_SCALE 1
#define FB_DIFF_THR_OFFSET 2
#define FB_DIFF_BIAS 3
#define FB_DIFF_EDGE_GAIN 4
#define FB_DIFF_DRIVE 5

/* new LIFDiff(data, opts) (src/lifdiff.js:84): uploads the network. tape_cap bounds the spike
 * tape (entries over all steps; 0: 64 N, at least 1M). */
int fb_diff_create(const fb_diff_net *net, int64_t tape_cap, fb_diff **out);
int fb_diff_destroy(fb_diff *d);

/* Replaces one per-neuron (or, for FB_DIFF_EDGE_GAIN, per-edge) array given at creation. */
int fb_diff_set(fb_diff *d, int32_t field, const float *values);

/* forward(steps, {seed, record}) (src/lifdiff.js:219-353): runs from reset; spike_count (f32[N],
 * host or device, may be null) receives the per-neuron spike totals (soft amplitudes summed).
 * record keeps the tape and a state checkpoint every p->checkpoint steps for fb_diff_backward. */
int fb_diff_forward(fb_diff *d, const fb_diff_params *p, int32_t steps, uint32_t seed, int32_t record,
                    float *spike_count);
/* fb_diff_forward with a drive schedule and/or a spike train (in may be null). */
int fb_diff_forward_ex(fb_diff *d, const fb_diff_params *p, int32_t steps, uint32_t seed, int32_t record,
                       float *spike_count, const fb_diff_inputs *in);

/* The recorded forward's spike tape: offsets i64[steps+1] (step t's spikes are entries
 * offsets[t] .. offsets[t+1]-1, forced spikes first), neuron indices and amplitudes (up to cap
 * entries; *len gets the total). */
int fb_diff_tape(fb_diff *d, int64_t *offsets, int32_t *idx, float *amp, int64_t cap, int64_t *len);

/* The recorded forward's spikes of nro readout neurons as a dense raster out f32[steps][nro]
 * (amplitudes; host or device). */
int fb_diff_raster(fb_diff *d, int32_t nro, const int32_t *readout, float *out);

/* backward(tape, dLdSpike, {truncate, lossFrom}) (src/lifdiff.js:494-686) over the recorded
 * forward. dL: f32[N] applied at every scored step (nro == 0), or f32[steps][nro] over the readout
 * neurons `readout` (a per-step generalisation of dLdSpikePerEpoch, :519-522). */
int fb_diff_backward(fb_diff *d, const float *dL, int32_t nro, const int32_t *readout, int32_t truncate,
                     int32_t loss_from, fb_diff_grads *g);

/* ---- batches of differentiable brains ------------------------------------------------------
 * No counterpart in the reference, which trains one LIFDiff at a time: B independent instances
 * (each its own network, drive, seed and length; one parameter set) advanced together, every
 * kernel launch covering the whole batch; a forward pass and a backward pass each run as one
 * captured CUDA graph (fb_diff_tuning). Arrays passed by the same pointer for the same field
 * of several instances are uploaded once and shared (fb_diff_batch_set on one of them sets it for
 * all). Each instance's results are those of fb_diff_* on that instance alone. */
typedef struct fb_diff_batch fb_diff_batch; /* opaque */

int fb_diff_batch_create(const fb_diff_net *nets, int32_t B, int64_t tape_cap, fb_diff_batch **out);
int fb_diff_batch_destroy(fb_diff_batch *b);
int fb_diff_batch_set(fb_diff_batch *b, int32_t inst, int32_t field, const float *values);

/* Forward of every instance from reset: steps[B] and seeds[B]; spike_counts (may be null)
 * receives the instances' f32[N_b] spike totals back to back. */
/* Launch shape of the per-step kernels (the autotuner's knobs): blocks per member of the
 * thread-per-neuron kernels (256 threads; at most the member's tile count is used) and of the
 * warp-per-arrival kernels. 0 restores the default (one tile per block for one member, about
 * four waves over the batch otherwise; 304 blocks over the batch). Results do not depend on it.
 * step_launches: 0 (default) runs a forward, and a backward's replays and reverse steps, as one
 * CUDA graph launch each, captured at the first pass with the same step counts, checkpoint
 * interval, launch shape and scalar parameters and kept (up to four per batch); 1 launches every
 * step's kernels from the host instead. Results do not depend on it either. */
typedef struct fb_diff_tuning {
  int32_t neuron_blocks, arrival_blocks, step_launches;
} fb_diff_tuning;
int fb_diff_batch_set_tuning(fb_diff_batch *b, const fb_diff_tuning *t);

int fb_diff_batch_forward(fb_diff_batch *b, const fb_diff_params *p, const int32_t *steps,
                          const uint32_t *seeds, int32_t record, float *spike_counts);
/* ... with per-member inputs in[B] (may be null, as may any member's pointers). */
int fb_diff_batch_forward_ex(fb_diff_batch *b, const fb_diff_params *p, const int32_t *steps,
                             const uint32_t *seeds, int32_t record, float *spike_counts,
                             const fb_diff_inputs *in);
int fb_diff_batch_tape(fb_diff_batch *b, int32_t inst, int64_t *offsets, int32_t *idx, float *amp,
                       int64_t cap, int64_t *len);
int fb_diff_batch_raster(fb_diff_batch *b, int32_t inst, int32_t nro, const int32_t *readout, float *out);
/* Every member's readout raster of the recorded forward in one call: member k's steps x nro[k]
 * amplitudes into out[k] (device memory), with one upload of the member records and one
 * synchronisation for the whole batch (fb_diff_batch_raster per member costs both per call). */
int fb_diff_batch_rasters(fb_diff_batch *b, const int32_t *nro, const int32_t *const *readout, float *const *out);

/* Backward of every instance over its recorded forward: dL[b], nro[b] (null: all 0) and
 * readout[b] as in fb_diff_backward; g[b] receives instance b's gradients (host or device
 * pointers). */
int fb_diff_batch_backward(fb_diff_batch *b, const float *const *dL, const int32_t *nro,
                           const int32_t *const *readout, int32_t truncate, int32_t loss_from,
                           fb_diff_grads *g);

/* out f64[E] (host or device) = the per-edge gradients of instances insts[0..n) of the last
 * backward, summed in list order (the instances must have the same edge count). */
int fb_diff_batch_edge_sum(fb_diff_batch *b, int32_t n, const int32_t *insts, double *out);

/* ---- flyvis optic lobe ----------------------------------------------------------------------
 * The rate network of lif.c's fv_step (src/wasm/lif.c:82-93), as src/flyvis.js drives it (one
 * FlyVis per eye, sharing the model: src/brainsetup.js:21-23): B instances sharing one model
 * (graph by source: indptr[N+1], target[E], weight[E]; bias[N]; kdt[N] = dt / max(tau, dt) as
 * f32), each with its own v and input x. fb_flyvis_step advances every instance nsteps times,
 * each step lif.c's fv_step bit for bit (its per-target sum order kept, no atomics). */
typedef struct fb_flyvis fb_flyvis;
#define FB_FV_V 0 /* membrane / activity v */
#define FB_FV_X 1 /* external input x */
/* FlyVis constructor (src/flyvis.js:4-17): v starts at bias. Model arrays are host or device. */
int fb_flyvis_create(int32_t N, int64_t E, const int32_t *indptr, const int32_t *target, const float *weight,
                     const float *bias, const float *kdt, int32_t B, fb_flyvis **out);
int fb_flyvis_destroy(fb_flyvis *f);
/* FlyVis.reset (src/flyvis.js:24): v = bias, of instance b (b < 0: all). */
int fb_flyvis_reset(fb_flyvis *f, int32_t b);
/* FlyVis.setInput (src/flyvis.js:20-21) of instance b: x[idx[k]] = values[k] in list order. */
int fb_flyvis_set_input(fb_flyvis *f, int32_t b, int32_t n, const int32_t *idx, const float *values);
/* Whole-array access to instance b's v or x (N floats, host or device). */
int fb_flyvis_write(fb_flyvis *f, int32_t field, int32_t b, const float *values);
int fb_flyvis_read(fb_flyvis *f, int32_t field, int32_t b, float *out);
/* FlyVis.step (src/flyvis.js:22), nsteps times for every instance. */
int fb_flyvis_step(fb_flyvis *f, int32_t nsteps);
int fb_flyvis_last_ms(fb_flyvis *f, float *ms);
/* Device pointers of the current state, layout [N][B] (instance fastest); valid until the next
 * step (v is double-buffered). */
int fb_flyvis_state(fb_flyvis *f, float **v, float **x, int32_t *layout_b);

/* ---- allocation-free step ----------------------------------------------------------------- */

/* A caller-owned brain for fb_lif_step_noalloc: the fields of the reference's Brain header
 * (src/wasm/lif.c:4-25, as LIFWasm._writeHeader fills it) with every array a DEVICE pointer the
 * caller allocated, plus the edge count E (= indptr[N]). Sizes: f32[N] v gE gI refr trace adapt
 * res bias thr drive sign; u32[N] spikeCount; u32[N+1] indptr; u32[E] indices; f32[E] weights;
 * i32[nslots * N] ring; i32[nslots] ringCount; i32[N] driven (the first nDriven entries are the
 * driven list, in insertion order). A fresh brain has v = vRest, res = 1, everything else zero. */
typedef struct fb_brain_view {
  int32_t N, nslots, head, coba;
  float dt, vRest, vThresh, vReset, tRef, adaptInc, depU;
  float dE, dTr, dA, kRec, kM, dtS, eExc, eInh, cE, cI;
  uint32_t rng;
  float *v, *gE, *gI, *refr, *trace, *adapt, *res, *bias, *thr, *drive, *sign;
  uint32_t *spikeCount;
  const uint32_t *indptr, *indices;
  const float *weights;
  int32_t *ring, *ringCount;
  int32_t *driven;
  int32_t nDriven;
  int32_t nFired, lastSlot;
  float bgEvents, bgAmp, bgAcc, preInh;
  int64_t E;
} fb_brain_view;

/* nsteps brain steps on caller-owned memory, allocating nothing -- no counterpart in the
 * reference (whose lif_step allocates nothing either, but also runs no GPU kernels). For callers
 * that may not call cudaMalloc/cudaFree: a host application that hands out every byte of device
 * memory from its own pool (an engine with a fixed device budget), or a real-time control loop
 * (the embodied fly steps its brain twice per simulated millisecond) that cannot take the
 * device-wide synchronisation an allocation or a free may imply. The step's scratch is a
 * file-scope __device__ array of 64 MiB that every GPU loading this library holds until exit; a
 * brain must fit it (about N = 20,000 neurons with 1.2M edges and a 19-slot ring), larger ones are
 * rejected with FB_EINVAL (use fb_brains_create). Results are those of fb_step, bit for bit.
 * Before anything is written the call checks, on the device, every index the step will follow
 * (indptr from 0 to E and non-decreasing, targets, the driven list, the ring lists and counts);
 * a violation returns FB_EINVAL with the brain untouched. A row that names one target more than
 * once has those contributions added in an unspecified order (fb_graph_create keeps row order). On success the view's head, rng, bgAcc,
 * nFired and lastSlot hold the state after the last step, and ring[lastSlot * N ...] its fired
 * list. On FB_ETIMEOUT or FB_EOVERFLOW the device arrays may be partly advanced while the view's
 * scalars are those from before the call: the brain is no longer consistent and must be rebuilt.
 * stream: a cudaStream_t (NULL: the legacy default stream); the call synchronises it (once after
 * the index check, once at the end) before returning. The first call on a device sets the device
 * up: it looks up the scratch array's device address and writes the xorshift jump tables into it,
 * then synchronises the device. Every call shares the one array and keeps the last call's
 * contents, so each call clears what must start at zero first; calls that overlap on the GPU race
 * on the array: serialise them. */
int fb_lif_step_noalloc(fb_brain_view *brain, int32_t nsteps, void *stream);

/* ---- the reference's compressed data files (host decoders, no device work) -------------------
 * FLYG, the connectome CSR the web app loads (graph.flyg; src/codec/graph.js:70-108, read by
 * src/data.js:28), and FLYN, its per-neuron table (neurons.flyn; src/codec/neurons.js:25-37), both
 * range coded (src/codec/rc.js). The decoded arrays are those of graph_w{min_weight}.bin (rows by
 * presynaptic neuron, each ascending by target; weights = synapse counts) and neurons.bin.
 * fb_flyg_sizes reads the sizes to allocate: indptr[N+1], indices[E], weights[E]. A corrupt
 * stream returns FB_EINVAL (the outputs are then undefined). */
typedef struct fb_flyg_header {
  uint32_t N, E, min_weight, pad;
} fb_flyg_header;
int fb_flyg_sizes(const uint8_t *buf, size_t len, fb_flyg_header *h);
int fb_flyg_decode(const uint8_t *buf, size_t len, uint32_t *indptr, uint32_t *indices, uint16_t *weights);
/* FLYN: N, then per neuron body_ids[N], soma[N][3] (voxels; NaN when absent), cls[N], nt[N],
 * superclass[N], side[N]. */
int fb_flyn_count(const uint8_t *buf, size_t len, uint32_t *N);
int fb_flyn_decode(const uint8_t *buf, size_t len, int64_t *body_ids, float *soma, uint16_t *cls, uint8_t *nt,
                   uint8_t *superclass, uint8_t *side);

#ifdef __cplusplus
}
#endif
#endif /* FLYBRAIN_H */
