"""Benchmark of the GB300 brain step on the full-scale synthetic connectome.

Workload (N=1): the 165,122-neuron, ~11M-edge synthetic graph, 2,000 seeded drive neurons at
U(100, 200) Hz, dt 0.1 ms, current-based LIF; the timed window simulates 2,000 ms (20,000 brain
steps) from rest. One bench step = 1,000 brain steps (100 ms simulated) in one persistent launch.

  value : synaptic events/s (events = spikes x out-degree, delivered) over the timed window,
          device time of the step launches (CUDA events on the launching stream), state in HBM
  e2e   : the same metric through the C ABI with host buffers: each bench step uploads the drive
          set from host memory, runs, and reads spike counts + the last fired list back (into
          pinned buffers; the events are counted from those after the timed region)
  cpu_baseline : the oracle port of lif_step (1 core: the reference kernel is serial) on a
          bounded sample of the same workload
  extra legs (each switchable by FB_BENCH_<LEG>=0), each with its own cpu_baseline except the
  scatter leg (a phase of a kernel, timed alone):
          high_activity (the headline plus a 6 mV tonic bias: ~97% of spikes recurrent),
          scatter (the grid kernel's delivery phase timed alone, 256 trials under that bias),
          adjoint, adjoint_batched, adjoint_uneven (float32 and, beside it, float64 -- the
          reference's arithmetic), batched (256 trials; split over ranks when N > 1), flyvis
          (64 eyes), embodied (the per-millisecond call pattern of the simulated fly)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Over N GPUs (torchrun, one rank per GPU): the single-trial legs run as independent replicas
(value = all ranks' events over the slowest rank's time); the batched ensemble's trials are split
over the ranks (rank r runs trials r, r + N, ...), the batched adjoint's in contiguous blocks whose
per-edge gradients are summed in global trial order by a chained hand-over (flybrain.shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "fly-brain_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "synaptic events/s & sim-s/wall-s at 165k LIF; batched fwd+adjoint vs plain fwd"
BRAIN_STEPS_PER_BENCH_STEP = int(os.environ.get("FB_BRAIN_STEPS", "1000"))
L2_FLUSH_BYTES = 512 << 20
# DRAM bytes (read + write) per brain step of the single-trial full-scale launch, from one ncu
# capture of a 100-step launch of each kernel (profiles/); traffic grows in proportion to steps.
DRAM_BYTES_PER_STEP_SINGLE = {
    "grid": 16.826112e6 / 100,    # fb::step_kernel
    "lagged": (52.875264e6 + 0.801792e6) / 100,   # fb::lagged_kernel
}
# DRAM bytes (read + write) per trial-step of the batched grid kernel, from one ncu capture of a
# 100-step launch over 32 full-scale trials (profiles/step_kernel_batched_32_trials.txt:
# 12.51 GB read + 6.95 GB written over 3,200 trial-steps); the bench's launch is scaled by its
# trial-steps (the update streams every trial's state, so traffic grows in proportion).
DRAM_BYTES_PER_TRIAL_STEP_BATCHED = (12.51e9 + 6.95e9) / 3200
HIGH_ACTIVITY_BIAS_MV = 6.0
KERNEL_NAME = {
    "grid": "fb::step_kernel (persistent, two grid barriers per step)",
    "lagged": "fb::lagged_kernel (persistent, delay-scheduled)",
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.stop = gpu, [], threading.Event()

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 4 + k and r[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("FB_BENCH_BACKEND") != "gloo" else "gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(x, world, op):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.MAX if world > 1 else None)


def sum_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.SUM if world > 1 else None)


def replica_throughput(events, seconds, world):
    """Whole-job throughput of independent replicas: the events of every rank over the slowest
    rank's time (each rank times its own timed region between barriers)."""
    return sum_over_ranks(events, world) / max_over_ranks(seconds, world)


def algorithmic_bytes(N, steps, spikes, events):
    """Bytes the step must move (per brain step: 64 B of state per neuron; per delivered spike
    20 B of row/sign/resource access; 16 B per synaptic event; 16 B per emitted spike)."""
    return 64.0 * N * steps + 20.0 * spikes + 16.0 * events + 16.0 * spikes


def cpu_baseline(g, idx, hz, params, sample_steps, bias_mv=0.0, warm_steps=200):
    """The oracle port of lif_step on one host core over sample_steps brain steps (after
    warm_steps from rest)."""
    from oracle import oracle as O
    O.build(ref=False)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, params, seed=1, backend="port")
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
    if bias_mv:
        ob.setBias(np.arange(g.N, dtype=np.int32), bias_mv)
    ob.run(warm_steps)  # warm caches (and, with a bias, the activity)
    sc0 = ob.spikeCount.astype(np.int64)
    t0 = time.perf_counter()
    ob.run(sample_steps)
    dt = time.perf_counter() - t0
    ev = float(((ob.spikeCount.astype(np.int64) - sc0) * g.outdeg()).sum())
    return ev / dt, dt, ev


def cpu_batched(g, spec, params, graphs, trials, sample_steps):
    """The batched ensemble on the host cores: as many of the trials as there are host threads,
    each an oracle brain with its own compiled weights (read back from the device), seed and drive,
    advanced together by ob_run_many (OpenMP, one trial per thread; the reference shares one graph
    across flies the same way, src/brainsetup.js:10-28). Trial-seconds per wall-second."""
    from oracle import oracle as O
    O.build(ref=False)
    threads = int(O.lib("port").ob_threads())
    n = min(threads, len(trials))
    brains = []
    for k in range(n):
        b = int(trials[k])
        w, sg = graphs[k].read()
        ob = O.OracleBrain(g.N, g.indptr, g.indices, w, sg, params, seed=int(spec["seeds"][b]))
        idx, hz = spec["drives"][b]
        for i, h in zip(idx.tolist(), hz.tolist()):
            ob.setDriveOne(i, h)
        brains.append(ob)
    O.run_many(brains, [50] * n)  # warm caches
    sc0 = [ob.spikeCount.astype(np.int64) for ob in brains]
    outdeg = g.outdeg().astype(np.int64)
    t0 = time.perf_counter()
    O.run_many(brains, [sample_steps] * n)
    secs = time.perf_counter() - t0
    ev = sum(float(((ob.spikeCount.astype(np.int64) - c) * outdeg).sum()) for ob, c in zip(brains, sc0))
    trial_s = n * sample_steps * params["dt"] / 1000.0
    return dict(value=trial_s / secs, unit="trial-s per wall-s", cores=n, kind="port", events_per_s=ev / secs,
                sample=f"{n} of the trials ({sample_steps} brain steps each after 50 warm-up steps), oracle port "
                       f"of lif_step, one trial per host thread ({secs:.1f} s)")


def cpu_adjoint(problems, steps, readouts, label):
    """The restated CPU adjoint (oracle/lifdiff.c: LIFDiff's forward with tape and checkpoints,
    replay and reverse sweep, src/lifdiff.js:219-686) on `problems`, one per host thread, each a
    recorded forward of `steps` steps and its backward with a per-step readout gradient.
    Trial-seconds of gradient per wall-second."""
    import concurrent.futures as cf

    def one(k):
        prob = problems[k]
        _, tape = prob.forward(steps, seed=k + 1, checkpoint=100)
        rng = np.random.default_rng(k)
        dL = np.zeros((steps, prob.N), np.float32)
        dL[:, readouts[k]] = (rng.standard_normal((steps, readouts[k].shape[0])) * 1e-3).astype(np.float32)
        prob.backward(tape, dL)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=len(problems)) as ex:
        list(ex.map(one, range(len(problems))))
    secs = time.perf_counter() - t0
    trial_s = len(problems) * steps * 0.1 / 1000.0
    return dict(value=trial_s / secs, unit="trial-s of gradient per wall-s", cores=len(problems), kind="port",
                seconds_per_trial_s=secs / trial_s,
                sample=f"{label}: {len(problems)} x {steps} steps, recorded forward + backward (oracle "
                       f"restatement of LIFDiff in double, one problem per host thread, {secs:.1f} s)")


def run_ours(args, rank, world):
    import torch
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda, workload

    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0")))
    g, idx, hz, _ = workload("full", seed=1)
    outdeg = g.outdeg().astype(np.int64)
    brain = LIFCuda(DeviceGraph(g), SYNTH_PARAMS, seed=1)
    brain._batch.set_drive(0, idx, hz)
    S = BRAIN_STEPS_PER_BENCH_STEP
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        brain.run(S)
    brain.reset()
    torch.cuda.synchronize()

    # ---- device-timed region: K launches of S brain steps, L2 flushed between launches ----
    launch_ms, events, spikes = [], 0.0, 0.0
    sc_prev = brain.spikeCount.astype(np.int64)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            brain.run(S)
            launch_ms.append(brain._batch.last_ms())
            sc = brain.spikeCount.astype(np.int64)
            d = sc - sc_prev
            events += float((d * outdeg).sum())
            spikes += float(d.sum())
            sc_prev = sc
    torch.cuda.synchronize()
    barrier(world)
    dev_s = max_over_ranks(sum(launch_ms) / 1e3, world)
    tot_events = sum_over_ranks(events, world)
    sim_s = args.steps * S * SYNTH_PARAMS["dt"] / 1000.0

    # ---- end to end through the C ABI with host buffers ----
    brain.reset()
    # inputs and results in pinned host memory
    h_idx = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int32)).pin_memory().numpy()
    h_hz = torch.from_numpy(np.ascontiguousarray(hz, dtype=np.float64)).pin_memory().numpy()
    # (one result buffer per bench step: the events are counted from them after the timed region,
    # since that accounting is the metric's, not part of the call a user makes)
    h_scs = [torch.empty(g.N, dtype=torch.int32).pin_memory().numpy().view(np.uint32) for _ in range(args.steps)]
    h_fired = torch.empty(g.N, dtype=torch.int32).pin_memory().numpy()
    e2e_events, h2d, d2h = 0.0, 0, 0
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        brain._batch.set_drive(0, h_idx, h_hz)
        h2d += h_idx.nbytes + h_hz.nbytes
        brain.run(S)
        brain._batch.read("spikeCount", 0, out=h_scs[k])
        fired = brain._batch.fired(0, out=h_fired)
        d2h += g.N * 4 + fired.nbytes
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    sc_prev = np.zeros(g.N, dtype=np.int64)
    for h_sc in h_scs:
        sc = h_sc.astype(np.int64)
        e2e_events += float(((sc - sc_prev) * outdeg).sum())
        sc_prev = sc
    e2e_events = sum_over_ranks(e2e_events, world)

    peak, kind = peaks()
    from flybrain import _native as nat
    sched = "lagged" if brain._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED else "grid"
    per_launch_bytes = algorithmic_bytes(g.N, S, spikes / args.steps, events / args.steps)
    achieved = per_launch_bytes / (np.mean(launch_ms) / 1e3) / 1e9
    res = dict(
        metric=METRIC, value=tot_events / dev_s, unit="synaptic events/s", n_gpus=world,
        steps=args.steps, warmup=args.warmup, ms_per_step=1e3 * dev_s / args.steps,
        higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
        data="synthetic (seeded connectome-shaped graph; no dataset)",
        config=dict(workload="plain forward, full scale: N=165,122 synthetic connectome, "
                    f"E={g.E:,} edges, 2,000 drive neurons at U(100,200) Hz, dt 0.1 ms, "
                    f"{args.steps * S} brain steps ({sim_s * 1e3:.0f} ms simulated)",
                    neurons=g.N, edges=g.E, brain_steps_per_step=S,
                    delivery="exact (reference per-target order)",
                    l2="flushed between timed launches (512 MiB write)", parallelism=f"replicas x{world}"),
        sim_s_per_wall_s=sim_s / dev_s, realtime_factor=sim_s / dev_s, spikes=spikes,
        events=tot_events,
        e2e=dict(value=e2e_events / e2e_s, unit="synaptic events/s", h2d_bytes_per_step=h2d // args.steps,
                 d2h_bytes_per_step=d2h // args.steps, sim_s_per_wall_s=sim_s / e2e_s),
        # the lagged schedule launches the step kernel and the ring bookkeeping kernel
        gpu_launches=args.steps * (2 if sched == "lagged" else 1),
        schedule=sched,
        roofline=dict(bound="hbm", achieved=achieved, peak=peak, unit="GB/s", frac=achieved / peak,
                      peak_kind=kind, traffic=DRAM_BYTES_PER_STEP_SINGLE[sched] * S,
                      kernel=KERNEL_NAME[sched], algorithmic_bytes_per_launch=per_launch_bytes),
        clocks=clk.summary(),
    )
    del brain
    torch.cuda.empty_cache()
    if os.environ.get("FB_BENCH_ACTIVE", "1") == "1":
        res["high_activity"] = run_high_activity(g, idx, hz, args)
        torch.cuda.empty_cache()
    precisions = [x for x in os.environ.get("FB_ADJ_PRECISIONS", "f32,f64").split(",") if x]
    if os.environ.get("FB_BENCH_ADJOINT", "1") == "1":
        res["adjoint"] = by_precision(precisions, lambda pr: run_adjoint(g, idx, hz, prec=pr, cpu=pr == precisions[0]))
        torch.cuda.empty_cache()
    if os.environ.get("FB_BENCH_ADJOINT_BATCH", "1") == "1":
        plain_per_trial_s = dev_s / sim_s

        def batched_adj(pr):
            ab = run_adjoint_batched(g, idx, hz, n_trials=int(os.environ.get("FB_ADJ_TRIALS", "64")),
                                     steps=int(os.environ.get("FB_ADJ_STEPS", "5000")), prec=pr, rank=rank,
                                     world=world, cpu=pr == precisions[0])
            ab["plain_single_trial_forward_per_trial_s"] = plain_per_trial_s
            ab["cost_vs_plain_single_trial_forward"] = ab["fwd_bwd_per_trial_s"] / plain_per_trial_s
            torch.cuda.empty_cache()
            return ab

        res["adjoint_batched"] = by_precision(precisions, batched_adj)
        res["adjoint_uneven"] = by_precision(
            precisions, lambda pr: run_adjoint_uneven(n_inst=int(os.environ.get("FB_ADJ_UNEVEN", "128")), prec=pr,
                                                      cpu=pr == precisions[0]))
        torch.cuda.empty_cache()
    if os.environ.get("FB_BENCH_BATCHED", "1") == "1":
        torch.cuda.empty_cache()
        bt = run_batched(g, args, n_trials=int(os.environ.get("FB_BATCH_TRIALS", "256")), rank=rank, world=world)
        bt["cost_vs_plain_per_trial_s"] = (1.0 / bt["trial_s_per_wall_s"]) / (dev_s / sim_s)
        res["batched"] = bt
    if os.environ.get("FB_BENCH_SCATTER", "1") == "1":
        torch.cuda.empty_cache()
        res["scatter"] = run_scatter(g, idx, hz)
    if os.environ.get("FB_BENCH_FLYVIS", "1") == "1":
        torch.cuda.empty_cache()
        res["flyvis"] = run_flyvis(n_eyes=int(os.environ.get("FB_FLYVIS_EYES", "64")))
    if os.environ.get("FB_BENCH_EMBODIED", "1") == "1":
        torch.cuda.empty_cache()
        res["embodied"] = run_embodied(g)
    if rank == 0:
        sample = int(os.environ.get("FB_CPU_SAMPLE_STEPS", "4000"))
        v, secs, ev = cpu_baseline(g, idx, hz, SYNTH_PARAMS, sample)
        res["cpu_baseline"] = dict(value=v, unit="synaptic events/s", cores=1, kind="port",
                                   sample=f"{sample} brain steps of the same workload from rest "
                                          f"({secs:.1f} s, oracle port of lif_step, 1 thread)")
        print(json.dumps(res), flush=True)


def run_high_activity(g, idx, hz, args, bias_mv=HIGH_ACTIVITY_BIAS_MV, launches=5):
    """High-activity variant of the full-scale forward: the headline's graph and drive plus a
    tonic bias of `bias_mv` on every neuron (setBias), which holds the network about 1 mV below
    threshold, so that almost every spike is a recurrent threshold crossing (about 60 Hz mean rate
    and 50k synaptic events per step, against about 1.5k in the headline, where nearly every spike
    is a driven one). Times the delivery and threshold cascade the headline barely exercises:
    `launches` launches of the bench step's length from rest, L2 flushed between them."""
    import torch
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda
    from flybrain import _native as nat
    S = BRAIN_STEPS_PER_BENCH_STEP
    brain = LIFCuda(DeviceGraph(g), SYNTH_PARAMS, seed=1)
    brain._batch.set_drive(0, idx, hz)
    brain.setBias(np.arange(g.N, dtype=np.int32), bias_mv)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    brain.run(S)  # warm-up
    brain.reset()
    outdeg = g.outdeg().astype(np.int64)
    driven = np.zeros(g.N, bool)
    driven[idx] = True
    sc_prev = brain.spikeCount.astype(np.int64)
    ms, events, spikes, dspikes = [], 0.0, 0.0, 0.0
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(launches):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            brain.run(S)
            ms.append(brain._batch.last_ms())
            sc = brain.spikeCount.astype(np.int64)
            d = sc - sc_prev
            events += float((d * outdeg).sum())
            spikes += float(d.sum())
            dspikes += float(d[driven].sum())
            sc_prev = sc
    secs = sum(ms) / 1e3
    sim_s = launches * S * SYNTH_PARAMS["dt"] / 1000.0
    sched = "lagged" if brain._batch.last_schedule() == nat.FB_SCHEDULE_LAGGED else "grid"
    peak, kind = peaks()
    byts = algorithmic_bytes(g.N, S, spikes / launches, events / launches)
    ach = byts / (np.mean(ms) / 1e3) / 1e9
    del brain
    sample = int(os.environ.get("FB_CPU_ACTIVE_SAMPLE_STEPS", "1000"))
    v, csecs, _ = cpu_baseline(g, idx, hz, SYNTH_PARAMS, sample, bias_mv=bias_mv, warm_steps=300)
    return dict(bias_mv=bias_mv, launches=launches, brain_steps=launches * S, events_per_s=events / secs,
                ms_per_1000_steps=1e3 * secs / (launches * S) * 1000, realtime_factor=sim_s / secs,
                spikes_per_step=spikes / (launches * S), recurrent_fraction=1.0 - dspikes / max(spikes, 1.0),
                events_per_step=events / (launches * S), schedule=sched, gpu_launches=launches * (2 if sched == "lagged" else 1),
                roofline=dict(bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak, peak_kind=kind,
                              traffic=None, kernel=KERNEL_NAME[sched], algorithmic_bytes_per_launch=byts),
                clocks=clk.summary(),
                cpu_baseline=dict(value=v, unit="synaptic events/s", cores=1, kind="port",
                                  sample=f"{sample} brain steps after 300 from rest, same bias ({csecs:.1f} s, "
                                         "oracle port of lif_step, 1 thread)"),
                config=f"the headline workload (N={g.N:,}, 2,000 drive neurons at U(100,200) Hz) plus a tonic "
                       f"{bias_mv} mV bias on every neuron; {launches} launches of {S} steps from rest, L2 flushed "
                       "between launches")


def by_precision(precisions, fn):
    """A leg's result in its first precision, with each further precision's result beside it
    under its own key (e.g. "f64")."""
    out = None
    for pr in precisions:
        r = fn(pr)
        if out is None:
            out = r
        else:
            out[pr] = r
    return out


def run_scatter(g, idx, hz, n_trials=256, bias_mv=6.0, warm=300, steps=100):
    """The scatter on its own: the grid kernel's delivery phase (each arriving spike's edges into
    the per-target buckets: edge record, W*s, an atomic slot claim and the bucket store) under
    load -- n_trials trials of the full graph with the headline drive and a tonic bias_mv bias on
    every neuron, timed by the kernel's phase timer over `steps` steps after `warm` steps from rest.
    Bandwidth in the phase's algorithmic bytes (16 B per synaptic event + 20 B per arrival) over the
    delivery phase's time, against the measured HBM peak; the update phase beside it in its 64 B
    per neuron. The phase timer's own cost is inside the phase times; the same steps without it are
    reported as plain_ms_per_step."""
    from flybrain import SYNTH_PARAMS, BrainBatch, DeviceGraph
    dg = DeviceGraph(g)
    outdeg = g.outdeg().astype(np.int64)
    bb = BrainBatch([dg] * n_trials, SYNTH_PARAMS, list(range(1, n_trials + 1)))
    bv = np.full(g.N, bias_mv, np.float32)
    for b in range(n_trials):
        bb.set_drive(b, idx, hz)
        bb.write("bias", b, bv)
    bb.step(warm)

    def counts():
        return np.stack([bb.read("spikeCount", b).astype(np.int64) for b in range(n_trials)])

    sc0 = counts()
    bb.step(steps)
    plain_ms = bb.last_ms()
    sc1 = counts()
    bb.profile(True)
    bb.step(steps)
    ph = bb.phase_times()
    bb.profile(False)
    sc2 = counts()
    d = sc2 - sc1
    events, arrivals = float((d * outdeg).sum()), float(d.sum())
    peak, kind = peaks()
    dbytes = 16.0 * events + 20.0 * arrivals
    ubytes = 64.0 * g.N * n_trials * steps
    deliver_s, update_s = ph["deliver"] / 1e3, ph["update"] / 1e3
    out = dict(trials=n_trials, bias_mv=bias_mv, steps=steps, events_per_trial_step=events / steps / n_trials,
               plain_ms_per_step=plain_ms / steps, plain_events_per_trial_step=float(((sc1 - sc0) * outdeg).sum()) / steps / n_trials,
               phase_ms_per_step={k: v / steps for k, v in ph.items() if k in ("serial", "deliver", "barrier1", "update", "barrier2")},
               roofline=dict(bound="hbm", achieved=dbytes / deliver_s / 1e9, peak=peak, unit="GB/s",
                             frac=dbytes / deliver_s / 1e9 / peak, peak_kind=kind, traffic=None,
                             kernel="fb::step_kernel, delivery phase", algorithmic_bytes=dbytes),
               update_gbs=ubytes / update_s / 1e9, update_frac=ubytes / update_s / 1e9 / peak,
               config=f"{n_trials} trials x N={g.N:,}, 2,000 drive neurons at U(100,200) Hz and a tonic {bias_mv} mV bias on "
                      f"every neuron; {steps} steps after {warm} from rest, phase-timed")
    del bb
    return out


def run_embodied(g, ms=1000, sensory=3000, seed=3):
    """The embodied loop's call pattern (src/sim/fly.js:151-192): every simulated millisecond the
    host rewrites the drive of the sensory neurons (setDrive), the brain takes two steps of
    dt 0.5 ms, and the spike counts come back for the motor readout, all through the public API
    with pinned host buffers. Reports microseconds per simulated millisecond (wall clock, every
    transfer and launch inside) and the real-time factor."""
    import torch
    from flybrain import SYNTH_PARAMS, DeviceGraph, LIFCuda
    rng = np.random.default_rng(seed)
    brain = LIFCuda(DeviceGraph(g), dict(SYNTH_PARAMS, dt=0.5), seed=seed)
    b = brain._batch
    sens = torch.from_numpy(np.sort(rng.choice(g.N, sensory, replace=False)).astype(np.int32)).pin_memory().numpy()
    rates = torch.from_numpy(rng.uniform(0, 200, (ms, sensory))).pin_memory().numpy()
    h_sc = torch.empty(g.N, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    outdeg = g.outdeg().astype(np.int64)

    def loop(n):
        for t in range(n):
            b.set_drive(0, sens, rates[t % ms])
            b.step(2)
            b.read("spikeCount", 0, out=h_sc)

    loop(50)  # warm-up
    sc0 = h_sc.astype(np.int64)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loop(ms)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ev = float(((h_sc.astype(np.int64) - sc0) * outdeg).sum())
    return dict(sim_ms=ms, brain_steps_per_ms=2, sensory_drives_per_ms=sensory,
                us_per_sim_ms=wall / ms * 1e6, realtime_factor=(ms / 1000.0) / wall, events_per_s=ev / wall,
                h2d_bytes_per_ms=sens.nbytes + rates[0].nbytes, d2h_bytes_per_ms=h_sc.nbytes,
                gpu_launches_per_ms=2,
                config=f"N={g.N:,} synthetic connectome at dt 0.5 ms; per simulated ms: drive of {sensory:,} "
                       "sensory neurons rewritten, 2 brain steps, all spike counts read back (pinned buffers)")


def run_flyvis(n_eyes=64, steps=200, seed=1):
    """The flyvis optic lobe (lif.c's fv_step) for n_eyes eyes (two per fly) sharing one
    flyvis-shaped model (N=45,669 nodes, ~1.5 M synapses, dt 20 ms), each with its own
    luminance input: eye-steps per second and synaptic operations (edges x eyes) per second,
    against the oracle port of fv_step on the host cores. Inputs are set once; each timed step is
    the whole batch's fv_step."""
    import torch
    from oracle import oracle as O
    from flybrain.flyvis import FlyVis, synth_flyvis
    m = synth_flyvis(seed=seed)
    rng = np.random.default_rng(seed)
    fv = FlyVis(m, B=n_eyes)
    for b in range(n_eyes):
        fv.setInput(rng.uniform(0, 1, 721).astype(np.float32), b)
    fv.step(10)  # warm-up
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        fv.step(steps)
        ms = fv.last_ms()
    secs = ms / 1e3
    N, E = m["N"], m["E"]
    # compulsory bytes per step: the transposed graph (source id + weight per edge) and
    # bias/kdt/pointers once, each eye's v read and written and x read
    byts = E * 8 + N * 12 + n_eyes * N * 12
    peak, kind = peaks()
    ach = byts * steps / secs / 1e9
    # the host baseline: the oracle port of fv_step, eyes spread over the host threads
    cpu_eyes, cpu_steps = min(16, n_eyes), 5
    v = np.tile(m["bias"], (cpu_eyes, 1)).astype(np.float32)
    x = np.zeros_like(v)
    t0 = time.perf_counter()
    O.fv_run(m, v, x, cpu_steps)
    cpu_s = time.perf_counter() - t0
    threads = int(O.lib("port").ob_threads())
    return dict(eyes=n_eyes, nodes=N, synapses=E, steps=steps, ms_per_step=ms / steps,
                eye_steps_per_s=n_eyes * steps / secs, synaptic_ops_per_s=E * n_eyes * steps / secs,
                sim_s_per_wall_s=steps * m["dt"] / secs,
                roofline=dict(bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak, peak_kind=kind,
                              traffic=None, note="the per-edge state gathers are served from L2 (the eyes' v is "
                                                 f"{n_eyes * N * 4 / 1e6:.1f} MB); HBM carries the compulsory bytes"),
                clocks=clk.summary(), gpu_launches=steps,
                cpu_baseline=dict(value=cpu_eyes * cpu_steps / cpu_s, unit="eye-steps/s", cores=threads, kind="port",
                                  sample=f"{cpu_eyes} eyes x {cpu_steps} steps, oracle port of fv_step"),
                config=f"{n_eyes} eyes sharing a synthetic flyvis-shaped model (N={N}, E={E}, dt 20 ms), own "
                       "luminance inputs; one launch per step, state [N][eyes] in HBM")


def run_batched(g, args, n_trials=256, seed=7, rank=0, world=1):
    """Batched ensemble: n_trials independent brains over the full graph's topology in one
    persistent launch (flybrain.ensemble). Each trial: its own seed, duration U(200, 2000) ms,
    drive set of U{500..4000} neurons at U(50, 250) Hz, and per-cell-type outgoing gains
    lognormal(0, 0.2) over 64 types compiled into its weights (writeGraph's outScale, on the
    device). Over several ranks, rank r runs trials r, r + world, ... (no exchange); the value is
    every rank's trial-seconds over the slowest rank's launch time."""
    import torch
    from flybrain.ensemble import build_ensemble, ensemble_spec
    from flybrain.shard import trials_of_rank
    from flybrain.synth import SYNTH_PARAMS
    p = dict(SYNTH_PARAMS, wSyn=0.275, inhGain=1.0, minSyn=1)
    spec = ensemble_spec(g.N, n_trials, seed=seed, dt=p["dt"])
    mine = trials_of_rank(n_trials, rank, world, "interleaved")
    batch, graphs, _ = build_ensemble(g, spec, p, mine)
    steps = spec["steps"][mine]
    batch.step(args.warmup * 10)  # warm-up
    from flybrain.autotune import tune_brains
    tune = tune_brains(batch, steps=100, key=f"bench-ensemble|B={len(mine)}|N={g.N}|E={g.E}")
    batch.reset(-1)  # back to rest
    outdeg = g.outdeg().astype(np.int64)
    torch.cuda.synchronize()
    barrier(world)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        batch.step_uneven(steps)
        ms = batch.last_ms()
    barrier(world)
    events = spikes = 0.0
    readout = []
    for b in range(len(mine)):
        sc = batch.read("spikeCount", b).astype(np.int64)
        events += float((sc * outdeg).sum())
        spikes += float(sc.sum())
        readout.append(float(sc[:1000].sum()) / (steps[b] * p["dt"] / 1000.0) / 1000.0)
    secs_local = ms / 1e3
    secs = max_over_ranks(secs_local, world)
    trial_sim_s = sum_over_ranks(float(steps.sum()) * p["dt"] / 1000.0, world)
    events_all = sum_over_ranks(events, world)
    byts = algorithmic_bytes(g.N, float(steps.sum()), spikes, events)
    peak, kind = peaks()
    ach = byts / secs_local / 1e9
    traffic = DRAM_BYTES_PER_TRIAL_STEP_BATCHED * float(steps.sum())
    res = dict(trials=n_trials, trials_this_rank=int(len(mine)), neurons=g.N, edges=g.E,
               trial_steps_total=int(steps.sum()), max_steps=int(steps.max()), trial_sim_s=trial_sim_s, wall_s=secs,
               trial_s_per_wall_s=trial_sim_s / secs, events_per_s=events_all / secs, spikes=spikes,
               mean_readout_rate_hz=float(np.mean(readout)),
               roofline=dict(bound="hbm", achieved=ach, peak=peak, unit="GB/s", frac=ach / peak,
                             peak_kind=kind, traffic=traffic, algorithmic_bytes=byts,
                             dram_gbs=traffic / secs_local / 1e9, dram_frac=traffic / secs_local / 1e9 / peak,
                             traffic_note="DRAM bytes scaled from a 32-trial ncu capture of the same kernel by "
                                          "trial-steps; achieved/frac count lif.c's algorithmic bytes, dram_gbs/"
                                          "dram_frac what DRAM actually carried"),
               clocks=clk.summary(), gpu_launches=1,
               tuning=dict(blocks_per_sm=tune["blocks_per_sm"], item_chunks=tune["item_chunks"],
                           cached=tune["cached"], candidates=len(tune.get("table", []))),
               config=f"{n_trials} trials x N=165,122, own seeds, durations U(200,2000) ms, drives "
                      "U{500..4000} neurons at U(50,250) Hz, 64 cell-type gains lognormal(0,0.2); "
                      "one persistent launch, uneven steps; state in HBM (no L2 flush needed: "
                      "the batch's state is ~60 GB)" + (f"; trials split over {world} ranks" if world > 1 else ""))
    if rank == 0:
        sample = int(os.environ.get("FB_CPU_BATCH_SAMPLE_STEPS", "200"))
        res["cpu_baseline"] = cpu_batched(g, spec, p, graphs, mine, sample)
    return res


def run_adjoint(g, idx, hz, steps=5000, seed=3, prec="f32", cpu=True):
    """The differentiable workload: surrogate-gradient LIF (fast-sigmoid slope 25/mV, beta 0.04)
    on the full graph, 500 ms at dt 0.1 ms, checkpoint every 100 steps; loss = MSE between 20 ms
    low-pass rates of 1,000 seeded readout neurons and a seeded 0-80 Hz target; gradients for
    every edge gain, every neuron's bias and 64 cell-type gains through the autograd function.
    The adjoint is bounded with the reference's adjClip (100, the value of its loom refit) since
    the steep surrogate's adjoint overflows on this graph otherwise. Arithmetic: float32
    intermediates, or prec="f64" for the reference's double). Reports forward+backward
    time against the plain (unrecorded) forward of the same window, and the library's own
    forward/backward times."""
    import torch
    from flybrain.autograd import DiffContext, LIFDiffFunction, lowpass_rates
    from flybrain.diff import DiffNet
    rng = np.random.default_rng(seed)
    data = dict(N=g.N, indptr=g.indptr, indices=g.indices, weights=g.counts.astype(np.float32), sign=g.sign)
    opts = dict(dt=0.1, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2,
                delay=1.8, wSyn=0.275, coba=False, soft=False, surrogateBeta=0.04, adjClip=100.0,
                checkpoint=100, adaptInc=0.0, depU=0.0, precision=prec, edgeGain=np.ones(g.E, np.float32),
                bias=np.zeros(g.N, np.float32), outScale=np.ones(g.N, np.float32))
    net = DiffNet(data, opts, tape_cap=1 << 26)
    for i, h in zip(idx.tolist(), hz.tolist()):
        net.setDriveOne(i, h)
    readout = np.sort(rng.choice(g.N, 1000, replace=False))
    dctx = DiffContext(net, g.cell_type, readout, steps)
    target = torch.as_tensor(rng.uniform(0, 80, (1, 1000)), dtype=torch.float32, device="cuda")
    eg = torch.ones(g.E, device="cuda", requires_grad=True)
    bias = torch.zeros(g.N, device="cuda", requires_grad=True)
    tg = torch.as_tensor(rng.lognormal(0, 0.2, 64), dtype=torch.float32, device="cuda").requires_grad_()

    def clock(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    net.forward(steps, record=False)  # warm-up (allocations, the pass's CUDA graph)
    _, plain = clock(lambda: net.forward(steps, record=False))
    net.forward(steps, record=True)  # warm-up (the recorded pass's graph)
    _, lib_fwd = clock(lambda: net.forward(steps, record=True))
    dro = np.zeros((steps, readout.shape[0]), np.float32)
    net.backward(dro, readout=readout)  # warm-up (arena allocation)
    _, lib_bwd = clock(lambda: net.backward(dro, readout=readout))
    for p_ in (eg, bias, tg):
        p_.grad = None

    def fwd():
        raster = LIFDiffFunction.apply(eg, bias, tg, dctx)
        return ((lowpass_rates(raster, 0.1) - target) ** 2).mean()

    # warm-up of the whole autograd path: the first float64 cumsum of a process loads (on some
    # builds JIT-compiles) torch's scan kernel, seconds that belong to no step
    fwd().backward()
    for p_ in (eg, bias, tg):
        p_.grad = None
    loss, fwd_s = clock(fwd)
    _, bwd_s = clock(loss.backward)
    sim_s = steps * 0.1 / 1000
    ge, gb, gt = eg.grad, bias.grad, tg.grad
    out = dict(neurons=g.N, edges=g.E, steps=steps, checkpoint=100, sim_s=sim_s, precision=prec,
                plain_forward_s=plain, library_forward_recorded_s=lib_fwd, library_backward_s=lib_bwd,
                autograd_forward_s=fwd_s, autograd_backward_s=bwd_s,
                fwd_bwd_per_trial_s=(fwd_s + bwd_s) / sim_s, plain_per_trial_s=plain / sim_s,
                cost_vs_plain_forward=(fwd_s + bwd_s) / plain, loss=float(loss.detach()),
                spikes=int(net.tape()[0][-1]),
                grads=dict(edge_nonzero=int((ge != 0).sum()), edge_finite=bool(torch.isfinite(ge).all()),
                           bias_nonzero=int((gb != 0).sum()), type_gain=[float(x) for x in gt[:4]]),
                config="surrogate-gradient LIF (beta 0.04, adjClip 100), N=165,122, 500 ms at dt 0.1 ms, "
                       "K=100; MSE of 20 ms low-pass rates of 1,000 readouts vs a 0-80 Hz target; "
                       "gradients for every edge gain, bias and 64 type gains (autograd)")
    del net, dctx
    if os.environ.get("FB_BENCH_GRAD_CHECK", "1") == "1" and cpu:
        out["grad_check"] = grad_check_full(g, idx, hz, data)
    if cpu:
        from oracle.lifdiff_oracle import DiffProblem
        cs = int(os.environ.get("FB_CPU_ADJ_SAMPLE_STEPS", "300"))
        prob = DiffProblem(g.N, g.indptr, g.indices, g.counts.astype(np.float32), g.sign, params=ADJ_OPTS,
                           driven=idx, drive_hz=hz, edgeGain=np.ones(g.E, np.float32), outScale=np.ones(g.N, np.float32))
        out["cpu_baseline"] = cpu_adjoint([prob], cs, [readout.astype(np.int32)], "the same network and readouts")
        out["cpu_baseline"]["vs_gpu_fwd_bwd"] = out["cpu_baseline"]["seconds_per_trial_s"] / out["fwd_bwd_per_trial_s"]
    return out


def grad_check_full(g, idx, hz, data, steps=500, seed=3, n=(3, 3, 2)):
    """Gradient accuracy at full scale: the adjoint leg's network in the smooth form
    scripts/grad_check.mjs checks (soft spikes, its surrogate width of 1.5 mV, no adjoint clipping:
    with the leg's steep surrogate the smooth model is silent at rest and no parameter moves the
    loss), 500 steps, the leg's loss (in float64) through the autograd function; n = (edge gains,
    biases, type gains) parameters drawn among the 4n of each kind with the largest gradients,
    against central finite differences of the forward in double (steps 4e-2, 0.4 mV and 4e-3: the
    float32 state and the tape's 1e-4 spike cut put noise of a fixed size into the loss, so smaller
    steps measure that noise rather than the slope). The float64 and the float32 adjoints are
    compared with the same differences; tests/test_grad_check_scale_gpu.py checks 32 parameters."""
    import torch
    from flybrain.autograd import DiffContext, finite_difference_check
    from flybrain.diff import DiffNet

    def context(prec):
        rng = np.random.default_rng(seed)
        net = DiffNet(data, dict(ADJ_OPTS, soft=True, surrogateBeta=1.5, adjClip=0.0, precision=prec,
                                 edgeGain=np.ones(g.E, np.float32), bias=np.zeros(g.N, np.float32),
                                 outScale=np.ones(g.N, np.float32)))
        for i, h in zip(idx.tolist(), hz.tolist()):
            net.setDriveOne(i, h)
        readout = np.sort(rng.choice(g.N, 1000, replace=False))
        target = torch.as_tensor(rng.uniform(0, 80, (1, 1000)), dtype=torch.float32, device="cuda")
        return DiffContext(net, g.cell_type, readout, steps, seed=seed), target

    d64, target = context("f64")
    d32, _ = context("f32")
    rng = np.random.default_rng(seed + 1)
    eg = torch.ones(g.E, device="cuda", requires_grad=True)
    bias = torch.zeros(g.N, device="cuda", requires_grad=True)
    tg = torch.as_tensor(rng.lognormal(0, 0.2, 64), dtype=torch.float32, device="cuda").requires_grad_()
    t0 = time.perf_counter()
    r = finite_difference_check(d64, target, eg, bias, tg, n_edge=n[0], n_bias=n[1], n_type=n[2],
                                h=dict(edge=4e-2, bias=0.4, type=4e-3), seed=5, fd_precision="f64",
                                others={"f32": d32})
    r["seconds"] = time.perf_counter() - t0
    r["config"] = (f"soft spikes (surrogate width 1.5 mV, scripts/grad_check.mjs's), no adjoint clipping, "
                   f"N={g.N:,}, {steps} steps, K=100; {r['params']} parameters against FP64 central differences "
                   "(h: edge 4e-2, bias 0.4 mV, type 4e-3); max_rel/median_rel: float64 adjoint, others.f32: "
                   "float32 adjoint")
    r["rows"] = [dict(kind=x["kind"], index=x["index"], rel=x["rel"], rel_f32=x["rel_f32"]) for x in r["rows"]]
    del d64, d32
    torch.cuda.empty_cache()
    return r


ADJ_OPTS = dict(dt=0.1, vRest=-52.0, vThresh=-45.0, vReset=-52.0, tauM=20.0, tauSyn=5.0, tRef=2.2, delay=1.8,
                wSyn=0.275, coba=False, soft=False, surrogateBeta=0.04, adjClip=100.0, checkpoint=100,
                adaptInc=0.0, depU=0.0)


def _adj_loss_grads(batch, readouts, targets, dt):
    """Rasters of every member, MSE of 20 ms low-pass rates against the member's target trace,
    and its gradient with respect to each raster (torch autograd over the filter). All members
    at once: the rasters in one library call into a [members, steps, readouts] buffer padded to
    the longest member (members of equal readout counts), one filter over all columns, each
    member's loss over its own steps."""
    import torch
    from flybrain.autograd import lowpass_rates
    B = batch.B
    R = {int(r.shape[0]) for r in readouts}
    if len(R) != 1:  # readout sets of different sizes: member by member
        dls, loss = [], 0.0
        for b in range(B):
            r = torch.zeros((batch._steps[b], readouts[b].shape[0]), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            batch.raster(b, readouts[b], out=r)
            r.requires_grad_()
            L = ((lowpass_rates(r, dt) - targets[b]) ** 2).mean()
            L.backward()
            dls.append(r.grad.detach().contiguous())
            loss += float(L.detach())
        torch.cuda.synchronize()
        return dls, loss / B
    R = R.pop()
    steps = [int(x) for x in batch._steps]
    T = max(steps)
    P = torch.zeros((B, T, R), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    batch.rasters(readouts, [P[b, : steps[b]] for b in range(B)])
    P.requires_grad_()
    rates = lowpass_rates(P.permute(1, 0, 2).reshape(T, B * R), dt).reshape(T, B, R)
    tgt = torch.stack([t.reshape(-1) for t in targets]).to(rates.dtype)  # [B, R]
    valid = (torch.arange(T, device="cuda")[:, None] < torch.as_tensor(steps, device="cuda")[None, :]).to(rates.dtype)
    per = (((rates - tgt[None]) ** 2).sum(2) * valid).sum(0) / (torch.as_tensor(steps, device="cuda").to(rates.dtype) * R)
    per.sum().backward()
    dls = [P.grad[b, : steps[b]] for b in range(B)]
    torch.cuda.synchronize()
    return dls, float(per.mean().detach())


def _tune_adjoint(batch, seeds, readouts, rng, key, steps=400):
    """The autotuner's pick of K and the per-step launch shape for `batch`, from a recorded forward
    and backward of `steps` steps per member with a random readout-loss gradient."""
    from flybrain.autotune import tune_diff
    dls = [rng.standard_normal((steps, r.shape[0])).astype(np.float32) * 1e-3 for r in readouts]
    r = tune_diff(batch, [steps] * batch.B, seeds, dls, readouts, Ks=(50, 100, 200), key=key)
    return dict(checkpoint=r["checkpoint"], neuron_blocks=r["neuron_blocks"], arrival_blocks=r["arrival_blocks"],
                cached=r["cached"], candidates=len(r.get("table", [])), tuning_s=sum(x["s"] for x in r.get("table", [])))


def run_adjoint_batched(g, idx, hz, n_trials=64, steps=5000, seed=5, prec="f32", rank=0, world=1, cpu=True):
    """Batched forward+adjoint: n_trials trials of the differentiable workload (surrogate slope
    25/mV, adjClip 100, 500 ms at dt 0.1 ms, K=100, float32 intermediates) sharing the full graph
    and its edge gains, each with its own seed and target trace, in one batch (fb_diff_batch_*);
    gradients for every edge (summed over trials in trial order), bias and type gain. Cost per
    trial-second against the plain single-trial forward. Over several ranks, rank r runs one
    contiguous block of the trials and the per-edge gradients are summed in global trial order
    across ranks (flybrain.shard.ordered_sum: the same float64 additions as one process)."""
    import torch
    from flybrain.diff import DiffBatch, DiffNet
    from flybrain.shard import ordered_sum, trials_of_rank
    rng = np.random.default_rng(seed)
    data = dict(N=g.N, indptr=g.indptr, indices=g.indices, weights=g.counts.astype(np.float32), sign=g.sign)
    eg = np.ones(g.E, np.float32)
    mine = trials_of_rank(n_trials, rank, world, "blocks")
    n_all, n_trials = n_trials, int(len(mine))
    members = []
    for _ in range(n_trials):
        n = DiffNet(data, dict(ADJ_OPTS, edgeGain=eg), _defer=True)
        for i, h in zip(idx.tolist(), hz.tolist()):
            n.setDriveOne(i, h)
        members.append(n)
    params = dict(ADJ_OPTS, precision=prec)
    t0 = time.perf_counter()
    batch = DiffBatch(members, params)
    create_s = time.perf_counter() - t0
    readout = np.sort(rng.choice(g.N, 1000, replace=False)).astype(np.int32)
    readouts = [readout] * n_trials
    all_targets = [rng.uniform(0, 80, (1, 1000)) for _ in range(n_all)]
    targets = [torch.as_tensor(all_targets[b], dtype=torch.float32, device="cuda") for b in mine.tolist()]
    seeds = [int(b) + 1 for b in mine.tolist()]

    def clock(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    batch.forward(200, seeds, counts=False)  # warm-up
    tune = _tune_adjoint(batch, seeds, readouts, rng, f"bench-adjoint|B={n_trials}|N={g.N}|E={g.E}")
    # each pass runs once untimed first: its first run captures the pass as a CUDA graph (timed
    # apart, `first_calls`), the timed run replays it
    _, plain0 = clock(lambda: batch.forward(steps, seeds, record=False, counts=False))
    _, plain_s = clock(lambda: batch.forward(steps, seeds, record=False, counts=False))
    _, fwd0 = clock(lambda: batch.forward(steps, seeds, record=True, counts=False))
    _, fwd_s = clock(lambda: batch.forward(steps, seeds, record=True, counts=False))
    _adj_loss_grads(batch, readouts, targets, 0.1)  # warm-up of the filter at these shapes
    (dls, loss), loss_s = clock(lambda: _adj_loss_grads(batch, readouts, targets, 0.1))
    _, bwd0 = clock(lambda: batch.backward(dls, readouts, device="cuda", edge=False))
    first = dict(plain_forward_s=plain0, forward_recorded_s=fwd0, backward_s=bwd0,
                 note="first run of each pass at these shapes, capturing it as a CUDA graph")
    gs, bwd_s = clock(lambda: batch.backward(dls, readouts, device="cuda"))
    ge = torch.zeros(g.E, dtype=torch.float64, device="cuda")
    if world == 1:
        _, sum_s = clock(lambda: batch.edge_sum(out=ge))
    else:  # this rank's trials in order, continued across ranks in global trial order
        def cross():
            per = []
            for b in range(n_trials):
                x = torch.zeros(g.E, dtype=torch.float64, device="cuda")
                batch.edge_sum(insts=[b], out=x)
                per.append(x)
            return ordered_sum(per, n_all, rank, world, (g.E,), device="cuda")
        ge, sum_s = clock(cross)
    trial_s = n_trials * steps * 0.1 / 1000
    total = fwd_s + loss_s + bwd_s + sum_s
    trial_s = sum_over_ranks(trial_s, world)
    total = max_over_ranks(total, world)
    spikes = sum(int(batch.tape(b)[0][-1]) for b in range(min(n_trials, 4)))
    out = dict(trials=n_all, trials_this_rank=n_trials, neurons=g.N, edges=g.E, steps=steps, checkpoint=batch.p["checkpoint"],
                precision=prec, tuning=tune, first_calls=first,
                create_s=create_s, plain_batch_forward_s=plain_s, forward_recorded_s=fwd_s, loss_s=loss_s,
                backward_s=bwd_s, edge_sum_s=sum_s, trial_s=trial_s,
                fwd_bwd_per_trial_s=total / trial_s, plain_batch_forward_per_trial_s=plain_s / trial_s,
                trial_s_of_gradient_per_wall_s=trial_s / total, loss=loss, spikes_first4=spikes,
                grads=dict(edge_nonzero=int((ge != 0).sum()), edge_finite=bool(torch.isfinite(ge).all()),
                           bias_nonzero=int(sum(int((x["bias"] != 0).sum()) for x in gs))),
                config=f"{n_all} trials sharing the N=165,122 graph and its edge gains, own seeds and "
                       "target traces; surrogate slope 25/mV, adjClip 100, 500 ms at dt 0.1 ms, K and "
                       "launch shape autotuned" + (f"; contiguous trial blocks over {world} ranks, per-edge "
                                                  "gradients summed in trial order" if world > 1 else ""))
    del batch, members, gs, dls
    torch.cuda.empty_cache()
    if cpu and rank == 0:
        from oracle import oracle as O
        from oracle.lifdiff_oracle import DiffProblem
        O.build(ref=False)
        nt = max(1, min(int(O.lib("port").ob_threads()), n_trials))
        cs = int(os.environ.get("FB_CPU_ADJ_BATCH_SAMPLE_STEPS", "200"))
        probs = [DiffProblem(g.N, g.indptr, g.indices, data["weights"], g.sign, params=ADJ_OPTS, driven=idx,
                             drive_hz=hz, edgeGain=eg, outScale=np.ones(g.N, np.float32)) for _ in range(nt)]
        out["cpu_baseline"] = cpu_adjoint(probs, cs, [readout] * nt, f"{nt} of the trials")
    return out


def run_adjoint_uneven(n_inst=128, seed=11, prec="f32", cpu=True):
    """Batched uneven adjoint: n_inst instances over separately seeded synthetic subgraphs of
    5,000-60,000 neurons, each 100-400 ms (dt 0.1 ms) with its own drive (1% of neurons at
    150 Hz) and target trace; forward+backward of the whole batch against its plain forward."""
    import torch
    from flybrain.diff import DiffBatch, DiffNet
    from flybrain.synth import synth_graph
    rng = np.random.default_rng(seed)
    import concurrent.futures as cf
    import multiprocessing as mp
    members, readouts, targets, steps = [], [], [], []
    t0 = time.perf_counter()
    sizes = [int(rng.integers(5000, 60001)) for _ in range(n_inst)]
    # the graphs are generated on the host cores by spawned workers (this process holds a CUDA
    # context, so it is not forked)
    with cf.ProcessPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)),
                                mp_context=mp.get_context("spawn")) as ex:
        graphs = list(ex.map(synth_graph, sizes, [1000 + k for k in range(n_inst)]))
    for k in range(n_inst):
        N, sg = sizes[k], graphs[k]
        n = DiffNet(dict(N=N, indptr=sg.indptr, indices=sg.indices, weights=sg.counts.astype(np.float32),
                         sign=sg.sign), dict(ADJ_OPTS), _defer=True)
        for i in rng.choice(N, max(1, N // 100), replace=False):
            n.setDriveOne(int(i), 150.0)
        members.append(n)
        steps.append(int(rng.integers(1000, 4001)))
        ro = np.sort(rng.choice(N, min(200, N), replace=False)).astype(np.int32)
        readouts.append(ro)
        targets.append(torch.as_tensor(rng.uniform(0, 80, (1, ro.shape[0])), dtype=torch.float32, device="cuda"))
    gen_s = time.perf_counter() - t0
    batch = DiffBatch(members, dict(ADJ_OPTS, precision=prec))
    seeds = list(range(1, n_inst + 1))

    def clock(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    batch.forward([200] * n_inst, seeds, counts=False)  # warm-up
    tune = _tune_adjoint(batch, seeds, readouts, rng, f"bench-uneven|B={n_inst}|N={sum(batch.N)}")
    # each pass runs once untimed first: its first run captures the pass as a CUDA graph (timed
    # apart, `first_calls`), the timed run replays it
    _, plain0 = clock(lambda: batch.forward(steps, seeds, record=False, counts=False))
    _, plain_s = clock(lambda: batch.forward(steps, seeds, record=False, counts=False))
    _, fwd0 = clock(lambda: batch.forward(steps, seeds, record=True, counts=False))
    _, fwd_s = clock(lambda: batch.forward(steps, seeds, record=True, counts=False))
    _adj_loss_grads(batch, readouts, targets, 0.1)  # warm-up of the filter at these shapes
    (dls, loss), loss_s = clock(lambda: _adj_loss_grads(batch, readouts, targets, 0.1))
    _, bwd0 = clock(lambda: batch.backward(dls, readouts, device="cuda", edge=False))
    first = dict(plain_forward_s=plain0, forward_recorded_s=fwd0, backward_s=bwd0,
                 note="first run of each pass at these shapes, capturing it as a CUDA graph")
    _, bwd_s = clock(lambda: batch.backward(dls, readouts, device="cuda"))
    trial_s = sum(steps) * 0.1 / 1000
    total = fwd_s + loss_s + bwd_s
    out = dict(instances=n_inst, neurons_total=int(sum(batch.N)), edges_total=int(sum(batch.E)),
                steps_min=min(steps), steps_max=max(steps), precision=prec, graph_gen_s=gen_s,
                checkpoint=batch.p["checkpoint"], tuning=tune, first_calls=first,
                plain_forward_s=plain_s, forward_recorded_s=fwd_s, loss_s=loss_s, backward_s=bwd_s,
                trial_s=trial_s, trial_s_of_gradient_per_wall_s=trial_s / total,
                trial_s_of_plain_forward_per_wall_s=trial_s / plain_s, cost_vs_plain_forward=total / plain_s,
                loss=loss,
                config=f"{n_inst} instances over synthetic subgraphs of 5,000-60,000 neurons, 100-400 ms at "
                       "dt 0.1 ms, own drive/seed/target; surrogate slope 25/mV, adjClip 100, K and launch "
                       "shape autotuned")
    if cpu:
        from oracle import oracle as O
        from oracle.lifdiff_oracle import DiffProblem
        O.build(ref=False)
        nt = max(1, min(int(O.lib("port").ob_threads()), n_inst))
        cs = int(os.environ.get("FB_CPU_ADJ_BATCH_SAMPLE_STEPS", "200"))
        probs = []
        for k in range(nt):
            m = members[k]
            hz = m.drive[list(m.drivenSet)]
            probs.append(DiffProblem(m.N, m.indptr, m.indices, m.counts, m.sign, params=ADJ_OPTS,
                                     driven=np.asarray(list(m.drivenSet), np.int32), drive_hz=hz))
        out["cpu_baseline"] = cpu_adjoint(probs, cs, readouts[:nt], f"the first {nt} instances")
    return out


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path: lif_step as the reference build (when the
    reference compiled here) or its oracle port, on this machine's host cores."""
    if rank != 0:
        return
    from flybrain import SYNTH_PARAMS, workload
    from oracle import oracle as O
    backend = "ref" if os.path.exists(O.REF_LIB) else "port"
    O.build(ref=False)
    g, idx, hz, _ = workload("full", seed=1)
    outdeg = g.outdeg().astype(np.int64)
    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, SYNTH_PARAMS, seed=1, backend=backend)
    for i, h in zip(idx.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
    S = int(os.environ.get("FB_REF_SAMPLE_STEPS", str(BRAIN_STEPS_PER_BENCH_STEP)))  # the window of our arm
    for _ in range(args.warmup):
        ob.run(S)
    ob.reset()
    sc_prev = ob.spikeCount.astype(np.int64)
    ev = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ob.run(S)
        sc = ob.spikeCount.astype(np.int64)
        ev += float(((sc - sc_prev) * outdeg).sum())
        sc_prev = sc
    secs = time.perf_counter() - t0
    sim_s = args.steps * S * SYNTH_PARAMS["dt"] / 1000.0
    v = ev / secs
    sample = f"{args.steps} x {S} brain steps of the full-scale workload (lif_step is serial: 1 thread)"
    print(json.dumps(dict(
        impl="reference", metric=METRIC, value=v, unit="synaptic events/s", n_gpus=world,
        steps=args.steps, warmup=args.warmup, ms_per_step=1e3 * secs / args.steps,
        higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
        data="synthetic (seeded connectome-shaped graph; no dataset)",
        config=dict(workload="plain forward, full scale: N=165,122 synthetic connectome, 2,000 drive "
                    "neurons at U(100,200) Hz, dt 0.1 ms", brain_steps_per_step=S),
        sim_s_per_wall_s=sim_s / secs,
        cpu_baseline=dict(value=v, unit="synaptic events/s", cores=1,
                          kind="reference" if backend == "ref" else "port", sample=sample),
        e2e=dict(value=v, unit="synaptic events/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0),
    )), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    rank, world = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
