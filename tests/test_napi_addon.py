"""The Node-API addon (fly-brain_gb300/napi/flybrain_napi.c, the LIFWasm object of
src/lifwasm.js:36-87 over the C ABI). Node is not installed, so the addon is compiled with gcc
against tests/napi/node_api.h (the Node-API declarations it uses) and driven through
tests/napi/napi_runtime.c, a minimal runtime with Node's argument semantics:

- host: a scripted session against a stand-in C ABI (tests/napi/fake_flybrain.c) that prints every
  call -- what each method passes down, what each getter returns, every error path;
- GPU: a brain on the real libflybrain driven through the addon (drive, bias, background, pulse,
  addG, setThr, step, run, reset, state getters) against the oracle doing the same, bit for bit."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAPI = os.path.join(ROOT, "tests", "napi")
ADDON = os.path.join(ROOT, "fly-brain_gb300", "napi", "flybrain_napi.c")
PARAM_NAMES = ("dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "traceTau", "adaptInc",
               "adaptTau", "depU", "depTau", "eExc", "eInh", "bgRate", "bgAmp", "preInh")


def _compile(out, extra_sources=(), extra_args=()):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror", "-DFLYBRAIN_NAPI_NO_MODULE", "-I", NAPI, "-I",
           os.path.join(ROOT, "include"), ADDON, os.path.join(NAPI, "napi_runtime.c"), os.path.join(NAPI, "driver.c"),
           *extra_sources, "-o", out, *extra_args, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


EXPECTED_MARSHAL = """\
new LIFNative() -> throws: new LIFNative({N, indptr, indices, weights, sign, params, seed})
new LIFNative({}) -> throws: LIFNative: N > 0 expected
new LIFNative({N, indptr: Float32Array}) -> throws: LIFNative: indptr must be a Uint32Array of N + 1
new LIFNative({..., seed: 1.5}) -> throws: LIFNative: seed must be an integer in [0, 2^32)
graph_create N=4 E=4 indptr_last=4 indices0=1 w0=0.5 sign0=1
brains_create B=1 stride=0 dt=0.1 vThresh=-40 tauM=10 bgRate=3 coba=1 seed=7
new LIFNative({...}) -> object
N -> 4
nAwake -> 4
step n=1
fired b=0 cap=4
step() -> Int32Array[3] 7 3 5
set_drive b=0 n=1 2:150
setDriveOne(2, 150) -> undefined
set_drive b=0 n=2 1:80 3:80
setDrive(Int32Array [1, 3], 80) -> undefined
set_drive b=0 n=2 0:0 2:0
setDrive([0, 2], 0) -> undefined
set_bias b=0 n=1 3:-1.5
setBias(3, -1.5) -> undefined
set_thr b=0 n=1 1:2
setThr(1, 2) -> undefined
add_g b=0 n=1 0:0.25:0
addG(0, 0.25) -> undefined
add_g b=0 n=1 1:0.5:0.75
addG(1, 0.5, 0.75) -> undefined
pulse b=0 n=1 2:1
pulse(Uint32Array [2], 1) -> undefined
set_background b=0 20 1.5
setBackground(20, 1.5) -> undefined
step n=10
run(10) -> 3
t -> 1.1
read field=0 b=0
v -> Float32Array[4] 0 0.5 1 1.5
read field=10 b=0
spikeCount -> Uint32Array[4] 1000 1001 1002 1003
set_params b=0 dt=0.1 vThresh=-40 tauM=12 bgRate=20 bgAmp=1.5 coba=0
setParams({tauM: 12, coba: false}) -> undefined
set_params b=0 dt=0.5 vThresh=-40 tauM=12 bgRate=20 bgAmp=1.5 coba=0
setParams({dt: 0.5, ...}) -> throws: fb_set_params: the ring depth would change
setParams(3) -> throws: LIFNative.setParams(q): an object of numbers
wake() -> undefined
flush() -> undefined
reset b=0
reset() -> undefined
t -> 0
set_drive b=0 n=1 9:10
setDrive(Int32Array [9], 10) -> throws: set_drive: neuron 9 out of range
setDriveOne(true, 10) -> throws: LIFNative.setDriveOne(i, rate): numbers expected
setBias(Float32Array [1], 1) -> throws: LIFNative.setBias(ix, mv): an index list and a number
run() -> throws: LIFNative.run(n): a step count >= 0
brains_destroy
graph_destroy
destroy() -> undefined
dispose() -> undefined
step() -> throws: LIFNative.step: not a live brain
v -> throws: LIFNative: not a live brain
collected
"""


def test_addon_marshalling_against_a_stand_in_library(tmp_path):
    """Every method and getter passes its arguments down as the C ABI expects (index lists as
    typed arrays, arrays of numbers or one number, one value broadcast over the list, addG's
    missing increment as 0, params by name over the defaults, the seed as given), returns
    LIFWasm's results (the fired list as an Int32Array, state as Float32Array / Uint32Array, t in
    ms), merges setParams over the parameters in force (LIFGpu's Object.assign) and keeps them when
    the library refuses, turns a failing call into a thrown Error with the library's message, and
    frees the brain once (destroy, dispose, then collection)."""
    exe = str(tmp_path / "driver")
    _compile(exe, [os.path.join(NAPI, "fake_flybrain.c")])
    r = subprocess.run([exe, "marshal"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout == EXPECTED_MARSHAL


def _write_input(path, g, p, seed, drive, bias, bg, steps, pulse, addg, thr):
    with open(path, "wb") as f:
        f.write(struct.pack("<iqi", g.N, int(g.indices.shape[0]), seed))
        f.write(np.array([float(p[k]) for k in PARAM_NAMES] + [1.0 if p.get("coba") else 0.0], "<f8").tobytes())
        f.write(np.asarray(g.indptr, "<u4").tobytes())
        f.write(np.asarray(g.indices, "<u4").tobytes())
        f.write(np.asarray(g.weights, "<f4").tobytes())
        f.write(np.asarray(g.sign, "<f4").tobytes())
        f.write(struct.pack("<i", len(drive[0])))
        f.write(np.asarray(drive[0], "<i4").tobytes())
        f.write(np.asarray(drive[1], "<f8").tobytes())
        f.write(struct.pack("<i", len(bias[0])))
        f.write(np.asarray(bias[0], "<i4").tobytes())
        f.write(struct.pack("<ddd", bias[1], bg[0], bg[1]))
        f.write(struct.pack("<iiii", *steps))
        f.write(struct.pack("<i", len(pulse[0])))
        f.write(np.asarray(pulse[0], "<i4").tobytes())
        f.write(struct.pack("<d", pulse[1]))
        f.write(struct.pack("<id", addg[0], addg[1]))
        f.write(struct.pack("<id", thr[0], thr[1]))


class _Reader:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        self.o = 0

    def take(self, fmt, n=1):
        dt = np.dtype(fmt)
        x = np.frombuffer(self.b, dt, n, self.o)
        self.o += dt.itemsize * n
        return x

    def fired(self):
        n = int(self.take("<i4")[0])
        return self.take("<i4", n).copy()


@pytest.mark.gpu
def test_addon_on_the_gpu_matches_the_oracle(tmp_path):
    """A 3,000-neuron conductance-based brain with depression and adaptation, built and driven
    through the addon on libflybrain: every fired list
    (steps, after a pulse / addG / setThr, after a 300-step run, after reset), the run's fired
    count, t, v and spikeCount equal the oracle's under the same calls."""
    from flybrain import DEFAULTS, SYNTH_PARAMS, builder, synth_graph
    from oracle import oracle as O
    exe = str(tmp_path / "driver")
    lib = os.path.dirname(builder.LIB)
    _compile(exe, extra_args=["-L", lib, "-lflybrain", f"-Wl,-rpath,{lib}"])
    g = synth_graph(3000, 5)
    p = dict(DEFAULTS, **dict(SYNTH_PARAMS, coba=True, depU=0.1, adaptInc=0.2))
    rng = np.random.default_rng(5)
    drv = rng.choice(g.N, 60, replace=False)
    hz = rng.uniform(100, 250, 60)
    bias_ix = rng.choice(g.N, 50, replace=False)
    pulse_ix = rng.choice(g.N, 40, replace=False)
    steps = (200, 100, 300, 50)
    args = dict(drive=(drv, hz), bias=(bias_ix, 1.5), bg=(20.0, 1.0), steps=steps, pulse=(pulse_ix, 6.0),
                addg=(int(pulse_ix[0]), 3.0), thr=(int(drv[1]), 2.5))
    _write_input(str(tmp_path / "in.bin"), g, p, 3, **args)
    r = subprocess.run([exe, "run", str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = _Reader(str(tmp_path / "out.bin"))

    ob = O.OracleBrain(g.N, g.indptr, g.indices, g.weights, g.sign, p, seed=3)
    for i, h in zip(drv.tolist(), hz.tolist()):
        ob.setDriveOne(i, h)
    ob.setBias(bias_ix, 1.5)
    ob.setBackground(20.0, 1.0)
    total = 0
    for _ in range(steps[0]):
        f = ob.step()
        np.testing.assert_array_equal(out.fired(), f)
        total += f.shape[0]
    ob.pulse(pulse_ix, 6.0)
    ob.addG(int(pulse_ix[0]), 3.0)
    ob.setThr(int(drv[1]), 2.5)
    for _ in range(steps[1]):
        np.testing.assert_array_equal(out.fired(), ob.step())
    nf = ob.run(steps[2])
    assert out.take("<f8")[0] == nf[-1]
    np.testing.assert_array_equal(out.fired(), ob.step())
    assert out.take("<f8")[0] == pytest.approx(ob.t)
    assert out.take("<f4", g.N).tobytes() == ob.v.tobytes()
    assert out.take("<u4", g.N).tobytes() == ob.spikeCount.astype("<u4").tobytes()
    ob.reset()
    for _ in range(steps[3]):
        np.testing.assert_array_equal(out.fired(), ob.step())
    assert out.o == len(out.b)
    assert total > 100 and int(ob.spikeCount.sum()) > 0
