"""The adjoint test problem of scripts/grad_check.mjs, rebuilt: the 600-neuron induced subgraph of
the real connectome (tests/golden/adjoint/real_subgraph_counts.npz), soft spikes, and every
per-neuron structure the gradients are taken through (sizeLog, thrMask, biasMask, logGain,
outScale, thrOffset), seeded with numpy instead of grad_check's LCG."""
import os

import numpy as np

from conftest import GOLDEN

EXC_SIGN = np.array([0, 1, -1, -1, 1, 1, 1, -1], np.float32)  # src/lif.js:5
# scripts/grad_check.mjs:65-67
P0 = dict(soft=True, tRef=0.0, minSyn=3.0, coba=True, wSyn=0.5, sizeAlpha=0.6, inhGain=0.8,
          eInh=-76.0, vThresh=-45.0, kcThreshold=2.0, laminaBias=14.0, adaptInc=0.4, depU=0.15,
          surrogateBeta=1.5)
# scripts/grad_check.mjs:92-93
H = dict(wSyn=2e-3, sizeAlpha=2e-3, inhGain=2e-3, eInh=2e-1, vThresh=1e-2, kcThreshold=1e-2,
         laminaBias=1e-2, adaptInc=2e-3, depU=2e-3)


def grad_check_inputs(seed=12345):
    z = np.load(os.path.join(GOLDEN, "adjoint", "real_subgraph_counts.npz"))
    n = int(z["N"])
    rng = np.random.default_rng(seed)
    ins = dict(N=n, indptr=z["indptr"], indices=z["indices"], counts=z["counts"].astype(np.float32),
               sign=EXC_SIGN[z["nt"]],
               sizeLog=rng.uniform(-1, 1, n).astype(np.float32),
               thrMask=(rng.random(n) < 0.2).astype(np.uint8),
               biasMask=(np.arange(n) < n / 4).astype(np.uint8),
               logGain=((rng.random(n) - 0.5) * 0.2).astype(np.float32),
               outScale=(0.5 + rng.random(n)).astype(np.float32),
               thrOffset=((rng.random(n) - 0.5) * 4).astype(np.float32))
    target = np.nonzero(rng.random(n) < 0.3)[0]
    return ins, target


def within_tolerance(a, fd, h, L):
    """scripts/grad_check.mjs:98: |a - fd| <= 1e-3 |fd| + 4e-6 |L| / h."""
    tol = 1e-3 * abs(fd) + 4e-6 * abs(L) / h
    return abs(a - fd) <= tol, abs(a - fd) / max(1e-12, abs(fd))
