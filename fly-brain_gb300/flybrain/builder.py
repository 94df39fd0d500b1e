"""Builds libflybrain.so (the C ABI of include/flybrain.h) for sm_103a with nvcc, in-tree.

Translation units compile in parallel; the result lands in flybrain/_lib/. No CMake, no torch
extension machinery: the library exports plain C symbols and links the CUDA runtime statically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libflybrain.so")
CHECK_LIB = os.path.join(OUT_DIR, "libflybrain_check.so")
SOURCES = ["fb_step.cu", "fb_api.cu", "fb_graph.cu", "fb_noalloc.cu", "fb_adjoint.cu", "fb_lagged.cu", "fb_flyvis.cu", "fb_codec.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--fmad=false"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflybrain.so")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    """checked=True builds libflybrain_check.so: every data-dependent index in the step kernel is
    bounds-checked (a failure is recorded and reported by fb_step, the access skipped)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj_check" if checked else "obj")
    lib = CHECK_LIB if checked else LIB
    flags = FLAGS + (["-DFB_CHECK"] if checked else [])
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "flybrain.h"))
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(obj_dir, s.replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            jobs.append([cc, *ARCH, *flags, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(obj_dir, s.replace(".cu", ".o")) for s in srcs]
    if force or jobs or _stale(lib, objs):
        run([cc, "-shared", *ARCH, "-o", lib, *objs, "-lcudart_static"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, checked="--checked" in sys.argv))
