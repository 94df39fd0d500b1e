"""The C ABI: libflybrain.so builds for sm_103a, loads, and exports every entry point that
include/flybrain.h declares (no compute without a GPU)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "flybrain.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fb_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from flybrain import _native
    return _native.load()


def test_library_exports_every_declared_symbol(lib):
    from flybrain import _native
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (fb_\w+)", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, missing
    assert set(declared()) <= set(_native.SIGNATURES), "ctypes signatures missing"


def test_library_is_sm103a_only(lib):
    from flybrain import _native
    out = subprocess.run(["cuobjdump", "--list-elf", _native.lib_path()], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout
    assert all("sm_103" in line for line in out.stdout.splitlines() if ".cubin" in line)


def test_errors_without_gpu_are_reported(lib):
    """With no device (this container) a create call fails with a status, never a crash."""
    import ctypes as C
    import numpy as np
    from flybrain import _native
    ip = np.zeros(2, dtype=np.uint32)
    h = C.c_void_p()
    rc = lib.fb_graph_create(1, 0, _native.ptr(ip), None, None, _native.ptr(np.zeros(1, np.float32)), C.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert rc == 0
        lib.fb_graph_destroy(h)
    else:
        assert rc != 0 and lib.fb_last_error()
    assert lib.fb_version() >= 100
    # argument validation happens before any device work
    assert lib.fb_graph_create(0, 0, None, None, None, None, C.byref(h)) == _native.FB_EINVAL
