"""ctypes binding of libflybrain.so (include/flybrain.h).

The library is the only compute path: if it is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import builder as _build

FB_OK = 0
FB_EINVAL, FB_ECUDA, FB_ENOMEM, FB_ETIMEOUT, FB_EOVERFLOW, FB_ESTATE, FB_ENODEV = -1, -2, -3, -4, -5, -6, -7
FB_DELIVER_EXACT, FB_DELIVER_SEQUENTIAL, FB_DELIVER_FAST = 0, 1, 2
FB_SCHEDULE_AUTO, FB_SCHEDULE_GRID, FB_SCHEDULE_LAGGED = 0, 1, 2
FIELDS = {"v": 0, "gE": 1, "gI": 2, "refr": 3, "trace": 4, "adapt": 5, "res": 6, "bias": 7,
          "thr": 8, "drive": 9, "spikeCount": 10}

# Every symbol the header declares, with its ctypes signature (restype, argtypes).
P, I32, I64, U32, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_double
PI32, PI64, PU32, PF = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_uint32), C.POINTER(C.c_float)


class FbParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "traceTau",
        "adaptInc", "adaptTau", "depU", "depTau", "eExc", "eInh", "bgRate", "bgAmp", "preInh")] + [
        ("coba", C.c_int32), ("reserved", C.c_int32)]


class FbCompileParams(C.Structure):
    _fields_ = [("wSyn", C.c_double), ("inhGain", C.c_double), ("minSyn", C.c_double), ("preInh", C.c_double)]


class FbBrainView(C.Structure):
    """fb_brain_view: the reference Brain header with device-pointer arrays."""
    _fields_ = ([("N", C.c_int32), ("nslots", C.c_int32), ("head", C.c_int32), ("coba", C.c_int32)]
                + [(k, C.c_float) for k in ("dt", "vRest", "vThresh", "vReset", "tRef", "adaptInc", "depU",
                                            "dE", "dTr", "dA", "kRec", "kM", "dtS", "eExc", "eInh", "cE", "cI")]
                + [("rng", C.c_uint32)]
                + [(k, C.c_void_p) for k in ("v", "gE", "gI", "refr", "trace", "adapt", "res", "bias",
                                             "thr", "drive", "sign", "spikeCount", "indptr", "indices",
                                             "weights", "ring", "ringCount", "driven")]
                + [("nDriven", C.c_int32), ("nFired", C.c_int32), ("lastSlot", C.c_int32)]
                + [(k, C.c_float) for k in ("bgEvents", "bgAmp", "bgAcc", "preInh")]
                + [("E", C.c_int64)])


class FbFlygHeader(C.Structure):
    _fields_ = [(k, C.c_uint32) for k in ("N", "E", "min_weight", "pad")]


class FbDiffParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "dt", "vRest", "vThresh", "vReset", "tauM", "tauSyn", "tRef", "delay", "wSyn", "adaptInc",
        "adaptTau", "depU", "depTau", "minSyn", "eExc", "eInh", "inhGain", "sizeAlpha",
        "maxSizeScale", "boostCap", "kcThreshold", "laminaBias", "surrogateBeta", "adjClip")] + [
        (k, C.c_int32) for k in ("coba", "soft", "checkpoint", "precision", "drive_soft", "exact32",
                                 "drive_epoch", "pad")]


class FbDiffNet(C.Structure):
    _fields_ = [("N", C.c_int32), ("nDriven", C.c_int32), ("E", C.c_int64)] + [
        (k, C.c_void_p) for k in ("indptr", "indices", "counts", "edge_gain", "sign", "size_log",
                                  "in_scale", "log_gain", "out_scale", "thr_offset", "beta", "bias",
                                  "thr_mask", "bias_mask", "sensory", "drive", "driven")] + [
        ("nDriveIdx", C.c_int32), ("pad", C.c_int32), ("drive_idx", C.c_void_p)]


class FbDiffGrads(C.Structure):
    _fields_ = [("params", C.c_double * 9), ("clamped_params", C.c_int32),
                ("clamped_log_gain", C.c_int32), ("log_gain", C.c_void_p), ("edge", C.c_void_p),
                ("bias", C.c_void_p), ("out_scale", C.c_void_p), ("drive", C.c_void_p),
                ("clamped_drive", C.c_int32), ("pad", C.c_int32)]


class FbTuning(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("blocks_per_sm", "item_chunks", "max_blocks_per_sm", "sms", "sub_grab", "timeout_us",
                                               "lag_driven_blocks", "pad")]


class FbDiffTuning(C.Structure):
    _fields_ = [("neuron_blocks", C.c_int32), ("arrival_blocks", C.c_int32), ("step_launches", C.c_int32)]


class FbDiffInputs(C.Structure):
    _fields_ = [("drive_at", C.c_void_p), ("train_off", C.c_void_p), ("train_idx", C.c_void_p)]


SIGNATURES = {
    "fb_version": (C.c_int, []),
    "fb_last_error": (C.c_char_p, []),
    "fb_device_info": (C.c_int, [PI32, PI32, PI32]),
    "fb_default_params": (None, [C.POINTER(FbParams)]),
    "fb_graph_create": (C.c_int, [I32, I64, P, P, P, P, C.POINTER(P)]),
    "fb_graph_create_shared": (C.c_int, [P, P, P, C.POINTER(P)]),
    "fb_graph_set_sign": (C.c_int, [P, P]),
    "fb_graph_compile": (C.c_int, [P, P, P, P, P, P, P, C.POINTER(FbCompileParams), C.POINTER(P)]),
    "fb_graph_read": (C.c_int, [P, P, P]),
    "fb_graph_info": (C.c_int, [P, PI32, PI64]),
    "fb_graph_destroy": (C.c_int, [P]),
    "fb_brains_create": (C.c_int, [P, I32, C.POINTER(FbParams), I32, P, C.POINTER(P)]),
    "fb_brains_destroy": (C.c_int, [P]),
    "fb_brains_set_mode": (C.c_int, [P, I32]),
    "fb_step": (C.c_int, [P, I32, P]),
    "fb_step_uneven": (C.c_int, [P, P, P]),
    "fb_record": (C.c_int, [P, I32, I64]),
    "fb_spike_log": (C.c_int, [P, I32, P, I32, P, I64, PI64, PI64]),
    "fb_fired": (C.c_int, [P, I32, P, I32, PI32]),
    "fb_ring_read": (C.c_int, [P, I32, P, P, P]),
    "fb_set_drive": (C.c_int, [P, I32, P, P, I32]),
    "fb_set_bias": (C.c_int, [P, I32, P, P, I32]),
    "fb_set_thr": (C.c_int, [P, I32, P, P, I32]),
    "fb_add_g": (C.c_int, [P, I32, P, P, P, I32]),
    "fb_pulse": (C.c_int, [P, I32, P, P, I32]),
    "fb_reset": (C.c_int, [P, I32]),
    "fb_set_background": (C.c_int, [P, I32, D, D]),
    "fb_set_params": (C.c_int, [P, I32, C.POINTER(FbParams)]),
    "fb_read": (C.c_int, [P, I32, I32, P]),
    "fb_write": (C.c_int, [P, I32, I32, P]),
    "fb_scalars": (C.c_int, [P, I32, PI32, PU32, PI32, PI32, PI32, PI64]),
    "fb_last_step_ms": (C.c_int, [P, PF]),
    "fb_profile": (C.c_int, [P, I32]),
    "fb_phase_times": (C.c_int, [P, C.POINTER(C.c_double), I32]),
    "fb_lif_step_noalloc": (C.c_int, [C.POINTER(FbBrainView), I32, P]),
    "fb_diff_default_params": (None, [C.POINTER(FbDiffParams)]),
    "fb_diff_create": (C.c_int, [C.POINTER(FbDiffNet), I64, C.POINTER(P)]),
    "fb_diff_destroy": (C.c_int, [P]),
    "fb_diff_set": (C.c_int, [P, I32, P]),
    "fb_diff_forward": (C.c_int, [P, C.POINTER(FbDiffParams), I32, U32, I32, P]),
    "fb_diff_forward_ex": (C.c_int, [P, C.POINTER(FbDiffParams), I32, U32, I32, P, C.POINTER(FbDiffInputs)]),
    "fb_diff_tape": (C.c_int, [P, P, P, P, I64, PI64]),
    "fb_diff_raster": (C.c_int, [P, I32, P, P]),
    "fb_diff_backward": (C.c_int, [P, P, I32, P, I32, I32, C.POINTER(FbDiffGrads)]),
    "fb_brains_set_schedule": (C.c_int, [P, I32]),
    "fb_last_schedule": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "fb_brains_set_tuning": (C.c_int, [P, C.POINTER(FbTuning)]),
    "fb_brains_tuning": (C.c_int, [P, C.POINTER(FbTuning)]),
    "fb_debug_trip_wait": (C.c_int, [P, I32]),
    "fb_diff_batch_set_tuning": (C.c_int, [P, C.POINTER(FbDiffTuning)]),
    "fb_diff_batch_create": (C.c_int, [C.POINTER(FbDiffNet), I32, I64, C.POINTER(P)]),
    "fb_diff_batch_destroy": (C.c_int, [P]),
    "fb_diff_batch_set": (C.c_int, [P, I32, I32, P]),
    "fb_diff_batch_forward": (C.c_int, [P, C.POINTER(FbDiffParams), P, P, I32, P]),
    "fb_diff_batch_forward_ex": (C.c_int, [P, C.POINTER(FbDiffParams), P, P, I32, P, P]),
    "fb_diff_batch_tape": (C.c_int, [P, I32, P, P, P, I64, PI64]),
    "fb_diff_batch_raster": (C.c_int, [P, I32, I32, P, P]),
    "fb_diff_batch_rasters": (C.c_int, [P, P, P, P]),
    "fb_diff_batch_backward": (C.c_int, [P, P, P, P, I32, I32, C.POINTER(FbDiffGrads)]),
    "fb_diff_batch_edge_sum": (C.c_int, [P, I32, P, P]),
    "fb_flyvis_create": (C.c_int, [I32, I64, P, P, P, P, P, I32, C.POINTER(P)]),
    "fb_flyvis_destroy": (C.c_int, [P]),
    "fb_flyvis_reset": (C.c_int, [P, I32]),
    "fb_flyvis_set_input": (C.c_int, [P, I32, I32, P, P]),
    "fb_flyvis_write": (C.c_int, [P, I32, I32, P]),
    "fb_flyvis_read": (C.c_int, [P, I32, I32, P]),
    "fb_flyvis_step": (C.c_int, [P, I32]),
    "fb_flyvis_last_ms": (C.c_int, [P, C.POINTER(C.c_float)]),
    "fb_flyvis_state": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(C.c_int32)]),
    "fb_flyg_sizes": (C.c_int, [P, C.c_size_t, C.POINTER(FbFlygHeader)]),
    "fb_flyg_decode": (C.c_int, [P, C.c_size_t, P, P, P]),
    "fb_flyn_count": (C.c_int, [P, C.c_size_t, PU32]),
    "fb_flyn_decode": (C.c_int, [P, C.c_size_t, P, P, P, P, P, P]),
}


class FlyBrainError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def lib_path() -> str:
    """libflybrain.so, or its index-checked build when FLYBRAIN_CHECKED=1."""
    return _build.CHECK_LIB if os.environ.get("FLYBRAIN_CHECKED") == "1" else _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libflybrain.so (building it first if absent); raises if that is impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FlyBrainError(FB_ENODEV, f"{path} is not built")
        _build.build(checked=os.environ.get("FLYBRAIN_CHECKED") == "1")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != FB_OK:
        msg = load().fb_last_error()
        raise FlyBrainError(rc, msg.decode() if msg else "")


def ptr(a) -> C.c_void_p:
    """Address of a contiguous numpy array, or of a torch tensor (host or device)."""
    if a is None:
        return C.c_void_p(0)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)
