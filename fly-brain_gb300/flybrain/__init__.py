"""GB300-native brain step of the fly connectome LIF model (the reference's lif_step + LIFDiff).

Public surface:
  LIFCuda, BrainBatch, DeviceGraph   -- the LIFWasm brain-model API on the sm_103a kernels
  synth_graph, drive_set, workload   -- seeded synthetic connectome-shaped workloads
  FlyVis, synth_flyvis, parse_flyvis -- the flyvis optic lobe (lif.c's fv_step), batched over eyes
  connectome, calibrate, neuromod     -- the connectome tables, the calibrated brain built on them and
                                         its octopamine / hunger controller
  build                               -- compile libflybrain.so in-tree (nvcc, sm_103a)
"""
from .builder import build
from .synth import Graph, SYNTH_PARAMS, drive_set, synth_graph, workload
from .brain import DEFAULTS, BrainBatch, DeviceGraph, LIFCuda
from .flyvis import FlyVis, parse_flyvis, synth_flyvis
from . import _native, calibrate, connectome, neuromod

__all__ = ["build", "Graph", "SYNTH_PARAMS", "drive_set", "synth_graph", "workload", "DEFAULTS",
           "BrainBatch", "DeviceGraph", "LIFCuda", "FlyVis", "parse_flyvis", "synth_flyvis", "_native",
           "calibrate", "connectome", "neuromod"]
