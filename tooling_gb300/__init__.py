"""GB300-native batched stepping for newt (hwang2409/tooling, newt/).

The compute path is ``libnewt_gpu.so`` (hand-written sm_103a CUDA behind the
C ABI in include/newt_gpu.h); this package is its Python host binding, the
model/scene builders and the build step.
"""
from . import model, scenes
from .api import Engine, NewtError, STEP_BATCHED, STEP_PLAIN, load_library

__all__ = ["Engine", "NewtError", "STEP_BATCHED", "STEP_PLAIN", "load_library", "model", "scenes"]
