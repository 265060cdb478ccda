"""sphgb -- GB300-native SPH step (iwoplaza/cuda-sph's voxel strategy) on sm_103a.

Python host code over libsphgb.so (hand-written CUDA kernels, C ABI in
include/sphgb.h).  Mirrors the reference's data classes, pipe builder,
serializer, config names and strategy API.
"""
from .config import SPHConstants
from .data_classes import Pipe, Segment, SimulationParameters, SimulationState
from .pipe_builder import PipeBuilder

__all__ = ["Pipe", "Segment", "SimulationParameters", "SimulationState", "PipeBuilder",
           "SPHConstants", "GB300SPHStrategy", "AbstractSPHStrategy", "SceneBatch", "SceneSpec",
           "StateGenerator"]


def __getattr__(name):
    # the GPU-facing modules import torch lazily
    if name in ("GB300SPHStrategy", "AbstractSPHStrategy", "VoxelSPHStrategy"):
        from . import strategies
        return getattr(strategies, name)
    if name in ("SceneBatch", "SceneSpec"):
        from . import device
        return getattr(device, name)
    if name == "StateGenerator":
        from .state_generator import StateGenerator
        return StateGenerator
    raise AttributeError(name)
