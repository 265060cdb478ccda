"""Strategy API, interface-compatible with the reference's
``sim/src/sph/strategies/abstract_sph_strategy.py`` (iwoplaza/cuda-sph).

``GB300SPHStrategy`` drops in where the reference constructs
``VoxelSPHStrategy(params)`` (state_generator.py:21-23):
``compute_next_state(old_state) -> SimulationState`` takes and returns host
FP64 arrays in original particle order, exactly like the reference (which
uploads, runs its kernels and downloads every step, :65-84).  The step runs
entirely on the GPU through libsphgb.so.  For runs that keep the state on the
device, ``advance(n)`` steps without host copies and ``state()`` reads it back.
"""
from __future__ import annotations

from abc import ABC, abstractmethod

import numpy as np

from . import config
from .config import SPHConstants
from .data_classes import SimulationParameters, SimulationState
from .device import SceneBatch, SceneSpec


class AbstractSPHStrategy(ABC):
    """abstract_sph_strategy.py:16-46: owns params and dt = 1 / fps."""

    def __init__(self, params: SimulationParameters):
        self.params = params
        self.dt = 1 / self.params.fps
        self.old_state: SimulationState = None
        self.new_state: SimulationState = None

    @abstractmethod
    def compute_next_state(self, old_state: SimulationState) -> SimulationState:
        ...


class GB300SPHStrategy(AbstractSPHStrategy):
    """The reference's voxel step on a GB300, one scene.

    ``constants`` default to this package's config module values (the
    reference's config.py defaults); ``mode`` defaults to ``config.SIM_MODE``
    ('BOX' or 'PIPE'), which the reference also reads at step time
    (abstract_sph_strategy.py:102).
    """

    def __init__(self, params: SimulationParameters, constants: SPHConstants = None,
                 mode: str = None, device: str = "cuda"):
        super().__init__(params)
        self.constants = constants if constants is not None else config.constants_from_module()
        self.mode = mode if mode is not None else config.SIM_MODE
        if self.mode not in ('BOX', 'PIPE'):
            raise Exception(f'Wrong simulation mode! ({self.mode})')
        self.scenes = SceneBatch([SceneSpec(params, self.constants, self.mode)], device=device)

    def compute_next_state(self, old_state: SimulationState) -> SimulationState:
        self.old_state = old_state
        pos, vel, rho = self.scenes.compute_next_state_host(
            np.asarray(old_state.position, dtype=np.float64).reshape(-1, 3),
            np.asarray(old_state.velocity, dtype=np.float64).reshape(-1, 3))
        self.new_state = SimulationState(pos, vel, rho)
        return self.new_state

    # -- device-resident use --------------------------------------------
    def load(self, state: SimulationState) -> None:
        self.scenes.load_states([state])

    def advance(self, n_steps: int = 1, use_graph: bool = True) -> None:
        self.scenes.step(n_steps, use_graph=use_graph)

    def state(self) -> SimulationState:
        return self.scenes.states()[0]


# the reference selects strategies by name (state_generator.py:21-23)
VoxelSPHStrategy = GB300SPHStrategy
