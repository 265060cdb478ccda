"""State iterator, interface-compatible with the reference's
``sim/src/state_generator.py`` (iwoplaza/cuda-sph).

``StateGenerator(start_state, params)`` yields one SimulationState per frame
for ``duration * fps`` frames.  With ``steps_per_frame > 1`` the state stays on
the device between saved frames (``advance``) and only every k-th step is
copied back, which the reference cannot do (it copies every step).
"""
from __future__ import annotations

import logging
from timeit import default_timer as timer

from . import config
from .data_classes import SimulationParameters, SimulationState

logger = logging.getLogger(__name__)


class StateGenerator:
    def __init__(self, start_state: SimulationState, params: SimulationParameters,
                 constants=None, mode=None, steps_per_frame: int = 1, device: str = "cuda"):
        from .strategies import GB300SPHStrategy
        if config.SIM_STRATEGY not in ('GB300', 'VOXEL'):
            raise Exception(f'Unsupported strategy {config.SIM_STRATEGY!r} (this build provides '
                            "'GB300'; 'VOXEL' maps to it)")
        self.current_state = start_state
        self.current_frame_idx = 0
        self.n_frames = params.duration * params.fps // max(1, steps_per_frame)
        self.steps_per_frame = max(1, int(steps_per_frame))
        self.sph_strategy = GB300SPHStrategy(params, constants=constants, mode=mode, device=device)
        if self.steps_per_frame > 1:
            self.sph_strategy.load(start_state)

    def __next__(self) -> SimulationState:
        if self.current_frame_idx >= self.n_frames:
            raise StopIteration
        t0 = timer()
        if self.steps_per_frame == 1:
            self.current_state = self.sph_strategy.compute_next_state(self.current_state)
        else:
            self.sph_strategy.advance(self.steps_per_frame)
            self.current_state = self.sph_strategy.state()
        logger.info("frame %d / %d computed in %.4f s", self.current_frame_idx, self.n_frames,
                    timer() - t0)
        self.current_frame_idx += 1
        return self.current_state

    def __iter__(self) -> "StateGenerator":
        return self
