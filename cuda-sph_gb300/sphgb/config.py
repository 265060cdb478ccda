"""Simulation configuration with the reference's names (iwoplaza/cuda-sph
``config.py``), without import-time side effects.

The reference freezes its physics constants into the kernels at JIT time
(``from config import INF_R, ...``) and builds a random start state when the
module is imported (config.py:123-132).  Here the same names exist as module
defaults, and the values a simulation uses travel with it at run time as an
``SPHConstants`` (one per scene), so scenes with different constants can
share a launch.  ``params``/``start_state`` builders are plain functions.
"""
from __future__ import annotations

import math
import pathlib
from dataclasses import dataclass, replace

import numpy as np

from .data_classes import Pipe, Segment, SimulationParameters, SimulationState
from .pipe_builder import PipeBuilder

SIM_MODE = 'BOX'        # 'BOX' or 'PIPE'
SIM_STRATEGY = 'GB300'  # the reference also accepts 'NAIVE' and 'VOXEL'
DURATION = 15
FPS = 20
PARTICLE_COUNT = 20_000
MASS = 1.0
RHO_0 = 1.0
INF_R = 2.0
VISC = 0.5
K = 10.0
DAMP = 0.7
INF_R_2 = INF_R ** 2
INF_R_6 = INF_R ** 6
INF_R_9 = INF_R ** 9
W_CONST = 315.0 / (64.0 * np.pi * INF_R_9)
GRAD_W_CONST = -45.0 / (np.pi * INF_R_6)
LAP_W_CONST = 45.0 / (np.pi * INF_R_6)
MAX_NEIGHBOURS = 32
NEIGHBOURING_VOXELS_COUNT = 27
VOXEL_SIZE = [INF_R, INF_R, INF_R]
BOX_SPACE_SIZE = [20 * INF_R, 20 * INF_R, 20 * INF_R]
PIPE_SPACE_SIZE = [20 * INF_R, 3 * INF_R, 3 * INF_R]
GRAVITY = [0.0, -2.0, 0.0]
HORIZONTAL_FORCE = [2.0, 0.0, 0.0]

ROOT_PROJ_DIRNAME = pathlib.Path.cwd()   # Saver/Loader paths are relative to this
ASSETS_DIRNAME = 'vis/assets'
PARAMS_FILENAME = 'params.json'
OUT_DIRNAME = 'out'

RESPAWN_SEED = 16435234                  # abstract_sph_strategy.py:27


def f32(x):
    """Round to the nearest FP32 value (returned as float64 / ndarray)."""
    return np.asarray(x, dtype=np.float32).astype(np.float64)


@dataclass(frozen=True)
class SPHConstants:
    """Per-scene physics constants (config.py:18-30 in the reference).

    ``walk_dims`` is 'ceil' (the voxel table's dims, the reference's
    documented intent) or 'truncated' (the reference's actual walk, which
    builds neighbour voxel ids with int(space/voxel),
    voxel_sph_strategy.py:110-116).  ``max_neighbours <= 0`` removes the cap.
    """
    mass: float = MASS
    rho_0: float = RHO_0
    inf_r: float = INF_R
    visc: float = VISC
    k: float = K
    damp: float = DAMP
    max_neighbours: int = MAX_NEIGHBOURS
    walk_dims: str = 'ceil'
    seed: int = RESPAWN_SEED

    def rounded(self) -> "SPHConstants":
        """Constants rounded to FP32, the precision the device uses."""
        return replace(self, mass=float(f32(self.mass)), rho_0=float(f32(self.rho_0)),
                       inf_r=float(f32(self.inf_r)), visc=float(f32(self.visc)),
                       k=float(f32(self.k)), damp=float(f32(self.damp)))

    @property
    def w_const(self):
        return 315.0 / (64.0 * np.pi * self.inf_r ** 9)

    @property
    def grad_w_const(self):
        return -45.0 / (np.pi * self.inf_r ** 6)

    @property
    def lap_w_const(self):
        return 45.0 / (np.pi * self.inf_r ** 6)


def constants_from_module() -> SPHConstants:
    """SPHConstants from this module's (possibly edited) globals."""
    return SPHConstants(mass=MASS, rho_0=RHO_0, inf_r=INF_R, visc=VISC, k=K, damp=DAMP,
                        max_neighbours=MAX_NEIGHBOURS)


def build_pipe() -> Pipe:
    """The reference's default pipe (config.py:68-76)."""
    return (PipeBuilder().with_starting_radius(1)
            .add_roller_segment(1)
            .add_increasing_segment(1, 1.2)
            .add_roller_segment(1)
            .add_lessening_segment(1, 1.2)
            .add_roller_segment(1)
            .transform(PIPE_SPACE_SIZE[0], PIPE_SPACE_SIZE[1])
            .get_result())


def create_params_pipe(pipe: Pipe = None) -> SimulationParameters:
    """config.py:44-53."""
    return SimulationParameters(
        particle_count=PARTICLE_COUNT, external_force=np.asarray(HORIZONTAL_FORCE),
        duration=DURATION, fps=FPS, pipe=pipe if pipe is not None else build_pipe(),
        space_size=np.asarray(PIPE_SPACE_SIZE), voxel_size=np.asarray(VOXEL_SIZE))


def create_params_box() -> SimulationParameters:
    """config.py:56-65."""
    return SimulationParameters(
        particle_count=PARTICLE_COUNT, external_force=np.asarray(GRAVITY),
        duration=DURATION, fps=FPS, pipe=Pipe([Segment()]),
        space_size=np.asarray(BOX_SPACE_SIZE), voxel_size=np.asarray(VOXEL_SIZE))


def start_state_box_wall(n: int = PARTICLE_COUNT, seed: int = 0) -> SimulationState:
    """Seeded version of config.py:79-97: a wall of particles in the first
    tenth of the box along x, velocity (1.5, -5, -5) +- 0.5."""
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)) * np.asarray(BOX_SPACE_SIZE, dtype=np.float64)
    pos[:, 0] *= 0.1
    vel = np.asarray([1.5, -5.0, -5.0]) + (rng.random((n, 3)) - 0.5)
    return SimulationState(f32(pos), f32(vel), np.zeros(n))


def start_state_inside_pipe(pipe: Pipe, n: int = PARTICLE_COUNT, seed: int = 0) -> SimulationState:
    """Seeded version of config.py:100-120: uniform x along the pipe, radius
    sqrt(U) * 0.98 R(x), zero velocity."""
    rng = np.random.default_rng(seed)
    length = pipe.get_length()
    c = pipe.segments[0].start_point
    pos = np.zeros((n, 3))
    for i in range(n):
        x = rng.random() * length
        r = math.sqrt(rng.random()) * pipe.radius_at(x) * 0.98
        th = rng.random() * 2.0 * math.pi
        pos[i] = (x, c[1] + r * math.cos(th), c[2] + r * math.sin(th))
    return SimulationState(f32(pos), np.zeros((n, 3)), np.zeros(n))
