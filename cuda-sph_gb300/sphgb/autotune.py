"""Autotuner for the launch choices of a batch of scenes.

Tunes what changes speed but not results:
* the density kernel variant: one warp per voxel run, a lane per candidate
  (SPHGB_DENSITY_WARP), or one thread per particle with its own walk
  (SPHGB_DENSITY_THREAD); both skip voxels beyond h and stop at the cap;
* the block size of the per-particle sort kernels;
* the member count above which a voxel is sorted by a block of its own.

And, for scenes without a neighbour cap only, the cell-size ratio: the voxel
edge as a multiple of h (>= 1, so the 27-voxel walk still covers h).  With the
reference's cap the voxel size is part of the result (the walk order decides
which 32 neighbours count), so capped scenes keep their own voxel size.

Each candidate is timed with CUDA events over a few steps of the batch's own
start states (sphgb_ctx_step_profiled), after one untimed step.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, replace
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import _capi
from .data_classes import SimulationState
from .device import SceneBatch, SceneSpec

VARIANTS = (_capi.DENSITY_WARP, _capi.DENSITY_THREAD)
SORT_BLOCKS = (128, 256, 512)
BIG_VOXEL = (32, 64, 256)
CELL_RATIOS = (1.0, 1.25, 1.5)


@dataclass
class Tuning:
    sort_block: int = 256
    density_variant: int = _capi.DENSITY_WARP
    big_voxel: int = 64
    cell_ratio: float = 1.0
    ms_per_step: float = float("nan")

    def apply(self, batch: SceneBatch) -> None:
        batch.set_tuning(self.sort_block, self.density_variant, self.big_voxel)


def _time(batch: SceneBatch, states, steps: int) -> float:
    batch.load_states(states)
    batch.step(1)
    batch.load_states(states)
    return sum(batch.step_profiled(steps).values())


def with_cell_ratio(spec: SceneSpec, ratio: float) -> SceneSpec:
    h = spec.constants.inf_r
    vs = np.full(3, float(np.float32(h * ratio)))
    return replace(spec, params=replace(spec.params, voxel_size=vs))


def autotune(pairs: Sequence[Tuple[SceneSpec, SimulationState]], steps: int = 3,
             device: str = "cuda") -> Tuple[Tuning, List[Tuning]]:
    """Return (best tuning, every candidate with its time)."""
    specs = [p[0] for p in pairs]
    states = [p[1] for p in pairs]
    uncapped = all(s.constants.max_neighbours <= 0 for s in specs)
    ratios = CELL_RATIOS if uncapped else (1.0,)
    tried: List[Tuning] = []
    for ratio in ratios:
        rs = [with_cell_ratio(s, ratio) for s in specs] if ratio != 1.0 else specs
        batch = SceneBatch(rs, device=device)
        for variant, block, big in itertools.product(VARIANTS, SORT_BLOCKS, BIG_VOXEL):
            t = Tuning(block, variant, big, ratio)
            t.apply(batch)
            t.ms_per_step = _time(batch, states, steps)
            tried.append(t)
        batch.close()
    best = min(tried, key=lambda t: t.ms_per_step)
    return best, tried


def summary(tried: List[Tuning]) -> Dict[str, float]:
    names = {_capi.DENSITY_WARP: "warp", _capi.DENSITY_THREAD: "thread"}
    return {f"{names[t.density_variant]}/b{t.sort_block}/big{t.big_voxel}/r{t.cell_ratio}":
            round(t.ms_per_step, 4) for t in tried}
