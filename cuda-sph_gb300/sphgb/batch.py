"""Many independent scenes advanced together.

The batched path puts every scene in one context: one voxel table (scene
ranges side by side), one sort, one warp-cooperative density launch and one
force launch per step for all scenes, and the whole multi-step sequence
captured once as a CUDA graph (one launch for all steps).  Each scene's
result is bit-identical to running it alone: scenes never share voxels,
neighbours or sums, and per-scene sums run in a fixed order.

The plain path is the reference's way of working, one scene per strategy
object and so one scene per kernel launch (the reference creates one
VoxelSPHStrategy per run, sim/src/state_generator.py:21-23), here on the same
GPU kernels.
"""
from __future__ import annotations

import time
from typing import List, Sequence, Tuple

from .data_classes import SimulationState
from .device import SceneBatch, SceneSpec


def particle_steps(specs: Sequence[SceneSpec], steps: int) -> int:
    return sum(s.n for s in specs) * steps


def run_batched(pairs: Sequence[Tuple[SceneSpec, SimulationState]], steps: int,
                device: str = "cuda", repeats: int = 1) -> Tuple[float, List[SimulationState]]:
    """Advance all scenes `steps` steps in one graph launch; returns (seconds
    of the fastest repeat, final states).  Each repeat reloads the start states."""
    import torch
    specs = [p[0] for p in pairs]
    batch = SceneBatch(specs, device=device)
    best = float("inf")
    for r in range(repeats + 1):            # the first run captures the graph
        batch.load_states([p[1] for p in pairs])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        batch.step(steps, use_graph=True)
        e1.record()
        torch.cuda.synchronize()
        if r > 0 or repeats == 0:
            best = min(best, e0.elapsed_time(e1) / 1e3)
    states = batch.states()
    batch.close()
    return best, states


def run_plain(pairs: Sequence[Tuple[SceneSpec, SimulationState]], steps: int,
              device: str = "cuda", use_graph: bool = False) -> Tuple[float, List[SimulationState]]:
    """Advance the scenes one after another, one context (strategy) per scene;
    returns (seconds, final states).  Contexts are created before timing."""
    import torch
    batches = [SceneBatch([spec], device=device) for spec, _ in pairs]
    for b, (_, st) in zip(batches, pairs):
        b.load_states([st])
        if use_graph:                       # capture outside the timed region
            b.step(steps, use_graph=True)
            b.load_states([st])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for b in batches:
        b.step(steps, use_graph=use_graph)
    e1.record()
    torch.cuda.synchronize()
    seconds = max(e0.elapsed_time(e1) / 1e3, 0.0)
    del t0
    states = [b.states()[0] for b in batches]
    for b in batches:
        b.close()
    return seconds, states
