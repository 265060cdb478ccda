"""Continuous batching of scene requests on one GPU.

Requests (a scene, its start state and a step count) arrive over time.  The
server keeps every admitted scene's state resident in HBM inside one
multi-scene context and advances all of them together, tick by tick:

* at a tick boundary, requests that have arrived are admitted in arrival
  order while the HBM budget allows (per-particle and per-voxel footprint of
  the state and of the step's scratch);
* admitted scenes join the running batch: the context is re-packed (scratch
  buffers that are big enough are reused), running scenes keep their state
  and step counters on the device, new scenes' start states are copied in;
* the tick advances every active scene by up to K steps, K = the largest
  number of steps any active scene still needs (at most max_tick_steps).  Each
  scene's request is its step limit on the device
  (sphgb_ctx_set_step_limits), so a scene that reaches it inside the tick is
  frozen there and is never stepped past its request;
* scenes whose steps are done retire at the next tick boundary: their state
  is copied out, memory frees up and queued requests can be admitted; the
  retirements and admissions of one boundary are one re-pack (the running
  state is exported once, the context reconfigured once).

While the GPU runs a tick (kernel launches are asynchronous), the host
generates and uploads the states of requests that arrived meanwhile, so their
preparation overlaps the running work.  A scene's result does not depend on
the mix it ran in: scenes share no voxels, neighbours or sums, re-packing
moves state exactly, and the respawn stream is keyed by the scene's own step
counter.
"""
from __future__ import annotations

import collections
import math
import time
from dataclasses import dataclass, field
from typing import Callable, Deque, List, Optional

import numpy as np

from .data_classes import SimulationState
from .device import SceneBatch, SceneSpec

# HBM bytes per particle for a scene resident in the batch: bound state
# (pos, vel 16 B each, rho, pid 4 B), the step's sorted copies (36 B), ids and
# ranks (12 B), force inputs (32 B), neighbour list (132 B), density tasks (8 B),
# export staging (56 B) and the FP64 accumulator (48 B both buffers, pipe scenes)
BYTES_PER_PARTICLE = 40 + 36 + 12 + 32 + 132 + 8 + 56
BYTES_PER_PIPE_PARTICLE = 48
BYTES_PER_VOXEL = 8


def footprint(spec: SceneSpec) -> int:
    space = np.asarray(spec.params.space_size, dtype=np.float64)
    voxel = np.asarray(spec.params.voxel_size, dtype=np.float64)
    voxels = int(np.prod(np.ceil(space / voxel))) + 1
    per = BYTES_PER_PARTICLE + (BYTES_PER_PIPE_PARTICLE if spec.mode == 'PIPE' else 0)
    return spec.n * per + voxels * BYTES_PER_VOXEL


@dataclass
class Request:
    rid: int
    spec: SceneSpec
    state: SimulationState
    steps: int
    arrival: float = 0.0                 # seconds after the server starts
    admitted: Optional[float] = None
    finished: Optional[float] = None
    remaining: int = 0
    result: Optional[SimulationState] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclass
class ServeStats:
    requests: int
    wall_s: float
    particle_steps: int
    ticks: int
    repacks: int
    max_active: int
    latencies: List[float] = field(default_factory=list)
    gpu_s: float = 0.0          # device time of the ticks' steps (CUDA events)
    repack_s: float = 0.0       # host wall time in re-packs (retirements with admissions)

    @property
    def throughput(self) -> float:
        return self.particle_steps / self.wall_s

    @property
    def gpu_busy(self) -> float:
        """Fraction of the wall time the GPU spent stepping scenes."""
        return self.gpu_s / self.wall_s if self.wall_s else 0.0

    def pct(self, q: float) -> float:
        return float(np.percentile(self.latencies, q)) if self.latencies else float("nan")


class SceneServer:
    def __init__(self, hbm_budget_bytes: float = 150e9, max_tick_steps: int = 64,
                 device: str = "cuda", clock: Callable[[], float] = time.perf_counter):
        self.budget = float(hbm_budget_bytes)
        self.max_tick = int(max_tick_steps)
        self.device = device
        self.clock = clock
        self.batch: Optional[SceneBatch] = None
        self.active: List[Request] = []
        self.used = 0

    # -- batch maintenance -----------------------------------------------
    def _rebuild(self, done: List[Request], admitted: List[Request], now: float) -> None:
        """One membership change: finished scenes are copied out, the rest keep
        their device state and step counters, admitted scenes start from their
        start states.  The running state is exported once for both."""
        import torch
        dev = torch.device(self.device)
        keep = [r for r in self.active if r.remaining > 0]
        parts_pos, parts_vel, steps = [], [], []
        if self.active and (done or admitted):
            pos, vel, rho = self.batch.export_aos_f64()      # device, FP64, original order
            old_steps = self.batch.steps.clone()
            for r in done:
                k = self._index[r.rid]
                off, n = self.batch.scene_offsets[k], self.batch.scene_sizes[k]
                r.result = SimulationState(pos[off:off + n].cpu().numpy(),
                                           vel[off:off + n].cpu().numpy(),
                                           rho[off:off + n].cpu().numpy())
                r.finished = now
            for r in keep:
                k = self._index[r.rid]
                off, n = self.batch.scene_offsets[k], self.batch.scene_sizes[k]
                parts_pos.append(pos[off:off + n])
                parts_vel.append(vel[off:off + n])
                steps.append(old_steps[k:k + 1])
        for r in admitted:
            parts_pos.append(torch.as_tensor(np.asarray(r.state.position, dtype=np.float64),
                                             device=dev).reshape(-1, 3))
            parts_vel.append(torch.as_tensor(np.asarray(r.state.velocity, dtype=np.float64),
                                             device=dev).reshape(-1, 3))
            steps.append(torch.zeros(1, dtype=torch.int32, device=dev))
        reqs = keep + admitted
        if not reqs:
            self.batch_reset()
            return
        specs = [r.spec for r in reqs]
        pos_all = torch.cat(parts_pos).contiguous()
        vel_all = torch.cat(parts_vel).contiguous()
        step_all = torch.cat(steps)
        if self.batch is None:
            self.batch = SceneBatch(specs, device=self.device)
            self.batch.steps.copy_(step_all)
        else:
            self.batch.reconfigure(specs, steps=step_all)
        self.batch.load_aos_device(pos_all, vel_all, reset_steps=False)
        # every scene stops at its request (step counters count from its start)
        self.batch.set_step_limits([r.steps for r in reqs])
        self.active = reqs
        self._index = {r.rid: k for k, r in enumerate(reqs)}

    # -- the loop ------------------------------------------------------------
    def run(self, requests: List[Request], prepare: Callable[[Request], None] = None) -> ServeStats:
        """Serve `requests` (sorted by arrival time, seconds from now).
        ``prepare(req)`` (optional) builds req.spec / req.state lazily; it is
        called for requests that have arrived while the GPU runs a tick."""
        import torch
        t0 = self.clock()
        schedule: Deque[Request] = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue: Deque[Request] = collections.deque()
        finished: List[Request] = []
        ticks = repacks = max_active = 0
        gpu_s = repack_s = 0.0
        total = len(requests)
        ready = set()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)

        def arrive(now):
            while schedule and schedule[0].arrival <= now:
                r = schedule.popleft()
                if prepare is not None and r.rid not in ready:
                    prepare(r)
                    ready.add(r.rid)
                queue.append(r)

        done: List[Request] = []          # finished in the last tick, not yet copied out
        while len(finished) < total:
            now = self.clock() - t0
            arrive(now)
            admitted = []
            while queue and self.used + footprint(queue[0].spec) <= self.budget:
                r = queue.popleft()
                r.admitted = now
                r.remaining = r.steps
                self.used += footprint(r.spec)
                admitted.append(r)
            if queue and not self.active and not admitted and not done:
                raise MemoryError(f"request {queue[0].rid} needs {footprint(queue[0].spec)} bytes, "
                                  f"over the {self.budget:.0f}-byte HBM budget")
            if done or admitted:
                # one re-pack per tick for retirements and admissions together
                t_r = self.clock()
                self._rebuild(done, admitted, now)
                repack_s += self.clock() - t_r
                repacks += 1
                finished.extend(done)
                done = []
                if len(finished) == total:
                    break
            if not self.active:
                # idle: wait for the next arrival
                if schedule:
                    time.sleep(max(0.0, min(schedule[0].arrival - (self.clock() - t0), 0.01)))
                continue
            max_active = max(max_active, len(self.active))
            k = min(self.max_tick, max(r.remaining for r in self.active))
            ev0.record()
            self.batch.step(k)                       # asynchronous
            ev1.record()
            # overlap: prepare requests that arrive while the GPU works
            if prepare is not None:
                for r in schedule:
                    if r.arrival > self.clock() - t0 + 0.05:
                        break
                    if r.rid not in ready:
                        prepare(r)
                        ready.add(r.rid)
            torch.cuda.synchronize()
            gpu_s += ev0.elapsed_time(ev1) / 1e3
            ticks += 1
            for r in self.active:
                r.remaining = max(0, r.remaining - k)    # the device froze it at 0
            done = [r for r in self.active if r.remaining == 0]
            for r in done:
                self.used -= footprint(r.spec)     # its memory is free for admissions
        wall = self.clock() - t0
        ps = sum(r.spec.n * r.steps for r in finished)
        return ServeStats(requests=total, wall_s=wall, particle_steps=ps, ticks=ticks,
                          repacks=repacks, max_active=max_active,
                          latencies=[r.latency for r in finished], gpu_s=gpu_s,
                          repack_s=repack_s)

    def batch_reset(self) -> None:
        self.active = []
        self._index = {}

    def close(self) -> None:
        if self.batch is not None:
            self.batch.close()
            self.batch = None


def poisson_requests(rate: float, count: int, seed: int = 4, make=None) -> List[Request]:
    """`count` requests with exponential inter-arrival times of mean 1/rate;
    `make(rng)` returns (spec, state, steps) (default: scenes.served_request)."""
    from . import scenes
    rng = np.random.default_rng(seed)
    make = make or scenes.served_request
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate) if math.isfinite(rate) and rate > 0 else 0.0
        spec, st, steps = make(rng)
        out.append(Request(rid=i, spec=spec, state=st, steps=steps, arrival=t))
    return out
