"""Seeded synthetic scenes with the shapes of the benchmark configurations.

All positions, velocities and constants are FP32-representable.

* ``config0``: dam-break box, 16x32x16 lattice (8,192 particles), spacing 0.02,
  jitter +-0.002, box [0,1]^3, h 0.045, mass 0.008, rho0 1000, K 3, visc 3.5,
  g (0,-9.81,0), restitution 0.5, dt 5e-4.
* ``config1``: pipe flow, 262,144 particles uniform in the first segment of a
  three-segment pipe along x (radii 0.10/0.06/0.10, length 0.5 each, axis
  y = z = 0.1, space 1.5 x 0.2 x 0.2), v = (1,0,0) + N(0, 0.05^2), h 0.02,
  no gravity, dt 2e-4; mass = rho0 * volume(first segment) / N.  The device
  interpolates a segment's radius between its row and the next row of
  Pipe.to_numpy (util_kernels.py:56-69), so the first segment is the cone
  0.10 -> 0.06 and particles are placed inside that cone.
* ``config2``: 4,194,304-particle dam break, 128x256x128 lattice, spacing
  0.005, jitter +-0.0005, box [0,2]^3, h 0.0112, mass 1.25e-4.
* ``config3_specs``: 256 independent boxes, N log-uniform in [1024, 65536]
  (rounded to 2 nx^3 particles, lattice nx x 2nx x nx), edge L uniform in
  [0.5, 2], gravity 9.81 in a uniform direction, spacing min(0.02, 0.9 L/2nx),
  mass 1000 s^3, h 1.93 s (about 30 neighbours).
* ``served_request``: one request of the served workload: 70 % box / 30 %
  pipe, N log-uniform in [2048, 524288], steps uniform in [100, 2000].  Box
  requests are config 0 scaled to N (same spacing, h and mass; the box edge
  grows to 1.25 x the block height), pipe requests config 1 scaled to N (h
  scaled to keep its neighbour count).
"""
from __future__ import annotations

import math

import numpy as np

from .config import SPHConstants, f32
from .data_classes import Pipe, Segment, SimulationParameters, SimulationState
from .device import SceneSpec

C0 = dict(rho_0=1000.0, k=3.0, visc=3.5, damp=0.5)


def box_dam_break(nx=16, ny=32, nz=16, spacing=0.02, jitter=0.002, box=(1.0, 1.0, 1.0),
                  h=0.045, mass=0.008, gravity=(0.0, -9.81, 0.0), dt=5e-4, seed=0,
                  max_neighbours=32, walk_dims='ceil'):
    """Jittered lattice block in the box corner; ids in C order of the
    (ix, iy, iz) index grid."""
    rng = np.random.default_rng(seed)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([ix, iy, iz], axis=-1).reshape(-1, 3).astype(np.float64)
    pos = (base + 0.5) * spacing + rng.uniform(-jitter, jitter, size=base.shape)
    n = len(pos)
    hh = float(f32(h))
    params = SimulationParameters(
        particle_count=n, external_force=f32(gravity), duration=1, fps=1.0 / float(f32(dt)),
        pipe=Pipe([Segment()]), space_size=f32(box), voxel_size=np.asarray([hh, hh, hh]))
    const = SPHConstants(mass=float(f32(mass)), inf_r=hh, max_neighbours=max_neighbours,
                         walk_dims=walk_dims, **C0).rounded()
    state = SimulationState(f32(pos), np.zeros((n, 3)), np.zeros(n))
    return SceneSpec(params, const, 'BOX'), state


def config0(seed=0, **kw):
    return box_dam_break(seed=seed, **kw)


def config2(seed=2, **kw):
    return box_dam_break(nx=128, ny=256, nz=128, spacing=0.005, jitter=0.0005,
                         box=(2.0, 2.0, 2.0), h=0.0112, mass=1.25e-4, seed=seed, **kw)


def pipe_flow(n=262_144, radii=(0.10, 0.06, 0.10), seg_len=0.5, axis=0.10, space=(1.5, 0.2, 0.2),
              h=0.02, v0=1.0, sigma=0.05, dt=2e-4, seed=1, rho_0=1000.0, max_neighbours=32):
    """Pipe of cylinders of the given radii laid end to end along x."""
    rng = np.random.default_rng(seed)
    segs = [Segment(start_point=(i * seg_len, axis, axis), start_radius=r, end_radius=r,
                    length=seg_len) for i, r in enumerate(radii)]
    pipe = Pipe(segs)
    r0, r1 = radii[0], radii[1]     # device radius of segment 0: r0 -> r1 (next row)
    vol = math.pi * seg_len / 3.0 * (r0 * r0 + r0 * r1 + r1 * r1)
    pos = np.empty((0, 3))
    while len(pos) < n:
        m = 2 * (n - len(pos)) + 1024
        x = rng.uniform(0.0, seg_len, m)
        y = rng.uniform(-r0, r0, m)
        z = rng.uniform(-r0, r0, m)
        R = r0 + (r1 - r0) * (x / seg_len)
        ok = (y * y + z * z) <= (0.999 * R) ** 2
        pos = np.concatenate([pos, np.stack([x, y + axis, z + axis], axis=1)[ok]])
    pos = pos[:n]
    vel = np.zeros((n, 3))
    vel[:, 0] = v0
    vel += rng.normal(0.0, sigma, size=(n, 3))
    hh = float(f32(h))
    params = SimulationParameters(
        particle_count=n, external_force=np.zeros(3), duration=1, fps=1.0 / float(f32(dt)),
        pipe=pipe, space_size=f32(space), voxel_size=np.asarray([hh, hh, hh]))
    const = SPHConstants(mass=float(f32(rho_0 * vol / n)), inf_r=hh, rho_0=rho_0, k=3.0,
                         visc=3.5, damp=0.5, max_neighbours=max_neighbours).rounded()
    return SceneSpec(params, const, 'PIPE'), SimulationState(f32(pos), f32(vel), np.zeros(n))


def config1(seed=1, **kw):
    return pipe_flow(seed=seed, **kw)


def config3_specs(n_scenes=256, seed=3, n_min=1024, n_max=65536, steps=50):
    """The batched workload: list of (SceneSpec, SimulationState)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_scenes):
        n_target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        nx = max(2, int(round((n_target / 2.0) ** (1.0 / 3.0))))
        L = rng.uniform(0.5, 2.0)
        g = rng.normal(size=3)
        g = 9.81 * g / np.linalg.norm(g)
        s = min(0.02, 0.9 * L / (2 * nx))
        spec, st = box_dam_break(nx=nx, ny=2 * nx, nz=nx, spacing=s, jitter=s / 10.0,
                                 box=(L, L, L), h=1.93 * s, mass=1000.0 * s ** 3,
                                 gravity=tuple(g), seed=int(rng.integers(1 << 31)))
        out.append((spec, st))
    return out


def served_request(rng, n_min=2048, n_max=524_288, box_frac=0.7):
    """One request: (SceneSpec, SimulationState, steps)."""
    n_target = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
    steps = int(rng.integers(100, 2001))
    seed = int(rng.integers(1 << 31))
    if rng.uniform() < box_frac:
        # config 0 scaled to N: its spacing, h and mass, the box grown to fit
        # the block (the reference's formulas are stable there, unlike at the
        # smaller h a fixed box would need)
        nx = max(2, int(round((n_target / 2.0) ** (1.0 / 3.0))))
        edge = max(1.0, 1.25 * 2 * nx * 0.02)
        spec, st = box_dam_break(nx=nx, ny=2 * nx, nz=nx, box=(edge, edge, edge), seed=seed)
    else:
        n = int(n_target)
        spec, st = pipe_flow(n=n, h=0.02 * (262_144 / n) ** (1.0 / 3.0), seed=seed)
    return spec, st, steps
