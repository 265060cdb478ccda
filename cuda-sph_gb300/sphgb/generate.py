"""Start states generated on the device (sphgb_generate).

The reference builds its start states with Python loops on the host
(config.py:79-121: ``__start_state_box_wall``, ``__start_state_inside_pipe``)
and fills a pipe on the GPU with ``spawn_particles_inside_pipe_kernel``
(sim/src/sph/kernels/base_kernels.py:130-143).  These functions produce the
same kinds of state directly in HBM, FP64 (n, 3) position and velocity in
particle-id order, ready for ``SceneBatch.load_aos_device``.  The random
numbers are Philox4x32-10 draws keyed by (seed, particle id), so a state is
the same for any launch shape and on any GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _capi
from .config import SPHConstants, f32
from .data_classes import Pipe, Segment, SimulationParameters
from .device import SceneSpec


def _run(gen: _capi.Generator, n: int, pipe: Optional[Pipe] = None, device="cuda"):
    import torch
    pos = torch.empty((max(n, 1), 3), dtype=torch.float64, device=device)
    vel = torch.empty((max(n, 1), 3), dtype=torch.float64, device=device)
    table, rows = None, 0
    if pipe is not None:
        t = np.ascontiguousarray(pipe.to_numpy(), dtype=np.float64)
        table = torch.from_numpy(t).to(device)
        rows = len(t)
    # the table is copied on the current stream, so the kernel runs there too
    stream = torch.cuda.current_stream(pos.device).cuda_stream
    _capi.call("sphgb_generate", C.byref(gen), None if table is None else table.data_ptr(), rows,
               int(n), pos.data_ptr(), vel.data_ptr(), stream)
    if table is not None:
        # keep the table alive until the kernel has read it
        torch.cuda.current_stream(pos.device).synchronize()
    return pos[:n], vel[:n]


def lattice_generator(nx, ny, nz, spacing, jitter, origin=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0),
                      sigma=0.0, seed=0) -> _capi.Generator:
    g = _capi.Generator()
    g.kind = _capi.GEN_LATTICE
    g.lattice[:] = [int(nx), int(ny), int(nz)]
    g.spacing, g.jitter = float(spacing), float(jitter)
    g.origin[:] = [float(x) for x in origin]
    g.velocity[:] = [float(x) for x in velocity]
    g.velocity_sigma = float(sigma)
    g.seed = int(seed)
    return g


def box_wall_generator(space_size: Sequence[float], wall_fraction=0.1,
                       base_velocity=(1.5, -5.0, -5.0), spread=1.0, seed=0) -> _capi.Generator:
    """config.py:79-97: positions uniform in [0, f*Sx) x [0, Sy) x [0, Sz),
    velocities base + U(-spread/2, spread/2) per axis."""
    g = _capi.Generator()
    g.kind = _capi.GEN_BOX_WALL
    g.extent[:] = [float(space_size[0]) * wall_fraction, float(space_size[1]), float(space_size[2])]
    g.velocity[:] = [float(x) for x in base_velocity]
    g.velocity_spread = float(spread)
    g.seed = int(seed)
    return g


def pipe_fill_generator(pipe: Pipe, x_range: Optional[Tuple[float, float]] = None, fill=0.98,
                        velocity=(0.0, 0.0, 0.0), sigma=0.0, seed=0) -> _capi.Generator:
    """config.py:100-121 (x uniform in [0, pipe length), r = sqrt(u) R(x) 0.98,
    angle uniform) with the pipe radius of the reference's kernels."""
    g = _capi.Generator()
    g.kind = _capi.GEN_PIPE_FILL
    if x_range is None:
        x_range = (0.0, pipe.get_length())
    g.x_range[:] = [float(x_range[0]), float(x_range[1])]
    g.fill = float(fill)
    g.velocity[:] = [float(x) for x in velocity]
    g.velocity_sigma = float(sigma)
    g.seed = int(seed)
    return g


def generate(gen: _capi.Generator, n: int, pipe: Optional[Pipe] = None, device="cuda"):
    """(pos, vel) FP64 (n, 3) device tensors for the generator, written on
    the current stream."""
    return _run(gen, n, pipe, device)


def box_wall(n: int, space_size=(40.0, 20.0, 20.0), seed=0, device="cuda"):
    """The reference's BOX start state (config.py:79-97) for n particles."""
    return generate(box_wall_generator(space_size, seed=seed), n, device=device)


def inside_pipe(n: int, pipe: Pipe, seed=0, device="cuda"):
    """The reference's PIPE start state (config.py:100-121) for n particles."""
    return generate(pipe_fill_generator(pipe, seed=seed), n, pipe=pipe, device=device)


def dam_break_scene(nx=128, ny=256, nz=128, spacing=0.005, jitter=0.0005, box=(2.0, 2.0, 2.0),
                    h=0.0112, mass=1.25e-4, gravity=(0.0, -9.81, 0.0), dt=5e-4, seed=2,
                    max_neighbours=32, device="cuda"):
    """A dam-break block generated in HBM: (SceneSpec, pos, vel).  Defaults:
    the 4,194,304-particle box (128 x 256 x 128 lattice, spacing 0.005,
    jitter +-0.0005, box [0,2]^3, h 0.0112, mass 1.25e-4)."""
    n = nx * ny * nz
    hh = float(f32(h))
    params = SimulationParameters(
        particle_count=n, external_force=f32(gravity), duration=1, fps=1.0 / float(f32(dt)),
        pipe=Pipe([Segment()]), space_size=f32(box), voxel_size=np.asarray([hh, hh, hh]))
    const = SPHConstants(mass=float(f32(mass)), inf_r=hh, max_neighbours=max_neighbours,
                         rho_0=1000.0, k=3.0, visc=3.5, damp=0.5).rounded()
    pos, vel = generate(lattice_generator(nx, ny, nz, spacing, jitter, seed=seed), n, device=device)
    return SceneSpec(params, const, 'BOX'), pos, vel


def pipe_flow_scene(n=262_144, radii=(0.10, 0.06, 0.10), seg_len=0.5, axis=0.10,
                    space=(1.5, 0.2, 0.2), h=0.02, v0=1.0, sigma=0.05, dt=2e-4, seed=1,
                    rho_0=1000.0, max_neighbours=32, device="cuda"):
    """Pipe flow generated in HBM: particles in the first segment (the cone
    r0 -> r1 of the kernels' radius), v = (v0, 0, 0) + N(0, sigma^2)."""
    import math
    segs = [Segment(start_point=(i * seg_len, axis, axis), start_radius=r, end_radius=r,
                    length=seg_len) for i, r in enumerate(radii)]
    pipe = Pipe(segs)
    r0, r1 = radii[0], radii[1]
    vol = math.pi * seg_len / 3.0 * (r0 * r0 + r0 * r1 + r1 * r1)
    hh = float(f32(h))
    params = SimulationParameters(
        particle_count=n, external_force=np.zeros(3), duration=1, fps=1.0 / float(f32(dt)),
        pipe=pipe, space_size=f32(space), voxel_size=np.asarray([hh, hh, hh]))
    const = SPHConstants(mass=float(f32(rho_0 * vol / n)), inf_r=hh, rho_0=rho_0, k=3.0,
                         visc=3.5, damp=0.5, max_neighbours=max_neighbours).rounded()
    gen = pipe_fill_generator(pipe, x_range=(0.0, seg_len), fill=0.999, velocity=(v0, 0.0, 0.0),
                              sigma=sigma, seed=seed)
    pos, vel = generate(gen, n, pipe=pipe, device=device)
    return SceneSpec(params, const, 'PIPE'), pos, vel
