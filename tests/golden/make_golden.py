"""Generate golden vectors by running the reference's own step code on the CPU.

Usage (in a container that has the reference checked out read-only)::

    python tests/golden/make_golden.py /path/to/cuda-sph

It imports the reference (iwoplaza/cuda-sph) with ``numba_shim`` installed as
``numba``, so ``VoxelSPHStrategy.compute_next_state``
(``sim/src/sph/strategies/abstract_sph_strategy.py:31-46``) and the kernels it
launches (``sim/src/sph/kernels/{voxel,base,util}_kernels.py``) execute as
written, one simulated thread at a time.  Two minimal interventions are needed
to import the reference on Python >= 3.11 and are applied only while importing:

* ``common/data_classes.py:73-85`` uses ndarray dataclass defaults, which
  Python 3.11+ rejects; the ``dataclass`` decorator is wrapped to turn such
  defaults into ``default_factory`` copies (the values are unchanged).
* kernel constants are frozen from ``config`` at import time
  (``voxel_kernels.py:5``, ``base_kernels.py:2``); each case sets the constants
  on the ``config`` module (derived ones by the formulas of ``config.py:24-32``)
  and re-imports the kernel and strategy modules.

Each case stores, per step, the input state (FP32-representable doubles), the
reference's intermediates (voxel ids, the sorted voxel/particle map, voxel_begin,
the ordered neighbour list of ``get_neighbours``) and its outputs (density,
pressure term, viscosity term, result force, next position and velocity) in
``tests/golden/<case>.npz``.  It also runs the reference's own pipe-geometry
tests (``sim/tests/test_collisions.py``) under the shim and records their
inputs and outputs in ``tests/golden/pipe_kats.npz``.

The uncapped neighbour count is produced by the same ``get_neighbours`` with
``MAX_NEIGHBOURS`` raised to 4096.
"""
from __future__ import annotations

import dataclasses
import importlib
import math
import os
import sys
import unittest

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numba_shim  # noqa: E402

numba_shim.install()

REF_MODULES = [
    "sim.src.sph.kernels.util_kernels",
    "sim.src.sph.kernels.base_kernels",
    "sim.src.sph.kernels.voxel_kernels",
    "sim.src.sph.kernels.naive_kernels",
    "sim.src.sph.strategies.abstract_sph_strategy",
    "sim.src.sph.strategies.naive_sph_strategy",
    "sim.src.sph.strategies.voxel_sph_strategy",
    "sim.src.sph",
    "sim.src.sph.thread_layout",
]


def _import_reference(ref_root: str):
    sys.path.insert(0, ref_root)
    orig = dataclasses.dataclass

    def patched(cls=None, /, **kw):
        def wrap(c):
            for name, val in list(vars(c).items()):
                if isinstance(val, np.ndarray):
                    setattr(c, name, dataclasses.field(
                        default_factory=lambda v=val: v.copy()))
            return orig(c, **kw)
        return wrap if cls is None else wrap(cls)

    dataclasses.dataclass = patched
    try:
        import common.data_classes  # noqa: F401
        import config  # noqa: F401
    finally:
        dataclasses.dataclass = orig
    import common.pipe_builder  # noqa: F401
    return sys.modules["config"]


def _set_constants(config, *, mass, rho_0, inf_r, visc, k, damp, max_neighbours=32,
                   sim_mode="BOX"):
    """Constants as config.py:13-32 defines them (derived ones recomputed)."""
    config.SIM_MODE = sim_mode
    config.MASS = mass
    config.RHO_0 = rho_0
    config.INF_R = inf_r
    config.VISC = visc
    config.K = k
    config.DAMP = damp
    config.INF_R_2 = inf_r ** 2
    config.INF_R_6 = inf_r ** 6
    config.INF_R_9 = inf_r ** 9
    config.W_CONST = 315.0 / (64.0 * np.pi * config.INF_R_9)
    config.GRAD_W_CONST = -45.0 / (np.pi * config.INF_R_6)
    config.LAP_W_CONST = 45.0 / (np.pi * config.INF_R_6)
    config.MAX_NEIGHBOURS = max_neighbours
    config.NEIGHBOURING_VOXELS_COUNT = 27
    config.VOXEL_SIZE = [inf_r, inf_r, inf_r]


def _reload_kernels():
    for m in REF_MODULES:
        sys.modules.pop(m, None)
    # the package first, as sim/src/state_generator.py:6-9 does (its __init__
    # imports the strategies; importing a strategy module first is circular)
    importlib.import_module("sim.src.sph")
    vk = importlib.import_module("sim.src.sph.kernels.voxel_kernels")
    bk = importlib.import_module("sim.src.sph.kernels.base_kernels")
    vs = importlib.import_module("sim.src.sph.strategies.voxel_sph_strategy")
    return vk, bk, vs


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def _neighbour_lists(vk, strategy, position, cap):
    """Ordered neighbour list of every particle from the reference's get_neighbours."""
    from numba import cuda
    n = position.shape[0]
    out = np.full((n, cap), -1, dtype=np.int32)
    counts = np.zeros(n, dtype=np.int32)
    d_pos = cuda.to_device(position)

    def kernel(out, counts, position, voxel_size, space_dim, voxel_begin, vmap):
        i = cuda.blockIdx.x * cuda.blockDim.x + cuda.threadIdx.x
        if i >= position.shape[0]:
            return
        nb = cuda.local.array(cap, np.int32)
        c = vk.get_neighbours(nb, i, position, voxel_size, space_dim, voxel_begin, vmap)
        counts[i] = c
        for t in range(c):
            out[i, t] = nb[t]

    kern = cuda.jit(kernel)
    block = 128
    kern[(n + block - 1) // block, block](
        out, counts, d_pos, strategy.d_voxel_size, strategy.d_space_dim,
        strategy.d_voxel_begin, strategy.d_voxel_particle_map)
    return out, counts


def run_case(config, name, *, params_kw, consts, state, steps, mode="BOX", seed=16435234):
    from common.data_classes import SimulationParameters, SimulationState
    _set_constants(config, sim_mode=mode, **consts)
    vk, bk, vs = _reload_kernels()
    params = SimulationParameters(**params_kw)
    strat = vs.VoxelSPHStrategy(params)
    rec = {k: [] for k in (
        "position_in", "velocity_in", "voxel_ids", "map_voxel", "map_pid", "voxel_begin",
        "space_dim_walk", "neigh_list", "neigh_count", "neigh_count_uncapped",
        "density", "pressure_term", "viscosity_term", "result_force",
        "position_out", "velocity_out")}
    cur = state
    numba_shim.DeviceArray.oob_reads = 0
    for step in range(steps):
        numba_shim.set_rng_step(step)
        nxt = strat.compute_next_state(cur)
        rec["position_in"].append(np.array(cur.position))
        rec["velocity_in"].append(np.array(cur.velocity))
        rec["voxel_ids"].append(np.array(strat.voxels, dtype=np.int32))
        rec["map_voxel"].append(np.array(strat.voxel_particle_map["voxel_id"]))
        rec["map_pid"].append(np.array(strat.voxel_particle_map["particle_id"]))
        rec["voxel_begin"].append(np.array(strat.voxel_begin, dtype=np.int32))
        rec["space_dim_walk"].append(np.array(strat.space_dim, dtype=np.int32))
        nl, nc = _neighbour_lists(vk, strat, np.array(cur.position), config.MAX_NEIGHBOURS)
        rec["neigh_list"].append(nl)
        rec["neigh_count"].append(nc)
        rec["density"].append(strat.d_new_density.copy_to_host())
        rec["pressure_term"].append(strat.d_new_pressure_term.copy_to_host())
        rec["viscosity_term"].append(strat.d_new_viscosity_term.copy_to_host())
        rec["result_force"].append(np.array(strat.result_force))
        rec["position_out"].append(np.array(nxt.position))
        rec["velocity_out"].append(np.array(nxt.velocity))
        cur = SimulationState(f32(nxt.position), f32(nxt.velocity), np.array(nxt.density))
    # uncapped neighbour counts with the same code and MAX_NEIGHBOURS raised
    _set_constants(config, sim_mode=mode, **dict(consts, max_neighbours=4096))
    vk2, _, vs2 = _reload_kernels()
    for step in range(steps):
        s2 = vs2.VoxelSPHStrategy(params)
        s2.old_state = SimulationState(rec["position_in"][step], rec["velocity_in"][step],
                                       np.zeros(params.particle_count))
        s2._initialize_computation()
        _, nc = _neighbour_lists(vk2, s2, rec["position_in"][step], 4096)
        rec["neigh_count_uncapped"].append(nc)
    pipe_rows = params.pipe.to_numpy() if mode == "PIPE" else np.zeros((0, 5))
    out = {k: np.stack(v) for k, v in rec.items()}
    out.update(
        mode=np.array(mode),
        space_size=np.asarray(params.space_size, dtype=np.float64),
        voxel_size=np.asarray(params.voxel_size, dtype=np.float64),
        external_force=np.asarray(params.external_force, dtype=np.float64),
        fps=np.array(params.fps, dtype=np.float64),
        dt=np.array(strat.dt, dtype=np.float64),
        mass=np.array(consts["mass"]), rho_0=np.array(consts["rho_0"]),
        inf_r=np.array(consts["inf_r"]), visc=np.array(consts["visc"]),
        k=np.array(consts["k"]), damp=np.array(consts["damp"]),
        max_neighbours=np.array(32), pipe_rows=pipe_rows, seed=np.array(seed, dtype=np.uint64),
        oob_reads=np.array(numba_shim.DeviceArray.oob_reads),
    )
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: N={params.particle_count} steps={steps} "
          f"oob_reads={numba_shim.DeviceArray.oob_reads} -> {os.path.relpath(path)}")


def lattice_state(nx, ny, nz, spacing, jitter, seed):
    rng = np.random.default_rng(seed)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([ix, iy, iz], axis=-1).reshape(-1, 3).astype(np.float64)
    pos = (base + 0.5) * spacing + rng.uniform(-jitter, jitter, size=base.shape)
    return f32(pos), np.zeros_like(pos)


def pipe_state(pipe, n, seed, space):
    rng = np.random.default_rng(seed)
    length = pipe.get_length()
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    for i in range(n):
        x = rng.uniform(0.0, length)
        r_max = pipe.radius_at(x)
        r = math.sqrt(rng.uniform()) * r_max * 0.98
        th = rng.uniform() * 2.0 * math.pi
        c = pipe.segments[0].start_point
        pos[i] = (x, c[1] + r * math.cos(th), c[2] + r * math.sin(th))
    vel[:, 0] = rng.uniform(-30.0, 60.0, n)
    vel[:, 1:] = rng.uniform(-20.0, 20.0, (n, 2))
    return f32(pos), f32(vel)


def collision_kats():
    """Run sim/tests/test_collisions.py under the shim and record its vectors."""
    _reload_kernels()
    sys.modules.pop("sim.tests.test_collisions", None)
    tc = importlib.import_module("sim.tests.test_collisions")
    suite = unittest.defaultTestLoader.loadTestsFromTestCase(tc.CollisionTests)
    res = unittest.TextTestRunner(verbosity=0, stream=open(os.devnull, "w")).run(suite)
    print(f"reference test_collisions under the shim: ran={res.testsRun} "
          f"failures={len(res.failures)} errors={len(res.errors)}")
    if res.failures or res.errors:
        for _, tb in res.failures + res.errors:
            print(tb)
        raise SystemExit("reference KATs do not pass under the shim")
    # recorded vectors: the same inputs the tests use, outputs from the same kernels
    from common.pipe_builder import PipeBuilder
    from numba import cuda
    bk = sys.modules["sim.src.sph.kernels.base_kernels"]
    out = {}
    pipe = PipeBuilder().add_roller_segment(1.0).add_increasing_segment(1.0, 3.0).get_result().to_numpy()
    pos = np.array([[-0.1, 0, 2], [0.5, 3, 4], [1, 0, 0], [2.5, 0, -5], [5, 5, 5]], dtype=np.float64)
    seg = np.array([bk.find_segment(p, pipe) for p in pos], dtype=np.int32)
    out.update(find_segment_pipe=pipe, find_segment_pos=pos, find_segment_out=seg)
    pipe2 = PipeBuilder().add_increasing_segment(4, 1).add_lessening_segment(6, 1.5).get_result().to_numpy()
    xb = np.array([bk.calc_x_at_segment_beginning(pipe2, s) for s in (0, 1, 2)])
    out.update(x_begin_pipe=pipe2, x_begin_out=xb)
    pipe3 = PipeBuilder().add_increasing_segment(1, 1).add_lessening_segment(1, 1.5).get_result().to_numpy()
    pos3 = np.array([[0.5, 0.5, 0.5], [0.76, 0.9, 0.9], [0.01, 1, 0.5], [1.25, 0.8, 0.8],
                     [1.5, 1.25, 1.40], [1.99, 1.3, 1.6], [2.2, 1, 1], [2.6, 1, 1],
                     [2.95, 0.2, 0.2]], dtype=np.float64)
    segs3 = np.array([0, 0, 0, 1, 1, 1, 2, 2, 2], dtype=np.int32)
    iso = np.array([bool(bk.is_out_of_pipe(p, pipe3, s)) for p, s in zip(pos3, segs3)])
    rad = np.array([bk.calc_radius_in_position(p, pipe3, s) for p, s in zip(pos3, segs3)])
    out.update(is_out_pipe=pipe3, is_out_pos=pos3, is_out_seg=segs3, is_out_out=iso, radius_out=rad)
    pipe4 = PipeBuilder().add_increasing_segment(1, 1).add_lessening_segment(2, 1.5).get_result().to_numpy()
    # collision resolution: the test's own case plus a spread of outside points
    rng = np.random.default_rng(7)
    cp = [np.array([1.3, 1.5, 0.0])]
    cv = [np.array([-0.5, 0.0, 0.0])]
    while len(cp) < 64:
        x = rng.uniform(0.05, 3.95)
        s = bk.find_segment(np.array([x, 0, 0]), pipe4)
        R = bk.calc_radius_in_position(np.array([x, 0, 0]), pipe4, s)
        th = rng.uniform(0, 2 * math.pi)
        r = R * rng.uniform(1.01, 1.3)
        p = np.array([x, r * math.cos(th), r * math.sin(th)])
        v = rng.uniform(-1, 1, 3)
        v[1:] += 0.5 * np.array([math.cos(th), math.sin(th)])
        cp.append(p)
        cv.append(v)
    cp = np.array(cp)
    cv = np.array(cv)
    cp_out = cp.copy()
    cv_out = cv.copy()
    cseg = np.zeros(len(cp), dtype=np.int32)
    cout = np.zeros(len(cp), dtype=bool)
    for i in range(len(cp)):
        cseg[i] = bk.find_segment(cp_out[i], pipe4)
        if bk.is_out_of_pipe(cp_out[i], pipe4, cseg[i]):
            bk.solve_collision(cp_out[i], cv_out[i], pipe4, cseg[i])
        cout[i] = bk.is_out_of_pipe(cp_out[i], pipe4, cseg[i])
    out.update(collide_pipe=pipe4, collide_pos_in=cp, collide_vel_in=cv,
               collide_seg=cseg, collide_pos_out=cp_out, collide_vel_out=cv_out,
               collide_still_out=cout)
    path = os.path.join(HERE, "pipe_kats.npz")
    np.savez_compressed(path, **out)
    print(f"pipe KATs -> {os.path.relpath(path)}")


def main(ref_root):
    config = _import_reference(ref_root)
    from common.data_classes import SimulationState, Pipe, Segment
    from common.pipe_builder import PipeBuilder

    collision_kats()

    c0 = dict(mass=float(np.float32(0.008)), rho_0=1000.0, inf_r=float(np.float32(0.045)),
              visc=3.5, k=3.0, damp=0.5)
    # (1) config-0-like dam break in a box whose size is not a multiple of h:
    #     the reference walks truncated dims (voxel_sph_strategy.py:110-116)
    pos, vel = lattice_state(8, 12, 6, 0.02, 0.002, seed=100)
    h = c0["inf_r"]
    # one step only: most particles then walk the wrong cells, find no neighbour,
    # get density 0 and leave the step with non-finite velocity and position
    run_case(config, "box_unaligned", consts=c0, state=SimulationState(pos, vel, np.zeros(len(pos))),
             steps=1, params_kw=dict(
                 particle_count=len(pos), external_force=np.array([0.0, -9.81, 0.0]),
                 duration=1, fps=2000, pipe=Pipe([Segment()]),
                 space_size=f32([0.5, 0.5, 0.5]), voxel_size=np.array([h, h, h])))
    # (2) same lattice density with the box an exact multiple of h: ceil == truncated dims
    h2 = 0.0625
    s2 = h2 / 2.25
    ca = dict(mass=float(np.float32(1000.0 * s2 ** 3)), rho_0=1000.0, inf_r=h2,
              visc=3.5, k=3.0, damp=0.5)
    pos, vel = lattice_state(8, 12, 6, s2, s2 / 10.0, seed=101)
    run_case(config, "box_aligned", consts=ca, state=SimulationState(pos, vel, np.zeros(len(pos))),
             steps=3, params_kw=dict(
                 particle_count=len(pos), external_force=np.array([0.0, -9.81, 0.0]),
                 duration=1, fps=2000, pipe=Pipe([Segment()]),
                 space_size=np.array([0.5, 0.5, 0.5]), voxel_size=np.array([h2, h2, h2])))
    # (3) the reference's own default constants (config.py:15-35), box wall start
    #     state distribution of config.py:79-97 (seeded, FP32-rounded), smaller box
    rng = np.random.default_rng(102)
    n = 600
    box = [10.0, 10.0, 10.0]
    pos = rng.random((n, 3))
    pos[:, 0] *= box[0] * 0.1
    pos[:, 1] *= box[1]
    pos[:, 2] *= box[2]
    vel = np.array([1.5, -5.0, -5.0]) + (rng.random((n, 3)) - 0.5) * 1.0
    cd = dict(mass=1.0, rho_0=1.0, inf_r=2.0, visc=0.5, k=10.0, damp=0.7)
    run_case(config, "box_defaults", consts=cd,
             state=SimulationState(f32(pos), f32(vel), np.zeros(n)), steps=2,
             params_kw=dict(particle_count=n, external_force=np.array([0.0, -2.0, 0.0]),
                            duration=1, fps=20, pipe=Pipe([Segment()]),
                            space_size=np.array(box), voxel_size=np.array([2.0, 2.0, 2.0])))
    # (4) pipe enclosure built exactly as config.py:68-76 (PIPE_SPACE_SIZE = 20h x 3h x 3h)
    pipe = (PipeBuilder().with_starting_radius(1).add_roller_segment(1)
            .add_increasing_segment(1, 1.2).add_roller_segment(1)
            .add_lessening_segment(1, 1.2).add_roller_segment(1)
            .transform(40.0, 6.0).get_result())
    n = 500
    pos, vel = pipe_state(pipe, n, seed=103, space=[40.0, 6.0, 6.0])
    run_case(config, "pipe_defaults", consts=cd, mode="PIPE",
             state=SimulationState(pos, vel, np.zeros(n)), steps=2,
             params_kw=dict(particle_count=n, external_force=np.array([2.0, 0.0, 0.0]),
                            duration=1, fps=20, pipe=pipe,
                            space_size=np.array([40.0, 6.0, 6.0]),
                            voxel_size=np.array([2.0, 2.0, 2.0])))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py /path/to/cuda-sph")
    main(sys.argv[1])
