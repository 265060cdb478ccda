"""The fused, device-resident step (SceneBatch / sphgb_ctx_step): identical to
the stage-by-stage path, to its CUDA-graph replay, alone or batched, and
within FP32 tolerance of the oracle through the host-buffer entry point."""
import numpy as np
import pytest

from gpu_util import run_stages, torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu


def _scenes():
    from sphgb import scenes
    return {
        "config0": scenes.config0(),
        "pipe": scenes.pipe_flow(n=20_000, seed=11, h=0.02 * (262_144 / 20_000) ** (1 / 3)),
        "uncapped": scenes.box_dam_break(nx=10, ny=20, nz=10, max_neighbours=0, seed=4),
        "truncated": scenes.box_dam_break(nx=10, ny=20, nz=10, box=(0.7, 0.7, 0.7),
                                          walk_dims='truncated', seed=5),
        # lattice spacing above h: about one particle in five has no neighbour,
        # density 0 and non-finite force factors, so the force pass defers it
        # to its second launch (the plain re-sum)
        "sparse": scenes.box_dam_break(nx=8, ny=8, nz=8, spacing=0.05, jitter=0.01, seed=6),
    }


@pytest.mark.parametrize("name", ["config0", "pipe", "uncapped", "truncated", "sparse"])
def test_fused_step_bit_identical_to_stages(name):
    """The fused step reads the density pass's neighbour list; the stage path
    walks again.  Same neighbours, order and arithmetic: identical bits.  The
    uncapped and sparse scenes send particles through the force pass's second
    launch (a walk, the plain re-sum); the stage path has one launch."""
    torch_cuda()
    from sphgb.device import SceneBatch
    spec, st = _scenes()[name]
    g = run_stages(spec, st.position, st.velocity, step=0)
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(1)
    out = b.states()[0]
    np.testing.assert_array_equal(out.density, g["density"])
    np.testing.assert_array_equal(out.velocity, g["velocity_out"])
    np.testing.assert_array_equal(out.position, g["position_out"])
    b.close()


def test_graph_replay_equals_eager():
    torch_cuda()
    from sphgb.device import SceneBatch
    spec, st = _scenes()["config0"]
    outs = []
    for use_graph in (False, True):
        b = SceneBatch([spec])
        b.load_states([st])
        for _ in range(3):
            b.step(2, use_graph=use_graph)
        outs.append(b.states()[0])
        b.close()
    for f in ("position", "velocity", "density"):
        np.testing.assert_array_equal(getattr(outs[0], f), getattr(outs[1], f))


def test_batched_scenes_identical_to_alone():
    """Scenes advanced together give bit-identical states and conservation sums
    to each scene advanced alone (different constants, modes and sizes)."""
    torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    picks = [_scenes()["config0"], _scenes()["pipe"],
             scenes.box_dam_break(nx=6, ny=12, nz=6, spacing=0.03, h=0.0675, mass=0.027, seed=9,
                                  gravity=(1.0, -9.0, 3.0))]
    together = SceneBatch([p[0] for p in picks])
    together.load_states([p[1] for p in picks])
    together.step(4, use_graph=True)
    t_states = together.states()
    t_cons = together.conservation()
    for k, (spec, st) in enumerate(picks):
        alone = SceneBatch([spec])
        alone.load_states([st])
        alone.step(4, use_graph=True)
        a = alone.states()[0]
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(a, f), getattr(t_states[k], f), err_msg=f"{k} {f}")
        np.testing.assert_array_equal(alone.conservation()[0], t_cons[k])
        alone.close()
    together.close()


def test_host_entry_matches_oracle():
    """sphgb_compute_next_state_host (FP64 AoS host buffers in and out) against
    the oracle's step on the same input."""
    torch_cuda()
    from sphgb.strategies import GB300SPHStrategy
    spec, st = _scenes()["config0"]
    strat = GB300SPHStrategy(spec.params, constants=spec.constants, mode=spec.mode)
    out = strat.compute_next_state(st)
    sp = ref.params_from_spec(spec)
    pos, vel, rho = ref.step(sp, st.position, st.velocity, step_index=0)
    assert np.max(np.abs(out.density - rho) / rho) < 1e-5
    assert np.max(np.abs(out.position - pos)) < 1e-6
    # velocities: cancellation in F makes a relative bound meaningless; bound by
    # the term scale like the stage tests (here via the step's own magnitude)
    assert np.max(np.abs(out.velocity - vel)) < 2e-4 * (np.abs(vel).max() + 1.0)
    # the strategy keeps the reference's attributes
    assert strat.old_state is st and strat.new_state is out and strat.dt == 1 / spec.params.fps


@pytest.mark.parametrize("order", ["slot", "particle", "pipelined", "auto"])
@pytest.mark.parametrize("name", ["config0", "pipe", "sparse", "uncapped", "truncated"])
def test_host_entry_bit_identical_to_device_path(name, order):
    """Calls of sphgb_compute_next_state_host in a row (uploads and downloads
    spread over streams; the force pass in slot order, in particle-order
    ranges, in ranges pipelined behind a density pass in buckets, or chosen by
    timing all three) give the same bits as loading the state and stepping it
    on the device.  The uncapped and truncated scenes cannot be pipelined and
    fall back to particle order."""
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st = _scenes()[name]
    dev = SceneBatch([spec])
    dev.load_states([st])
    host = SceneBatch([spec])
    host.set_host_order({"slot": _capi.HOST_ORDER_SLOT, "particle": _capi.HOST_ORDER_PARTICLE,
                         "pipelined": _capi.HOST_ORDER_PIPELINED,
                         "auto": _capi.HOST_ORDER_AUTO}[order])
    pos, vel = st.position, st.velocity
    for _ in range(8 if order == "auto" else 2):   # auto: three orders run, timed, then chosen
        dev.step(1)
        want = dev.states()[0]
        pos, vel, rho = host.compute_next_state_host(pos, vel)
        np.testing.assert_array_equal(pos, want.position)
        np.testing.assert_array_equal(vel, want.velocity)
        np.testing.assert_array_equal(rho, want.density)
    dev.close()
    host.close()


@pytest.mark.parametrize("shape", [(3, 7, 5), (1, 5, 1), (9, 11, 7)])
def test_host_entry_particle_ranges_uneven_counts(shape):
    """Particle-order ranges when the particle count does not split evenly
    into the ranges (105 particles), or is below their number (5 particles:
    some ranges empty): same bits as the slot-order call.  The pipelined
    order runs on 693 particles (uneven ranges and buckets) and falls back to
    particle order on the two smaller scenes."""
    torch_cuda()
    from sphgb import _capi, scenes
    from sphgb.device import SceneBatch
    nx, ny, nz = shape
    spec, st = scenes.box_dam_break(nx=nx, ny=ny, nz=nz, seed=21)
    outs = []
    for order in (_capi.HOST_ORDER_SLOT, _capi.HOST_ORDER_PARTICLE, _capi.HOST_ORDER_PIPELINED):
        b = SceneBatch([spec])
        b.set_host_order(order)
        outs.append(b.compute_next_state_host(st.position, st.velocity))
        b.close()
    for other in outs[1:]:
        for a, c in zip(outs[0], other):
            np.testing.assert_array_equal(a, c)


def test_trajectory_config0_200_steps():
    """200 free-running fused steps of the 8,192-particle dam break, every
    step pinned by a shadow step of the FP64 oracle: from the GPU's own state
    before step k, the oracle computes step k, and the GPU's step k must match
    it with the tolerances of a single step (test_gpu_parity): the neighbour
    rows the step's force pass read and their counts bit for bit, density
    1e-5, next velocity and position within the bounds of the term scales.
    Particles whose box wall response fired on one side only (an FP32 and an
    FP64 position on either side of a wall) may differ by the reflection; at
    most 2 per step and 10 over the run.

    The two trajectories themselves separate over time, because the
    reference's capped walk makes the dynamics chaotic (a pair crossing r = h
    changes which particle is the 32nd neighbour); their distance is printed
    as information, with only loose statistical bounds."""
    torch_cuda()
    from sphgb.device import SceneBatch
    from test_gpu_parity import oracle_step_dict, rho_one, step_errors
    from test_gpu_full_size import _lists_without_self
    spec, st = _scenes()["config0"]
    sp = ref.params_from_spec(spec)
    b = SceneBatch([spec])
    b.load_states([st])
    pos, vel = st.position.copy(), st.velocity.copy()     # free-running oracle
    n = len(pos)
    space = np.asarray(sp.space_size[:])
    cur = b.states()[0]
    flips_total = 0
    for k in range(200):
        # shadow: the oracle's step k from the GPU's own state
        gpos = np.asarray(cur.position, dtype=np.float64)
        gvel = np.asarray(cur.velocity, dtype=np.float64)
        exp, scales, _ = oracle_step_dict(spec, gpos, gvel, step=k)
        b.step(1)
        nxt = b.states()[0]
        lst, cnt = (t.cpu().numpy() for t in b.step_neighbours())
        ok = np.isfinite(gpos).all(1) & np.all((gpos >= 0) & (gpos < space), axis=1)
        want, kk = _lists_without_self(exp["neigh_list"])
        np.testing.assert_array_equal(cnt[ok], kk[ok], err_msg=f"step {k}")
        np.testing.assert_array_equal(lst[ok], want[ok], err_msg=f"step {k}")
        g = {"density": nxt.density, "velocity_out": nxt.velocity, "position_out": nxt.position}
        for what in ("velocity_out", "position_out"):
            fa, fb = np.isfinite(g[what][ok]), np.isfinite(exp[what][ok])
            assert np.array_equal(fa, fb), (k, what, "non-finite pattern")
        e_rho, _, _, nv, nx = step_errors(g, exp, ok, scales, sp.dt, list(sp.external_force),
                                          sp.inf_r, None, rho_one(spec))
        assert e_rho < 1e-5, (k, e_rho)
        over = (nv.max(axis=1) > 1.0) | (nx.max(axis=1) > 1.0)
        if over.any():
            # only particles the wall response moved on one side may differ
            x_in = gpos[ok][over]
            free_g = np.all(np.abs(x_in + nxt.velocity[ok][over] * sp.dt
                                   - nxt.position[ok][over]) <= 1e-6, axis=1)
            free_o = np.all(np.abs(x_in + exp["velocity_out"][ok][over] * sp.dt
                                   - exp["position_out"][ok][over]) <= 1e-6, axis=1)
            assert not np.any(free_g & free_o), (k, "off-wall particle outside its bound")
            flips_total += int(over.sum())
            assert over.sum() <= 2, (k, int(over.sum()))
        cur = nxt
        # free-running comparison, information only
        pos, vel, rho = ref.step(sp, pos, vel, step_index=k)
        step = k + 1
        if step in (1, 10, 50, 100, 150, 200):
            fin = np.isfinite(nxt.position).all(1) & np.isfinite(pos).all(1)
            dx = np.linalg.norm(nxt.position - pos, axis=1)[fin]
            drho = abs(nxt.density.mean() - rho.mean()) / rho.mean()
            print(f"step {step}: shadow rho {e_rho:.1e}, vel/bound {nv.max():.2f}, "
                  f"pos/bound {nx.max():.2f}; free-running |dx| median {np.median(dx):.2e} "
                  f"max {dx.max():.2e}, mean rho rel diff {drho:.1e}, non-finite gpu "
                  f"{n - np.isfinite(nxt.position).all(1).sum()}")
            assert drho < 1e-2 and (~fin).sum() <= 0.01 * n
    assert flips_total <= 10
    b.close()


def test_conservation_sums_match_fp64_sums_of_the_state():
    """sphgb_ctx_conservation (FP64, fixed order) against numpy FP64 sums of
    the same state: relative 1e-12 (only the summation order differs).  Two
    boxes after three steps and a pipe flow as loaded (the pipe's FP64
    position accumulator is what is summed)."""
    torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    boxes = [scenes.config0(), scenes.box_dam_break(nx=10, ny=20, nz=10, seed=4,
                                                   gravity=(1.0, -9.0, 3.0))]
    pipe = [scenes.pipe_flow(n=20_000, seed=11, h=0.02 * (262_144 / 20_000) ** (1 / 3))]
    for pairs, steps in ((boxes, 3), (pipe, 0)):
        b = SceneBatch([s for s, _ in pairs])
        b.load_states([st for _, st in pairs])
        b.step(steps)
        cons = b.conservation()
        states = b.states()
        for k, (spec, _) in enumerate(pairs):
            st = states[k]
            assert np.isfinite(st.position).all() and np.isfinite(st.velocity).all()
            m = np.float64(np.float32(spec.constants.mass))
            g = np.asarray(spec.params.external_force, dtype=np.float32).astype(np.float64)
            v2 = (st.velocity ** 2).sum(1)
            pot = -m * (st.position @ g)
            want = np.array([m * spec.n, *(m * st.velocity.sum(0)), 0.5 * m * v2.sum(),
                             pot.sum(), 0.5 * m * v2.sum() + pot.sum(), spec.n])
            scale = np.array([m * spec.n] + [m * np.abs(st.velocity).sum() + 1e-300] * 3
                             + [0.5 * m * v2.sum() + 1e-300] + [np.abs(pot).sum() + 1e-300]
                             + [np.abs(pot).sum() + 0.5 * m * v2.sum() + 1e-300] + [spec.n])
            err = np.abs(cons[k] - want) / scale
            assert err.max() < 1e-12, (k, cons[k], want)
        b.close()


@pytest.mark.parametrize("name", ["config0", "pipe", "uncapped", "truncated"])
def test_density_variants_bit_identical(name):
    """The two density kernels (warp per voxel run with a lane per
    candidate, thread per particle) keep the same neighbours in the same order and sum
    them the same way: identical states after several steps."""
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st = _scenes()[name]
    outs = []
    for variant in (_capi.DENSITY_WARP, _capi.DENSITY_THREAD):
        b = SceneBatch([spec])
        b.set_tuning(256, variant, 64)
        b.load_states([st])
        b.step(4, use_graph=True)
        outs.append(b.states()[0])
        b.close()
    for o in outs[1:]:
        np.testing.assert_array_equal(o.density, outs[0].density)
        np.testing.assert_array_equal(o.velocity, outs[0].velocity)
        np.testing.assert_array_equal(o.position, outs[0].position)


def test_density_variants_identical_on_dense_voxels():
    """Voxels far above 32 particles (many tasks per voxel, thousands of
    candidates per walk, several staged chunks) and a scene whose block
    starts at a voxel boundary."""
    torch_cuda()
    from sphgb import _capi, scenes
    from sphgb.device import SceneBatch
    cases = [scenes.box_dam_break(nx=24, ny=24, nz=24, spacing=0.004, jitter=0.0004,
                                  h=0.03, mass=6.4e-5, seed=12),
             scenes.pipe_flow(n=30_000, seed=13, h=0.02)]
    for spec, st in cases:
        outs = []
        for variant in (_capi.DENSITY_WARP, _capi.DENSITY_THREAD):
            b = SceneBatch([spec])
            b.set_tuning(256, variant, 64)
            b.load_states([st])
            b.step(2)
            outs.append(b.states()[0])
            b.close()
        for o in outs[1:]:
            np.testing.assert_array_equal(o.density, outs[0].density)
            np.testing.assert_array_equal(o.velocity, outs[0].velocity)


def test_host_entry_page_locked_buffers_match_pageable():
    """sphgb_compute_next_state_host gives the same bits from page-locked
    host arrays as from pageable ones."""
    torch = torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    for spec, st in (scenes.config0(), scenes.pipe_flow(n=20_000, seed=11,
                                                         h=0.02 * (262_144 / 20_000) ** (1 / 3))):
        n = spec.n
        # a fresh context for each call: the step index keys the pipe's respawn draws
        a = SceneBatch([spec])
        pageable = a.compute_next_state_host(np.array(st.position), np.array(st.velocity))
        a.close()
        b = SceneBatch([spec])
        pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()  # noqa
        hp, hv = pin((n, 3)), pin((n, 3))
        hp[:] = st.position
        hv[:] = st.velocity
        op, ov, orho = pin((n, 3)), pin((n, 3)), pin((n,))
        locked = b.compute_next_state_host(hp, hv, op, ov, orho)
        for a, c in zip(pageable, locked):
            np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(op, pageable[0])
        np.testing.assert_array_equal(orho, pageable[2])
        b.close()


def test_host_order_rejects_unknown_values():
    """sphgb_ctx_set_host_order takes AUTO, SLOT, PARTICLE or PIPELINED only; a refused
    value leaves the context usable and its results unchanged."""
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st = _scenes()["config0"]
    b = SceneBatch([spec])
    with pytest.raises(_capi.SphgbError, match="order must be") as e:
        b.set_host_order(7)
    assert e.value.code == -1
    ref_b = SceneBatch([spec])
    got = b.compute_next_state_host(st.position, st.velocity)
    want = ref_b.compute_next_state_host(st.position, st.velocity)
    for a, c in zip(got, want):
        np.testing.assert_array_equal(a, c)
    b.close()
    ref_b.close()
