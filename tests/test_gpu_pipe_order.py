"""The pipelined order of the host-buffer entry point on seeded random scenes:
the same bits as loading the state and stepping it on the device, over two
calls in a row (the second starts from the first's output).

The scenes are lattice blocks of random sizes (at least 512 particles, so
the order applies) and spacings, with random velocities, in four kinds:
- as generated (particle ids follow space: each bucket depends on the next);
- with the particle ids shuffled (every bucket depends on the last one, and
  the downloads wait for the whole density pass);
- with host-made non-finite and out-of-box positions (the overflow entry
  keeps arrival order, so a range can complete only with a later bucket);
- with a quarter of the particles in one dense cluster (the big-voxel sort,
  capped lists).
"""
import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu

KINDS = ["lattice", "shuffled", "nonfinite", "cluster"]


def _case(kind, seed):
    from sphgb import scenes
    from sphgb.data_classes import SimulationState
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers(8, 19, size=3))
    spacing = float(rng.uniform(0.015, 0.03))
    spec, st = scenes.box_dam_break(nx=nx, ny=ny, nz=nz, spacing=spacing, jitter=spacing / 10,
                                    seed=seed)
    pos = st.position.copy()
    n = len(pos)
    vel = rng.normal(0.0, 0.1, size=(n, 3))
    if kind == "shuffled":
        perm = rng.permutation(n)
        pos, vel = pos[perm], vel[perm]
    elif kind == "nonfinite":
        k = rng.choice(n, size=max(3, n // 100), replace=False)
        pos[k[0::3], 0] = np.nan
        pos[k[1::3], 1] = np.inf
        pos[k[2::3], 2] = 5.0            # outside the unit box
    elif kind == "cluster":
        k = rng.choice(n, size=n // 4, replace=False)
        pos[k] = pos[k[0]] + rng.uniform(-1e-3, 1e-3, size=(len(k), 3))
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    return spec, SimulationState(f32(pos), f32(vel), np.zeros(n))


@pytest.mark.parametrize("seed", [101, 202])
@pytest.mark.parametrize("kind", KINDS)
def test_pipelined_order_bit_identical_on_random_scenes(kind, seed):
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st = _case(kind, seed)
    assert spec.params.particle_count >= 512
    dev = SceneBatch([spec])
    dev.load_states([st])
    host = SceneBatch([spec])
    host.set_host_order(_capi.HOST_ORDER_PIPELINED)
    pos, vel = st.position, st.velocity
    for call in range(2):
        dev.step(1)
        want = dev.states()[0]
        pos, vel, rho = host.compute_next_state_host(pos, vel)
        for got, ref, what in ((pos, want.position, "position"), (vel, want.velocity, "velocity"),
                               (rho, want.density, "density")):
            np.testing.assert_array_equal(got, ref, err_msg=f"{kind} seed {seed} call {call} {what}")
    dev.close()
    host.close()
