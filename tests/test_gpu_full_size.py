"""The benchmark's own scene at full size: the 4,194,304-particle dam-break box
(spacing 0.005, h 0.0112, [0,2]^3 box, a 5.7 M-voxel table).  One fused step
against the FP64 oracle's step of the same input over every particle; the
fused step (warp-cooperative density pass, forces over its neighbour list)
against the stage-by-stage path (thread walks) bit for bit; and the
host-buffer entry point against the device-resident path bit for bit, in both
force-pass orders."""
import numpy as np
import pytest

from gpu_util import run_stages, torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def config2():
    from sphgb import scenes
    spec, st = scenes.config2()
    assert spec.params.particle_count == 4_194_304
    return spec, st


@pytest.fixture(scope="module")
def fused(config2):
    torch_cuda()
    from sphgb.device import SceneBatch
    spec, st = config2
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(1)
    out = b.states()[0]
    b.close()
    return out


def test_full_size_step_matches_oracle(config2, fused):
    """Tolerances as for the small scenes: density 1e-5 relative, position 1e-6
    absolute, velocity 2e-4 of the largest (the force is a difference of terms
    of similar size, so a relative bound per particle means nothing)."""
    spec, st = config2
    sp = ref.params_from_spec(spec)
    pos, vel, rho = ref.step(sp, st.position, st.velocity, step_index=0)
    assert np.all(np.isfinite(fused.density)) and np.all(np.isfinite(fused.position))
    assert np.max(np.abs(fused.density - rho) / rho) < 1e-5
    assert np.max(np.abs(fused.position - pos)) < 1e-6
    assert np.max(np.abs(fused.velocity - vel)) < 2e-4 * (np.abs(vel).max() + 1.0)


def test_full_size_fused_step_bit_identical_to_stages(config2, fused):
    spec, st = config2
    g = run_stages(spec, st.position, st.velocity, step=0)
    np.testing.assert_array_equal(fused.density, g["density"])
    np.testing.assert_array_equal(fused.velocity, g["velocity_out"])
    np.testing.assert_array_equal(fused.position, g["position_out"])


@pytest.mark.parametrize("order", ["slot", "particle"])
def test_full_size_host_entry_bit_identical_to_device_path(config2, fused, order):
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st = config2
    host = SceneBatch([spec])
    host.set_host_order({"slot": _capi.HOST_ORDER_SLOT, "particle": _capi.HOST_ORDER_PARTICLE}[order])
    pos, vel, rho = host.compute_next_state_host(st.position, st.velocity)
    host.close()
    np.testing.assert_array_equal(pos, fused.position)
    np.testing.assert_array_equal(vel, fused.velocity)
    np.testing.assert_array_equal(rho, fused.density)
