"""Empty and tiny scenes on the GPU: a scene of no particles (alone, through
the host-buffer entry point, and inside a batch of others), and scenes of one
and two particles against the FP64 oracle.  A lone particle has density 0, so
its step divides by zero exactly as the reference's does
(base_kernels.py:46-52): the infinities and NaNs must land in the same places."""
import numpy as np
import pytest

from gpu_util import torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu


def _box(n_per_axis, seed):
    from sphgb import scenes
    nx, ny, nz = n_per_axis
    return scenes.box_dam_break(nx=nx, ny=ny, nz=nz, seed=seed)


def test_empty_scene_alone():
    torch_cuda()
    from sphgb.device import SceneBatch
    spec, st = _box((0, 0, 0), seed=1)
    assert spec.n == 0
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(3)
    b.step(2, use_graph=True)
    out = b.states()[0]
    assert out.position.shape == (0, 3) and out.velocity.shape == (0, 3)
    assert out.density.shape == (0,)
    pos, vel, rho = b.compute_next_state_host(st.position, st.velocity)
    assert pos.shape == (0, 3) and rho.shape == (0,)
    b.close()


def test_batch_with_empty_scene_matches_alone():
    """An empty scene between two others changes nothing for them."""
    torch_cuda()
    from sphgb.device import SceneBatch
    picks = [_box((6, 12, 6), seed=2), _box((0, 0, 0), seed=3), _box((5, 9, 4), seed=4)]
    together = SceneBatch([p[0] for p in picks])
    together.load_states([p[1] for p in picks])
    together.step(3, use_graph=True)
    got = together.states()
    for k in (0, 2):
        alone = SceneBatch([picks[k][0]])
        alone.load_states([picks[k][1]])
        alone.step(3, use_graph=True)
        a = alone.states()[0]
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(a, f), getattr(got[k], f), err_msg=f"{k} {f}")
        alone.close()
    assert got[1].position.shape == (0, 3)
    together.close()


def _same_with_nonfinite(a, b, atol):
    """Equal non-finite pattern (NaN where NaN, the same infinities), finite
    values within atol."""
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    inf = np.isinf(a) | np.isinf(b)
    np.testing.assert_array_equal(a[inf], b[inf])
    fin = np.isfinite(a) & np.isfinite(b)
    assert np.all(np.abs(a[fin] - b[fin]) <= atol * (1.0 + np.abs(b[fin])))


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 1, 1)])
def test_one_and_two_particles_match_oracle(shape):
    torch_cuda()
    from sphgb.device import SceneBatch
    spec, st = _box(shape, seed=5)
    sp = ref.params_from_spec(spec)
    b = SceneBatch([spec])
    b.load_states([st])
    pos, vel = st.position.copy(), st.velocity.copy()
    for k in range(3):
        pos, vel, rho = ref.step(sp, pos, vel, step_index=k)
        b.step(1)
        g = b.states()[0]
        _same_with_nonfinite(g.density, rho, 1e-5)
        _same_with_nonfinite(g.velocity, vel, 1e-4)
        _same_with_nonfinite(g.position, pos, 1e-6)
    b.close()


def test_context_refuses_more_particles_than_its_index_range():
    """A context is limited to 2^29 particles (its kernels index per-particle
    FP64 rows in 32-bit arithmetic); one more is refused with SPHGB_ERR_RANGE
    before any allocation."""
    torch_cuda()
    import ctypes as C
    from sphgb import _capi
    from sphgb.device import scene_params
    spec, _ = _box((2, 2, 2), seed=6)
    lib = _capi.load()
    sp = scene_params(spec)
    sp.particle_count = (1 << 29) + 1
    ctx = C.c_void_p()
    rc = lib.sphgb_ctx_create(C.byref(sp), 1, None, 0, C.byref(ctx))
    assert rc == -5 and not ctx.value, (rc, _capi.last_error())
    assert "2^29" in _capi.last_error()
    # two scenes whose sum crosses the limit are refused the same way
    sps = (_capi.SceneParams * 2)(scene_params(spec), scene_params(spec))
    sps[0].particle_count = 1 << 28
    sps[1].particle_count = (1 << 28) + 1
    rc = lib.sphgb_ctx_create(sps, 2, None, 0, C.byref(ctx))
    assert rc == -5 and not ctx.value
