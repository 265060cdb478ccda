"""Start states generated on the device (sphgb_generate) and the headless
point-field vertex stage (sphgb_point_field), against the oracle.

Lattice and box-wall states use only Philox uniforms, additions and
multiplications: bit-identical to the oracle.  The pipe fill and normal
deviates call cos, sin and log, whose last bit may differ between CUDA's and
the C library's implementations: positions within 1e-15 m (radii ~0.1 m,
about 10 ulp) or 2e-15 relative, velocities within 1e-14 m/s.  The point field is FP32 with one
rounding per operation in both: bit-identical.
"""
import numpy as np
import pytest

from gpu_util import torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu

TOL_TRIG_POS = 1e-15    # absolute, metres
TOL_TRIG_VEL = 1e-14    # absolute, m/s
TOL_TRIG_REL = 2e-15    # relative to the pipe radius, for radii far from 1 (about 8 ulp)


def _np(t):
    return t.cpu().numpy()


def _oracle_gen(g_capi):
    """The same generator as an oracle struct."""
    g = ref.Generator()
    for name, _ in ref.Generator._fields_:
        v = getattr(g_capi, name)
        if hasattr(v, "__len__"):
            getattr(g, name)[:] = list(v)
        else:
            setattr(g, name, v)
    return g


def test_lattice_bit_identical_to_oracle_at_4m():
    torch_cuda()
    from sphgb import generate as G
    g = G.lattice_generator(128, 256, 128, 0.005, 0.0005, seed=2)
    n = 128 * 256 * 128
    pos, vel = G.generate(g, n)
    rp, rv = ref.generate(_oracle_gen(g), n)
    np.testing.assert_array_equal(_np(pos), rp)
    np.testing.assert_array_equal(_np(vel), rv)
    # every particle within the jitter of its lattice site
    i = np.arange(n)
    site = (np.stack([i // (256 * 128), (i // 128) % 256, i % 128], 1) + 0.5) * 0.005
    assert np.abs(rp - site).max() <= 0.0005 * (1 + 1e-12)


def test_box_wall_bit_identical_to_oracle():
    torch_cuda()
    from sphgb import generate as G
    g = G.box_wall_generator((40.0, 20.0, 20.0), seed=9)
    pos, vel = G.generate(g, 200_000)
    rp, rv = ref.generate(_oracle_gen(g), 200_000)
    np.testing.assert_array_equal(_np(pos), rp)
    np.testing.assert_array_equal(_np(vel), rv)
    # config.py:80-95 ranges
    assert (rp >= 0).all() and (rp < [4.0, 20.0, 20.0]).all()
    assert (np.abs(rv - [1.5, -5.0, -5.0]) <= 0.5).all()


def test_pipe_fill_matches_oracle_and_stays_inside():
    torch_cuda()
    from sphgb import generate as G
    from sphgb.pipe_builder import PipeBuilder
    pipe = (PipeBuilder().with_starting_radius(1).add_roller_segment(1)
            .add_increasing_segment(1, 1.2).add_roller_segment(1)
            .add_lessening_segment(1, 1.2).add_roller_segment(1)
            .transform(40.0, 20.0).get_result())          # config.py:68-76
    g = G.pipe_fill_generator(pipe, seed=4)
    n = 100_000
    pos, vel = G.generate(g, n, pipe=pipe)
    rp, rv = ref.generate(_oracle_gen(g), n, pipe=pipe.to_numpy())
    gp = _np(pos)
    np.testing.assert_array_equal(gp[:, 0], rp[:, 0])
    # radii ~10 here: a few ulp of the radius (y = axis + r cos(theta))
    np.testing.assert_allclose(gp, rp, rtol=0, atol=TOL_TRIG_REL * pipe.to_numpy()[:, 3].max())
    np.testing.assert_array_equal(_np(vel), rv)
    table = pipe.to_numpy()
    for k in range(0, n, 997):
        seg = ref.find_segment(rp[k], table)
        assert seg >= 0
        r = np.hypot(rp[k, 1] - table[0, 1], rp[k, 2] - table[0, 2])
        assert r <= 0.98 * ref.radius_in_position(rp[k], table, seg) * (1 + 1e-12)
        assert not ref.is_out_of_pipe(rp[k], table, seg)


def test_generated_pipe_flow_velocity_normal_and_steps_like_host_load():
    torch = torch_cuda()
    from sphgb import generate as G
    from sphgb.data_classes import SimulationState
    from sphgb.device import SceneBatch
    spec, pos, vel = G.pipe_flow_scene(n=50_000, seed=8)
    g = G.pipe_fill_generator(spec.params.pipe, x_range=(0.0, 0.5), fill=0.999,
                              velocity=(1.0, 0.0, 0.0), sigma=0.05, seed=8)
    rp, rv = ref.generate(_oracle_gen(g), 50_000, pipe=spec.params.pipe.to_numpy())
    np.testing.assert_allclose(_np(pos), rp, rtol=0, atol=TOL_TRIG_POS)
    np.testing.assert_allclose(_np(vel), rv, rtol=0, atol=TOL_TRIG_VEL)
    dv = rv - [1.0, 0.0, 0.0]
    assert np.abs(dv.mean(0)).max() < 4 * 0.05 / np.sqrt(50_000)
    assert np.abs(dv.std(0) / 0.05 - 1).max() < 0.02
    # loading the device-generated state equals loading the same values from the host
    a = SceneBatch([spec])
    a.load_aos_device(pos, vel)
    a.step(3)
    b = SceneBatch([spec])
    b.load_states([SimulationState(_np(pos), _np(vel), np.zeros(50_000))])
    b.step(3)
    sa, sb = a.states()[0], b.states()[0]
    np.testing.assert_array_equal(sa.position, sb.position)
    np.testing.assert_array_equal(sa.velocity, sb.velocity)
    np.testing.assert_array_equal(sa.density, sb.density)
    assert np.isfinite(sa.density).all()
    a.close()
    b.close()
    torch.cuda.synchronize()


def test_generator_rejects_bad_arguments():
    torch_cuda()
    from sphgb import _capi
    from sphgb import generate as G
    g = G.lattice_generator(4, 4, 4, 0.1, 0.0)
    with pytest.raises(_capi.SphgbError):
        G.generate(g, 65)                       # n != nx*ny*nz
    g = _capi.Generator()
    g.kind = _capi.GEN_PIPE_FILL
    with pytest.raises(_capi.SphgbError):
        G.generate(g, 10)                       # no pipe table
    g.kind = 7
    with pytest.raises(_capi.SphgbError):
        G.generate(g, 10)


def _view_proj():
    # a perspective projection and a look-at view, FP32 (row-major numpy)
    f, near, far, aspect = 1.0 / np.tan(np.radians(30.0)), 0.1, 100.0, 16 / 9
    proj = np.array([[f / aspect, 0, 0, 0], [0, f, 0, 0],
                     [0, 0, (far + near) / (near - far), 2 * far * near / (near - far)],
                     [0, 0, -1, 0]], dtype=np.float32)
    view = np.eye(4, dtype=np.float32)
    view[:3, 3] = [-0.5, -0.4, -3.0]
    model = np.diag([1.0, 1.0, 1.0, 1.0]).astype(np.float32)
    model[:3, 3] = [0.1, 0.0, -0.2]
    return proj, model, view


def test_point_field_bit_identical_to_oracle():
    torch = torch_cuda()
    from sphgb.point_field import point_field, _mat
    rng = np.random.default_rng(3)
    n = 100_003
    pos = rng.uniform(-1, 2, size=(n, 4)).astype(np.float32)
    rho = rng.uniform(0, 30, size=n).astype(np.float32)
    rho[:6] = [0.0, 10.0, 25.0, np.nan, np.inf, -1.0]
    proj, model, view = _view_proj()
    for stride in (4, 3):
        p = pos[:, :stride].copy()
        clip, col, size = point_field(torch.as_tensor(p, device="cuda"),
                                      torch.as_tensor(rho, device="cuda"), proj, model, view)
        rc, rcol, rsize = ref.point_field(p, stride, rho, _mat(proj), _mat(model), _mat(view))
        np.testing.assert_array_equal(_np(clip), rc)
        np.testing.assert_array_equal(_np(col), rcol)
        np.testing.assert_array_equal(_np(size), rsize)
    assert np.all((rsize >= 1) & (rsize <= 13))
    assert np.all(rcol[:, 3] == 0.5)


def test_point_field_of_a_scene_batch():
    torch = torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    from sphgb.point_field import frame_attributes, _mat
    spec, st = scenes.config0()
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(2)
    proj, model, view = _view_proj()
    clip, col, size, pid = frame_attributes(b, proj, model, view)
    torch.cuda.synchronize()
    p = _np(b.pos)[:spec.n]
    rc, rcol, rsize = ref.point_field(p, 4, _np(b.rho)[:spec.n], _mat(proj), _mat(model),
                                      _mat(view))
    np.testing.assert_array_equal(_np(clip), rc)
    np.testing.assert_array_equal(_np(size), rsize)
    assert sorted(_np(pid).tolist()) == list(range(spec.n))
    b.close()
