"""The oracle's start-state generators and point-field stage on their own
(CPU): the distributions and ranges of config.py:79-121, the Box-Muller
moments, the keying of every draw by particle id, and the shader formulas of
vis/assets/point_field.vert:14-23 on hand-computed cases."""
import numpy as np

from oracle import ref


def _gen(kind, **kw):
    g = ref.Generator()
    g.kind = kind
    for k, v in kw.items():
        if isinstance(v, (list, tuple)):
            getattr(g, k)[:] = list(v)
        else:
            setattr(g, k, v)
    return g


def test_lattice_sites_jitter_and_id_order():
    g = _gen(ref.GEN_LATTICE, lattice=(3, 5, 4), spacing=0.02, jitter=0.002, origin=(1, 2, 3),
             seed=11)
    p, v = ref.generate(g, 60)
    i = np.arange(60)
    idx = np.stack([i // 20, (i // 4) % 5, i % 4], 1)
    site = np.array([1, 2, 3]) + (idx + 0.5) * 0.02
    assert np.abs(p - site).max() <= 0.002
    assert np.abs(p - site).max() > 0.0015          # the jitter is used
    assert (v == 0).all()


def test_draws_are_keyed_by_particle_id():
    g = _gen(ref.GEN_BOX_WALL, extent=(1, 2, 3), velocity=(1.5, -5, -5), velocity_spread=1.0,
             seed=5)
    p1, v1 = ref.generate(g, 1000)
    p2, v2 = ref.generate(g, 5000)
    np.testing.assert_array_equal(p1, p2[:1000])
    np.testing.assert_array_equal(v1, v2[:1000])
    g.seed = 6
    p3, _ = ref.generate(g, 1000)
    assert not np.array_equal(p1, p3)


def test_box_wall_ranges_and_means():
    g = _gen(ref.GEN_BOX_WALL, extent=(4, 20, 20), velocity=(1.5, -5, -5), velocity_spread=1.0,
             seed=1)
    n = 200_000
    p, v = ref.generate(g, n)
    assert (p >= 0).all() and (p < [4, 20, 20]).all()
    np.testing.assert_allclose(p.mean(0), [2, 10, 10], rtol=0.01)
    assert (np.abs(v - [1.5, -5, -5]) <= 0.5).all()
    np.testing.assert_allclose(v.mean(0), [1.5, -5, -5], atol=0.005)


def test_pipe_fill_inside_radius_and_normal_velocity():
    # one cone segment 0.1 -> 0.06 over [0, 0.5), then a cylinder
    pipe = np.array([[0.0, 0.1, 0.1, 0.10, 0.5],
                     [0.5, 0.1, 0.1, 0.06, 0.5],
                     [1.0, 0.1, 0.1, 0.06, 0.0]])
    g = _gen(ref.GEN_PIPE_FILL, x_range=(0.0, 1.0), fill=0.98, velocity=(1.0, 0, 0),
             velocity_sigma=0.05, seed=3)
    n = 100_000
    p, v = ref.generate(g, n, pipe=pipe)
    assert (p[:, 0] >= 0).all() and (p[:, 0] < 1.0).all()
    R = np.where(p[:, 0] < 0.5, 0.1 + (0.06 - 0.1) * p[:, 0] / 0.5, 0.06)
    r = np.hypot(p[:, 1] - 0.1, p[:, 2] - 0.1)
    assert (r <= 0.98 * R * (1 + 1e-12)).all()
    # r = sqrt(u) R: (r / 0.98 R)^2 is uniform on [0, 1)
    q = (r / (0.98 * R)) ** 2
    assert abs(q.mean() - 0.5) < 0.005
    dv = v - [1.0, 0, 0]
    assert np.abs(dv.mean(0)).max() < 4 * 0.05 / np.sqrt(n)
    assert np.abs(dv.std(0) / 0.05 - 1).max() < 0.01


def test_point_field_formulas():
    eye = np.eye(4, dtype=np.float32).reshape(16)
    pos = np.array([[0.0, 0.0, 10.0], [1.0, 2.0, 0.5], [0.0, 0.0, -1.0], [0, 0, 100.0]],
                   dtype=np.float32)
    rho = np.array([0.0, 10.0, 5.0, np.nan], dtype=np.float32)
    clip, col, size = ref.point_field(pos, 3, rho, eye, eye, eye)
    np.testing.assert_array_equal(clip[:, :3], pos)
    assert (clip[:, 3] == 1).all()
    # t = 0: colour (0.1, 0.7, 0.5), size (40 + 20) / z clamped to [1, 13]
    np.testing.assert_allclose(col[0], [0.1, 0.7, 0.5, 0.5], rtol=1e-7)
    assert size[0] == np.float32(6.0)
    # t = 1: colour 0.7 * (0.3, 0.4, 1), size 40 / 0.5 -> 13
    np.testing.assert_allclose(col[1], [0.21, 0.28, 0.7, 0.5], rtol=1e-6)
    assert size[1] == 13.0
    assert size[2] == 1.0                       # behind the camera
    assert size[3] == 1.0 and col[3][2] == np.float32(0.7)   # NaN density: t = 1
