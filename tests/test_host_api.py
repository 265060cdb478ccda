"""Host-side mirror of the reference's interface (CPU only).

The pipe and builder cases restate the reference's own tests
(common/tests/test_pipe.py, common/tests/test_pipe_builder.py,
common/tests/test_saving_loading.py) against this package's classes.
"""
import numpy as np
import pytest

from sphgb import config
from sphgb.config import SPHConstants
from sphgb.data_classes import Pipe, Segment, SimulationParameters, SimulationState
from sphgb.pipe_builder import PipeBuilder


def test_segment_to_numpy():                       # test_pipe.py:14-19
    assert np.all(Segment(start_radius=4.5).to_numpy() == np.array([0, 0, 0, 4.5, 1]))


def test_simple_pipe_to_numpy():                   # test_pipe.py:21-26
    assert np.all(Pipe([Segment()]).to_numpy() == np.array([[0, 0, 0, 1, 1], [1, 0, 0, 1, 1]]))


def test_pipe_to_numpy():                          # test_pipe.py:28-35
    pipe = PipeBuilder().with_starting_radius(3).add_roller_segment(1).add_increasing_segment(1, 2).get_result()
    expected = np.array([[0, 0, 0, 3, 1], [1, 0, 0, 1, 1], [2, 0, 0, 1, 1], [3, 0, 0, 3, 1]])
    assert np.all(pipe.to_numpy() == expected)


def test_builder_basic_and_first_segment():       # test_pipe_builder.py:12-30
    assert PipeBuilder().get_result() == Pipe([Segment()])
    pipe = (PipeBuilder().with_starting_position((1, 2, 3)).with_starting_length(20)
            .with_starting_radius(4).with_ending_radius(5).get_result())
    assert pipe == Pipe([Segment(start_point=(1, 2, 3), start_radius=4, end_radius=5, length=20)])


@pytest.mark.parametrize("build,msg", [
    (lambda: PipeBuilder().with_starting_length(-10), PipeBuilder._NEGATIVE_LENGTH_MESSAGE),
    (lambda: PipeBuilder().with_starting_radius(-1), PipeBuilder._NEGATIVE_RADIUS_MESSAGE),
    (lambda: PipeBuilder().with_ending_radius(-1), PipeBuilder._NEGATIVE_RADIUS_MESSAGE),
    (lambda: PipeBuilder().add_roller_segment(20).with_starting_radius(1),
     PipeBuilder._FIRST_SEGMENT_MESSAGE),
    (lambda: PipeBuilder().add_lessening_segment(1, -10), PipeBuilder._NEGATIVE_CHANGE_MESSAGE),
])
def test_builder_errors(build, msg):               # test_pipe_builder.py:32-53, 106-117
    with pytest.raises(AssertionError) as e:
        build()
    assert str(e.value) == msg


def test_builder_segments():                       # test_pipe_builder.py:55-104
    assert PipeBuilder().with_ending_radius(4).add_roller_segment(30).get_result() == \
        Pipe([Segment(end_radius=4), Segment((1, 0, 0), 4, 4, 30)])
    assert PipeBuilder().with_ending_radius(7).add_lessening_segment(length=1, change=6).get_result() == \
        Pipe([Segment(end_radius=7), Segment((1, 0, 0), 7, 1, 1)])
    assert PipeBuilder().with_ending_radius(5).add_increasing_segment(length=1, change=5).get_result() == \
        Pipe([Segment(end_radius=5), Segment((1, 0, 0), 5, 10, 1)])
    got = (PipeBuilder().with_starting_radius(10).with_ending_radius(5).add_roller_segment(length=1)
           .add_increasing_segment(1, 5).get_result())
    assert got == Pipe([Segment(start_radius=10, end_radius=5), Segment((1, 0, 0), 5, 5, 1),
                        Segment((2, 0, 0), np.float64(5), 10, 1)])


def test_builder_transform():                      # test_pipe_builder.py:118-130
    pipe = (PipeBuilder().add_increasing_segment(2., 3.).add_roller_segment(1.)
            .add_increasing_segment(2., 3.).transform(600, 600, 70).get_result())
    expected = (PipeBuilder().with_starting_position((0., 300., 300.)).with_starting_radius(10.)
                .with_ending_radius(10.).with_starting_length(100.).add_increasing_segment(200., 30.)
                .add_roller_segment(100.).add_increasing_segment(200., 30.).get_result().to_numpy())
    assert np.all(pipe.to_numpy() == expected)


def test_reference_default_pipe_layout():
    """config.py:68-76 pipe, as the reference's golden run recorded it."""
    import os
    from helpers import GOLDEN_DIR
    d = np.load(os.path.join(GOLDEN_DIR, "pipe_defaults.npz"))
    np.testing.assert_array_equal(config.build_pipe().to_numpy(), d["pipe_rows"])


def test_serializer_round_trip(tmp_path, monkeypatch):   # test_saving_loading.py:12-56
    from sphgb.serializer import Loader, Saver
    monkeypatch.setattr(config, "ROOT_PROJ_DIRNAME", tmp_path)
    params = SimulationParameters(pipe=Pipe([Segment(), Segment((1.0, 0.0, 0.0), 1, 4, 5)]))
    Saver("data", params)
    loaded = Loader("data").load_simulation_parameters()
    for name in vars(params):
        a, b = getattr(params, name), getattr(loaded, name)
        assert type(a) is type(b)
        assert np.all(a == b) if isinstance(a, np.ndarray) else a == b
    saver = Saver("data2", SimulationParameters())
    s1 = SimulationState(position=np.asarray([0, 1, 0]))
    s2 = SimulationState(position=np.asarray([0, 2, 0]))
    saver.save_next_state(s1)
    saver.save_next_state(s2)
    ld = Loader("data2")
    for k, s in enumerate((s1, s2)):
        got = ld.load_simulation_state(k)
        for name in vars(s):
            assert np.all(getattr(got, name) == getattr(s, name))
    # same file names as the reference's saver (saver.py:28-36)
    assert sorted(p.name for p in (tmp_path / "data2").iterdir()) == sorted(
        ["params.json"] + [f"{n}_{k}.npy" for n in ("position", "velocity", "density") for k in (0, 1)])


def test_loader_missing_dir_raises(tmp_path, monkeypatch):
    from sphgb.serializer import Loader
    monkeypatch.setattr(config, "ROOT_PROJ_DIRNAME", tmp_path)
    with pytest.raises(Exception, match="does not exists"):
        Loader("nope")


def test_config_names_and_constants():
    for name in ("SIM_MODE", "SIM_STRATEGY", "DURATION", "FPS", "PARTICLE_COUNT", "MASS", "RHO_0",
                 "INF_R", "VISC", "K", "DAMP", "INF_R_2", "INF_R_6", "INF_R_9", "W_CONST",
                 "GRAD_W_CONST", "LAP_W_CONST", "MAX_NEIGHBOURS", "NEIGHBOURING_VOXELS_COUNT",
                 "VOXEL_SIZE", "BOX_SPACE_SIZE", "PIPE_SPACE_SIZE", "GRAVITY", "HORIZONTAL_FORCE",
                 "PARAMS_FILENAME", "OUT_DIRNAME"):
        assert hasattr(config, name), name
    c = config.constants_from_module()
    assert c.w_const == pytest.approx(config.W_CONST)
    r = SPHConstants(inf_r=0.045, mass=0.008).rounded()
    assert r.inf_r == float(np.float32(0.045)) and r.mass == float(np.float32(0.008))
    p = config.create_params_box()
    assert list(p.space_size) == config.BOX_SPACE_SIZE
    st = config.start_state_box_wall(n=100, seed=1)
    assert st.position.shape == (100, 3) and np.all(st.position[:, 0] <= 0.1 * config.BOX_SPACE_SIZE[0])
    pipe = config.build_pipe()
    st = config.start_state_inside_pipe(pipe, n=50, seed=1)
    r = np.hypot(st.position[:, 1] - 3.0, st.position[:, 2] - 3.0)
    assert np.all(r <= np.array([pipe.radius_at(x) for x in st.position[:, 0]]))


def test_scene_generators_shapes():
    from sphgb import scenes
    spec, st = scenes.config0()
    assert spec.n == 8192 and st.position.shape == (8192, 3)
    assert np.all(st.position.astype(np.float32).astype(np.float64) == st.position)
    assert np.all((st.position > 0) & (st.position < 0.7))
    spec, st = scenes.pipe_flow(n=5000, seed=1)
    rows = spec.params.pipe.to_numpy()
    assert rows.shape == (4, 5) and np.allclose(rows[:, 3], [0.10, 0.06, 0.10, 0.10])
    x = st.position[:, 0]
    R = 0.10 - 0.04 * x / 0.5
    assert np.all(np.hypot(st.position[:, 1] - 0.1, st.position[:, 2] - 0.1) <= R + 1e-7)
    b = scenes.config3_specs(n_scenes=8, seed=3)
    for spec, st in b:
        assert 1024 // 2 <= spec.n <= 2 * 65536 and len(st.position) == spec.n
        L = spec.params.space_size[0]
        assert np.all(st.position < L)
