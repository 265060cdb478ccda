"""The steps either side of the path: frames written from device-resident
state (AsyncFrameSaver) in the reference's on-disk format, and the
StateGenerator driver (sim/src/state_generator.py:14-56)."""
import os

import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def test_async_saver_writes_the_reference_format(tmp_path, monkeypatch):
    torch = torch_cuda()
    from sphgb import config, scenes
    from sphgb.device import SceneBatch
    from sphgb.serializer import Loader, Saver
    from sphgb.serializer.saver import AsyncFrameSaver
    monkeypatch.setattr(config, "ROOT_PROJ_DIRNAME", str(tmp_path))
    spec, st = scenes.config0()
    spec_b, st_b = scenes.box_dam_break(nx=6, ny=12, nz=6, seed=3)
    batch = SceneBatch([spec_b, spec])           # the saved scene is the second one
    batch.load_states([st_b, st])
    saver = AsyncFrameSaver("frames", spec.params, depth=2)
    expect = []
    for _ in range(5):
        batch.step(2, use_graph=True)
        saver.save(batch, index=1)               # overlaps with the next steps
        expect.append(batch.states()[1])
    saver.close()
    torch.cuda.synchronize()
    # same files as the synchronous Saver writes (saver.py:28-46)
    Saver("frames_sync", spec.params)
    assert (sorted(os.listdir(tmp_path / "frames"))
            == sorted(["params.json"] + [f"{k}_{e}.npy" for e in range(5)
                                         for k in ("position", "velocity", "density")]))
    with open(tmp_path / "frames" / "params.json") as a, \
            open(tmp_path / "frames_sync" / "params.json") as b:
        assert a.read() == b.read()
    ld = Loader("frames")
    for e, want in enumerate(expect):
        got = ld.load_simulation_state(e)
        assert got.position.dtype == np.float64 and got.position.shape == (spec.n, 3)
        np.testing.assert_array_equal(got.position, want.position)
        np.testing.assert_array_equal(got.velocity, want.velocity)
        np.testing.assert_array_equal(got.density, want.density)
    batch.close()


def test_state_generator_frames_equal_strategy_steps():
    """One frame per step through compute_next_state (host arrays, as the
    reference), and three steps per frame kept on the device: same states."""
    torch_cuda()
    import itertools
    from sphgb import config, scenes
    from sphgb.state_generator import StateGenerator
    from sphgb.strategies import GB300SPHStrategy
    spec, st = scenes.config0()
    gen = StateGenerator(st, spec.params, constants=spec.constants, mode='BOX')
    assert gen.n_frames >= 6
    strat = GB300SPHStrategy(spec.params, constants=spec.constants, mode='BOX')
    s = st
    for frame in itertools.islice(gen, 6):
        s = strat.compute_next_state(s)
        np.testing.assert_array_equal(frame.position, s.position)
        np.testing.assert_array_equal(frame.velocity, s.velocity)
        np.testing.assert_array_equal(frame.density, s.density)
    assert gen.current_frame_idx == 6
    gen3 = StateGenerator(st, spec.params, constants=spec.constants, mode='BOX',
                          steps_per_frame=3)
    out = list(itertools.islice(gen3, 2))
    np.testing.assert_array_equal(out[-1].position, s.position)
    np.testing.assert_array_equal(out[-1].velocity, s.velocity)
    np.testing.assert_array_equal(out[-1].density, s.density)
    assert config.SIM_STRATEGY in ('GB300', 'VOXEL')
