"""The autotuner only changes speed: every candidate gives the same results."""
import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def test_autotune_capped_scene_keeps_results_bit_identical():
    torch_cuda()
    from sphgb import scenes
    from sphgb.autotune import autotune, summary
    from sphgb.device import SceneBatch
    pairs = [scenes.config0(), scenes.pipe_flow(n=20_000, seed=3, h=0.045)]
    best, tried = autotune(pairs, steps=2)
    assert len(tried) == 18 and best in tried and best.cell_ratio == 1.0
    assert all(np.isfinite(t.ms_per_step) and t.ms_per_step > 0 for t in tried)
    print(summary(tried))
    outs = []
    for tuning in (None, best):
        b = SceneBatch([p[0] for p in pairs])
        if tuning is not None:
            tuning.apply(b)
        b.load_states([p[1] for p in pairs])
        b.step(3)
        outs.append(b.states())
        b.close()
    for a, c in zip(*outs):
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(a, f), getattr(c, f))


def test_autotune_uncapped_scene_tries_cell_ratios():
    """Without the cap the neighbour set does not depend on the voxel size
    (>= h): larger voxels give the same physics up to summation order."""
    torch_cuda()
    from sphgb import scenes
    from sphgb.autotune import autotune, with_cell_ratio
    from sphgb.device import SceneBatch
    spec, st = scenes.box_dam_break(nx=10, ny=20, nz=10, max_neighbours=0, seed=6)
    best, tried = autotune([(spec, st)], steps=1)
    assert {t.cell_ratio for t in tried} == {1.0, 1.25, 1.5}
    res = []
    for ratio in (1.0, 1.5):
        b = SceneBatch([with_cell_ratio(spec, ratio)])
        b.load_states([st])
        b.step(1)
        res.append(b.states()[0])
        b.close()
    assert np.max(np.abs(res[0].density - res[1].density) / res[0].density) < 1e-5
    assert np.max(np.abs(res[0].position - res[1].position)) < 1e-6
