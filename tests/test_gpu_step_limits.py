"""Per-scene step limits (sphgb_ctx_set_step_limits): one launch, or one
captured graph, advances each scene of a batch by its own number of steps.

A scene whose step counter reaches its limit is frozen; later steps leave its
position, velocity, density and counter unchanged.  Every scene must end
bit-identical to the same scene stepped alone for exactly its limit, in box
contexts (the two-launch force pass) and in contexts with a pipe scene (the
one-launch FP64 pass), with either density kernel, and checked mode must find
nothing wrong with the library's structures while scenes are frozen.
"""
import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def _pairs(with_pipe):
    from sphgb import scenes
    out = [scenes.config0(),
           scenes.box_dam_break(nx=10, ny=20, nz=10, seed=4, gravity=(1.0, -9.0, 3.0))]
    if with_pipe:
        out.append(scenes.pipe_flow(n=20_000, seed=11, h=0.02 * (262_144 / 20_000) ** (1 / 3)))
    return out


def _alone(spec, st, steps):
    from sphgb.device import SceneBatch
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(steps)
    out = b.states()[0]
    b.close()
    return out


def _same(a, b, label):
    for f in ("position", "velocity", "density"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f"{label} {f}")


@pytest.mark.parametrize("with_pipe", [False, True])
@pytest.mark.parametrize("variant", ["warp", "thread"])
def test_each_scene_stops_at_its_limit(with_pipe, variant):
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    pairs = _pairs(with_pipe)
    limits = [4, 9, 15][:len(pairs)]
    top = max(limits)
    b = SceneBatch([p[0] for p in pairs])
    b.set_tuning(256, {"warp": _capi.DENSITY_WARP, "thread": _capi.DENSITY_THREAD}[variant], 64)
    b.set_checks(True)
    b.load_states([p[1] for p in pairs])
    b.set_step_limits(limits)
    b.step(top, use_graph=True)
    got = b.states()
    assert b.steps.cpu().tolist() == limits
    structural = _capi.CHECK_VOXEL_TABLE | _capi.CHECK_NEIGHBOUR_LIST
    # the pipe flow blows up under the reference's formulas (non-finite
    # velocities, respawns), which sets the input and output bits; the
    # library's structures, frozen scenes included, must stay valid
    assert not b.check_word()[0] & structural
    for k, ((spec, st), lim) in enumerate(zip(pairs, limits)):
        _same(got[k], _alone(spec, st, lim), f"scene {k} at {lim} steps")
    # further steps leave every frozen scene as it is
    b.step(3)
    for k, g in enumerate(b.states()):
        _same(g, got[k], f"scene {k} frozen")
    assert b.steps.cpu().tolist() == limits
    # raising a limit in place (no new call) lets that scene go on
    b.step_limits[0] = limits[0] + 2
    b.step(2, use_graph=True)
    after = b.states()
    _same(after[0], _alone(pairs[0][0], pairs[0][1], limits[0] + 2), "scene 0 resumed")
    for k in range(1, len(pairs)):
        _same(after[k], got[k], f"scene {k} still frozen")
    bits = b.check_word()[0]
    assert not bits & structural
    if not with_pipe:
        assert bits == 0
    b.close()


def test_removing_the_limits_and_reconfiguring():
    torch_cuda()
    from sphgb.device import SceneBatch
    pairs = _pairs(False)
    b = SceneBatch([p[0] for p in pairs])
    b.load_states([p[1] for p in pairs])
    b.set_step_limits([0, 0])               # both frozen from the start
    b.step(2)
    for k, g in enumerate(b.states()):
        np.testing.assert_array_equal(g.position, pairs[k][1].position)
    b.set_step_limits(None)                 # no limits: both advance
    b.step(2)
    assert b.steps.cpu().tolist() == [2, 2]
    _same(b.states()[0], _alone(pairs[0][0], pairs[0][1], 2), "unlimited")
    b.set_step_limits([1, 1])
    b.reconfigure([p[0] for p in pairs])    # drops the limits with the old layout
    assert b.step_limits is None
    b.load_states([p[1] for p in pairs])
    b.step(2)
    assert b.steps.cpu().tolist() == [2, 2]
    with pytest.raises(ValueError):
        b.set_step_limits([1, 2, 3])
    # a host array is refused before any step could read it on the device
    import ctypes as C
    from sphgb import _capi
    host = (C.c_int32 * 2)(1, 1)
    assert _capi.load().sphgb_ctx_set_step_limits(b.handle, C.addressof(host)) == -1
    assert "device" in _capi.last_error()
    b.close()
