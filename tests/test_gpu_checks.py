"""Checked mode (sphgb_ctx_set_checks / sphgb_ctx_check_word): the device error
word that reports the inputs the reference leaves undefined.

The reference computes voxel ids of particles outside the box without a bound
(voxel_kernels.py:10-17, :89-105), walks never-written neighbour voxel entries
(:44, :64-65) and reads past voxel_begin (:70); non-finite coordinates are
not expected anywhere.  This library defines what happens there (clamped
voxel coordinates, an overflow entry for non-finite positions that no walk
visits), and checked mode reports that it happened.  The bad inputs here are
made on the host: NaN and out-of-box positions in an otherwise valid state.
The check kernel compares every index with its range before it uses it, so
none of this can fault; the structural bits (voxel table, neighbour list) must
stay clear, because the library's own structures are valid whatever the
input.
"""
import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def _bad_state():
    """config0 with three NaN positions and four finite positions outside the
    [0,1]^3 box."""
    from sphgb import scenes
    from sphgb.data_classes import SimulationState
    spec, st = scenes.config0()
    pos = np.array(st.position)
    nan_ids = [17, 4000, 8191]
    pos[17, 0] = np.nan
    pos[4000, 1] = np.nan
    pos[8191, 2] = np.inf
    out_ids = [5, 300, 2222, 7000]
    pos[5] = (-0.25, 0.3, 0.3)
    pos[300] = (0.5, 1.5, 0.5)
    pos[2222] = (0.2, 0.2, 1.0)      # exactly on the upper face: outside [0, 1)
    pos[7000] = (3.0, -1.0, 0.1)
    return spec, SimulationState(pos, np.array(st.velocity), np.array(st.density)), nan_ids, out_ids


def test_clean_scene_sets_no_bits():
    torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    spec, st = scenes.config0()
    b = SceneBatch([spec])
    b.set_checks(True)
    b.load_states([st])
    b.step(2)
    b.step(3, use_graph=True)
    assert b.check_word() == (0, None, 0)
    b.close()


def test_bad_inputs_set_their_bits_and_nothing_else():
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st, nan_ids, out_ids = _bad_state()
    b = SceneBatch([spec])
    b.load_states([st])
    b.step(1)
    assert b.check_word() == (0, None, 0)        # off by default: nothing recorded
    b.set_checks(True)
    b.load_states([st])
    b.step(1)
    bits, first, flagged = b.check_word(clear=True)
    assert bits & _capi.CHECK_NONFINITE_INPUT
    assert bits & _capi.CHECK_OUT_OF_DOMAIN
    assert bits & _capi.CHECK_NONFINITE_OUTPUT   # NaN in, NaN out (density 0)
    assert not bits & (_capi.CHECK_VOXEL_TABLE | _capi.CHECK_NEIGHBOUR_LIST), bits
    assert first == min(nan_ids + out_ids)
    assert flagged >= len(nan_ids) + len(out_ids)
    assert b.check_word() == (0, None, 0)        # cleared
    # the fused step's neighbour rows of the same step stay within the scene
    b.load_states([st])
    b.step(1, use_graph=True)
    lst, cnt = (t.cpu().numpy() for t in b.step_neighbours())
    assert np.all(cnt[nan_ids] == 0) and np.all(lst[nan_ids] == -1)
    assert lst.max() < spec.n and np.all((lst >= 0) == (np.arange(32)[None, :] < cnt[:, None]))
    assert b.check_word()[0] & _capi.CHECK_NONFINITE_INPUT
    b.close()


@pytest.mark.parametrize("order", ["slot", "particle", "pipelined"])
def test_host_entry_runs_the_checks(order):
    torch_cuda()
    from sphgb import _capi
    from sphgb.device import SceneBatch
    spec, st, nan_ids, out_ids = _bad_state()
    b = SceneBatch([spec])
    b.set_host_order({"slot": _capi.HOST_ORDER_SLOT, "particle": _capi.HOST_ORDER_PARTICLE,
                      "pipelined": _capi.HOST_ORDER_PIPELINED}[order])
    b.set_checks(True)
    b.compute_next_state_host(st.position, st.velocity)
    bits, first, _ = b.check_word()
    assert bits & _capi.CHECK_NONFINITE_INPUT and bits & _capi.CHECK_OUT_OF_DOMAIN
    assert not bits & (_capi.CHECK_VOXEL_TABLE | _capi.CHECK_NEIGHBOUR_LIST), bits
    assert first == min(nan_ids + out_ids)
    b.close()


def test_step_neighbours_needs_a_step():
    torch_cuda()
    from sphgb import _capi, scenes
    from sphgb.device import SceneBatch
    spec, st = scenes.config0()
    b = SceneBatch([spec])
    b.load_states([st])
    with pytest.raises(_capi.SphgbError, match="SPHGB_ERR_STATE"):
        b.step_neighbours()
    b.step(1)
    b.step_neighbours()
    b.neighbour_counts()            # re-sorts the context's buffers
    with pytest.raises(_capi.SphgbError, match="SPHGB_ERR_STATE"):
        b.step_neighbours()
    b.close()
