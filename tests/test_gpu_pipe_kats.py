"""The reference's only numeric pins, run through the C ABI on the GPU.

sim/tests/test_collisions.py:90-209 checks the pipe geometry of
util_kernels.py: find_segment (:105, [-1, 0, 1, 2, -1]),
calc_x_at_segment_beginning (:153, [0, 1, 5]), is_out_of_pipe (:178-180, nine
booleans) and "collision ends inside" (:184-209).  tests/golden/pipe_kats.npz
holds those inputs with the outputs the reference's own functions gave
(recorded by tests/golden/make_golden.py), plus 63 more outside points
resolved by the reference's solve_collision.  Every respawn on the GPU is
keyed by the Philox4x32-10 stream, so sphgb_philox_uniform is held bit for bit
to Random123's published known answers and to the Python restatement
(tests/golden/philox_ref.py).

Integers and booleans: exact.  FP64 outputs: within 1e-12 relative (the
device geometry is written in the reference's operation order with IEEE
double operations, so it is expected to be exact).
"""
import os
import sys

import numpy as np
import pytest

from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def kats():
    return dict(np.load(os.path.join(GOLDEN_DIR, "pipe_kats.npz")))


def test_find_segment_kat(kats):
    torch_cuda()
    from sphgb import kernels as K
    seg = K.find_segment(kats["find_segment_pos"], kats["find_segment_pipe"])
    np.testing.assert_array_equal(seg, kats["find_segment_out"])
    np.testing.assert_array_equal(seg, [-1, 0, 1, 2, -1])      # test_collisions.py:105


def test_x_at_segment_beginning_kat(kats):
    torch_cuda()
    from sphgb import kernels as K
    xb = K.calc_x_at_segment_beginning(kats["x_begin_pipe"], [0, 1, 2])
    np.testing.assert_array_equal(xb, kats["x_begin_out"])
    np.testing.assert_array_equal(xb, [0.0, 1.0, 5.0])          # test_collisions.py:153


def test_is_out_of_pipe_kat(kats):
    torch_cuda()
    from sphgb import kernels as K
    out, rad = K.is_out_of_pipe(kats["is_out_pos"], kats["is_out_pipe"], kats["is_out_seg"])
    np.testing.assert_array_equal(out, kats["is_out_out"])     # test_collisions.py:178-180
    np.testing.assert_allclose(rad, kats["radius_out"], rtol=1e-12, atol=0.0)


def test_solve_collision_kat(kats):
    """find_segment, then solve_collision when out of the pipe, for the
    reference test's own case (index 0: (1.3, 1.5, 0) moving -x, which must end
    inside, test_collisions.py:184-209) and 63 recorded outside points."""
    torch_cuda()
    from sphgb import kernels as K
    pipe = kats["collide_pipe"]
    pos, vel, seg = K.solve_collision(kats["collide_pos_in"], kats["collide_vel_in"], pipe)
    np.testing.assert_array_equal(seg, kats["collide_seg"])
    for got, want in ((pos, kats["collide_pos_out"]), (vel, kats["collide_vel_out"])):
        scale = np.maximum(np.abs(want), 1.0)
        err = np.abs(got - want) / scale
        assert err.max() < 1e-12, (np.unravel_index(err.argmax(), err.shape), err.max())
    # "collision ends inside": the resolved positions are inside (or, for the
    # recorded outside points where the reference's own resolution leaves the
    # particle out, out exactly as there)
    out, _ = K.is_out_of_pipe(pos, pipe, seg)
    np.testing.assert_array_equal(out, kats["collide_still_out"])
    assert not out[0]


def test_philox_known_answers_through_the_c_abi():
    """Random123's Philox4x32-10 known answers in the uniform the library
    draws: u = ((c0 << 21) | (c1 >> 11)) / 2^53 of the output words, with the
    counter (draw, step, pid, 0) and the key (seed low, seed high)."""
    torch_cuda()
    sys.path.insert(0, GOLDEN_DIR)
    from philox_ref import philox4x32_10, philox_uniform_f64
    from sphgb import kernels as K
    m = 0xFFFFFFFF

    def uniform_of(words):
        c0, c1 = words[0], words[1]
        return float(((c0 << 21) | (c1 >> 11))) / 2.0 ** 53

    # counter (0, 0, 0, 0), key (0, 0): draw 0, step 0, pid 0, seed 0
    kat0 = uniform_of((0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8))
    assert philox4x32_10((0, 0, 0, 0), (0, 0))[0] == 0x6627e8d5
    assert K.philox_uniform(0, [0], 0, 0)[0] == kat0
    # counter all ones but c3 (the library keeps c3 = 0): compare against the
    # restatement, which is itself pinned to the all-ones known answer
    assert philox4x32_10((m, m, m, m), (m, m)) == (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)
    seed = (m << 32) | m
    got = K.philox_uniform(seed, [-1], -1, -1)[0]
    assert got == philox_uniform_f64(seed, m, m, m)


def test_philox_stream_matches_restatement_bit_for_bit():
    """10,000 seeded (seed, pid, step, draw) tuples, the respawn stream's
    arguments, against the Python restatement."""
    torch_cuda()
    sys.path.insert(0, GOLDEN_DIR)
    from philox_ref import philox_uniform_f64
    from sphgb import kernels as K
    rng = np.random.default_rng(11)
    n_groups, per = 20, 500
    for _ in range(n_groups):
        seed = int(rng.integers(0, 2 ** 63))
        step = int(rng.integers(0, 2 ** 31))
        draw = int(rng.integers(0, 4))
        pids = rng.integers(0, 2 ** 31, per).astype(np.int32)
        got = K.philox_uniform(seed, pids, step, draw)
        want = np.array([philox_uniform_f64(seed, int(p), step, draw) for p in pids])
        np.testing.assert_array_equal(got, want)
        assert np.all((got >= 0.0) & (got < 1.0))
