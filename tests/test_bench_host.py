"""bench.py's host-side bookkeeping on CPU: the error against the oracle's step
(pipe scenes count the particles whose wall response fired apart), and the
committed ncu figures the JSON line reads (traffic and warp instructions per
particle of the dominant kernel, per workload)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _step(n=64, dt=1e-3, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    v = rng.random((n, 3)) - 0.5
    return x, v, dt, x + v * dt, np.ones(n)


def test_oracle_error_box():
    x, v, dt, p, r = _step()
    got = (p + 1e-8, v * (1 + 1e-7), r * (1 + 2e-7))
    e = bench.oracle_error(got, (p, v, r))
    assert abs(e["position_max_abs"] - 1e-8) < 1e-12
    assert abs(e["density_max_rel"] - 2e-7) < 1e-12
    assert e["particles_compared"] == len(p)
    assert "wall_response_particles" not in e


def test_oracle_error_pipe_counts_wall_particles_apart():
    x, v, dt, p, r = _step()
    want_p, want_v = p.copy(), v.copy()
    want_p[5] = [0.3, 0.1, 0.1]           # respawned in the FP64 step
    got_p, got_v = p.copy(), v.copy()
    got_p[5] = [0.30002, 0.1, 0.1]         # respawned too, within 1e-3 of |x|
    got_p[9] = [0.7, 0.05, 0.12]           # a wall decision that flipped
    e = bench.oracle_error((got_p, got_v, r), (want_p, want_v, r), pos_in=x, dt=dt)
    assert e["wall_response_particles"] == 2
    assert e["wall_within_1e-3"] == 1
    assert e["wall_position_max_abs"] > 0.1
    assert e["position_max_abs"] == 0.0 and e["velocity_max_abs_over_max"] == 0.0


def test_committed_profile_figures():
    assert bench.committed_traffic("density") > 1e8                   # the 4M box
    assert bench.committed_inst_per_particle("density") > 100
    assert bench.committed_inst_per_particle("density", "config1") > 100
    assert bench.committed_traffic("density", "box2m") is None        # no summary committed
    assert bench.committed_inst_per_particle("rank_gather") is None
