"""The oracle (oracle/ref_cpu.c) against golden vectors recorded from the
reference's own step code (tests/golden/make_golden.py).  CPU only.

Integer and index results (voxel ids, sorted order, voxel_begin, ordered
neighbour lists and counts) must be identical; floating-point results agree
to 1e-9 relative (the oracle is FP64 with the reference's operation order).
Particles outside [0, space) are excluded: the reference's voxel table loses
them (ids outside the table, voxel_sph_strategy.py:84-107) while this project
clamps them into the edge voxels.
"""
import os
import sys

import numpy as np
import pytest

from helpers import GOLDEN_DIR, ALIGNED_CASES, GOLDEN_CASES, golden_spec, in_domain, load_golden, rel_err
from oracle import ref

RTOL = 1e-9


def _cases():
    out = []
    for name in GOLDEN_CASES:
        out.append((name, "truncated"))
        if name in ALIGNED_CASES:
            out.append((name, "ceil"))
    return out


@pytest.mark.parametrize("name,walk", _cases())
def test_oracle_reproduces_reference_step(name, walk):
    d = load_golden(name)
    spec = golden_spec(d, walk)
    sp = ref.params_from_spec(spec, exact=True)
    pipe = d["pipe_rows"] if str(d["mode"]) == "PIPE" else None
    for s in range(d["position_in"].shape[0]):
        pos, vel = d["position_in"][s], d["velocity_in"][s]
        ok = in_domain(pos, d["space_size"])
        vox = ref.assign_voxels(sp, pos)
        np.testing.assert_array_equal(vox[ok], d["voxel_ids"][s][ok])
        spid, start, count = ref.organize(sp, vox)
        ref_map = d["map_pid"][s]
        np.testing.assert_array_equal(spid[ok[spid]], ref_map[ok[ref_map]])
        if ok.all():
            np.testing.assert_array_equal(np.where(count > 0, start, -1), d["voxel_begin"][s])
        lst, nc, nu = ref.neighbours(sp, pos, spid, start, count)
        np.testing.assert_array_equal(lst[ok], d["neigh_list"][s][ok])
        np.testing.assert_array_equal(nc[ok], d["neigh_count"][s][ok])
        np.testing.assert_array_equal(nu[ok], d["neigh_count_uncapped"][s][ok])
        rho = ref.density(sp, pos, spid, start, count)
        pt, vt, ps, vs = ref.forces(sp, pos, vel, rho, spid, start, count)
        x, v, f = ref.integrate(sp, pos, vel, rho, pt, vt, pipe=pipe, step=s)
        assert rel_err(rho[ok], d["density"][s][ok]) < RTOL
        assert rel_err(pt[ok], d["pressure_term"][s][ok], ps[ok] + 1e-300) < RTOL
        assert rel_err(vt[ok], d["viscosity_term"][s][ok], vs[ok] + 1e-300) < RTOL
        assert rel_err(x[ok], d["position_out"][s][ok], 1.0) < RTOL
        assert rel_err(v[ok], d["velocity_out"][s][ok], np.abs(v[ok]).max() + 1e-300) < RTOL


def test_truncated_walk_differs_from_ceil_on_unaligned_box():
    """The reference's truncated walk dims (voxel_sph_strategy.py:110-116)
    visit the wrong voxels when space/voxel is not an integer; the ceil walk
    finds every neighbour within h."""
    d = load_golden("box_unaligned")
    pos = d["position_in"][0]
    counts = {}
    for walk in ("truncated", "ceil"):
        sp = ref.params_from_spec(golden_spec(d, walk))
        spid, start, count = ref.organize(sp, ref.assign_voxels(sp, pos))
        counts[walk] = ref.neighbours(sp, pos, spid, start, count, with_list=False)[2]
    # brute-force uncapped count: every pair within h (FP64, the reference's predicate)
    h = float(np.float32(d["inf_r"]))
    diff = pos[:, None, :] - pos[None, :, :]
    brute = (np.sqrt(((diff[..., 0] ** 2 + diff[..., 1] ** 2) + diff[..., 2] ** 2)) <= h).sum(1)
    np.testing.assert_array_equal(counts["ceil"], brute)
    assert counts["truncated"].mean() < 0.5 * brute.mean()


def test_pipe_kats_from_reference_tests():
    """sim/tests/test_collisions.py cases, outputs recorded from the reference."""
    k = dict(np.load(os.path.join(GOLDEN_DIR, "pipe_kats.npz")))
    seg = [ref.find_segment(p, k["find_segment_pipe"]) for p in k["find_segment_pos"]]
    np.testing.assert_array_equal(seg, k["find_segment_out"])
    np.testing.assert_array_equal(seg, [-1, 0, 1, 2, -1])          # test_collisions.py:105
    xb = [ref.x_at_segment_beginning(k["x_begin_pipe"], s) for s in (0, 1, 2)]
    np.testing.assert_array_equal(xb, [0, 1, 5])                   # test_collisions.py:153
    iso = [ref.is_out_of_pipe(p, k["is_out_pipe"], s) for p, s in zip(k["is_out_pos"], k["is_out_seg"])]
    np.testing.assert_array_equal(iso, k["is_out_out"])
    rad = [ref.radius_in_position(p, k["is_out_pipe"], s) for p, s in zip(k["is_out_pos"], k["is_out_seg"])]
    np.testing.assert_allclose(rad, k["radius_out"], rtol=1e-15)
    for i in range(len(k["collide_pos_in"])):
        s = ref.find_segment(k["collide_pos_in"][i], k["collide_pipe"])
        assert s == k["collide_seg"][i]
        p, v = k["collide_pos_in"][i], k["collide_vel_in"][i]
        if ref.is_out_of_pipe(p, k["collide_pipe"], s):
            p, v = ref.solve_collision(p, v, k["collide_pipe"], s)
        np.testing.assert_allclose(p, k["collide_pos_out"][i], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(v, k["collide_vel_out"][i], rtol=1e-12, atol=1e-12)


def test_philox_c_matches_python():
    sys.path.insert(0, GOLDEN_DIR)
    from philox_ref import philox4x32_10, philox_uniform_f64
    rng = np.random.default_rng(5)
    for _ in range(200):
        seed = int(rng.integers(0, 2 ** 63))
        pid, step, draw = (int(rng.integers(0, 2 ** 31)) for _ in range(3))
        assert ref.philox_uniform(seed, pid, step, draw) == philox_uniform_f64(seed, pid, step, draw)
    # Random123's published Philox4x32-10 known answers (kat_vectors)
    assert philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)
    m = 0xFFFFFFFF
    assert philox4x32_10((m, m, m, m), (m, m)) == (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)
