"""The allocation-free voxel organisation, sphgb_organize_voxels_noalloc.

Some callers of this library cannot call cudaMalloc: their process forbids
device allocation after start-up, or every device byte has to come from an
allocator they own.  For them the voxel sort (hash, counting sort, voxel
table) has an entry point that takes no context and keeps its scratch in a
fixed array inside the library.  These tests check that it gives exactly the
output of the allocating entry point (sphgb_organize_voxels): same sorted
state, same voxel table, bit for bit, on consecutive calls with different
scenes, and that sizes beyond its limits are refused.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import to_device, torch_cuda

pytestmark = pytest.mark.gpu


def _clustered(n_nan=16):
    """262,144 particles (the entry point's limit) in a [0,1]^3 box with h 0.02
    (125,000 voxels): a lattice, of which 10,000 particles are packed into one
    voxel (sorted in global memory), 40 x 150 into 40 other voxels (sorted in
    shared memory; both above the 64 members that send a voxel to the
    big-voxel sort), n_nan with a NaN coordinate (the overflow entry) and a
    few outside the box (clamped into the table)."""
    from sphgb import scenes
    spec, st = scenes.box_dam_break(nx=64, ny=64, nz=64, spacing=0.0125, jitter=0.001,
                                    h=0.02, mass=0.002, seed=31)
    assert spec.n == 262_144
    rng = np.random.default_rng(32)
    pos = np.array(st.position, dtype=np.float64)
    perm = rng.permutation(spec.n)
    h = 0.02
    k = 0
    big = perm[k:k + 10_000]; k += 10_000
    pos[big] = (np.array([10, 11, 12]) + rng.uniform(0.05, 0.95, (len(big), 3))) * h
    for c in range(40):
        idx = perm[k:k + 150]; k += 150
        corner = np.array([5 + c, 20 + (c % 7), 30 + (c % 11)])
        pos[idx] = (corner + rng.uniform(0.05, 0.95, (len(idx), 3))) * h
    nan = perm[k:k + n_nan]; k += n_nan
    pos[nan, rng.integers(0, 3, n_nan)] = np.nan
    out = perm[k:k + 8]; k += 8
    pos[out] = rng.uniform(-0.5, 1.5, (8, 3))
    from sphgb.data_classes import SimulationState
    pos = np.asarray(pos, dtype=np.float32).astype(np.float64)
    return spec, SimulationState(pos, np.array(st.velocity), np.array(st.density))


def _scenes():
    from sphgb import scenes
    return [scenes.config0(),                                              # 8,192, 12,167 voxels
            scenes.box_dam_break(nx=40, ny=80, nz=40, spacing=0.01, jitter=0.001,
                                 h=0.0225, mass=0.001, seed=21),            # 128,000, 79,508 voxels
            _clustered(),
            scenes.config0(seed=7)]


def _allocating(spec, pos, vel):
    from sphgb import kernels as K
    from sphgb.device import SceneBatch
    batch = SceneBatch([spec])
    p4, v4, pid, _ = to_device(pos, vel)
    out = K.organize_voxels(batch, p4, v4, pid)
    torch = torch_cuda()
    torch.cuda.synchronize()
    res = [t.cpu().numpy() for t in (out[0], out[1], out[2], out[4], out[5])]
    batch.close()
    return res


def _noalloc(spec, pos, vel):
    torch = torch_cuda()
    from sphgb import _capi
    from sphgb.device import scene_params
    sp = scene_params(spec)
    n = spec.n
    p4, v4, pid, _ = to_device(pos, vel)
    pos_o, vel_o, pid_o = torch.empty_like(p4), torch.empty_like(v4), torch.empty_like(pid)
    nv = int(np.prod(np.ceil(np.asarray(sp.space_size[:]) / np.asarray(sp.voxel_size[:])))) + 1
    start = torch.full((nv,), -7, dtype=torch.int32, device="cuda")
    count = torch.full((nv,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _capi.call("sphgb_organize_voxels_noalloc", C.byref(sp), p4.data_ptr(), v4.data_ptr(),
               pid.data_ptr(), pos_o.data_ptr(), vel_o.data_ptr(), pid_o.data_ptr(),
               start.data_ptr(), count.data_ptr(), stream)
    torch.cuda.synchronize()
    assert n == len(pos)
    return [t.cpu().numpy() for t in (pos_o, vel_o, pid_o, start, count)]


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    torch_cuda()
    for spec, st in _scenes():
        ref = _allocating(spec, st.position, st.velocity)
        got = _noalloc(spec, st.position, st.velocity)
        pos_r, vel_r, pid_r, start_r, count_r = ref
        pos_g, vel_g, pid_g, start_g, count_g = got
        np.testing.assert_array_equal(count_g, count_r)
        occupied = count_r > 0
        np.testing.assert_array_equal(start_g[occupied], start_r[occupied])
        assert count_g.sum() == spec.n
        # The last table entry collects particles with a non-finite coordinate.
        # No walk visits it, and it keeps arrival order (which depends on the
        # order atomics land in): compare it as a set.  Everything before it
        # is in (voxel, particle id) order and must match bit for bit.
        m = spec.n - int(count_r[-1])
        np.testing.assert_array_equal(pid_g[:m], pid_r[:m])
        np.testing.assert_array_equal(pos_g[:m], pos_r[:m])
        np.testing.assert_array_equal(vel_g[:m], vel_r[:m])
        og, orr = np.argsort(pid_g[m:]), np.argsort(pid_r[m:])
        np.testing.assert_array_equal(pid_g[m:][og], pid_r[m:][orr])
        np.testing.assert_array_equal(pos_g[m:][og], pos_r[m:][orr])
        np.testing.assert_array_equal(vel_g[m:][og], vel_r[m:][orr])
        if spec.n == 262_144:
            # the clustered scene reaches both branches of the big-voxel sort
            # and the overflow entry
            big = np.flatnonzero(count_r[:-1] > 64)
            assert len(big) >= 41 and count_r[:-1].max() >= 10_000 and count_r[-1] == 16
            for v in big:
                assert np.all(np.diff(pid_g[start_r[v]:start_r[v] + count_r[v]]) > 0)


def test_noalloc_refuses_sizes_beyond_its_limits():
    from sphgb import _capi
    from sphgb.device import scene_params
    from sphgb import scenes
    spec, _ = scenes.config0()
    sp = scene_params(spec)
    sp.particle_count = 262_145
    lib = _capi.load()
    rc = lib.sphgb_organize_voxels_noalloc(C.byref(sp), None, None, None, None, None, None, None,
                                           None, None)
    assert rc == -5 and "262144" in _capi.last_error()
    sp = scene_params(spec)
    sp.voxel_size[0] = sp.voxel_size[1] = sp.voxel_size[2] = 0.001      # 1e9 voxels
    rc = lib.sphgb_organize_voxels_noalloc(C.byref(sp), None, None, None, None, None, None, None,
                                           None, None)
    assert rc == -5 and "4194304" in _capi.last_error()
