"""Degenerate inputs on the GPU: dense clusters (voxels of thousands of
particles) and non-finite positions.  The reference has undefined behaviour
for non-finite positions (int32 of NaN, voxel_kernels.py:12); here they go to
a per-scene overflow bucket that no walk visits.  The sorted order of every
finite particle must still be the oracle's (voxel, particle id) order, and a
step must complete."""
import numpy as np
import pytest

from gpu_util import run_stages, to_device, torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu


def cluster_scene(seed=0):
    from sphgb import scenes
    spec, st = scenes.box_dam_break(nx=20, ny=40, nz=20, seed=seed)     # 16,000 particles
    pos = st.position.copy()
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(pos))
    pos[idx[:3000]] = [0.3125, 0.3125, 0.3125]                        # smem bitonic path
    pos[idx[3000:12000]] = pos[idx[3000]]                             # global bitonic path
    pos[idx[12000:12100]] = np.nan                                    # overflow bucket
    pos[idx[12100:12110], 1] = np.inf
    return spec, pos.astype(np.float32).astype(np.float64), st.velocity, idx


def test_clusters_and_nonfinite_sort_exactly():
    torch = torch_cuda()
    from sphgb import kernels as K
    from sphgb.device import SceneBatch
    spec, pos, vel, idx = cluster_scene()
    batch = SceneBatch([spec])
    p4, v4, pid, _ = to_device(pos, vel)
    pS, vS, idS, _, start, count = K.organize_voxels(batch, p4, v4, pid)
    torch.cuda.synchronize()
    ids, count, start = idS.cpu().numpy(), count.cpu().numpy(), start.cpu().numpy()
    finite = np.isfinite(pos).all(axis=1)
    sp = ref.params_from_spec(spec)
    spid, rstart, rcount = ref.organize(sp, ref.assign_voxels(sp, np.where(finite[:, None], pos, 0)))
    nv = len(rcount)
    # finite particles: exactly the oracle's order, and they fill the table first
    np.testing.assert_array_equal(ids[:finite.sum()], spid[finite[spid]])
    # non-finite particles: the overflow bucket (last entry), in arrival order
    assert count[nv] == (~finite).sum()
    over = ids[start[nv]:start[nv] + count[nv]]
    np.testing.assert_array_equal(np.sort(over), np.nonzero(~finite)[0])
    assert count.max() >= 9000      # the cluster plus the voxel's own particles
    batch.close()


def test_step_on_degenerate_input_completes():
    torch_cuda()
    spec, pos, vel, idx = cluster_scene(seed=1)
    g = run_stages(spec, pos, vel)
    finite = np.isfinite(pos).all(axis=1)
    assert (g["neigh_count"][~finite] == 0).all()
    assert (g["neigh_count"][finite] >= 1).all()          # self at least
    assert (g["neigh_count"] <= 32).all()
