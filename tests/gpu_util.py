"""GPU-side test helpers: run every stage of one step through the C ABI and
return the results in original particle order (numpy)."""
from __future__ import annotations

import numpy as np


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def to_device(pos, vel):
    torch = torch_cuda()
    n = len(pos)
    p4 = torch.zeros((max(n, 1), 4), dtype=torch.float32, device="cuda")
    v4 = torch.zeros((max(n, 1), 4), dtype=torch.float32, device="cuda")
    p4[:n, :3] = torch.as_tensor(np.asarray(pos, dtype=np.float32), device="cuda")
    v4[:n, :3] = torch.as_tensor(np.asarray(vel, dtype=np.float32), device="cuda")
    pid = torch.arange(max(n, 1), dtype=torch.int32, device="cuda")
    p64 = torch.as_tensor(np.asarray(pos, dtype=np.float32).astype(np.float64), device="cuda")
    return p4[:n], v4[:n], pid[:n], p64


def run_stages(spec, pos, vel, step=0, cap=32):
    """All stages of one step on the GPU.  Returns a dict of numpy arrays in
    original particle order (lists hold original particle ids)."""
    torch = torch_cuda()
    from sphgb import kernels as K
    from sphgb.device import SceneBatch
    batch = SceneBatch([spec])
    n = len(pos)
    p4, v4, pid, p64 = to_device(pos, vel)
    pipe = spec.mode == 'PIPE'
    vox = K.assign_voxels_to_particles(batch, p4)
    pS, vS, idS, p64S, start, count = K.organize_voxels(batch, p4, v4, pid, p64 if pipe else None)
    lst, nc, nu = K.get_neighbours(batch, pS, start, count, cap=cap)
    rho = K.density(batch, pS, start, count)
    P, V = K.pressure_viscosity(batch, pS, vS, rho, start, count)
    steps = torch.full((1,), step, dtype=torch.int32, device="cuda")
    pN, vN, idN, p64N, F = K.integrate(batch, pS, vS, rho, idS, start, count, steps,
                                       p64S if pipe else None)
    torch.cuda.synchronize()
    ids = idS.cpu().numpy()
    out = dict(voxel=vox.cpu().numpy(), sorted_pid=ids, start=start.cpu().numpy(),
               count=count.cpu().numpy())

    def unsort(a):
        a = a.cpu().numpy()
        r = np.empty_like(a)
        r[ids] = a
        return r

    l = lst.cpu().numpy()
    lp = np.where(l >= 0, ids[np.clip(l, 0, max(n - 1, 0))], -1)
    out["neigh_list"] = np.empty_like(lp)
    out["neigh_list"][ids] = lp
    out["neigh_count"] = unsort(nc)
    out["neigh_count_uncapped"] = unsort(nu)
    out["density"] = unsort(rho).astype(np.float64)
    out["pressure_term"] = unsort(P)[:, :3].astype(np.float64)
    out["viscosity_term"] = unsort(V)[:, :3].astype(np.float64)
    out["result_force"] = unsort(F)[:, :3].astype(np.float64)
    assert np.array_equal(idN.cpu().numpy(), ids)
    if pipe:
        out["position_out"] = unsort(p64N)
    else:
        out["position_out"] = unsort(pN)[:, :3].astype(np.float64)
    out["velocity_out"] = unsort(vN)[:, :3].astype(np.float64)
    batch.close()
    return out
