"""Stage-level calls named after the reference's kernels
(sim/src/sph/kernels/{voxel,base,util}_kernels.py of iwoplaza/cuda-sph), on
torch device tensors.  Each launches the same CUDA kernels the fused step uses.

State tensors: pos/vel (N, 4) float32, pid (N,) int32, pos64 (N, 3) float64.
The voxel table is (start, count) int32 of ``scenes.n_voxels`` entries; the
reference's ``voxel_begin[v]`` is ``start[v]`` where ``count[v] > 0``, else -1.
"""
from __future__ import annotations

import numpy as np

from . import _capi


def _torch():
    import torch
    return torch


def _s(stream=None):
    torch = _torch()
    return (stream or torch.cuda.current_stream()).cuda_stream


def _p(t):
    return None if t is None else t.data_ptr()


def assign_voxels_to_particles(scenes, pos, stream=None):
    """voxel_kernels.py:89-105 -> voxel id per particle (int32)."""
    torch = _torch()
    out = torch.empty((max(pos.shape[0], 1),), dtype=torch.int32, device=pos.device)
    _capi.call("sphgb_assign_voxels", scenes.handle, pos.data_ptr(), out.data_ptr(), _s(stream))
    return out[:pos.shape[0]]


def organize_voxels(scenes, pos, vel, pid, pos64=None, stream=None):
    """voxel_sph_strategy.py:65-107 on the device: returns the voxel-sorted
    (pos, vel, pid, pos64) and the voxel table (start, count)."""
    torch = _torch()
    n = pos.shape[0]
    pos_o = torch.empty_like(pos)
    vel_o = torch.empty_like(vel)
    pid_o = torch.empty_like(pid)
    pos64_o = None if pos64 is None else torch.empty_like(pos64)
    nv = max(scenes.n_voxels, 1)
    start = torch.empty((nv,), dtype=torch.int32, device=pos.device)
    count = torch.empty((nv,), dtype=torch.int32, device=pos.device)
    _capi.call("sphgb_organize_voxels", scenes.handle, pos.data_ptr(), vel.data_ptr(),
               pid.data_ptr(), _p(pos64), pos_o.data_ptr(), vel_o.data_ptr(), pid_o.data_ptr(),
               _p(pos64_o), start.data_ptr(), count.data_ptr(), _s(stream))
    del n
    return pos_o, vel_o, pid_o, pos64_o, start, count


def get_neighbours(scenes, pos_sorted, start, count, cap=32, stream=None):
    """voxel_kernels.py:30-85 for every sorted slot: (list of sorted slots,
    capped count, uncapped count)."""
    torch = _torch()
    n = max(pos_sorted.shape[0], 1)
    lst = torch.empty((n, cap), dtype=torch.int32, device=pos_sorted.device)
    nc = torch.empty((n,), dtype=torch.int32, device=pos_sorted.device)
    nu = torch.empty((n,), dtype=torch.int32, device=pos_sorted.device)
    _capi.call("sphgb_neighbours", scenes.handle, pos_sorted.data_ptr(), start.data_ptr(),
               count.data_ptr(), lst.data_ptr(), int(cap), nc.data_ptr(), nu.data_ptr(), _s(stream))
    m = pos_sorted.shape[0]
    return lst[:m], nc[:m], nu[:m]


def density(scenes, pos_sorted, start, count, stream=None):
    """density_kernel, voxel_kernels.py:109-132."""
    torch = _torch()
    rho = torch.empty((max(pos_sorted.shape[0], 1),), dtype=torch.float32, device=pos_sorted.device)
    _capi.call("sphgb_density", scenes.handle, pos_sorted.data_ptr(), start.data_ptr(),
               count.data_ptr(), rho.data_ptr(), _s(stream))
    return rho[:pos_sorted.shape[0]]


def pressure_viscosity(scenes, pos_sorted, vel_sorted, rho_sorted, start, count, stream=None):
    """pressure_kernel + viscosity_kernel, voxel_kernels.py:136-211 -> (P, V) (N, 4)."""
    torch = _torch()
    n = max(pos_sorted.shape[0], 1)
    pt = torch.empty((n, 4), dtype=torch.float32, device=pos_sorted.device)
    vt = torch.empty((n, 4), dtype=torch.float32, device=pos_sorted.device)
    _capi.call("sphgb_forces", scenes.handle, pos_sorted.data_ptr(), vel_sorted.data_ptr(),
               rho_sorted.data_ptr(), start.data_ptr(), count.data_ptr(), pt.data_ptr(),
               vt.data_ptr(), _s(stream))
    m = pos_sorted.shape[0]
    return pt[:m], vt[:m]


def integrate(scenes, pos_sorted, vel_sorted, rho_sorted, pid_sorted, start, count, steps,
              pos64_sorted=None, stream=None):
    """Forces + integrating_kernel + wall response (base_kernels.py:30-98):
    returns next (pos, vel, pid, pos64, result_force)."""
    torch = _torch()
    pos_o = torch.empty_like(pos_sorted)
    vel_o = torch.empty_like(vel_sorted)
    pid_o = torch.empty_like(pid_sorted)
    f_o = torch.empty_like(pos_sorted)
    p64_o = None if pos64_sorted is None else torch.empty_like(pos64_sorted)
    _capi.call("sphgb_integrate", scenes.handle, pos_sorted.data_ptr(), vel_sorted.data_ptr(),
               rho_sorted.data_ptr(), pid_sorted.data_ptr(), _p(pos64_sorted), start.data_ptr(),
               count.data_ptr(), steps.data_ptr(), pos_o.data_ptr(), vel_o.data_ptr(),
               pid_o.data_ptr(), _p(p64_o), f_o.data_ptr(), _s(stream))
    return pos_o, vel_o, pid_o, p64_o, f_o


# ---- pipe geometry (util_kernels.py), FP64 ---------------------------------

def _dev_f64(a, device):
    torch = _torch()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device)


def find_segment(position, pipe, device="cuda"):
    """util_kernels.py:72-77 for each row of position (n, 3)."""
    torch = _torch()
    pos = _dev_f64(position, device)
    pp = _dev_f64(pipe, device)
    out = torch.empty((len(pos),), dtype=torch.int32, device=device)
    _capi.call("sphgb_pipe_find_segment", pos.data_ptr(), len(pos), pp.data_ptr(), len(pp),
               out.data_ptr(), _s())
    return out.cpu().numpy()


def is_out_of_pipe(position, pipe, segments, device="cuda"):
    """util_kernels.py:46-53 -> (bool array, radius at the position)."""
    torch = _torch()
    pos = _dev_f64(position, device)
    pp = _dev_f64(pipe, device)
    seg = torch.as_tensor(np.ascontiguousarray(segments, dtype=np.int32), device=device)
    out = torch.empty((len(pos),), dtype=torch.int32, device=device)
    rad = torch.empty((len(pos),), dtype=torch.float64, device=device)
    _capi.call("sphgb_pipe_is_out", pos.data_ptr(), seg.data_ptr(), len(pos), pp.data_ptr(),
               len(pp), out.data_ptr(), rad.data_ptr(), _s())
    return out.cpu().numpy().astype(bool), rad.cpu().numpy()


def calc_x_at_segment_beginning(pipe, segments, device="cuda"):
    """util_kernels.py:38-43."""
    torch = _torch()
    pp = _dev_f64(pipe, device)
    seg = torch.as_tensor(np.ascontiguousarray(segments, dtype=np.int32), device=device)
    out = torch.empty((len(seg),), dtype=torch.float64, device=device)
    _capi.call("sphgb_pipe_x_at_segment_beginning", seg.data_ptr(), len(seg), pp.data_ptr(),
               len(pp), out.data_ptr(), _s())
    return out.cpu().numpy()


def solve_collision(position, velocity, pipe, device="cuda"):
    """find_segment then, if out of the pipe, solve_collision (util_kernels.py:
    182-204), per row -> (position, velocity, segment)."""
    torch = _torch()
    pos = _dev_f64(position, device).clone()
    vel = _dev_f64(velocity, device).clone()
    pp = _dev_f64(pipe, device)
    seg = torch.empty((len(pos),), dtype=torch.int32, device=device)
    _capi.call("sphgb_pipe_solve_collision", pos.data_ptr(), vel.data_ptr(), len(pos),
               pp.data_ptr(), len(pp), seg.data_ptr(), _s())
    return pos.cpu().numpy(), vel.cpu().numpy(), seg.cpu().numpy()


def philox_uniform(seed, pids, step, draw, device="cuda"):
    """The respawn stream: uniforms in [0, 1) for (seed, particle id, step, draw)."""
    torch = _torch()
    pid = torch.as_tensor(np.ascontiguousarray(pids, dtype=np.int32), device=device)
    out = torch.empty((len(pid),), dtype=torch.float64, device=device)
    _capi.call("sphgb_philox_uniform", int(seed), pid.data_ptr(), len(pid), int(step), int(draw),
               out.data_ptr(), _s())
    return out.cpu().numpy()
