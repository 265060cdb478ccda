"""Headless point-field vertex stage (sphgb_point_field).

The reference's visualiser draws every particle as a GL point whose colour
and size come from its density (vis/assets/point_field.vert:14-23,
point_field.frag:5-9).  This module computes the same per-vertex values on
the device -- clip-space position, RGBA colour and point size -- into device
tensors, with no window, swapchain or graphics API.  ``frame_attributes``
takes them straight from a SceneBatch's device state.
"""
from __future__ import annotations

import numpy as np

from . import _capi


def _mat(m) -> np.ndarray:
    """4x4 matrix as 16 column-major FP32 values (a GLSL mat4 uniform)."""
    a = np.asarray(m, dtype=np.float32)
    if a.shape == (4, 4):
        a = a.T            # row-major numpy (m[row][col]) -> column-major
    a = np.ascontiguousarray(a.reshape(16), dtype=np.float32)
    return a


def point_field(pos, rho, proj, model, view, stream=None):
    """pos: (n, 3) or (n, 4) FP32 device tensor, rho: (n,) FP32 device tensor;
    proj/model/view: 4x4 (row-major numpy) or 16 column-major values.
    Returns (clip (n, 4), colour (n, 4), size (n,)) FP32 device tensors."""
    import torch
    if pos.dtype != torch.float32 or rho.dtype != torch.float32:
        raise TypeError("point_field takes FP32 positions and densities")
    pos = pos.contiguous()
    n = int(rho.shape[0])
    stride = int(pos.shape[1])
    clip = torch.empty((max(n, 1), 4), dtype=torch.float32, device=pos.device)
    colour = torch.empty((max(n, 1), 4), dtype=torch.float32, device=pos.device)
    size = torch.empty((max(n, 1),), dtype=torch.float32, device=pos.device)
    P, M, V = _mat(proj), _mat(model), _mat(view)
    if stream is None:
        stream = torch.cuda.current_stream(pos.device).cuda_stream
    _capi.call("sphgb_point_field", pos.data_ptr(), stride, rho.contiguous().data_ptr(), n,
               P.ctypes.data, M.ctypes.data, V.ctypes.data, clip.data_ptr(), colour.data_ptr(),
               size.data_ptr(), stream)
    return clip[:n], colour[:n], size[:n]


def frame_attributes(batch, proj, model, view):
    """Point-field attributes of every particle of a SceneBatch, in its
    device (voxel-sorted) order, together with the particle ids of that
    order: (clip, colour, size, pid)."""
    clip, colour, size = point_field(batch.pos, batch.rho, proj, model, view)
    return clip, colour, size, batch.pid
