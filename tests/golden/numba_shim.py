"""Minimal CPU stand-in for the parts of ``numba.cuda`` that the reference uses.

Test infrastructure only.  numba is not installed here, but the reference's GPU
code (``sim/src/sph/kernels/*.py`` of iwoplaza/cuda-sph) is ordinary Python
decorated with ``@cuda.jit``.  Installing this module as ``numba`` in
``sys.modules`` lets ``make_golden.py`` import and execute the reference's own
kernels and strategies, one simulated thread at a time, to record golden
input/output vectors.

What it emulates and how:

* ``cuda.jit`` / ``cuda.jit(device=True)`` return the Python function; a kernel
  is launched with ``kernel[grid, block](*args)``, which runs every thread in
  order, setting ``cuda.threadIdx.x``, ``cuda.blockIdx.x``, ``cuda.blockDim.x``.
* ``cuda.local.array`` returns a fresh numpy array.  numba leaves local arrays
  uninitialised; integer arrays are filled with ``-1`` here, which makes the
  never-written tail of ``neigh_voxels`` (``voxel_kernels.py:44,64-65``) read as
  "no voxel" -- the interpretation the rest of this project implements.
* device arrays are numpy arrays of class ``DeviceArray``; a scalar read one
  past the end of a 1-D array returns ``0`` instead of raising, which is what
  the ``while`` at ``voxel_kernels.py:70`` needs (its result does not depend on
  the value read, see ``make_golden.py``).  Such reads are counted.
* ``numba.cuda.random``: the reference draws respawn positions with numba's
  xoroshiro128p generator (``base_kernels.py:108-109``).  This shim replaces the
  stream with the project's own counter-based Philox4x32-10 keyed by
  ``(seed, thread index)`` with counter ``(step, draw)``, so that golden pipe
  vectors use exactly the uniforms the CUDA path uses.  ``set_rng_step`` sets
  the step before each strategy call.
"""
from __future__ import annotations

import sys
import types

import numpy as np

from philox_ref import philox_uniform_f64  # noqa: E402  (sibling module)


class DeviceArray(np.ndarray):
    """numpy array that tolerates a scalar read one past the end of axis 0."""

    oob_reads = 0

    def __getitem__(self, idx):
        if (self.ndim == 1 and isinstance(idx, (int, np.integer))
                and int(idx) == self.shape[0]):
            DeviceArray.oob_reads += 1
            return self.dtype.type(0)
        return super().__getitem__(idx)

    def copy_to_host(self):
        return np.array(self, copy=True).view(np.ndarray)


def _to_device(arr):
    return np.array(arr, copy=True).view(DeviceArray)


class _Dim:
    __slots__ = ("x", "y", "z")

    def __init__(self):
        self.x = 0
        self.y = 0
        self.z = 0


class _Kernel:
    def __init__(self, fn):
        self.fn = fn

    def __getitem__(self, cfg):
        grid, block = cfg
        grid = int(grid)
        block = int(block)

        def launch(*args):
            cuda.blockDim.x = block
            for b in range(grid):
                cuda.blockIdx.x = b
                for t in range(block):
                    cuda.threadIdx.x = t
                    self.fn(*args)

        return launch

    def __call__(self, *args, **kwargs):  # device-function style call
        return self.fn(*args, **kwargs)


def _jit(fn=None, device=False, **_kw):
    def wrap(f):
        return f if device else _Kernel(f)

    if fn is None:
        return wrap
    return wrap(fn)


class _Local:
    @staticmethod
    def array(shape, dtype):
        dt = np.dtype(dtype)
        if np.issubdtype(dt, np.integer):
            return np.full(shape, -1, dtype=dt)
        return np.zeros(shape, dtype=dt)


class _Device:
    compute_capability = (8, 6)


cuda = types.ModuleType("numba.cuda")
cuda.jit = _jit
cuda.local = _Local()
cuda.threadIdx = _Dim()
cuda.blockIdx = _Dim()
cuda.blockDim = _Dim()
cuda.to_device = _to_device
cuda.synchronize = lambda: None
cuda.get_current_device = lambda: _Device()

_rng = {"step": 0}


def set_rng_step(step: int) -> None:
    _rng["step"] = int(step)


class _RngStates:
    def __init__(self, n, seed):
        self.seed = int(seed)
        self.draws = {}


def create_xoroshiro128p_states(n, seed=0, **_kw):
    return _RngStates(n, seed)


def xoroshiro128p_uniform_float64(states, i):
    i = int(i)
    key = (i, _rng["step"])
    k = states.draws.get(key, 0)
    states.draws[key] = k + 1
    return philox_uniform_f64(states.seed, i, _rng["step"], k)


random_mod = types.ModuleType("numba.cuda.random")
random_mod.create_xoroshiro128p_states = create_xoroshiro128p_states
random_mod.xoroshiro128p_uniform_float64 = xoroshiro128p_uniform_float64
cuda.random = random_mod

numba = types.ModuleType("numba")
numba.cuda = cuda


def install() -> None:
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda
    sys.modules["numba.cuda.random"] = random_mod
