"""Device-resident scenes: the state of one or more independent scenes kept in
HBM and advanced by libsphgb.so.

Layout on the device (FP32 unless noted), for N particles over all scenes:
  pos   (N, 4)  x, y, z, unused        -- voxel-sorted slot order
  vel   (N, 4)  vx, vy, vz, unused
  rho   (N,)    density of the last step (computed from its start positions)
  pid   (N,)    int32 particle id within its scene at each slot
  pos64 (N, 3)  FP64 position accumulator (allocated when a scene is a pipe)
  steps (S,)    int32 steps taken per scene (keys the respawn random stream)
Scenes occupy consecutive slot ranges in the order given.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import ctypes as C
import numpy as np

from . import _capi
from .config import SPHConstants, f32
from .data_classes import SimulationParameters, SimulationState


@dataclass
class SceneSpec:
    """One scene: the reference's SimulationParameters plus its constants and
    enclosure mode ('BOX' or 'PIPE', the reference's config.SIM_MODE)."""
    params: SimulationParameters
    constants: SPHConstants = field(default_factory=SPHConstants)
    mode: str = 'BOX'

    @property
    def n(self) -> int:
        return int(self.params.particle_count)


def scene_params(spec: SceneSpec, pipe_row_offset: int = 0) -> _capi.SceneParams:
    """SphgbSceneParams for a scene, every value rounded to FP32 first."""
    p, c = spec.params, spec.constants.rounded()
    sp = _capi.SceneParams()
    sp.particle_count = int(p.particle_count)
    space = f32(np.asarray(p.space_size, dtype=np.float64))
    voxel = f32(np.asarray(p.voxel_size, dtype=np.float64))
    ext = f32(np.asarray(p.external_force, dtype=np.float64))
    for a in range(3):
        sp.space_size[a] = float(space[a])
        sp.voxel_size[a] = float(voxel[a])
        sp.external_force[a] = float(ext[a])
    sp.dt = float(f32(1.0 / float(p.fps)))
    sp.mass, sp.rho_0, sp.inf_r = c.mass, c.rho_0, c.inf_r
    sp.visc, sp.k, sp.damp = c.visc, c.k, c.damp
    sp.max_neighbours = int(c.max_neighbours)
    if spec.mode not in ('BOX', 'PIPE'):
        raise Exception(f'Wrong simulation mode! ({spec.mode})')
    sp.mode = _capi.MODE_PIPE if spec.mode == 'PIPE' else _capi.MODE_BOX
    if c.walk_dims not in ('ceil', 'truncated'):
        raise ValueError(f"walk_dims must be 'ceil' or 'truncated', not {c.walk_dims!r}")
    sp.walk_dims = _capi.WALK_TRUNCATED if c.walk_dims == 'truncated' else _capi.WALK_CEIL
    sp.pipe_rows = len(p.pipe.to_numpy()) if spec.mode == 'PIPE' else 0
    sp.pipe_row_offset = pipe_row_offset if spec.mode == 'PIPE' else 0
    sp.seed = int(c.seed)
    return sp


class SceneBatch:
    """Scenes resident on one GPU, advanced together by one launch sequence."""

    def __init__(self, specs: Sequence[SceneSpec], device: str = "cuda"):
        import torch
        self._torch = torch
        self.device = torch.device(device)
        self._ctx = None
        self.out_pos = self.out_vel = self.out_pid = self.out_pos64 = None
        self.step_limits = None
        self._configure(specs)

    def _tables(self, specs):
        rows, params = [], []
        for s in specs:
            params.append(scene_params(s, pipe_row_offset=len(rows)))
            if s.mode == 'PIPE':
                rows.extend(np.asarray(s.params.pipe.to_numpy(), dtype=np.float64))
        table = (np.ascontiguousarray(np.stack(rows), dtype=np.float64) if rows
                 else np.zeros((0, 5)))
        return (_capi.SceneParams * len(params))(*params), table, len(rows)

    def _configure(self, specs, steps=None):
        torch = self._torch
        specs = list(specs)
        if not specs:
            raise ValueError("need at least one scene")
        lib = _capi.load()
        arr, table, n_rows = self._tables(specs)
        pipe_ptr = table.ctypes.data if n_rows else None
        with torch.cuda.device(self.device):
            if self._ctx is None:
                handle = C.c_void_p()
                _capi.check(lib.sphgb_ctx_create(arr, len(specs), pipe_ptr, n_rows,
                                                 C.byref(handle)), "sphgb_ctx_create")
                self._ctx = handle
            else:
                _capi.check(lib.sphgb_ctx_reconfigure(self._ctx, arr, len(specs), pipe_ptr, n_rows),
                            "sphgb_ctx_reconfigure")
        self.specs = specs
        self._params, self.pipe_table = arr, table
        n = C.c_int64()
        v = C.c_int64()
        _capi.check(lib.sphgb_ctx_sizes(self._ctx, C.byref(n), C.byref(v)), "sphgb_ctx_sizes")
        self.n, self.n_voxels = int(n.value), int(v.value)
        self.scene_sizes = [s.n for s in self.specs]
        self.scene_offsets = list(np.concatenate([[0], np.cumsum(self.scene_sizes)[:-1]]).astype(int))
        self.any_pipe = any(s.mode == 'PIPE' for s in self.specs)
        dev = self.device
        self.pos = torch.zeros((max(self.n, 1), 4), dtype=torch.float32, device=dev)
        self.vel = torch.zeros((max(self.n, 1), 4), dtype=torch.float32, device=dev)
        self.rho = torch.zeros((max(self.n, 1),), dtype=torch.float32, device=dev)
        self.pid = torch.zeros((max(self.n, 1),), dtype=torch.int32, device=dev)
        self.pos64 = torch.zeros((max(self.n, 1) if self.any_pipe else 1, 3),
                                 dtype=torch.float64, device=dev)
        self.steps = (torch.zeros((len(self.specs),), dtype=torch.int32, device=dev)
                      if steps is None else steps.to(dev, torch.int32).contiguous())
        _capi.check(lib.sphgb_ctx_bind_state(
            self._ctx, self.pos.data_ptr(), self.vel.data_ptr(), self.rho.data_ptr(),
            self.pid.data_ptr(), self.pos64.data_ptr(), self.steps.data_ptr()),
            "sphgb_ctx_bind_state")
        self.out_pos = self.out_vel = self.out_pid = self.out_pos64 = None
        self.step_limits = None          # the context drops its limits on reconfiguration

    def reconfigure(self, specs: Sequence[SceneSpec], steps=None) -> None:
        """Replace the scenes, reusing the context's scratch where it fits.
        The state is reset (load new states afterwards); ``steps`` optionally
        gives each scene's step count (the respawn stream position)."""
        self._configure(specs, steps)

    def set_tuning(self, sort_block: int = 256, density_variant: int = _capi.DENSITY_WARP,
                   big_voxel: int = 64) -> None:
        """Launch tuning; results are unchanged (see sphgb_ctx_set_tuning)."""
        _capi.call("sphgb_ctx_set_tuning", self._ctx, int(sort_block), int(density_variant),
                   int(big_voxel))

    def set_host_order(self, order: int = _capi.HOST_ORDER_AUTO) -> None:
        """Force-pass order of compute_next_state_host; results are unchanged
        (see sphgb_ctx_set_host_order)."""
        _capi.call("sphgb_ctx_set_host_order", self._ctx, int(order))

    # -- helpers ---------------------------------------------------------
    def _stream(self, stream=None) -> int:
        torch = self._torch
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        return s.cuda_stream

    @property
    def handle(self):
        return self._ctx

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            _capi.load().sphgb_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_output(self, enable: bool = True) -> None:
        """With enable, every step writes its result to separate output
        tensors (self.out_pos, self.out_vel, self.out_pid, self.out_pos64) and
        leaves the bound state unchanged, so repeated steps all start from it."""
        torch = self._torch
        if enable:
            dev, n = self.device, max(self.n, 1)
            self.out_pos = torch.zeros((n, 4), dtype=torch.float32, device=dev)
            self.out_vel = torch.zeros((n, 4), dtype=torch.float32, device=dev)
            self.out_pid = torch.zeros((n,), dtype=torch.int32, device=dev)
            self.out_pos64 = torch.zeros((n if self.any_pipe else 1, 3), dtype=torch.float64,
                                         device=dev)
            _capi.call("sphgb_ctx_bind_output", self._ctx, self.out_pos.data_ptr(),
                       self.out_vel.data_ptr(), self.out_pid.data_ptr(),
                       self.out_pos64.data_ptr() if self.any_pipe else None)
        else:
            _capi.call("sphgb_ctx_bind_output", self._ctx, None, None, None, None)
            self.out_pos = self.out_vel = self.out_pid = self.out_pos64 = None

    # -- state in / out --------------------------------------------------
    def load_states(self, states: Sequence[SimulationState], stream=None) -> None:
        """Upload host states (SimulationState per scene, original particle order)."""
        torch = self._torch
        if len(states) != len(self.specs):
            raise ValueError("one state per scene")
        pos = np.concatenate([np.asarray(s.position, dtype=np.float64).reshape(-1, 3)
                              for s in states])
        vel = np.concatenate([np.asarray(s.velocity, dtype=np.float64).reshape(-1, 3)
                              for s in states])
        if len(pos) != self.n or len(vel) != self.n:
            raise ValueError("state sizes do not match the scenes' particle counts")
        self.load_aos_device(torch.from_numpy(np.ascontiguousarray(pos)).to(self.device),
                             torch.from_numpy(np.ascontiguousarray(vel)).to(self.device), stream)

    def load_aos_device(self, pos_aos, vel_aos, stream=None, reset_steps=True) -> None:
        """Load FP64 (N, 3) device tensors in original order (scene-concatenated)."""
        _capi.call("sphgb_ctx_load_aos_f64", self._ctx, pos_aos.data_ptr(), vel_aos.data_ptr(),
                   self._stream(stream))
        if reset_steps:
            self.steps.zero_()

    def export_aos_f64(self, stream=None):
        """(pos, vel, rho) as FP64 device tensors in original particle order."""
        torch = self._torch
        n = max(self.n, 1)
        pos = torch.empty((n, 3), dtype=torch.float64, device=self.device)
        vel = torch.empty((n, 3), dtype=torch.float64, device=self.device)
        rho = torch.empty((n,), dtype=torch.float64, device=self.device)
        _capi.call("sphgb_ctx_store_aos_f64", self._ctx, pos.data_ptr(), vel.data_ptr(),
                   rho.data_ptr(), self._stream(stream))
        return pos[:self.n], vel[:self.n], rho[:self.n]

    def states(self) -> List[SimulationState]:
        pos, vel, rho = (t.cpu().numpy() for t in self.export_aos_f64())
        out = []
        for off, n in zip(self.scene_offsets, self.scene_sizes):
            out.append(SimulationState(pos[off:off + n].copy(), vel[off:off + n].copy(),
                                       rho[off:off + n].copy()))
        return out

    # -- stepping and diagnostics ----------------------------------------
    def set_step_limits(self, limits=None) -> None:
        """Per-scene step limits (sphgb_ctx_set_step_limits): a sequence of one
        step count per scene, or a device int32 tensor, or None to remove
        them.  A scene whose step counter (self.steps) has reached its limit
        is frozen: later steps leave it unchanged.  The tensor is kept as
        self.step_limits; writing new values into it needs no new call."""
        torch = self._torch
        if limits is None:
            self.step_limits = None
            _capi.call("sphgb_ctx_set_step_limits", self._ctx, None)
            return
        t = torch.as_tensor(limits, dtype=torch.int32, device=self.device).contiguous()
        if t.numel() != len(self.specs):
            raise ValueError("one step limit per scene")
        self.step_limits = t
        _capi.call("sphgb_ctx_set_step_limits", self._ctx, t.data_ptr())

    def step(self, n_steps: int = 1, use_graph: bool = False, stream=None) -> None:
        _capi.call("sphgb_ctx_step", self._ctx, int(n_steps), 1 if use_graph else 0,
                   self._stream(stream))

    STAGES = ("hash", "scan", "scatter", "rank_gather", "density", "force_integrate",
              "step_counter")

    def step_profiled(self, n_steps: int = 1, stream=None) -> dict:
        """Step without a graph, timing every stage with CUDA events on the
        launching stream; returns mean milliseconds per step per stage."""
        out = (C.c_float * len(self.STAGES))()
        _capi.call("sphgb_ctx_step_profiled", self._ctx, int(n_steps), self._stream(stream), out)
        return dict(zip(self.STAGES, [float(v) for v in out]))

    def conservation(self, stream=None) -> np.ndarray:
        """(S, 8) FP64: mass, momentum xyz, kinetic, potential, total energy, particles."""
        torch = self._torch
        out = torch.zeros((len(self.specs), 8), dtype=torch.float64, device=self.device)
        _capi.call("sphgb_ctx_conservation", self._ctx, out.data_ptr(), self._stream(stream))
        return out.cpu().numpy()

    def neighbour_counts(self, stream=None):
        """(capped, uncapped) neighbour counts per particle, original order."""
        torch = self._torch
        n = max(self.n, 1)
        cap = torch.zeros((n,), dtype=torch.int32, device=self.device)
        unc = torch.zeros((n,), dtype=torch.int32, device=self.device)
        _capi.call("sphgb_ctx_neighbour_counts", self._ctx, cap.data_ptr(), unc.data_ptr(),
                   self._stream(stream))
        return cap[:self.n].cpu().numpy(), unc[:self.n].cpu().numpy()

    def step_neighbours(self, stream=None):
        """The latest step's neighbour lists as the force pass read them:
        (list (N, 32) int32 of scene-local particle ids in walk order, self
        left out, -1 padded; count (N,) int32, -1 above 32), original order,
        as device tensors (see sphgb_ctx_step_neighbours)."""
        torch = self._torch
        n = max(self.n, 1)
        lst = torch.empty((n, 32), dtype=torch.int32, device=self.device)
        cnt = torch.empty((n,), dtype=torch.int32, device=self.device)
        _capi.call("sphgb_ctx_step_neighbours", self._ctx, lst.data_ptr(), cnt.data_ptr(),
                   self._stream(stream))
        return lst[:self.n], cnt[:self.n]

    def set_checks(self, enable: bool = True) -> None:
        """Checked mode: validate every later step into the error word."""
        _capi.call("sphgb_ctx_set_checks", self._ctx, 1 if enable else 0)

    def check_word(self, clear: bool = False, stream=None):
        """(bits, smallest flagged original index or None, flagged
        particle-steps) of checked mode; synchronises the stream."""
        w = (C.c_uint32 * 3)()
        _capi.call("sphgb_ctx_check_word", self._ctx, w, 1 if clear else 0, self._stream(stream))
        return int(w[0]), (None if w[1] == 0xFFFFFFFF else int(w[1])), int(w[2])

    def compute_next_state_host(self, pos, vel, pos_out=None, vel_out=None, rho_out=None):
        """One step through the host-buffer entry point (one-scene batches)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        n = self.n
        pos_out = np.empty((n, 3)) if pos_out is None else pos_out
        vel_out = np.empty((n, 3)) if vel_out is None else vel_out
        rho_out = np.empty((n,)) if rho_out is None else rho_out
        _capi.call("sphgb_compute_next_state_host", self._ctx, pos.ctypes.data, vel.ctypes.data,
                   pos_out.ctypes.data, vel_out.ctypes.data, rho_out.ctypes.data)
        return pos_out, vel_out, rho_out
