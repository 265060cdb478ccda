"""ORACLE wrapper (test infrastructure, never product code).

ctypes bindings for oracle/ref_cpu.c, the FP64 CPU restatement of the
reference's voxel SPH step (iwoplaza/cuda-sph,
sim/src/sph/strategies/voxel_sph_strategy.py with the kernels it launches).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
and only as the checker or the timed CPU baseline.

Arrays are numpy FP64 AoS (N, 3) in original particle order, the layout of
SimulationState (common/data_classes.py:81-85).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

MODE_BOX, MODE_PIPE = 0, 1
WALK_CEIL, WALK_TRUNCATED = 0, 1


class SceneParams(C.Structure):
    """Same layout as SphgbSceneParams in include/sphgb.h."""
    _fields_ = [
        ("particle_count", C.c_int64),
        ("space_size", C.c_double * 3),
        ("voxel_size", C.c_double * 3),
        ("external_force", C.c_double * 3),
        ("dt", C.c_double),
        ("mass", C.c_double),
        ("rho_0", C.c_double),
        ("inf_r", C.c_double),
        ("visc", C.c_double),
        ("k", C.c_double),
        ("damp", C.c_double),
        ("max_neighbours", C.c_int32),
        ("mode", C.c_int32),
        ("walk_dims", C.c_int32),
        ("pipe_rows", C.c_int32),
        ("pipe_row_offset", C.c_int64),
        ("seed", C.c_uint64),
    ]


def make_params(*, n, space_size, voxel_size, external_force, dt, mass, rho_0, inf_r, visc,
                k, damp, max_neighbours=32, mode=MODE_BOX, walk_dims=WALK_CEIL, pipe_rows=0,
                seed=16435234) -> SceneParams:
    sp = SceneParams()
    sp.particle_count = int(n)
    for a in range(3):
        sp.space_size[a] = float(space_size[a])
        sp.voxel_size[a] = float(voxel_size[a])
        sp.external_force[a] = float(external_force[a])
    sp.dt, sp.mass, sp.rho_0, sp.inf_r = float(dt), float(mass), float(rho_0), float(inf_r)
    sp.visc, sp.k, sp.damp = float(visc), float(k), float(damp)
    sp.max_neighbours = int(max_neighbours)
    sp.mode, sp.walk_dims, sp.pipe_rows = int(mode), int(walk_dims), int(pipe_rows)
    sp.pipe_row_offset = 0
    sp.seed = int(seed)
    return sp


GEN_LATTICE, GEN_BOX_WALL, GEN_PIPE_FILL = 0, 1, 2


class Generator(C.Structure):
    """Same layout as SphgbGenerator in include/sphgb.h."""
    _fields_ = [
        ("kind", C.c_int32),
        ("lattice", C.c_int32 * 3),
        ("spacing", C.c_double),
        ("jitter", C.c_double),
        ("origin", C.c_double * 3),
        ("extent", C.c_double * 3),
        ("velocity", C.c_double * 3),
        ("velocity_spread", C.c_double),
        ("velocity_sigma", C.c_double),
        ("x_range", C.c_double * 2),
        ("fill", C.c_double),
        ("seed", C.c_uint64),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle.build_oracle import build  # noqa: WPS433
        path = build()
        L = C.CDLL(path)
        P = C.POINTER
        d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        sp = P(SceneParams)
        vp = C.c_void_p
        L.ref_derived.argtypes = [sp, i32, d]
        L.ref_assign_voxels.argtypes = [sp, C.c_int64, d, i32]
        L.ref_organize.argtypes = [sp, C.c_int64, i32, i32, i32, i32]
        L.ref_neighbours.argtypes = [sp, C.c_int64, d, i32, i32, i32, vp, C.c_int, vp, vp]
        L.ref_density.argtypes = [sp, C.c_int64, d, i32, i32, i32, d]
        L.ref_forces.argtypes = [sp, C.c_int64, d, d, d, i32, i32, i32, d, d, vp, vp]
        L.ref_integrate.argtypes = [sp, C.c_int64, d, d, d, d, d, vp, vp, C.c_int32]
        L.ref_step.argtypes = [sp, C.c_int64, d, d, d, vp, vp, vp, vp, C.c_int32]
        L.ref_philox_uniform.argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_int32]
        L.ref_philox_uniform.restype = C.c_double
        L.ref_x_at_segment_beginning.argtypes = [d, C.c_int]
        L.ref_x_at_segment_beginning.restype = C.c_double
        L.ref_radius_in_position.argtypes = [d, d, C.c_int]
        L.ref_radius_in_position.restype = C.c_double
        L.ref_find_segment.argtypes = [d, d, C.c_int]
        L.ref_is_out_of_pipe.argtypes = [d, d, C.c_int]
        L.ref_solve_collision.argtypes = [d, d, d, C.c_int]
        L.ref_collide_pipe_one.argtypes = [d, d, d, C.c_int, C.c_uint64, C.c_int32, C.c_int32]
        f32 = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.ref_generate.argtypes = [P(Generator), vp, C.c_int, C.c_int64, d, d]
        L.ref_point_field.argtypes = [f32, C.c_int, f32, C.c_int64, f32, f32, f32, f32, f32, f32]
        L.ref_num_threads.restype = C.c_int
        L.ref_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def derived(sp):
    dims = np.zeros(6, np.int32)
    consts = np.zeros(5, np.float64)
    lib().ref_derived(C.byref(sp), dims, consts)
    return dims[:3].copy(), dims[3:].copy(), consts


def assign_voxels(sp, pos):
    pos = _c(pos)
    out = np.zeros(len(pos), np.int32)
    lib().ref_assign_voxels(C.byref(sp), len(pos), pos, out)
    return out


def organize(sp, voxel):
    dims, _, _ = derived(sp)
    nv = int(np.prod(dims.astype(np.int64)))
    voxel = _c(voxel, np.int32)
    spid = np.zeros(len(voxel), np.int32)
    start = np.zeros(nv, np.int32)
    count = np.zeros(nv, np.int32)
    rc = lib().ref_organize(C.byref(sp), len(voxel), voxel, spid, start, count)
    assert rc == 0
    return spid, start, count


def neighbours(sp, pos, spid, start, count, with_list=True):
    pos = _c(pos)
    n = len(pos)
    cap = sp.max_neighbours if sp.max_neighbours > 0 else 0
    lst = np.full((n, cap), -1, np.int32) if (with_list and cap > 0) else None
    nc = np.zeros(n, np.int32)
    nu = np.zeros(n, np.int32)
    lib().ref_neighbours(C.byref(sp), n, pos, spid, start, count, _ptr(lst), cap, _ptr(nc), _ptr(nu))
    return lst, nc, nu


def density(sp, pos, spid, start, count):
    pos = _c(pos)
    rho = np.zeros(len(pos))
    rc = lib().ref_density(C.byref(sp), len(pos), pos, spid, start, count, rho)
    assert rc == 0
    return rho


def forces(sp, pos, vel, rho, spid, start, count):
    pos, vel, rho = _c(pos), _c(vel), _c(rho)
    n = len(pos)
    pt, vt, ps, vs = (np.zeros((n, 3)) for _ in range(4))
    rc = lib().ref_forces(C.byref(sp), n, pos, vel, rho, spid, start, count, pt, vt, _ptr(ps), _ptr(vs))
    assert rc == 0
    return pt, vt, ps, vs


def integrate(sp, pos, vel, rho, pt, vt, pipe=None, step=0):
    pos, vel = _c(pos).copy(), _c(vel).copy()
    force = np.zeros_like(pos)
    pipe = None if pipe is None else _c(pipe)
    lib().ref_integrate(C.byref(sp), len(pos), pos, vel, _c(rho), _c(pt), _c(vt),
                        _ptr(force), _ptr(pipe), int(step))
    return pos, vel, force


def step(sp, pos, vel, pipe=None, step_index=0, want_terms=False):
    """One compute_next_state.  Returns (pos, vel, rho[, pressure, viscosity, force])."""
    pos, vel = _c(pos).copy(), _c(vel).copy()
    n = len(pos)
    rho = np.zeros(n)
    pt = np.zeros((n, 3)) if want_terms else None
    vt = np.zeros((n, 3)) if want_terms else None
    ft = np.zeros((n, 3)) if want_terms else None
    pipe = None if pipe is None else _c(pipe)
    rc = lib().ref_step(C.byref(sp), n, pos, vel, rho, _ptr(pt), _ptr(vt), _ptr(ft), _ptr(pipe),
                        int(step_index))
    assert rc == 0
    if want_terms:
        return pos, vel, rho, pt, vt, ft
    return pos, vel, rho


def philox_uniform(seed, pid, step_, draw):
    return lib().ref_philox_uniform(int(seed), int(pid), int(step_), int(draw))


def find_segment(p, pipe):
    pipe = _c(pipe)
    return lib().ref_find_segment(_c(p), pipe, len(pipe))


def is_out_of_pipe(p, pipe, seg):
    return bool(lib().ref_is_out_of_pipe(_c(p), _c(pipe), int(seg)))


def radius_in_position(p, pipe, seg):
    return lib().ref_radius_in_position(_c(p), _c(pipe), int(seg))


def x_at_segment_beginning(pipe, seg):
    return lib().ref_x_at_segment_beginning(_c(pipe), int(seg))


def solve_collision(p, v, pipe, seg):
    p, v = _c(p).copy(), _c(v).copy()
    lib().ref_solve_collision(p, v, _c(pipe), int(seg))
    return p, v


def generate(gen, n, pipe=None):
    """Start state (pos, vel) FP64 (n, 3) of the generator (ref_cpu.c ref_generate)."""
    pos = np.empty((n, 3)); vel = np.empty((n, 3))
    table = None if pipe is None else _c(pipe)
    rows = 0 if pipe is None else len(table)
    ptr = None if table is None else table.ctypes.data_as(C.c_void_p)
    rc = lib().ref_generate(C.byref(gen), ptr, rows, int(n), pos, vel)
    if rc != 0:
        raise ValueError("invalid generator")
    return pos, vel


def point_field(pos, stride, rho, proj, model, view):
    """(clip (n,4), colour (n,4), size (n,)) FP32 of the point-field vertex stage."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)
    rho = np.ascontiguousarray(rho, dtype=np.float32)
    n = len(rho)
    m = [np.ascontiguousarray(x, dtype=np.float32).reshape(16) for x in (proj, model, view)]
    clip = np.empty((n, 4), np.float32); col = np.empty((n, 4), np.float32)
    size = np.empty(n, np.float32)
    lib().ref_point_field(pos, int(stride), rho, n, m[0], m[1], m[2], clip, col, size)
    return clip, col, size


def num_threads():
    return lib().ref_num_threads()


def set_num_threads(n):
    lib().ref_set_num_threads(int(n))


def params_from_spec(spec, pipe_rows=None, exact=False):
    """Oracle SceneParams for a scene description with ``params`` (the
    reference's SimulationParameters), ``constants`` and ``mode`` attributes.
    Every value is rounded to FP32 as the device rounds it, unless ``exact``
    (values as given, dt = 1 / fps in FP64 as the reference computes it)."""
    f = (lambda x: float(x)) if exact else (lambda x: float(np.float32(x)))  # noqa: E731
    p, c = spec.params, spec.constants
    mode = MODE_PIPE if spec.mode == 'PIPE' else MODE_BOX
    rows = 0
    if mode == MODE_PIPE:
        rows = len(p.pipe.to_numpy()) if pipe_rows is None else pipe_rows
    return make_params(
        n=p.particle_count, space_size=[f(v) for v in p.space_size],
        voxel_size=[f(v) for v in p.voxel_size], external_force=[f(v) for v in p.external_force],
        dt=f(1.0 / float(p.fps)), mass=f(c.mass), rho_0=f(c.rho_0), inf_r=f(c.inf_r),
        visc=f(c.visc), k=f(c.k), damp=f(c.damp), max_neighbours=c.max_neighbours, mode=mode,
        walk_dims=WALK_TRUNCATED if c.walk_dims == 'truncated' else WALK_CEIL,
        pipe_rows=rows, seed=c.seed)
