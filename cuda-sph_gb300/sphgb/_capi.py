"""ctypes binding of libsphgb.so (include/sphgb.h).

There is no fallback: if the library cannot be loaded, every entry point
raises.  Device pointers come from torch tensors (``tensor.data_ptr()``) and
streams from ``torch.cuda.current_stream().cuda_stream``.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

MODE_BOX, MODE_PIPE = 0, 1
WALK_CEIL, WALK_TRUNCATED = 0, 1
DENSITY_WARP, DENSITY_THREAD = 0, 1
HOST_ORDER_AUTO, HOST_ORDER_SLOT, HOST_ORDER_PARTICLE, HOST_ORDER_PIPELINED = 0, 1, 2, 3
# checked-mode bits of the error word (sphgb_ctx_set_checks)
CHECK_NONFINITE_INPUT, CHECK_OUT_OF_DOMAIN, CHECK_VOXEL_TABLE = 1, 2, 4
CHECK_NEIGHBOUR_LIST, CHECK_NONFINITE_OUTPUT = 8, 16

ERRORS = {
    -1: "SPHGB_ERR_INVALID",
    -2: "SPHGB_ERR_CUDA",
    -3: "SPHGB_ERR_NOMEM",
    -4: "SPHGB_ERR_STATE",
    -5: "SPHGB_ERR_RANGE",
}


class SphgbError(RuntimeError):
    """A libsphgb entry point returned a negative status."""

    def __init__(self, code, where, message):
        super().__init__(f"{where}: {ERRORS.get(code, code)}: {message}")
        self.code = code


class SceneParams(C.Structure):
    """SphgbSceneParams (include/sphgb.h)."""
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


GEN_LATTICE, GEN_BOX_WALL, GEN_PIPE_FILL = 0, 1, 2


class Generator(C.Structure):
    """SphgbGenerator (include/sphgb.h)."""
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


# (name, restype, argtypes) for every entry point declared in include/sphgb.h
_VP, _I, _I64, _U64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint64
SIGNATURES = [
    ("sphgb_abi_version", _I, []),
    ("sphgb_scene_params_size", _I, []),
    ("sphgb_last_error", C.c_char_p, []),
    ("sphgb_ctx_create", _I, [C.POINTER(SceneParams), _I, _VP, _I, C.POINTER(_VP)]),
    ("sphgb_ctx_destroy", _I, [_VP]),
    ("sphgb_ctx_reconfigure", _I, [_VP, C.POINTER(SceneParams), _I, _VP, _I]),
    ("sphgb_ctx_set_tuning", _I, [_VP, _I, _I, _I]),
    ("sphgb_ctx_sizes", _I, [_VP, C.POINTER(_I64), C.POINTER(_I64)]),
    ("sphgb_ctx_bind_state", _I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    ("sphgb_ctx_bind_output", _I, [_VP, _VP, _VP, _VP, _VP]),
    ("sphgb_ctx_load_aos_f64", _I, [_VP, _VP, _VP, _VP]),
    ("sphgb_ctx_store_aos_f64", _I, [_VP, _VP, _VP, _VP, _VP]),
    ("sphgb_ctx_set_step_limits", _I, [_VP, _VP]),
    ("sphgb_ctx_step", _I, [_VP, _I, _I, _VP]),
    ("sphgb_ctx_step_profiled", _I, [_VP, _I, _VP, C.POINTER(C.c_float)]),
    ("sphgb_compute_next_state_host", _I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    ("sphgb_ctx_set_host_order", _I, [_VP, _I]),
    ("sphgb_ctx_conservation", _I, [_VP, _VP, _VP]),
    ("sphgb_ctx_neighbour_counts", _I, [_VP, _VP, _VP, _VP]),
    ("sphgb_ctx_step_neighbours", _I, [_VP, _VP, _VP, _VP]),
    ("sphgb_ctx_set_checks", _I, [_VP, _I]),
    ("sphgb_ctx_check_word", _I, [_VP, C.POINTER(C.c_uint32), _I, _VP]),
    ("sphgb_assign_voxels", _I, [_VP, _VP, _VP, _VP]),
    ("sphgb_organize_voxels", _I, [_VP] + [_VP] * 10 + [_VP]),
    ("sphgb_organize_voxels_noalloc", _I, [C.POINTER(SceneParams)] + [_VP] * 9),
    ("sphgb_neighbours", _I, [_VP, _VP, _VP, _VP, _VP, _I, _VP, _VP, _VP]),
    ("sphgb_density", _I, [_VP, _VP, _VP, _VP, _VP, _VP]),
    ("sphgb_forces", _I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    ("sphgb_integrate", _I, [_VP] + [_VP] * 13 + [_VP]),
    ("sphgb_pipe_find_segment", _I, [_VP, _I, _VP, _I, _VP, _VP]),
    ("sphgb_pipe_is_out", _I, [_VP, _VP, _I, _VP, _I, _VP, _VP, _VP]),
    ("sphgb_pipe_x_at_segment_beginning", _I, [_VP, _I, _VP, _I, _VP, _VP]),
    ("sphgb_pipe_solve_collision", _I, [_VP, _VP, _I, _VP, _I, _VP, _VP]),
    ("sphgb_philox_uniform", _I, [_U64, _VP, _I, _I, _I, _VP, _VP]),
    ("sphgb_generator_size", _I, []),
    ("sphgb_generate", _I, [C.POINTER(Generator), _VP, _I, _I64, _VP, _VP, _VP]),
    ("sphgb_point_field", _I, [_VP, _I, _VP, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
]

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Load libsphgb.so (raises OSError/RuntimeError if it is not there)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise OSError(
                f"libsphgb.so not found at {path}; build it with "
                "`python -c \"import __graft_entry__ as g; g.build()\"` "
                "(there is no CPU fallback)")
    L = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if L.sphgb_abi_version() != 1:
        raise OSError("libsphgb ABI version mismatch")
    if L.sphgb_scene_params_size() != C.sizeof(SceneParams):
        raise OSError("SphgbSceneParams layout mismatch between libsphgb.so and the binding")
    if L.sphgb_generator_size() != C.sizeof(Generator):
        raise OSError("SphgbGenerator layout mismatch between libsphgb.so and the binding")
    _lib = L
    return L


def last_error() -> str:
    return load().sphgb_last_error().decode("utf-8", "replace")


def check(rc: int, where: str) -> None:
    if rc != 0:
        raise SphgbError(rc, where, last_error())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
