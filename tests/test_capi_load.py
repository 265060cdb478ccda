"""The C ABI library loads and exports exactly what include/sphgb.h declares
(CPU only: no compute calls)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from sphgb import _build, _capi

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "sphgb.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sphgb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _capi.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _build.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (sphgb_[a-z0-9_]+)\b", out))
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    extra = sorted(exported - set(names))
    assert not extra, f"exported but not declared: {extra}"
    for n in names:
        assert hasattr(lib, n)


def test_binding_covers_header(lib):
    assert sorted(n for n, _, _ in _capi.SIGNATURES) == declared_functions()


def test_abi_and_struct_layout(lib):
    assert lib.sphgb_abi_version() == 1
    assert lib.sphgb_scene_params_size() == C.sizeof(_capi.SceneParams)
    from oracle import ref
    assert C.sizeof(ref.SceneParams) == C.sizeof(_capi.SceneParams)


def test_invalid_arguments_are_rejected_without_a_gpu(lib):
    """Argument checks run before any CUDA call."""
    out = C.c_void_p()
    assert lib.sphgb_ctx_create(None, 0, None, 0, C.byref(out)) == -1
    assert "at least one scene" in _capi.last_error()
    p = _capi.SceneParams()
    p.particle_count = 10
    p.inf_r = -1.0
    p.dt = 0.1
    assert lib.sphgb_ctx_create(C.byref(p), 1, None, 0, C.byref(out)) == -1
    assert "inf_r" in _capi.last_error()
    assert lib.sphgb_ctx_step(None, 1, 0, None) == -1
    with pytest.raises(_capi.SphgbError):
        _capi.call("sphgb_ctx_step", None, 1, 0, None)
    assert lib.sphgb_compute_next_state_host(None, None, None, None, None, None) == -1
    assert "ctx is null" in _capi.last_error()
    assert lib.sphgb_ctx_set_host_order(None, _capi.HOST_ORDER_SLOT) == -1
    assert "ctx is null" in _capi.last_error()


def test_noalloc_refuses_misaligned_buffers_without_a_gpu(lib):
    """The allocation-free voxel sort moves positions and velocities as float4
    and the voxel table in int4 quads, so each buffer must be 16-byte aligned.
    The check runs before any CUDA call: the addresses here are never touched."""
    from sphgb import scenes
    from sphgb.device import scene_params
    spec, _ = scenes.config0()
    sp = scene_params(spec)
    base = 0x10000000
    good = [base + 0x100000 * k for k in range(8)]
    names = ["d_pos", "d_vel", "d_pid", "d_pos_out", "d_vel_out", "d_pid_out", "d_voxel_start",
             "d_voxel_count"]
    for i, name in enumerate(names):
        for off in (4, 8, 12):
            bufs = list(good)
            bufs[i] += off
            rc = lib.sphgb_organize_voxels_noalloc(C.byref(sp), *bufs, None)
            assert rc == -1, (name, off, rc)
            assert name in _capi.last_error() and "16-byte" in _capi.last_error()


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    monkeypatch.setattr(_capi, "_lib", None)
    monkeypatch.setattr(_capi, "lib_path", lambda: str(tmp_path / "missing.so"))
    with pytest.raises(OSError, match="no CPU fallback"):
        _capi.load()
