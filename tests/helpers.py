"""Shared test helpers: golden fixtures, scene conversions, comparisons."""
from __future__ import annotations

import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_CASES = ["box_unaligned", "box_aligned", "box_defaults", "pipe_defaults"]
# cases whose space is a multiple of the voxel size: ceil walk dims == truncated
ALIGNED_CASES = ["box_aligned", "box_defaults", "pipe_defaults"]


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, f"{name}.npz")))


def golden_spec(d, walk_dims="truncated"):
    """SceneSpec of a golden case (constants exactly as the reference ran them)."""
    from sphgb.config import SPHConstants
    from sphgb.data_classes import Pipe, Segment, SimulationParameters
    from sphgb.device import SceneSpec
    mode = str(d["mode"])
    rows = d["pipe_rows"]
    if mode == "PIPE":
        segs = []
        for r in range(len(rows) - 1):
            segs.append(Segment(start_point=tuple(rows[r, :3]), start_radius=rows[r, 3],
                                end_radius=rows[r + 1, 3], length=rows[r, 4]))
        pipe = Pipe(segs)
    else:
        pipe = Pipe([Segment()])
    params = SimulationParameters(
        particle_count=d["position_in"].shape[1], external_force=d["external_force"],
        duration=1, fps=float(d["fps"]), pipe=pipe, space_size=d["space_size"],
        voxel_size=d["voxel_size"])
    c = SPHConstants(mass=float(d["mass"]), rho_0=float(d["rho_0"]), inf_r=float(d["inf_r"]),
                     visc=float(d["visc"]), k=float(d["k"]), damp=float(d["damp"]),
                     max_neighbours=int(d["max_neighbours"]), walk_dims=walk_dims,
                     seed=int(d["seed"]))
    return SceneSpec(params, c, mode)


def in_domain(pos, space):
    return np.all((pos >= 0) & (pos < np.asarray(space)), axis=1)


def rel_err(a, b, scale=None):
    """max |a-b| / max(|b|, scale) over finite entries of b; non-finite masks must agree."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), f"non-finite pattern differs at {np.argwhere(fa != fb)[:5]}"
    if not fb.any():
        return 0.0
    den = np.abs(b)
    if scale is not None:
        den = np.fmax(den, np.broadcast_to(scale, den.shape))
    den = np.fmax(den, 1e-300)
    return float(np.max(np.abs(a[fb] - b[fb]) / den[fb]))
