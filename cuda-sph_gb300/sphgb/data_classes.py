"""Simulation data classes, interface-compatible with the reference's
``common/data_classes.py`` (iwoplaza/cuda-sph).

Same class names, field names, defaults and ``to_numpy`` layout.  The ndarray
defaults are produced by ``default_factory`` so the module imports on Python
3.11+ (the reference's class-level ndarray defaults, :73-85, raise there).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np


@dataclass
class Segment:
    """One pipe segment (common/data_classes.py:7-27): a truncated cone along x."""
    start_point: Tuple[np.float64, np.float64, np.float64] = (0.0, 0.0, 0.0)
    start_radius: np.float64 = 1.0
    end_radius: np.float64 = 1.0
    length: np.float64 = 1.0

    def to_numpy(self) -> np.ndarray:
        """Row ``[x0, y0, z0, start_radius, length]``."""
        x0, y0, z0 = self.start_point
        return np.array([x0, y0, z0, self.start_radius, self.length], dtype=np.float64)

    def radius_at(self, t: float):
        """Radius at x = t, linear between the end radii."""
        if self.start_radius == self.end_radius:
            return self.start_radius
        frac = (t - self.start_point[0]) / self.length
        return self.start_radius + (self.end_radius - self.start_radius) * frac


@dataclass(frozen=True)
class Pipe:
    """Sequence of segments (common/data_classes.py:30-67)."""
    segments: List[Segment] = field(default_factory=list)

    def to_numpy(self) -> np.ndarray:
        """Kernel pipe table: one row per segment plus a closing row.

        The closing row repeats the last segment's row with x advanced by its
        length and the radius set to its end radius (data_classes.py:34-44).
        The device kernels interpolate the radius of segment j between rows j
        and j + 1.
        """
        if not self.segments:
            return np.asarray([])
        rows = [s.to_numpy() for s in self.segments]
        tail = self.segments[-1].to_numpy()
        tail[0] += tail[4]
        tail[3] = self.segments[-1].end_radius
        rows.append(tail)
        return np.stack(rows)

    def get_length(self):
        return float(sum(s.length for s in self.segments))

    def find_segment(self, t: float):
        """Index of the segment whose closed x-interval holds t, or -1."""
        for i, s in enumerate(self.segments):
            if s.start_point[0] <= t <= s.start_point[0] + s.length:
                return i
        return -1

    def radius_at(self, t: float):
        return self.segments[self.find_segment(t)].radius_at(t)


@dataclass(frozen=True)
class SimulationParameters:
    """Run parameters (common/data_classes.py:70-78)."""
    particle_count: np.int32 = 100
    external_force: np.ndarray = field(default_factory=lambda: np.asarray([0, 0, 0]))
    duration: np.int32 = 10
    fps: np.int32 = 20
    pipe: Pipe = field(default_factory=lambda: Pipe([Segment()]))
    space_size: np.ndarray = field(default_factory=lambda: np.asarray([1, 1, 1]))
    voxel_size: np.ndarray = field(default_factory=lambda: np.asarray([1, 1, 1]))


@dataclass(frozen=True)
class SimulationState:
    """Particle state (common/data_classes.py:81-85): position (n, 3),
    velocity (n, 3), density (n,)."""
    position: np.ndarray = field(default_factory=lambda: np.asarray([[1, 1, 1]]))
    velocity: np.ndarray = field(default_factory=lambda: np.asarray([[1, 1, 1]]))
    density: np.ndarray = field(default_factory=lambda: np.asarray([1]))
