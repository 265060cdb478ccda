"""Fluent pipe builder, interface-compatible with the reference's
``common/pipe_builder.py`` (iwoplaza/cuda-sph): same methods, same
AssertionError messages, same ``transform`` rescaling.
"""
from __future__ import annotations

from typing import Tuple

from .data_classes import Pipe, Segment


class PipeBuilder:
    """Builds a Pipe segment by segment (pipe_builder.py:6-161).

    The first segment is configured with the ``with_*`` methods; every
    ``add_*`` call appends a segment that starts where the previous one ends,
    with the previous end radius as its start radius.
    """
    _FIRST_SEGMENT_MESSAGE = "First segment can't be change after adding new segments"
    _NEGATIVE_RADIUS_MESSAGE = "Radius must be positive"
    _NEGATIVE_CHANGE_MESSAGE = "Change must be positive"
    _NEGATIVE_LENGTH_MESSAGE = "Length must be positive"

    def __init__(self) -> None:
        self._editing_first = True
        self._pipe = Pipe(segments=[Segment()])

    def _first(self) -> Segment:
        assert self._editing_first, self._FIRST_SEGMENT_MESSAGE
        return self._pipe.segments[0]

    def with_starting_position(self, position: Tuple[float, float, float]) -> "PipeBuilder":
        self._first().start_point = position
        return self

    def with_starting_radius(self, radius: float) -> "PipeBuilder":
        seg = self._first()
        assert radius > 0, self._NEGATIVE_RADIUS_MESSAGE
        seg.start_radius = radius
        return self

    def with_ending_radius(self, radius: float) -> "PipeBuilder":
        seg = self._first()
        assert radius > 0, self._NEGATIVE_RADIUS_MESSAGE
        seg.end_radius = radius
        return self

    def with_starting_length(self, length: float) -> "PipeBuilder":
        seg = self._first()
        assert length > 0, self._NEGATIVE_LENGTH_MESSAGE
        seg.length = length
        return self

    def add_roller_segment(self, length) -> "PipeBuilder":
        """Append a cylinder of the given length."""
        self._editing_first = False
        assert length > 0, self._NEGATIVE_LENGTH_MESSAGE
        prev = self._pipe.segments[-1]
        x0, y0, z0 = prev.start_point
        self._pipe.segments.append(Segment(
            start_point=(x0 + prev.length, y0, z0),
            start_radius=prev.end_radius,
            end_radius=prev.end_radius,
            length=length))
        return self

    def add_lessening_segment(self, length, change) -> "PipeBuilder":
        """Append a cone whose end radius is ``change`` smaller than its start."""
        self.add_roller_segment(length)
        assert change > 0, self._NEGATIVE_CHANGE_MESSAGE
        last = self._pipe.segments[-1]
        assert change < last.end_radius, "After change radius must be positive"
        last.end_radius = last.end_radius - change
        return self

    def add_increasing_segment(self, length, change) -> "PipeBuilder":
        """Append a cone whose end radius is ``change`` larger than its start."""
        self.add_roller_segment(length)
        assert change > 0, self._NEGATIVE_CHANGE_MESSAGE
        last = self._pipe.segments[-1]
        last.end_radius = last.end_radius + change
        return self

    def transform(self, space_size_x: float, space_size_yz: float,
                  max_radius: float = None) -> "PipeBuilder":
        """Fit the pipe into a space: x from 0 to space_size_x, axis at
        y = z = space_size_yz / 2, radii scaled so the largest is max_radius
        (space_size_yz / 2 when not given)."""
        segs = self._pipe.segments
        scale_x = space_size_x / sum(s.length for s in segs)
        centre = space_size_yz / 2.0
        x = 0.0
        for s in segs:
            s.start_point = (x, centre, centre)
            s.length = s.length * scale_x
            x += s.length
        if not max_radius:
            max_radius = space_size_yz / 2.0
        biggest = 0.0
        for s in segs:
            biggest = max(biggest, s.start_radius, s.end_radius)
        scale_r = max_radius / biggest
        for s in segs:
            s.start_radius = s.start_radius * scale_r
            s.end_radius = s.end_radius * scale_r
        return self

    def get_result(self) -> Pipe:
        return self._pipe
