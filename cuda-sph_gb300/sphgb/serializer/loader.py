"""Frame reader, format-compatible with the reference's
``common/serializer/loader.py`` (iwoplaza/cuda-sph)."""
from __future__ import annotations

import json
import os
from dataclasses import fields

import numpy as np

from .. import config
from ..data_classes import Pipe, Segment, SimulationParameters, SimulationState


class Loader:
    """Reads params.json and per-epoch state files (loader.py:9-64)."""

    def __init__(self, out_dirname: str) -> None:
        self._folder = os.path.join(str(config.ROOT_PROJ_DIRNAME), out_dirname)
        if not os.path.exists(self._folder):
            raise Exception(f'Directory ({self._folder}) does not exists! '
                            f'Could not load simulation!')
        with open(os.path.join(self._folder, config.PARAMS_FILENAME)) as f:
            self._json = json.load(f)

    def load_simulation_parameters(self) -> SimulationParameters:
        values = {}
        for f in fields(SimulationParameters):
            if f.name == "pipe":
                values["pipe"] = self._load_pipe()
            elif f.type == "np.ndarray":
                values[f.name] = np.asarray(self._json[f.name])
            else:
                values[f.name] = self._json[f.name]
        return SimulationParameters(**values)

    def _load_pipe(self) -> Pipe:
        return Pipe([
            Segment(start_point=tuple(s["start_point"]), start_radius=s["start_radius"],
                    end_radius=s["end_radius"], length=s["length"])
            for s in self._json["pipe"]["segments"]])

    def load_simulation_state(self, epoch: int) -> SimulationState:
        arrays = {f.name: np.load(os.path.join(self._folder, f"{f.name}_{epoch}.npy"))
                  for f in fields(SimulationState)}
        return SimulationState(**arrays)
