"""Frame writer, format-compatible with the reference's
``common/serializer/saver.py`` (iwoplaza/cuda-sph).

On-disk format (unchanged): ``<out>/params.json`` holding
``dataclasses.asdict(params)`` (ndarrays as lists, sorted keys, indent 4) and,
per saved epoch k, ``position_k.npy``, ``velocity_k.npy`` and
``density_k.npy``.  ``AsyncFrameSaver`` writes the same files from
device-resident state: the device-to-host copy of a frame runs on a side
stream into pinned memory and the ``.npy`` files are written by a background
thread, so frames overlap with the next steps.
"""
from __future__ import annotations

import dataclasses
import json
import os
import queue
import threading

import numpy as np

from .. import config
from ..data_classes import SimulationParameters, SimulationState


def _out_path(out_dirname: str) -> str:
    return os.path.join(str(config.ROOT_PROJ_DIRNAME), out_dirname)


def write_params(folder: str, params: SimulationParameters) -> None:
    """params.json as saver.py:38-46 writes it."""
    d = dataclasses.asdict(params)
    for key, value in d.items():
        if type(value) is np.ndarray:
            d[key] = value.tolist()
    with open(os.path.join(folder, config.PARAMS_FILENAME), "w") as f:
        json.dump(d, f, default=lambda o: o.__dict__, sort_keys=True, indent=4)


class Saver:
    """Writes params.json once and one set of .npy files per epoch (saver.py:9-46)."""

    def __init__(self, out_dirname: str, params: SimulationParameters) -> None:
        self._folder = _out_path(out_dirname)
        if not os.path.exists(self._folder):
            os.mkdir(self._folder)
        write_params(self._folder, params)
        self._epoch = 0

    def save_next_state(self, state: SimulationState) -> None:
        for name, value in vars(state).items():
            np.save(os.path.join(self._folder, f"{name}_{self._epoch}"), value)
        self._epoch += 1


class AsyncFrameSaver:
    """Saver for device-resident scenes (same files as ``Saver``).

    ``save(scenes, index=0)`` snapshots one scene of a ``SceneBatch``: a side
    CUDA stream waits for the producer stream, converts the FP32 voxel-sorted
    state to FP64 arrays in original particle order and copies them into
    pinned host buffers; a writer thread then waits for that copy and writes
    the ``.npy`` files.  ``close()`` flushes everything.  At most ``depth``
    frames are in flight; ``save`` blocks when that many are queued.
    """

    def __init__(self, out_dirname: str, params: SimulationParameters, depth: int = 3) -> None:
        import torch
        self._torch = torch
        self._folder = _out_path(out_dirname)
        os.makedirs(self._folder, exist_ok=True)
        write_params(self._folder, params)
        self._epoch = 0
        self._stream = torch.cuda.Stream()
        self._free: "queue.Queue" = queue.Queue()
        self._todo: "queue.Queue" = queue.Queue()
        self._depth = depth
        self._bufs_made = 0
        self._error = None
        self._thread = threading.Thread(target=self._writer, daemon=True)
        self._thread.start()

    def _buffers(self, n):
        """A free set of pinned buffers for n particles (at most `depth` sets live)."""
        torch = self._torch
        while True:
            try:
                bufs = self._free.get_nowait()
            except queue.Empty:
                if self._bufs_made < self._depth:
                    self._bufs_made += 1
                    pin = dict(dtype=torch.float64, pin_memory=True)
                    return (torch.empty((n, 3), **pin), torch.empty((n, 3), **pin),
                            torch.empty((n,), **pin))
                bufs = self._free.get()
            if bufs[0].shape[0] == n:
                return bufs
            self._bufs_made -= 1   # wrong size: let it go

    def save(self, scenes, index: int = 0) -> None:
        if self._error:
            raise self._error
        torch = self._torch
        n = scenes.scene_sizes[index]
        hp, hv, hr = self._buffers(n)
        producer = torch.cuda.current_stream()
        self._stream.wait_stream(producer)
        with torch.cuda.stream(self._stream):
            dp, dv, dr = scenes.export_aos_f64(stream=self._stream)
            # the next steps rewrite the state in place: they wait for the
            # export (a short kernel), not for the copies to the host
            exported = torch.cuda.Event()
            exported.record(self._stream)
            lo = scenes.scene_offsets[index]
            hp.copy_(dp[lo:lo + n], non_blocking=True)
            hv.copy_(dv[lo:lo + n], non_blocking=True)
            hr.copy_(dr[lo:lo + n], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self._stream)
        producer.wait_event(exported)
        self._todo.put((self._epoch, ev, (hp, hv, hr)))
        self._epoch += 1

    def _writer(self):
        while True:
            item = self._todo.get()
            if item is None:
                return
            epoch, ev, (hp, hv, hr) = item
            try:
                ev.synchronize()
                for name, t in (("position", hp), ("velocity", hv), ("density", hr)):
                    np.save(os.path.join(self._folder, f"{name}_{epoch}"), t.numpy())
            except Exception as e:  # surfaced on the next save/close
                self._error = e
            self._free.put((hp, hv, hr))

    def close(self) -> None:
        self._todo.put(None)
        self._thread.join()
        if self._error:
            raise self._error
