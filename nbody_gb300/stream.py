"""Frame streams in the reference's on-disk format (nbg_stream_* in the C ABI).

DataStream mirrors nbody_data_stream (nbody/nbody_data_stream.h): open(),
write(data) for a frame in host memory, close().  write_engine() is the GPU
path: the frame is taken from the engine's device state, queued on the engine
stream and written by the library's writer thread, so the simulation does not
wait for the file system.  StreamReader mirrors the parts of
nbody_data_stream_reader (nbody/nbody_data_stream_reader.h) that read frames
back.
"""
from __future__ import annotations

import ctypes as C
import logging
import os
from typing import Optional

import numpy as np

from . import _lib

log = logging.getLogger("nbody_gb300")

SEPARATOR = "\t"  # nbody_data_stream::get_idx_separator


def make_idx_name(base: str) -> str:
    return base + ".idx"


def make_dat_name(base: str, part: int) -> str:
    return f"{base}{part}.dat"


def make_col_name(base: str) -> str:
    return base + ".col"


def make_mass_name(base: str) -> str:
    return base + ".mass"


class DataStream:
    """nbody_data_stream: returns 0 on success and -1 on failure, as the
    reference does."""

    def __init__(self):
        self._lib = _lib.load()
        self._w: Optional[int] = None
        self._header = False
        self._engine = None

    def open(self, name: str, max_part_size: int, append_to: "Optional[StreamReader]" = None,
             engine=None) -> int:
        self.close()
        h = C.c_void_p()
        eh = engine.handle if engine is not None else None
        st = self._lib.nbg_stream_open(eh, os.fsencode(name), int(max_part_size),
                                       1 if append_to is not None else 0, C.byref(h))
        if st != 0:
            log.warning("stream open %s failed (status %d)", name, st)
            return -1
        self._w = h.value
        self._engine = engine
        self._header = False
        return 0

    def _set_header(self, data) -> int:
        if self._header:
            return 0
        col = np.ascontiguousarray(data.get_color(), dtype=np.float32)
        mass = np.ascontiguousarray(data.mass, dtype=np.float64)
        st = self._lib.nbg_stream_set_header(self._w, data.get_count(), int(data.box_size),
                                             col.ctypes.data, mass.ctypes.data)
        self._header = st == 0
        return 0 if st == 0 else -1

    def _fail(self, what: str, st: int) -> int:
        log.warning("stream %s failed: %s", what,
                    self._lib.nbg_stream_last_error(self._w).decode(errors="replace"))
        return -1

    def write(self, data) -> int:
        """nbody_data_stream::write: one frame of `data` (host memory)."""
        if data is None or self._w is None:
            return -1
        if self._set_header(data) != 0:
            return -1
        v = np.ascontiguousarray(data.vertices, dtype=np.float64)
        u = np.ascontiguousarray(data.velocities, dtype=np.float64)
        st = self._lib.nbg_stream_write_host(self._w, v.ctypes.data, u.ctypes.data,
                                             int(data.get_step()), float(data.get_time()))
        return 0 if st == 0 else self._fail("write", st)

    def write_engine(self, engine, data) -> int:
        """A frame of the engine's current state y (device), labelled with
        data's step and time; returns once the copy is queued."""
        if self._w is None or engine is None:
            return -1
        if self._set_header(data) != 0:
            return -1
        st = self._lib.nbg_stream_write(self._w, engine.get_y().handle, int(data.get_step()),
                                        float(data.get_time()))
        return 0 if st == 0 else self._fail("write", st)

    def flush(self) -> int:
        if self._w is None:
            return -1
        return 0 if self._lib.nbg_stream_flush(self._w) == 0 else -1

    def close(self) -> int:
        if self._w is None:
            return 0
        st = self._lib.nbg_stream_close(self._w)
        self._w = None
        return 0 if st == 0 else -1

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StreamReader:
    """Reads frames of a stream (nbody/nbody_data_stream_reader.cpp)."""

    def __init__(self):
        self.frames = []  # (step, time, part, offset)
        self.coord_size = 0
        self.body_count = 0
        self.box_size = 0
        self.base = ""
        self._cur = 0

    def load(self, base: str) -> int:
        self.frames = []
        try:
            with open(make_idx_name(base)) as fh:
                lines = fh.read().split("\n")
        except OSError:
            return -1
        for line in lines:
            if not line:
                continue
            if line.startswith("#"):
                key, _, val = line.partition(" ")
                if key == "#coord_size":
                    self.coord_size = int(val)
                elif key == "#body_count":
                    self.body_count = int(val)
                elif key == "#box_size":
                    self.box_size = int(val)
                continue
            parts = line.split(SEPARATOR)
            if len(parts) != 4:
                return -1
            self.frames.append((int(parts[0]), float(parts[1]), int(parts[2]), int(parts[3])))
        self.base = base
        self._cur = 0
        return 0

    def get_frame_count(self) -> int:
        return len(self.frames)

    def get_steps_count(self) -> int:
        return self.frames[-1][0] if self.frames else 0

    def get_max_time(self) -> float:
        return self.frames[-1][1] if self.frames else 0.0

    def get_body_count(self) -> int:
        return self.body_count

    def get_coord_size(self) -> int:
        return self.coord_size

    def get_last_file_n(self) -> int:
        return self.frames[-1][2] if self.frames else 0

    def seek(self, frame: int) -> int:
        if frame < 0 or frame >= len(self.frames):
            return -1
        self._cur = frame
        return 0

    def read(self, data) -> int:
        """The current frame into data (vertices, velocities, step, time); advances."""
        if self._cur >= len(self.frames):
            return -1
        step, time, part, off = self.frames[self._cur]
        n = self.body_count
        try:
            with open(make_dat_name(self.base, part), "rb") as fh:
                fh.seek(off)
                raw = np.frombuffer(fh.read(48 * n), dtype=np.float64)
        except OSError:
            return -1
        if raw.size != 6 * n:
            return -1
        data.vertices = raw[:3 * n].reshape(n, 3).copy()
        data.velocities = raw[3 * n:].reshape(n, 3).copy()
        data.set_step(step)
        data.set_time(time)
        self._cur += 1
        return 0
