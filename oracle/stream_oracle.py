"""Oracle: the reference's frame stream writer restated in Python.

TEST INFRASTRUCTURE ONLY: the checker for the stream files the GB300 library
writes (nbody_gb300/csrc/nbg_stream.cu).  It follows
nbody/nbody_data_stream.cpp:
  * open (:168-196): part 0 and the index are opened (truncated, or appended
    to when continuing a stream whose last part number is given);
  * write (:107-160): the header is written with the first frame
    (write_header, :62-98: "#coord_size", "#body_count", "#box_size" lines,
    the .col and .mass files); a new part is opened when the current one's
    position has reached max_part_size; the frame is N vertices then N
    velocities (3 doubles per body); the index line is
    step TAB time TAB part TAB offset, the time printed as QTextStream
    prints a double by default (6 significant digits, shortest notation);
  * names (:206-229): <base>.idx, <base><part>.dat, <base>.col, <base>.mass.
"""
from __future__ import annotations

import os

import numpy as np


class OracleStream:
    def __init__(self, base: str, max_part_size: int, append_part: int | None = None):
        self.base = base
        self.max_part = int(max_part_size)
        os.makedirs(os.path.dirname(base) or ".", exist_ok=True)
        self.part = 0 if append_part is None else int(append_part)
        self.header_written = append_part is not None
        mode = "ab" if append_part is not None else "wb"
        self.dat = open(f"{base}{self.part}.dat", mode)
        self.idx = open(base + ".idx", "a" if append_part is not None else "w")

    def write(self, step: int, time: float, vertices, velocities, box_size: int, color, mass):
        n = len(mass)
        if not self.header_written:
            self.idx.write(f"#coord_size 8\n#body_count {n}\n#box_size {int(box_size)}\n")
            with open(self.base + ".col", "wb") as fh:
                fh.write(np.ascontiguousarray(color, dtype=np.float32).tobytes())
            with open(self.base + ".mass", "wb") as fh:
                fh.write(np.ascontiguousarray(mass, dtype=np.float64).tobytes())
            self.header_written = True
        if self.max_part > 0 and self.dat.tell() >= self.max_part:
            self.dat.close()
            self.part += 1
            self.dat = open(f"{self.base}{self.part}.dat", "wb")
        pos = self.dat.tell()
        self.dat.write(np.ascontiguousarray(vertices, dtype=np.float64).tobytes())
        self.dat.write(np.ascontiguousarray(velocities, dtype=np.float64).tobytes())
        self.dat.flush()
        self.idx.write(f"{int(step)}\t{float(time):g}\t{self.part}\t{pos}\n")
        self.idx.flush()

    def close(self):
        self.dat.close()
        self.idx.close()
