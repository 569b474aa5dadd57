"""ctypes binding of oracle/_ref/libnbody_ref.so: the reference's own CPU code.

TEST INFRASTRUCTURE ONLY (see oracle/ref_build.py and oracle/ref_glue.cpp):
the reference's engines, kd heap, solvers, Butcher tables, galaxy generator,
stream writer and conservation sums, compiled from its sources where they
lie.  load_ref() returns None when the sources are absent (the GPU host), so
the tests that pin the oracle against the reference skip there.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from .ref_build import build_ref

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class RefLib:
    def __init__(self, path):
        lib = C.CDLL(str(path))
        sz, dbl, i32 = C.c_size_t, C.c_double, C.c_int
        lib.ref_make_universe.argtypes = [sz, dbl, dbl, dbl, sz, C.c_void_p, C.c_void_p,
                                          C.POINTER(sz)]
        lib.ref_fcompute.argtypes = [C.c_char_p, sz, _dp, _dp, sz, dbl, _dp]
        lib.ref_solver_run.argtypes = [C.c_char_p, C.c_char_p, sz, _dp, _dp, dbl, _dp,
                                       C.POINTER(dbl), C.POINTER(C.c_uint64)]
        lib.ref_butcher_table.argtypes = [C.c_char_p, sz, C.POINTER(sz), _dp, _dp, _dp, _dp,
                                          C.POINTER(i32)]
        lib.ref_heap_build.argtypes = [sz, _dp, _dp, dbl, _dp, _dp, _dp,
                                       np.ctypeslib.ndpointer(dtype=np.int64,
                                                              flags="C_CONTIGUOUS")]
        lib.ref_stream_write.argtypes = [C.c_char_p, C.c_longlong, sz, sz, _dp, _dp,
                                         np.ctypeslib.ndpointer(dtype=np.uint64,
                                                                flags="C_CONTIGUOUS"), _dp]
        lib.ref_statistics.argtypes = [sz, _dp, _dp, _dp]
        for fn in (lib.ref_make_universe, lib.ref_fcompute, lib.ref_solver_run,
                   lib.ref_butcher_table, lib.ref_heap_build, lib.ref_stream_write,
                   lib.ref_statistics):
            fn.restype = i32
        self.lib = lib

    @staticmethod
    def _kv(params: dict) -> bytes:
        return ";".join(f"{k}={v}" for k, v in params.items()).encode()

    def make_universe(self, star_count: int, sx=100.0, sy=100.0, sz=100.0):
        """(y [6n], mass [n]) of nbody_data::make_universe."""
        n = C.c_size_t(0)
        self.lib.ref_make_universe(star_count, sx, sy, sz, 0, None, None, C.byref(n))
        y = np.zeros(6 * n.value)
        m = np.zeros(n.value)
        self.lib.ref_make_universe(star_count, sx, sy, sz, n.value, y.ctypes.data, m.ctypes.data,
                                   C.byref(n))
        return y, m

    def fcompute(self, engine: dict, y, mass, steps=1, mutate=0.0):
        """[steps][6n] f of the engine nbody_create_engine makes from `engine`."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        n = mass.size
        out = np.zeros(steps * 6 * n)
        rc = self.lib.ref_fcompute(self._kv(engine), n, y, mass, steps, mutate, out)
        if rc != 0:
            raise ValueError(f"ref_fcompute({engine}) = {rc}")
        return out.reshape(steps, 6 * n)

    def solver_run(self, solver: dict, engine: dict, y, mass, max_time):
        """(y, t, step) after nbody_solver::run to max_time."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        out = np.zeros_like(y)
        t = C.c_double(0.0)
        st = C.c_uint64(0)
        rc = self.lib.ref_solver_run(self._kv(solver), self._kv(engine), mass.size, y, mass,
                                     max_time, out, C.byref(t), C.byref(st))
        if rc != 0:
            raise ValueError(f"ref_solver_run({solver}, {engine}) = {rc}")
        return out, t.value, st.value

    def butcher_table(self, solver: dict):
        """(a [s][s], b1, b2, c, implicit, embedded) of a Butcher solver."""
        k = C.c_size_t(0)
        fl = C.c_int(0)
        z = np.zeros(1)
        rc = self.lib.ref_butcher_table(self._kv(solver), 0, C.byref(k), z, z, z, z, C.byref(fl))
        if rc != 0:
            raise ValueError(f"not a Butcher solver: {solver}")
        s = k.value
        a, b1, b2, c = np.zeros(s * s), np.zeros(s), np.zeros(s), np.zeros(s)
        self.lib.ref_butcher_table(self._kv(solver), s, C.byref(k), a, b1, b2, c, C.byref(fl))
        return a.reshape(s, s), b1, b2, c, bool(fl.value & 1), bool(fl.value & 2)

    def heap_build(self, y, mass, lam):
        """nbody_space_heap::build node arrays: (com [3][2n], mass, crit r^2, body)."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        n = mass.size
        com, m, r2 = np.zeros(3 * 2 * n), np.zeros(2 * n), np.zeros(2 * n)
        body = np.zeros(2 * n, dtype=np.int64)
        if self.lib.ref_heap_build(n, y, mass, lam, com, m, r2, body) != 0:
            raise ValueError("heap build failed")
        return com.reshape(3, 2 * n), m, r2, body

    def stream_write(self, base: str, max_part_size: int, frames, mass, steps, times):
        frames = np.ascontiguousarray(frames, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        steps = np.ascontiguousarray(steps, dtype=np.uint64)
        times = np.ascontiguousarray(times, dtype=np.float64)
        rc = self.lib.ref_stream_write(base.encode(), max_part_size, mass.size, len(steps),
                                       frames.reshape(-1), mass, steps, times)
        if rc != 0:
            raise ValueError(f"ref_stream_write = {rc}")

    def statistics(self, y, mass):
        """P[3], L[3], mass centre[3], total energy of print_statistics."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        out = np.zeros(10)
        if self.lib.ref_statistics(mass.size, y, mass, out) != 0:
            raise ValueError("ref_statistics failed")
        return out


_REF = None


def load_ref() -> Optional[RefLib]:
    """The reference build, or None when the reference's sources are absent."""
    global _REF
    if _REF is None:
        path = build_ref()
        if path is None:
            return None
        _REF = RefLib(path)
    return _REF
