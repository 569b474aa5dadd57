"""Oracle: the reference's 'simple' engine behind the nbody_engine interface.

TEST INFRASTRUCTURE ONLY: lets the restated solvers (nbody_gb300/solvers.py)
run on the CPU against the reference's golden vectors, so the solver
restatements are checked without a GPU; the GPU tests then run the same
solvers on the GB300 engine.  Forces are orc_fcompute_simple
(nbody/nbody_engine_simple.cpp:116-173) and the buffer algebra is the
oracle's restatement of nbody/nbody_engine_simple.cpp:245-419 (zero
coefficients skipped, Kahan-corrected fmaddn_corr).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .oracle import load_oracle


class Buf:
    __slots__ = ("a",)

    def __init__(self, n: int):
        self.a = np.zeros(n, dtype=np.float64)

    def size(self) -> int:
        return self.a.size * 8


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ptrs(bufs, count):
    arr = (C.POINTER(C.c_double) * max(count, 1))()
    for i in range(count):
        arr[i] = _ptr(bufs[i].a)
    return arr


class OracleEngine:
    def __init__(self):
        self.orc = load_oracle()
        lib = self.orc.lib
        dp = C.POINTER(C.c_double)
        lib.orc_fill.argtypes = [dp, C.c_double, C.c_size_t]
        lib.orc_fmadd_inplace.argtypes = [dp, dp, C.c_double, C.c_size_t]
        lib.orc_fmadd.argtypes = [dp, dp, dp, C.c_double, C.c_size_t]
        lib.orc_fmaddn_inplace.argtypes = [dp, C.POINTER(dp), dp, C.c_size_t, C.c_size_t]
        lib.orc_fmaddn.argtypes = [dp, dp, C.POINTER(dp), dp, C.c_size_t, C.c_size_t]
        lib.orc_fmaddn_corr.argtypes = [dp, dp, C.POINTER(dp), dp, C.c_size_t, C.c_size_t]
        self.lib = lib
        self.data = None
        self.y = None
        self.mass = None

    # -- nbody_engine ----------------------------------------------------------
    def init(self, data) -> bool:
        self.data = data
        n = data.get_count()
        self.y = Buf(6 * n)
        self.y.a[:] = data.to_state()
        self.mass = np.ascontiguousarray(data.mass, dtype=np.float64)
        return True

    def problem_size(self) -> int:
        return self.y.a.size

    def get_y(self):
        return self.y

    def get_time(self) -> float:
        return self.data.get_time()

    def set_time(self, t: float) -> None:
        self.data.set_time(t)

    def advise_time(self, dt: float) -> None:
        self.data.advise_time(dt)

    def get_data(self, data) -> None:
        data.from_state(self.y.a)

    def create_buffer(self, nbytes: int):
        return Buf(nbytes // 8)

    def create_buffers(self, nbytes: int, count: int):
        return [Buf(nbytes // 8) for _ in range(count)]

    def fcompute(self, t, y, f) -> None:
        f.a[:] = self.orc.fcompute_simple(y.a, self.mass)

    def copy_buffer(self, a, b) -> None:
        a.a[:] = b.a

    def fill_buffer(self, a, v: float) -> None:
        self.lib.orc_fill(_ptr(a.a), float(v), a.a.size)

    def fmadd_inplace(self, a, b, c: float) -> None:
        self.lib.orc_fmadd_inplace(_ptr(a.a), _ptr(b.a), float(c), a.a.size)

    def fmadd(self, a, b, c, d: float) -> None:
        self.lib.orc_fmadd(_ptr(a.a), _ptr(b.a), _ptr(c.a), float(d), a.a.size)

    def fmaddn_inplace(self, a, b, c, csize: int) -> None:
        cc = (C.c_double * max(csize, 1))(*c[:csize])
        self.lib.orc_fmaddn_inplace(_ptr(a.a), _ptrs(b, csize), cc, csize, a.a.size)

    def fmaddn(self, a, b, c, d, dsize: int) -> None:
        dd = (C.c_double * max(dsize, 1))(*d[:dsize])
        bp = _ptr(b.a) if b is not None else None
        self.lib.orc_fmaddn(_ptr(a.a), bp, _ptrs(c, dsize), dd, dsize, a.a.size)

    def fmaddn_corr(self, a, corr, b, c, csize: int) -> None:
        cc = (C.c_double * max(csize, 1))(*c[:csize])
        self.lib.orc_fmaddn_corr(_ptr(a.a), _ptr(corr.a), _ptrs(b, csize), cc, csize, a.a.size)

    def fmaxabs(self, a) -> float:
        return float(self.orc.fmaxabs(a.a))

    def clamp(self, y, b: float) -> None:
        self.orc.clamp(y.a, self.data.get_count(), b)
