"""ctypes binding and build recipe for the CPU oracle (nbody_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, where it is the checker.  The GB300 engine never imports
this module.

    from oracle.oracle import load_oracle
    orc = load_oracle()          # builds oracle/_build/libnbody_oracle.so if needed
    f = orc.fcompute_simple(y, mass)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "libnbody_oracle.so"
SRC = HERE / "nbody_oracle.c"

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build_oracle(force: bool = False) -> Path:
    """Compile nbody_oracle.c with gcc -fopenmp -ffp-contract=off."""
    BUILD_DIR.mkdir(exist_ok=True)
    if (not force and LIB.exists()
            and LIB.stat().st_mtime >= SRC.stat().st_mtime
            and LIB.stat().st_mtime >= (HERE / "nbody_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=c11", "-Wall", "-o", str(tmp), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class _Heap(C.Structure):
    """struct orc_heap (nbody_oracle.h)."""
    _fields_ = [("count", C.c_size_t), ("size", C.c_size_t),
                ("com", C.POINTER(C.c_double)), ("mass", C.POINTER(C.c_double)),
                ("r2", C.POINTER(C.c_double)), ("bmin", C.POINTER(C.c_double)),
                ("bmax", C.POINTER(C.c_double)), ("body_n", C.POINTER(C.c_int64)),
                ("lambda2", C.c_double)]


class Oracle:
    """Thin numpy-facing wrapper over the oracle C functions."""

    def __init__(self, path: Path):
        lib = C.CDLL(str(path))
        self.lib = lib
        u64 = C.c_uint64
        for name in ("orc_left_idx", "orc_rght_idx", "orc_parent_idx",
                     "orc_next_down", "orc_skip_idx"):
            fn = getattr(lib, name)
            fn.argtypes = [u64]
            fn.restype = u64
        lib.orc_next_up.argtypes = [u64, u64]
        lib.orc_next_up.restype = u64
        lib.orc_fcompute_simple.argtypes = [C.c_size_t, _dp, _dp, _dp, C.c_int]
        lib.orc_fcompute_block.argtypes = [C.c_size_t, _dp, _dp, _dp, C.c_int]
        lib.orc_fcompute_block_range.argtypes = [C.c_size_t, _dp, _dp, _dp, C.c_size_t,
                                                 C.c_size_t, C.c_int]
        lib.orc_accel_rows.argtypes = [C.c_size_t, _dp, _dp, C.c_double,
                                       C.c_void_p, C.c_size_t, _dp, C.c_int]
        lib.orc_fmaxabs.argtypes = [_dp, C.c_size_t]
        lib.orc_fmaxabs.restype = C.c_double
        lib.orc_statistics.argtypes = [C.c_size_t, _dp, _dp, _dp, C.c_int]
        lib.orc_solver_run.argtypes = [C.c_char_p, C.c_size_t, _dp, _dp,
                                       C.POINTER(C.c_double), C.c_double,
                                       C.c_double, C.c_double, C.c_size_t,
                                       C.c_size_t, C.c_double, C.c_int,
                                       C.POINTER(C.c_uint64)]
        lib.orc_solver_run.restype = C.c_int
        lib.orc_fcompute_bh.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_size_t,
                                        C.c_size_t, C.c_double, C.c_size_t,
                                        _dp, _dp, _dp, C.c_int]
        lib.orc_fcompute_bh.restype = C.c_int
        lib.orc_heap_free.argtypes = [C.c_void_p]
        lib.orc_heap_build.argtypes = [C.c_void_p, C.c_size_t, _dp, _dp, _dp, _dp,
                                       C.c_double]
        lib.orc_heap_build.restype = C.c_int
        lib.orc_heap_visits.argtypes = [C.c_void_p, _dp]
        lib.orc_heap_visits.restype = u64
        lib.orc_clamp.argtypes = [_dp, C.c_size_t, C.c_double]

    # -- heap index algebra ------------------------------------------------
    def next_down(self, i): return int(self.lib.orc_next_down(i))
    def skip_idx(self, i): return int(self.lib.orc_skip_idx(i))
    def next_up(self, i, n): return int(self.lib.orc_next_up(i, n))
    def parent_idx(self, i): return int(self.lib.orc_parent_idx(i))
    def left_idx(self, i): return int(self.lib.orc_left_idx(i))
    def rght_idx(self, i): return int(self.lib.orc_rght_idx(i))

    # -- engines -----------------------------------------------------------
    def fcompute_simple(self, y, mass, nthreads=1):
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        f = np.empty_like(y)
        self.lib.orc_fcompute_simple(mass.size, y, mass, f, nthreads)
        return f

    def fcompute_block(self, y, mass, nthreads=1):
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        f = np.empty_like(y)
        self.lib.orc_fcompute_block(mass.size, y, mass, f, nthreads)
        return f

    def fcompute_block_range(self, y, mass, f, row0, row1, nthreads=1):
        """Block engine over rows [row0, row1) only (writes those rows of f)."""
        self.lib.orc_fcompute_block_range(mass.size, y, mass, f, row0, row1, nthreads)

    def accel_rows(self, y, mass, eps, rows=None, nthreads=0):
        """FP64 softened direct-sum accelerations [len(rows), 3]."""
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        n = mass.size
        if nthreads <= 0:
            nthreads = os.cpu_count() or 1
        if rows is None:
            acc = np.empty((n, 3))
            self.lib.orc_accel_rows(n, y, mass, eps, None, n, acc, nthreads)
        else:
            rows = np.ascontiguousarray(rows, dtype=np.int64)
            acc = np.empty((rows.size, 3))
            self.lib.orc_accel_rows(n, y, mass, eps, rows.ctypes.data_as(C.c_void_p),
                                    rows.size, acc, nthreads)
        return acc

    def fcompute_bh(self, y, mass, lam, layout=2, traverse=1, steps=1,
                    build_rate=0, nthreads=1, mutate=None):
        """simple_bh over `steps` calls; returns the list of f per step.
        mutate(y) -> y is applied between steps (test_fcompute's y *= 1.99)."""
        heap = (C.c_byte * 128)()  # orc_heap storage (zeroed = empty tree)
        y = np.ascontiguousarray(y, dtype=np.float64).copy()
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        out = []
        try:
            for step in range(steps):
                f = np.empty_like(y)
                rc = self.lib.orc_fcompute_bh(C.addressof(heap), layout, traverse,
                                              step, build_rate, lam, mass.size,
                                              y, mass, f, nthreads)
                if rc != 0:
                    raise ValueError(f"orc_fcompute_bh failed: {rc}")
                out.append(f)
                if mutate is not None:
                    y = np.ascontiguousarray(mutate(y))
        finally:
            self.lib.orc_heap_free(C.addressof(heap))
        return out

    def heap_nodes(self, y, mass, lam):
        """The kd heap's node arrays after orc_heap_build: (com [3][2n],
        mass [2n], crit r^2 [2n], body [2n], bmin [3][2n], bmax [3][2n])."""
        heap = _Heap()
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        n = mass.size
        try:
            rc = self.lib.orc_heap_build(C.addressof(heap), n, y[:n].copy(), y[n:2 * n].copy(),
                                         y[2 * n:3 * n].copy(), mass, lam)
            if rc != 0:
                raise ValueError("heap build failed")
            sz = heap.size

            def arr(p, k):
                return np.ctypeslib.as_array(p, shape=(k,)).copy()
            com = arr(heap.com, 3 * sz).reshape(sz, 3).T.copy()
            out = (com, arr(heap.mass, sz), arr(heap.r2, sz), arr(heap.body_n, sz),
                   arr(heap.bmin, 3 * sz).reshape(sz, 3).T.copy(),
                   arr(heap.bmax, 3 * sz).reshape(sz, 3).T.copy())
        finally:
            self.lib.orc_heap_free(C.addressof(heap))
        return out

    def bh_visits(self, y, mass, lam, rows):
        """Stackless node visits for each row (kd heap at ratio lam)."""
        heap = (C.c_byte * 128)()
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        n = mass.size
        try:
            rc = self.lib.orc_heap_build(C.addressof(heap), n, y[:n].copy(),
                                         y[n:2 * n].copy(), y[2 * n:3 * n].copy(),
                                         mass, lam)
            if rc != 0:
                raise ValueError("heap build failed")
            res = []
            for r in rows:
                v = np.array([y[r], y[n + r], y[2 * n + r]])
                res.append(int(self.lib.orc_heap_visits(C.addressof(heap), v)))
        finally:
            self.lib.orc_heap_free(C.addressof(heap))
        return np.array(res)

    # -- buffer algebra ----------------------------------------------------
    def fmaxabs(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        return float(self.lib.orc_fmaxabs(a, a.size))

    def clamp(self, y, count, b):
        y = np.ascontiguousarray(y, dtype=np.float64).copy()
        self.lib.orc_clamp(y, count, b)
        return y

    def statistics(self, y, mass):
        y = np.ascontiguousarray(y, dtype=np.float64)
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        out = np.zeros(12)
        self.lib.orc_statistics(mass.size, y, mass, out, 1)
        return out

    # -- solvers -----------------------------------------------------------
    def solver_run(self, name, y, mass, max_time, min_step, max_step,
                   max_recursion=8, substep_subdivisions=8,
                   error_threshold=1e-4, correction=False, t0=0.0):
        y = np.ascontiguousarray(y, dtype=np.float64).copy()
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        t = C.c_double(t0)
        cnt = C.c_uint64(0)
        rc = self.lib.orc_solver_run(name.encode(), mass.size, y, mass, C.byref(t),
                                     max_time, min_step, max_step, max_recursion,
                                     substep_subdivisions, error_threshold,
                                     int(bool(correction)), C.byref(cnt))
        if rc != 0:
            raise ValueError(f"unknown solver {name}")
        return y, t.value, cnt.value


_ORACLE = None


def load_oracle() -> Oracle:
    global _ORACLE
    if _ORACLE is None:
        _ORACLE = Oracle(build_oracle())
    return _ORACLE
