"""Integrators that drive an engine only through the nbody_engine interface.

These restate the reference's solvers -- the unchanged callers of the hot
path -- so that the GB300 engine can be driven exactly as the reference's own
solver classes drive any engine:

  * euler          nbody/nbody_solver_euler.cpp:19-31
  * rk4            nbody/nbody_solver_rk4.cpp:19-48
  * rk_butcher     nbody/nbody_solver_rk_butcher.cpp:60-248 (explicit, embedded
                   error = fmaxabs(fmaddn(NULL, k, b2 - b1)), recursive
                   subdivision, optional Kahan correction)
  * tables         rkdp (nbody/nbody_solver_rkdp.cpp:30-62),
                   rkck (nbody/nbody_solver_rkck.cpp:30-62),
                   rkf  (nbody/nbody_solver_rkf.cpp:30-71)
  * run loop       nbody/nbody_solver.cpp:55-105 (dt = max_step every advise)

The Butcher coefficients are the published Dormand-Prince, Cash-Karp and
Fehlberg tables, written out in the same row layout the reference uses.
"""
from __future__ import annotations

from fractions import Fraction as Fr
from typing import List, Optional

F8 = 8  # sizeof(nbcoord_t)


class ButcherTable:
    def __init__(self, a, b1, b2, c, embedded=True):
        self.steps = len(c)
        self.a = [[float(x) for x in row] for row in a]
        self.b1 = [float(x) for x in b1]
        self.b2 = [float(x) for x in b2]
        self.c = [float(x) for x in c]
        self.embedded = embedded


def _t(*rows):
    return [list(r) for r in rows]


RKDP = ButcherTable(
    _t([0], [Fr(1, 5)], [Fr(3, 40), Fr(9, 40)], [Fr(44, 45), Fr(-56, 15), Fr(32, 9)],
       [Fr(19372, 6561), Fr(-25360, 2187), Fr(64448, 6561), Fr(-212, 729)],
       [Fr(9017, 3168), Fr(-355, 33), Fr(46732, 5247), Fr(49, 176), Fr(-5103, 18656)],
       [Fr(35, 384), 0, Fr(500, 1113), Fr(125, 192), Fr(-2187, 6784), Fr(11, 84), 0]),
    [Fr(35, 384), 0, Fr(500, 1113), Fr(125, 192), Fr(-2187, 6784), Fr(11, 84), 0],
    [Fr(5179, 57600), 0, Fr(7571, 16695), Fr(393, 640), Fr(-92097, 339200), Fr(187, 2100),
     Fr(1, 40)],
    [0, Fr(1, 5), Fr(3, 10), Fr(4, 5), Fr(8, 9), 1, 1])

RKCK = ButcherTable(
    _t([0], [Fr(1, 5)], [Fr(3, 40), Fr(9, 40)], [Fr(3, 10), Fr(-9, 10), Fr(6, 5)],
       [Fr(-11, 54), Fr(5, 2), Fr(-70, 27), Fr(35, 27)],
       [Fr(1631, 55296), Fr(175, 512), Fr(575, 13824), Fr(44275, 110592), Fr(253, 4096)]),
    [Fr(37, 378), 0, Fr(250, 621), Fr(125, 594), 0, Fr(512, 1771)],
    [Fr(2825, 27648), 0, Fr(18575, 48384), Fr(13525, 55296), Fr(277, 14336), Fr(1, 4)],
    [0, Fr(1, 5), Fr(3, 10), Fr(3, 5), 1, Fr(7, 8)])

RKF = ButcherTable(
    _t([0], [Fr(2, 27)], [Fr(1, 36), Fr(1, 12)], [Fr(1, 24), 0, Fr(1, 8)],
       [Fr(5, 12), 0, Fr(-25, 16), Fr(25, 16)], [Fr(1, 20), 0, 0, Fr(1, 4), Fr(1, 5)],
       [Fr(-25, 108), 0, 0, Fr(125, 108), Fr(-65, 27), Fr(125, 54)],
       [Fr(31, 300), 0, 0, 0, Fr(61, 225), Fr(-2, 9), Fr(13, 900)],
       [2, 0, 0, Fr(-53, 6), Fr(704, 45), Fr(-107, 9), Fr(67, 90), 3],
       [Fr(-91, 108), 0, 0, Fr(23, 108), Fr(-976, 135), Fr(311, 54), Fr(-19, 60), Fr(17, 6),
        Fr(-1, 12)],
       [Fr(2383, 4100), 0, 0, Fr(-341, 164), Fr(4496, 1025), Fr(-301, 82), Fr(2133, 4100),
        Fr(45, 82), Fr(45, 164), Fr(18, 41)],
       [Fr(3, 205), 0, 0, 0, 0, Fr(-6, 41), Fr(-3, 205), Fr(-3, 41), Fr(3, 41), Fr(6, 41), 0],
       [Fr(-1777, 4100), 0, 0, Fr(-341, 164), Fr(4496, 1025), Fr(-289, 82), Fr(2193, 4100),
        Fr(51, 82), Fr(33, 164), Fr(12, 41), 0, 1]),
    [Fr(41, 840), 0, 0, 0, 0, Fr(34, 105), Fr(9, 35), Fr(9, 35), Fr(9, 280), Fr(9, 280),
     Fr(41, 840), 0, 0],
    [0, 0, 0, 0, 0, Fr(34, 105), Fr(9, 35), Fr(9, 35), Fr(9, 280), Fr(9, 280), 0,
     Fr(41, 840), Fr(41, 840)],
    [0, Fr(2, 27), Fr(1, 9), Fr(1, 6), Fr(5, 12), Fr(1, 2), Fr(5, 6), Fr(1, 6), Fr(2, 3),
     Fr(1, 3), 1, 0, 1])

TABLES = {"rkdp": RKDP, "rkck": RKCK, "rkf": RKF}


class Solver:
    """nbody_solver (nbody/nbody_solver.h)."""

    def __init__(self):
        self._engine = None
        self.min_step = 0.0
        self.max_step = 0.0
        self.clamp_to_box = False

    def set_engine(self, e) -> None:
        self._engine = e

    def engine(self):
        return self._engine

    def set_time_step(self, min_step: float, max_step: float) -> None:
        self.min_step = float(min_step)
        self.max_step = float(max_step)

    def run(self, data, max_time: float, check=None, stream=None, dump_dt: float = 0.0,
            check_dt: float = 0.0) -> int:
        """nbody/nbody_solver.cpp:55-105.  Frames go to `stream` (a
        nbody_gb300.stream.DataStream) every dump_dt, the first at t = 0; a
        stream opened on the engine takes them from device memory.  `check`
        is called every check_dt (every step when check_dt is 0)."""
        dt = self.max_step
        last_check = data.get_time()
        last_dump = last_check

        def dump() -> int:
            if getattr(stream, "_engine", None) is self._engine:
                return stream.write_engine(self._engine, data)
            self._engine.get_data(data)
            return stream.write(data)

        if stream is not None and dump_dt > 0 and last_dump <= 0:
            if dump() != 0:
                return -1
            last_dump = data.get_time()
        while data.get_time() < max_time:
            if self.clamp_to_box:
                self._engine.clamp(self._engine.get_y(), data.box_size)
            self.advise(dt)
            t = data.get_time()
            if check is not None and (check_dt <= 0 or t >= last_check + check_dt - dt * 0.1):
                check(data)
                last_check = t
            if stream is not None and dump_dt > 0 and t >= last_dump + dump_dt - dt * 0.1:
                if dump() != 0:
                    return -1
                last_dump = t
        return 0

    def advise(self, dt: float) -> None:
        raise NotImplementedError


class SolverEuler(Solver):
    def __init__(self):
        super().__init__()
        self._dy = None

    def advise(self, dt: float) -> None:
        e = self._engine
        y = e.get_y()
        if self._dy is None:
            self._dy = e.create_buffer(F8 * e.problem_size())
        e.fcompute(e.get_time(), y, self._dy)
        e.fmadd_inplace(y, self._dy, dt)
        e.advise_time(dt)


class SolverRK4(Solver):
    def __init__(self):
        super().__init__()
        self._k: List = []
        self._tmp = None

    def advise(self, dt: float) -> None:
        e = self._engine
        y = e.get_y()
        t = e.get_time()
        if not self._k:
            ps = e.problem_size()
            self._k = e.create_buffers(F8 * ps, 4)
            self._tmp = e.create_buffer(F8 * ps)
        k, tmp = self._k, self._tmp
        e.fcompute(t, y, k[0])
        e.fmadd(tmp, y, k[0], dt / 2.0)
        e.fcompute(t + dt / 2.0, tmp, k[1])
        e.fmadd(tmp, y, k[1], dt / 2.0)
        e.fcompute(t + dt / 2.0, tmp, k[2])
        e.fmadd(tmp, y, k[2], dt)
        e.fcompute(t + dt, tmp, k[3])
        coeff = [dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0]
        e.fmaddn_inplace(y, k, coeff, 4)
        e.advise_time(dt)


class SolverRKButcher(Solver):
    """Explicit embedded Runge-Kutta with recursive step subdivision."""

    def __init__(self, table: ButcherTable, error_threshold=1e-4, max_recursion=8,
                 substep_subdivisions=8, correction=False):
        super().__init__()
        self.bt = table
        self.error_threshold = float(error_threshold)
        self.max_recursion = int(max_recursion)
        self.substep_subdivisions = int(substep_subdivisions)
        self.correction = bool(correction)
        self._k: List = []
        self._t = None
        self._ystack: List = []
        self._ycorr = None
        self._tcorr = None
        self.last_error = 0.0

    def advise(self, dt: float) -> None:
        e = self._engine
        self._sub_step(1, e.get_time(), dt, e.get_y(), 0)
        e.advise_time(dt)

    def _alloc(self):
        e = self._engine
        ps = e.problem_size()
        self._k = e.create_buffers(F8 * ps, self.bt.steps)
        self._t = e.create_buffer(F8 * ps)
        self._ystack = e.create_buffers(F8 * ps, self.max_recursion)
        if self.correction:
            self._ycorr = e.create_buffer(F8 * ps)
            self._tcorr = e.create_buffer(F8 * ps)
            e.fill_buffer(self._ycorr, 0.0)
            e.fill_buffer(self._tcorr, 0.0)

    def _stages(self, y, t, dt):
        """nbody/nbody_solver_rk_butcher.cpp:130-162."""
        e, bt = self._engine, self.bt
        for i in range(bt.steps):
            if i == 0:
                e.fcompute(t + bt.c[i] * dt, y, self._k[i])
                continue
            coeff = [dt * bt.a[i][n] for n in range(i)]
            if self.correction:
                e.copy_buffer(self._tcorr, self._ycorr)
                e.copy_buffer(self._t, y)
                e.fmaddn_corr(self._t, self._tcorr, self._k, coeff, i)
            else:
                e.fmaddn(self._t, y, self._k, coeff, i)
            e.fcompute(t + bt.c[i] * dt, self._t, self._k[i])

    def _sub_step(self, substeps, t, dt, y, level):
        """nbody/nbody_solver_rk_butcher.cpp:164-248."""
        e, bt = self._engine, self.bt
        if not self._k:
            self._alloc()
        for _ in range(substeps):
            self._stages(y, t, dt)
            max_error = 0.0
            if bt.embedded:
                coeff = [bt.b2[n] - bt.b1[n] for n in range(bt.steps)]
                e.fmaddn(self._t, None, self._k, coeff, bt.steps)
                max_error = e.fmaxabs(self._t)
            self.last_error = max_error
            can = bt.embedded and level < self.max_recursion and dt > self.min_step
            if can and max_error > self.error_threshold:
                new_dt = dt / float(self.substep_subdivisions)
                cy = self._ystack[level]
                e.copy_buffer(cy, y)
                self._sub_step(self.substep_subdivisions, t, new_dt, cy, level + 1)
                e.copy_buffer(y, cy)
            else:
                coeff = [bt.b2[n] * dt for n in range(bt.steps)]
                if self.correction:
                    e.fmaddn_corr(y, self._ycorr, self._k, coeff, len(self._k))
                else:
                    e.fmaddn_inplace(y, self._k, coeff, len(self._k))
            t += dt


def create_solver(param: dict) -> Optional[Solver]:
    """nbody_create_solver (nbody/nbody_solvers.cpp:17-110) for the solvers
    restated here; None for an unknown type."""
    kind = str(param.get("solver", ""))
    if kind == "euler":
        s: Solver = SolverEuler()
    elif kind == "rk4":
        s = SolverRK4()
    elif kind in TABLES:
        s = SolverRKButcher(TABLES[kind],
                            error_threshold=float(param.get("error_threshold", 1e-4)),
                            max_recursion=int(param.get("max_recursion", 8)),
                            substep_subdivisions=int(param.get("substep_subdivisions", 8)),
                            correction=bool(param.get("correction", False)))
    else:
        return None
    s.set_time_step(float(param.get("min_step", 1e-9)), float(param.get("max_step", 1e-2)))
    s.clamp_to_box = bool(param.get("clamp", False))
    return s
