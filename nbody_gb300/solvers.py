"""Integrators that drive an engine only through the nbody_engine interface.

These restate the reference's solvers -- the unchanged callers of the hot
path -- so that the GB300 engine can be driven exactly as the reference's own
solver classes drive any engine:

  * euler          nbody/nbody_solver_euler.cpp:19-31
  * rk4            nbody/nbody_solver_rk4.cpp:19-48
  * rk_butcher     nbody/nbody_solver_rk_butcher.cpp:60-248 (explicit, embedded
                   error = fmaxabs(fmaddn(NULL, k, b2 - b1)), recursive
                   subdivision, optional Kahan correction)
                   and its implicit branch (:107-130, fixed-point refinement of
                   the stage derivatives)
  * tables         rkdp (nbody/nbody_solver_rkdp.cpp:30-62),
                   rkck (nbody/nbody_solver_rkck.cpp:30-62),
                   rkf  (nbody/nbody_solver_rkf.cpp:30-71),
                   rkdverk (nbody/nbody_solver_rkdverk.cpp:29-70),
                   rkgl (nbody/nbody_solver_rkgl.cpp:29-60, implicit),
                   rklc (nbody/nbody_solver_rklc.cpp:29-60, implicit),
                   rkfeagin10/12/14 (nbody/nbody_solver_rkfeagin{10,12,14}.cpp,
                   loaded from feagin_tables.json)
  * midpoint       nbody/nbody_solver_midpoint.cpp:23-40
  * midpoint-st    nbody/nbody_solver_midpoint_stetter.cpp:23-76
  * trapeze        nbody/nbody_solver_trapeze.cpp:30-56
  * adams          nbody/nbody_solver_adams.cpp:30-100 (Adams-Bashforth,
                   rank 1..5, started by another solver)
  * bs             nbody/nbody_solver_bulirsch_stoer.cpp:7-120 with the Neville
                   extrapolator (nbody/nbody_extrapolator.cpp:103-181)
  * run loop       nbody/nbody_solver.cpp:55-105 (dt = max_step every advise)

The Butcher coefficients are the published Dormand-Prince, Cash-Karp,
Fehlberg, Verner (DVERK 6(5)), Gauss-Legendre and Lobatto IIIC tables,
written out in the same row layout the reference uses (the Gauss-Legendre
entries with the same double expressions in sqrt(15)).  The Feagin 10/12/14
tables (hundreds of 60-digit published coefficients) are data: the doubles
the reference's solvers hold, in feagin_tables.json.
"""
from __future__ import annotations

import math
from fractions import Fraction as Fr
from typing import List, Optional

F8 = 8  # sizeof(nbcoord_t)


class ButcherTable:
    def __init__(self, a, b1, b2, c, embedded=True, implicit=False):
        self.steps = len(c)
        self.a = [[float(x) for x in row] for row in a]
        self.b1 = [float(x) for x in b1]
        self.b2 = [float(x) for x in b2]
        self.c = [float(x) for x in c]
        self.embedded = embedded
        self.implicit = implicit


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

RKDVERK = ButcherTable(
    _t([0], [Fr(1, 6)], [Fr(4, 75), Fr(16, 75)], [Fr(5, 6), Fr(-8, 3), Fr(5, 2)],
       [Fr(-165, 64), Fr(55, 6), Fr(-425, 64), Fr(85, 96)],
       [Fr(12, 5), -8, Fr(4015, 612), Fr(-11, 36), Fr(88, 255)],
       [Fr(-8263, 15000), Fr(124, 75), Fr(-643, 680), Fr(-81, 250), Fr(2484, 10625), 0],
       [Fr(3501, 1720), Fr(-300, 43), Fr(297275, 52632), Fr(-319, 2322), Fr(24068, 84065), 0,
        Fr(3850, 26703)]),
    [Fr(3, 40), 0, Fr(875, 2244), Fr(23, 72), Fr(264, 1955), 0, Fr(125, 11592), Fr(43, 616)],
    [Fr(13, 160), 0, Fr(2375, 5984), Fr(5, 16), Fr(12, 85), Fr(3, 44), 0, 0],
    [0, Fr(1, 6), Fr(4, 15), Fr(2, 3), Fr(5, 6), 1, Fr(1, 15), 1])


def _gauss_legendre3() -> ButcherTable:
    """3-stage Gauss-Legendre; entries evaluated in double with sqrt(15) as
    written in the reference table."""
    r = math.sqrt(15.0)
    a = [[5.0 / 36.0, 2.0 / 9.0 - r / 15.0, 5.0 / 36.0 - r / 30.0],
         [5.0 / 36.0 + r / 24.0, 2.0 / 9.0, 5.0 / 36.0 - r / 24.0],
         [5.0 / 36.0 + r / 30.0, 2.0 / 9.0 + r / 15.0, 5.0 / 36.0]]
    return ButcherTable(a, [5.0 / 18.0, 4.0 / 9.0, 5.0 / 18.0], [-5.0 / 6.0, 8.0 / 3.0, -5.0 / 6.0],
                        [0.5 - r / 10.0, 0.5, 0.5 + r / 10.0], embedded=False, implicit=True)


RKGL = _gauss_legendre3()

RKLC = ButcherTable(
    [[Fr(1, 6), Fr(-1, 3), Fr(1, 6)], [Fr(1, 6), Fr(5, 12), Fr(-1, 12)],
     [Fr(1, 6), Fr(2, 3), Fr(1, 6)]],
    [Fr(1, 6), Fr(2, 3), Fr(1, 6)], [Fr(-1, 2), 2, Fr(-1, 2)], [0, Fr(1, 2), 1],
    embedded=True, implicit=True)

def _feagin_tables() -> dict:
    """The Feagin 10(8), 12(10) and 14(12) tables (nbody/nbody_solver_rkfeagin
    {10,12,14}.cpp: 17, 25 and 35 stages of T. Feagin's published 60-digit
    coefficients, as doubles), from feagin_tables.json beside this module
    (each double stored exactly, as float.hex)."""
    import json
    from pathlib import Path
    data = json.loads((Path(__file__).resolve().parent / "feagin_tables.json").read_text())
    out = {}
    for name, t in data["tables"].items():
        h = float.fromhex
        out[name] = ButcherTable([[h(x) for x in row] for row in t["a"]],
                                 [h(x) for x in t["b1"]], [h(x) for x in t["b2"]],
                                 [h(x) for x in t["c"]], embedded=t["embedded"],
                                 implicit=t["implicit"])
    return out


TABLES = {"rkdp": RKDP, "rkck": RKCK, "rkf": RKF, "rkdverk": RKDVERK, "rkgl": RKGL,
          "rklc": RKLC, **_feagin_tables()}


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
                 substep_subdivisions=8, correction=False, refine_steps_count=1):
        super().__init__()
        self.bt = table
        self.error_threshold = float(error_threshold)
        self.max_recursion = int(max_recursion)
        self.substep_subdivisions = int(substep_subdivisions)
        self.correction = bool(correction)
        self.refine_steps_count = int(refine_steps_count)
        self._k: List = []
        self._t = None
        self._tmpk = None
        self._ystack: List = []
        self._ycorr = None
        self._tcorr = None
        self.last_error = 0.0
        # instrumentation (no effect on the integration): accepted substeps,
        # those accepted above the threshold (at the recursion cap or the
        # minimum step), and the largest error of an accepted substep
        self.accepted_steps = 0
        self.capped_steps = 0
        self.max_accepted_error = 0.0

    def advise(self, dt: float) -> None:
        e = self._engine
        self._sub_step(1, e.get_time(), dt, e.get_y(), 0)
        e.advise_time(dt)

    def _alloc(self):
        e = self._engine
        ps = e.problem_size()
        self._k = e.create_buffers(F8 * ps, self.bt.steps)
        self._t = e.create_buffer(F8 * ps)
        self._tmpk = e.create_buffer(F8 * ps)
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

    def _stages_implicit(self, y, t, dt, first_approach):
        """nbody/nbody_solver_rk_butcher.cpp:107-130: the first call of the
        solver starts the stage derivatives from an Euler guess; later calls
        start from the previous step's; then refine_steps_count sweeps of
        k_i = f(y + dt sum_n a_in k_n)."""
        e, bt = self._engine, self.bt
        if first_approach:
            e.fcompute(t, y, self._tmpk)
            for i in range(bt.steps):
                e.fmadd(self._t, y, self._tmpk, dt * bt.c[i])
                e.fcompute(t + bt.c[i] * dt, self._t, self._k[i])
        for _ in range(self.refine_steps_count):
            for i in range(bt.steps):
                coeff = [dt * bt.a[i][n] for n in range(bt.steps)]
                e.fmaddn(self._t, y, self._k, coeff, len(self._k))
                e.fcompute(t + bt.c[i] * dt, self._t, self._k[i])

    def _sub_step(self, substeps, t, dt, y, level):
        """nbody/nbody_solver_rk_butcher.cpp:164-248."""
        e, bt = self._engine, self.bt
        first_approach = False
        if not self._k:
            self._alloc()
            first_approach = True
        for _ in range(substeps):
            if bt.implicit:
                self._stages_implicit(y, t, dt, first_approach)
            else:
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
                self.accepted_steps += 1
                self.capped_steps += int(max_error > self.error_threshold)
                self.max_accepted_error = max(self.max_accepted_error, max_error)
                coeff = [bt.b2[n] * dt for n in range(bt.steps)]
                if self.correction:
                    e.fmaddn_corr(y, self._ycorr, self._k, coeff, len(self._k))
                else:
                    e.fmaddn_inplace(y, self._k, coeff, len(self._k))
            t += dt


class SolverMidpoint(Solver):
    """nbody/nbody_solver_midpoint.cpp:23-40."""

    def __init__(self):
        super().__init__()
        self._k1 = self._k2 = self._tmp = None

    def advise(self, dt: float) -> None:
        e = self._engine
        if self._k1 is None:
            ps = e.problem_size()
            self._k1, self._k2, self._tmp = (e.create_buffer(F8 * ps) for _ in range(3))
        y, t = e.get_y(), e.get_time()
        e.fcompute(t, y, self._k1)
        e.fmadd(self._tmp, y, self._k1, dt / 2.0)
        e.fcompute(t + dt / 2.0, self._tmp, self._k2)
        e.fmadd_inplace(y, self._k2, dt)
        e.advise_time(dt)


class SolverMidpointStetter(Solver):
    """Stetter's two-sequence midpoint rule, nbody/nbody_solver_midpoint_stetter.cpp:23-76:
    u_{k+1} = u_k + dt f(v_k + dt/2 f(u_k)), v_{k+1} = v_k + dt/2 (f(u_k) + f(u_{k+1})),
    y = (u + v) / 2; f(u_{k+1}) is reused as the next step's f(u_k)."""

    def __init__(self):
        super().__init__()
        self._fu: List = []
        self._uv: List = []
        self._tmp = self._du = None
        self._uv_initiated = False

    def reset(self) -> None:
        self._uv_initiated = False

    def advise(self, dt: float) -> None:
        e = self._engine
        y, t = e.get_y(), e.get_time()
        first = not self._fu
        if first:
            ps = e.problem_size()
            self._tmp = e.create_buffer(F8 * ps)
            self._du = e.create_buffer(F8 * ps)
            self._fu = e.create_buffers(F8 * ps, 2)
            self._uv = e.create_buffers(F8 * ps, 2)
        if not self._uv_initiated or first:
            e.copy_buffer(self._uv[0], y)
            e.copy_buffer(self._uv[1], y)
            first = True
            self._uv_initiated = True
        fu, uv = self._fu, self._uv
        if first:
            e.fcompute(t, uv[0], fu[0])
        e.fmadd(self._tmp, uv[1], fu[0], dt / 2.0)
        e.fcompute(t + dt / 2.0, self._tmp, self._du)
        e.fmadd_inplace(uv[0], self._du, dt)
        e.fcompute(t + dt, uv[0], fu[1])
        e.fmaddn_inplace(uv[1], fu, [dt / 2.0, dt / 2.0], 2)
        e.fmaddn(y, None, uv, [0.5, 0.5], len(uv))
        fu[0], fu[1] = fu[1], fu[0]
        e.advise_time(dt)


class SolverTrapeze(Solver):
    """nbody/nbody_solver_trapeze.cpp:30-56: Euler predictor, then
    refine_steps_count corrector sweeps of the trapezoidal rule."""

    def __init__(self, refine_steps_count: int = 1):
        super().__init__()
        self.refine_steps_count = int(refine_steps_count)
        self._f: List = []
        self._pred = None

    def advise(self, dt: float) -> None:
        e = self._engine
        y, t = e.get_y(), e.get_time()
        if not self._f:
            ps = e.problem_size()
            self._f = e.create_buffers(F8 * ps, 2)
            self._pred = e.create_buffer(F8 * ps)
        e.fcompute(t, y, self._f[0])
        e.fmadd(self._pred, y, self._f[0], dt)
        for sweep in range(self.refine_steps_count + 1):
            coeff = [dt / 2.0, dt / 2.0]
            e.fcompute(t, self._pred, self._f[1])
            if sweep == self.refine_steps_count:
                e.fmaddn_inplace(y, self._f, coeff, 2)
            else:
                e.fmaddn(self._pred, y, self._f, coeff, 2)
        e.advise_time(dt)


_ADAMS = {1: [1.0], 2: [3.0 / 2.0, -1.0 / 2.0], 3: [23.0 / 12.0, -4.0 / 3.0, 5.0 / 12.0],
          4: [55.0 / 24.0, -59.0 / 24.0, 37.0 / 24.0, -3.0 / 8.0],
          5: [1901.0 / 720.0, -1387.0 / 360.0, 109.0 / 30.0, -637.0 / 360.0, 251.0 / 720.0]}


class SolverAdams(Solver):
    """Adams-Bashforth of rank 1..5, nbody/nbody_solver_adams.cpp:30-100; the
    first rank + 1 steps are made by the starter solver while the ring of
    derivatives fills."""

    def __init__(self, starter: Solver, rank: int = 1, correction: bool = False):
        super().__init__()
        self.starter = starter
        self.rank = int(rank)
        self.correction = bool(correction)
        self._f: List = []
        self._corr = None
        self._step = 0

    def reset(self) -> None:
        if self._corr is not None:
            self._engine.fill_buffer(self._corr, 0.0)
        self._step = 0

    def advise(self, dt: float) -> None:
        e = self._engine
        a = _ADAMS[self.rank]
        y, t = e.get_y(), e.get_time()
        fnum = self._step % self.rank
        if not self._f:
            self.starter.set_engine(e)
            self._f = e.create_buffers(F8 * e.problem_size(), self.rank)
            if self.correction:
                self._corr = e.create_buffer(F8 * e.problem_size())
                e.fill_buffer(self._corr, 0.0)
        if self._step > self.rank:
            e.fcompute(t, y, self._f[fnum])
            coeff = [0.0] * self.rank
            for n in range(self.rank):
                coeff[(self.rank + fnum - n) % self.rank] = a[n] * dt
            if self.correction:
                e.fmaddn_corr(y, self._corr, self._f, coeff, self.rank)
            else:
                e.fmaddn_inplace(y, self._f, coeff, self.rank)
            e.advise_time(dt)
        else:
            e.fcompute(t, y, self._f[fnum])
            self.starter.advise(dt)
        self._step += 1


class NevilleExtrapolator:
    """nbody/nbody_extrapolator.cpp:103-181: polynomial extrapolation to a zero
    step in (step count)^order, one table row per level."""

    def __init__(self, engine, order: int, substeps):
        self.e = engine
        self.steps = [int(s ** order) if order != 1 else int(s) for s in substeps]
        ps = engine.problem_size()
        self.table = engine.create_buffers(F8 * ps, len(substeps))
        self.prev = engine.create_buffers(F8 * ps, len(substeps))
        self.diff = engine.create_buffer(F8 * ps)

    def update_table(self, k: int, y) -> None:
        e = self.e
        self.table, self.prev = self.prev, self.table
        e.copy_buffer(self.table[0], y)
        for j in range(k):
            s1 = float(self.steps[k])
            s2 = float(self.steps[k - j - 1])
            sd = s1 - s2
            e.fmaddn(self.table[j + 1], None, [self.table[j], self.prev[j]], [s1 / sd, -s2 / sd], 2)

    def estimate_error(self, level: int) -> float:
        if level == 0:
            return float("inf")
        self.e.fmadd(self.diff, self.table[level], self.table[level - 1], -1.0)
        return self.e.fmaxabs(self.diff)

    def extrapolate(self, level: int, y) -> None:
        self.e.copy_buffer(y, self.table[level])


def _bs_steps(n: int) -> List[int]:
    """nbody/nbody_solver_bulirsch_stoer.cpp:7-39 (Bulirsch sequence 2, 4, 6, 8, 12, ...)."""
    steps: List[int] = []
    if n > 0:
        steps.append(2)
    if n > 1:
        steps.append(4)
    if n > 2:
        steps.append(6)
    for j in range(3, n):
        steps.append(2 * steps[j - 2])
    return steps


class SolverBulirschStoer(Solver):
    """nbody/nbody_solver_bulirsch_stoer.cpp:41-120: Stetter midpoint sequences
    of 2, 4, 6, 8, ... substeps, Neville extrapolation in (substeps)^2, stop at
    the first level >= 2 whose estimate is below the threshold."""

    def __init__(self, max_level: int = 8, error_threshold: float = 1e-11):
        super().__init__()
        self.max_level = int(max_level)
        self.error_threshold = float(error_threshold)
        self.sub_steps = _bs_steps(self.max_level)
        self._y0 = None
        self._ext = None
        self._internal = None

    def advise(self, dt: float) -> None:
        e = self._engine
        if self._y0 is None:
            self._y0 = e.create_buffer(F8 * e.problem_size())
            self._ext = NevilleExtrapolator(e, 2, self.sub_steps)
            self._internal = SolverMidpointStetter()
            self._internal.set_engine(e)
        y, t0 = e.get_y(), e.get_time()
        e.copy_buffer(self._y0, y)
        for level in range(self.max_level):
            e.copy_buffer(y, self._y0)
            e.set_time(t0)
            n = self.sub_steps[level]
            sub_dt = dt / n
            self._internal.reset()
            for _ in range(n):
                self._internal.advise(sub_dt)
            self._ext.update_table(level, y)
            if level < 2:
                continue
            if self._ext.estimate_error(level) < self.error_threshold or level == self.max_level - 1:
                self._ext.extrapolate(level, y)
                break
        e.set_time(t0)
        e.advise_time(dt)


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
                            correction=bool(param.get("correction", False)),
                            refine_steps_count=int(param.get("refine_steps_count", 1)))
    elif kind == "midpoint":
        s = SolverMidpoint()
    elif kind == "midpoint-st":
        s = SolverMidpointStetter()
    elif kind == "trapeze":
        s = SolverTrapeze(int(param.get("refine_steps_count", 1)))
    elif kind == "adams":
        starter = create_solver(dict(param, solver=param.get("starter_solver", "euler")))
        if starter is None:
            return None
        s = SolverAdams(starter, int(param.get("rank", 1)), bool(param.get("correction", False)))
    elif kind == "bs":
        s = SolverBulirschStoer(int(param.get("max_level", 8)),
                                float(param.get("error_threshold", 1e-11)))
    else:
        return None
    s.set_time_step(float(param.get("min_step", 1e-9)), float(param.get("max_step", 1e-2)))
    s.clamp_to_box = bool(param.get("clamp", False))
    return s
