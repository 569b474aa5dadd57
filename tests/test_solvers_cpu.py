"""The restated solvers (nbody_gb300/solvers.py) on the oracle's 'simple'
engine against the reference's golden vectors
(test/solver/test_nbody_solver.cpp:150-260: 16 bodies from
initial_state.txt to t = 0.3, steps [1e-3, 3e-2], Butcher solvers with
max_recursion 1, substep_subdivisions 2, refine_steps_count 1,
error_threshold 1e-5; end state within 1e-12).  test_solvers_gpu.py runs
the same cases on the GB300 engine."""
import pytest

from nbody_gb300.data import NBodyData
from nbody_gb300.solvers import TABLES, create_solver
from oracle.engine_oracle import OracleEngine
from conftest import GOLDEN

CASES = [
    ("adams5", {"solver": "adams", "rank": 5}),
    ("adams5-corr", {"solver": "adams", "rank": 5, "correction": True}),
    ("bulirsch-stoer", {"solver": "bs", "max_level": 4, "min_step": 1e-5}),
    ("euler", {"solver": "euler"}),
    ("midpoint", {"solver": "midpoint"}),
    ("midpoint-st", {"solver": "midpoint-st"}),
    ("rk4", {"solver": "rk4"}),
    ("rkck", {"solver": "rkck"}),
    ("rkdp", {"solver": "rkdp", "correction": False}),
    ("rkdp-corr", {"solver": "rkdp", "correction": True}),
    ("rkdverk", {"solver": "rkdverk"}),
    ("rkf", {"solver": "rkf"}),
    ("rkfeagin10", {"solver": "rkfeagin10"}),
    ("rkfeagin10-corr", {"solver": "rkfeagin10", "correction": True}),
    ("rkfeagin12", {"solver": "rkfeagin12"}),
    ("rkfeagin14", {"solver": "rkfeagin14"}),
    ("rkgl", {"solver": "rkgl"}),
    ("rklc", {"solver": "rklc"}),
    ("trapeze2", {"solver": "trapeze", "refine_steps_count": 2}),
]


def run_case(engine, param, golden):
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    assert engine.init(d)
    p = dict(param)
    if p["solver"] in TABLES:  # the test's Butcher settings
        p.update(max_recursion=1, substep_subdivisions=2, refine_steps_count=1,
                 error_threshold=1e-5)
    s = create_solver(p)
    s.set_time_step(1e-3, 3e-2)
    s.set_engine(engine)
    assert s.run(d, 0.3) == 0
    engine.get_data(d)
    expected = NBodyData.load(str(GOLDEN / f"{golden}.txt"))
    return d, expected


@pytest.mark.parametrize("golden,param", CASES, ids=[c[0] for c in CASES])
def test_solver_golden_on_oracle_engine(golden, param):
    d, expected = run_case(OracleEngine(), param, golden)
    assert d.is_equal(expected, 1e-12)


def test_invalid_solver_params():
    assert create_solver({"solver": "invalid"}) is None
    assert create_solver({"solver": "adams", "starter_solver": "invalid"}) is None


@pytest.mark.parametrize("name", sorted(TABLES))
def test_butcher_table_check(name):
    """test/solver/test_nbody_solver.cpp:87-140: weights sum to 1 and each
    row of a sums to its c."""
    t = TABLES[name]
    eps = 10 * 2.220446049250313e-16
    assert abs(sum(t.b1) - 1.0) < eps and abs(sum(t.b2) - 1.0) < eps
    for i in range(t.steps):
        jmax = t.steps if t.implicit else i
        row = t.a[i][:jmax]
        amax = max([abs(a) for a in row], default=0.0) if jmax else 1.0
        amax = amax if amax > 0 else 1.0
        assert abs(sum(row) - t.c[i]) / amax < eps, (name, i)
