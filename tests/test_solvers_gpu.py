"""The reference's solver golden vectors reproduced through the GB300 engine.

test/solver/test_nbody_solver.cpp:43-145: 16-body initial_state.txt, run to
t = 0.3 with steps [1e-3, 3e-2] (max_recursion 1, substep_subdivisions 2,
error_threshold 1e-5), end state within 1e-12 absolute of test/data/<name>.txt.
The solvers drive the engine only through the nbody_engine interface.
"""
import pytest

from nbody_gb300.data import NBodyData
from nbody_gb300.solvers import create_solver
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = [("euler", {"solver": "euler"}), ("rk4", {"solver": "rk4"}),
         ("rkdp", {"solver": "rkdp", "correction": False}),
         ("rkdp-corr", {"solver": "rkdp", "correction": True}),
         ("rkck", {"solver": "rkck"}), ("rkf", {"solver": "rkf"})]


@pytest.mark.parametrize("golden,param", CASES, ids=[c[0] for c in CASES])
def test_solver_golden_on_gpu(make_engine, golden, param):
    e = make_engine(precision="fp64")
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    assert e.init(d)
    s = create_solver(dict(param, max_recursion=1, substep_subdivisions=2,
                           error_threshold=1e-5))
    s.set_time_step(1e-3, 3e-2)
    s.set_engine(e)
    s.run(d, 0.3)
    e.get_data(d)
    expected = NBodyData.load(str(GOLDEN / f"{golden}.txt"))
    assert d.is_equal(expected, 1e-12)
