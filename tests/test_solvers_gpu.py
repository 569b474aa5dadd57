"""The reference's solver golden vectors reproduced through the GB300 engine.

test/solver/test_nbody_solver.cpp:43-260: 16-body initial_state.txt, run to
t = 0.3 with steps [1e-3, 3e-2] (Butcher solvers: max_recursion 1,
substep_subdivisions 2, refine_steps_count 1, error_threshold 1e-5), end
state within 1e-12 absolute of test/data/<name>.txt.  The solvers drive the
engine only through the nbody_engine interface; the same cases run on the
oracle's engine in test_solvers_cpu.py.
"""
import pytest

from test_solvers_cpu import CASES, run_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("golden,param", CASES, ids=[c[0] for c in CASES])
def test_solver_golden_on_gpu(make_engine, golden, param):
    d, expected = run_case(make_engine(precision="fp64"), param, golden)
    assert d.is_equal(expected, 1e-12)
