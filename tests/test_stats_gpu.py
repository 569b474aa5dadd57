"""GPU FP64 conservation sums against the oracle's Kahan restatement of
print_statistics (nbody/nbody_data.cpp:57-145)."""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["golden16", "universe128", "cube3000", "plummer8192"])
def test_statistics_match_oracle(make_engine, oracle, case):
    if case == "golden16":
        d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    elif case == "universe128":
        d = NBodyData.make_universe(64)
    elif case == "cube3000":
        d = NBodyData.uniform_cube(3000, seed=2)
    else:
        d = NBodyData.plummer(8192, seed=3)
    e = make_engine(precision="fp64")
    assert e.init(d)
    got = e.statistics()
    ref = oracle.statistics(d.to_state(), d.mass)
    # FP64 sums in different orders differ by rounding of their terms, so the
    # bound scales with the sum of the terms' magnitudes (momentum and angular
    # momentum can cancel to far below them: make_universe's two black holes
    # of mass 999 move in opposite directions)
    m, r, v = d.mass[:, None], d.vertices, d.velocities
    p_abs = (m * np.abs(v)).sum(axis=0).max()
    l_abs = (m * np.abs(np.cross(r, v))).sum(axis=0).max()
    scale = np.array([max(np.abs(ref[0:3]).max(), p_abs)] * 3 +
                     [max(np.abs(ref[3:6]).max(), l_abs)] * 3 +
                     [abs(ref[6]), abs(ref[7]), 1, 1, 1, ref[11]])
    scale = np.maximum(scale, 1e-300)
    err = np.abs(got - ref) / np.maximum(scale, np.abs(ref[8:11]).max() * (np.arange(12) >= 8))
    print(f"\n{case}: max rel {err.max():.2e}")
    assert np.all(np.abs(got - ref) <= 1e-12 * np.maximum(scale, 1e-12) + 1e-15)


def test_print_statistics_tracks_drift(make_engine, oracle):
    """nbody_data::print_statistics with the engine's GPU sums: the first
    call fixes the initial values (zero drift), later calls report the
    percent drifts of P, L and E against them, equal to the same drifts
    from the oracle's host sums of the states get_data returns."""
    from nbody_gb300.solvers import create_solver
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    e = make_engine(precision="fp64")
    assert e.init(d)
    s = create_solver({"solver": "rk4"})
    s.set_engine(e)
    s.set_time_step(1e-2, 1e-2)
    line0 = d.print_statistics(e)
    assert "dP 0.000e+00" in line0 and "dE 0.000e+00" in line0 and line0.startswith("#00000000")
    st0 = oracle.statistics(d.to_state(), d.mass)
    for _ in range(20):
        s.advise(1e-2)
    line = d.print_statistics(e)
    st1 = oracle.statistics(d.to_state(), d.mass)
    e0, e1 = st0[6] + st0[7], st1[6] + st1[7]
    de = abs(100.0 * (e1 - e0) / e0)
    dp = abs(100.0 * np.linalg.norm(st1[0:3] - st0[0:3]) / np.linalg.norm(st0[0:3]))
    print("\n" + line)
    assert d.get_step() == 20 and abs(d.get_time() - 0.2) < 1e-12
    assert abs(d.get_energy_err() - de) <= 1e-9 * max(de, 1e-3)
    # momentum is conserved to rounding: both drifts are rounding noise
    assert d.get_impulce_err() < 1e-9 and dp < 1e-9
    assert f"dE {d.get_energy_err():.3e}" in line
