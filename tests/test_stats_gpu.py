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
    scale = np.array([np.abs(ref[0:3]).max(), np.abs(ref[0:3]).max(), np.abs(ref[0:3]).max(),
                      np.abs(ref[3:6]).max(), np.abs(ref[3:6]).max(), np.abs(ref[3:6]).max(),
                      abs(ref[6]), abs(ref[7]), 1, 1, 1, ref[11]])
    scale = np.maximum(scale, 1e-300)
    err = np.abs(got - ref) / np.maximum(scale, np.abs(ref[8:11]).max() * (np.arange(12) >= 8))
    print(f"\n{case}: max rel {err.max():.2e}")
    assert np.all(np.abs(got - ref) <= 1e-12 * np.maximum(scale, 1e-12) + 1e-15)
