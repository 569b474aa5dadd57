"""Copy the reference's golden vectors into tests/golden/.

The reference (drons/nbody) pins its solvers with 16-body end states after
t = 0.3 (test/solver/test_nbody_solver.cpp:43-145): the initial state
test/data/initial_state.txt and one end state per solver, compared at 1e-12
absolute.  Its table loader is pinned with three malformed tables.  The
reference is not on the machine the GPU tests run on, so the files travel
with the tests.  Run from the repository root:

    python tests/golden/make_fixtures.py /path/to/reference
"""
import shutil
import sys
from pathlib import Path

FILES = ["initial_state", "euler", "rk4", "rkdp", "rkdp-corr", "rkck", "rkf",
         "midpoint", "rkdverk", "rkfeagin10", "rkfeagin12", "rkfeagin14",
         "rkgl", "rklc", "adams5", "adams5-corr", "bulirsch-stoer",
         "midpoint-st", "rkfeagin10-corr", "trapeze2",
         # the table loader's fixtures (test/stream/test_nbody_stream.cpp:344-372)
         "inv_column", "inv_columns_count", "inv_radius"]


def main(ref_root: str) -> None:
    src = Path(ref_root) / "test" / "data"
    dst = Path(__file__).resolve().parent
    for name in FILES:
        shutil.copyfile(src / f"{name}.txt", dst / f"{name}.txt")
        print("copied", name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_fixtures.py /path/to/reference")
    main(sys.argv[1])
