"""Write nbody_gb300/feagin_tables.json: the Feagin 10, 12 and 14 Butcher
tables (T. Feagin's published coefficients, 17, 25 and 35 stages) as the
reference's solvers hold them (nbody/nbody_solver_rkfeagin{10,12,14}.cpp,
60-digit decimals parsed to double), taken from the reference build
(oracle/_ref) through nbody_solver_rk_butcher::table().  Each double is
stored exactly (float.hex); explicit tables keep row i as its i entries.

TEST INFRASTRUCTURE: run where the reference's sources are present:
    python -m oracle.make_feagin_tables
tests/test_ref_pin.py checks the committed file against the reference.
"""
import json
from pathlib import Path

from oracle.ref_oracle import load_ref

OUT = Path(__file__).resolve().parent.parent / "nbody_gb300" / "feagin_tables.json"


def main():
    ref = load_ref()
    if ref is None:
        raise SystemExit("the reference's sources are needed")
    tables = {}
    for name in ("rkfeagin10", "rkfeagin12", "rkfeagin14"):
        a, b1, b2, c, implicit, embedded = ref.butcher_table({"solver": name})
        s = len(c)
        rows = [[float(a[i, j]).hex() for j in range(s if implicit else i)] for i in range(s)]
        tables[name] = {"steps": s, "a": rows, "b1": [float(x).hex() for x in b1],
                        "b2": [float(x).hex() for x in b2], "c": [float(x).hex() for x in c],
                        "implicit": implicit, "embedded": embedded}
    OUT.write_text(json.dumps({"source": "T. Feagin's Runge-Kutta 10(8), 12(10), 14(12) "
                                         "coefficients as the reference's solvers hold them",
                               "tables": tables}, indent=0))
    print(OUT, {k: v["steps"] for k, v in tables.items()})


if __name__ == "__main__":
    main()
