"""The oracle restatement and the committed fixtures against the reference's
own code.

oracle/_ref/libnbody_ref.so is the reference's CPU sources (nbody/*.cpp,
unchanged) compiled here against the Qt-API shim (oracle/ref_build.py).
These tests pin oracle/nbody_oracle.c, the galaxy generator of
nbody_gb300/data.py, the Butcher tables of nbody_gb300/solvers.py and the
stream format to what the reference itself computes -- bit for bit where the
arithmetic is the same -- so that the GPU parity tests, which compare
against the oracle, inherit the pin.  They need the reference's sources and
skip where those are absent (the GPU host).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from conftest import GOLDEN

ref_oracle = pytest.importorskip("oracle.ref_oracle")


@pytest.fixture(scope="module")
def ref():
    r = ref_oracle.load_ref()
    if r is None:
        pytest.skip("the reference's sources are not present on this host")
    return r


@pytest.mark.parametrize("stars", [8, 64, 512])
def test_make_universe_equals_reference(ref, stars):
    """nbody_data::make_universe (nbody/nbody_data.cpp:263-324), the input of
    the reference's engine tests, bit for bit."""
    y, m = ref.make_universe(stars)
    d = NBodyData.make_universe(stars)
    assert np.array_equal(d.to_state(), y)
    assert np.array_equal(d.mass, m)


def _inputs():
    y, m = NBodyData.make_universe(64).to_state(), NBodyData.make_universe(64).mass
    c = NBodyData.uniform_cube(1024, seed=11)
    return [("universe128", y, m), ("cube1024", c.to_state(), c.mass)]


@pytest.mark.parametrize("engine", ["simple", "openmp", "block"])
@pytest.mark.parametrize("case", [0, 1])
def test_direct_engines_equal_reference(ref, oracle, engine, case):
    """simple / openmp / block fcompute (nbody/nbody_engine_{simple,openmp,
    block}.cpp) equal the oracle's restatement bit for bit."""
    _, y, m = _inputs()[case]
    f_ref = ref.fcompute({"engine": engine}, y, m)[0]
    f = oracle.fcompute_block(y, m) if engine == "block" else oracle.fcompute_simple(y, m)
    assert np.array_equal(f, f_ref)


@pytest.mark.parametrize("lam", [3.1623, 1.1111, 1e8])
@pytest.mark.parametrize("layout", ["heap", "heap_stackless"])
@pytest.mark.parametrize("trav", ["cycle", "nested_tree"])
@pytest.mark.parametrize("rate", [0, 2])
@pytest.mark.parametrize("case", [0, 1])
def test_simple_bh_equals_reference(ref, oracle, lam, layout, trav, rate, case):
    """simple_bh (nbody/nbody_engine_simple_bh.cpp:16-194) over the kd heap
    (nbody/nbody_space_heap.cpp, nbody_space_heap_stackless.cpp) through the
    reference's factory, as test_nbody_engine_compare drives it
    (test/engine/test_nbody_engine.cpp:472-550, 1358-1559): two steps, y *=
    1.99 between, tree_build_rate 0 and 2 (the second step refits).  The
    oracle restatement, which the GPU FP64 walk is tested against, equals it
    bit for bit."""
    _, y, m = _inputs()[case]
    f_ref = ref.fcompute({"engine": "simple_bh", "distance_to_node_radius_ratio": lam,
                          "traverse_type": trav, "tree_layout": layout,
                          "tree_build_rate": rate}, y, m, steps=2, mutate=0.99)
    f = oracle.fcompute_bh(y, m, lam, layout={"heap": 1, "heap_stackless": 2}[layout],
                           traverse={"cycle": 0, "nested_tree": 1}[trav], steps=2,
                           build_rate=rate, mutate=lambda v: v + 0.99 * v)
    for s in range(2):
        assert np.array_equal(f[s], f_ref[s]), s


@pytest.mark.parametrize("n,kind", [(128, "universe"), (1024, "cube"), (4096, "plummer")])
@pytest.mark.parametrize("lam", [2.0, 3.1623])
def test_kd_heap_nodes_equal_reference(ref, oracle, n, kind, lam):
    """nbody_space_heap::build (nbody/nbody_space_heap.cpp:13-37,119-190):
    every node's mass centre, mass and critical radius, and every leaf's
    body, bit for bit (the GPU kd build is tested node for node against the
    oracle)."""
    d = {"universe": lambda: NBodyData.make_universe(n // 2),
         "cube": lambda: NBodyData.uniform_cube(n, seed=3),
         "plummer": lambda: NBodyData.plummer(n, seed=4)}[kind]()
    y, m = d.to_state(), d.mass
    c_ref, m_ref, r_ref, b_ref = ref.heap_build(y, m, lam)
    com, mass, r2, body, _, _ = oracle.heap_nodes(y, m, lam)
    assert np.array_equal(com[:, 1:], c_ref[:, 1:])
    assert np.array_equal(mass[1:], m_ref[1:])
    assert np.array_equal(r2[1:], r_ref[1:])
    assert np.array_equal(body[n:], b_ref[n:])


GOLDEN_CASES = [
    ("adams5", {"solver": "adams", "rank": 5}),
    ("adams5-corr", {"solver": "adams", "rank": 5, "correction": "true"}),
    ("bulirsch-stoer", {"solver": "bs", "max_level": 4}),
    ("euler", {"solver": "euler"}),
    ("midpoint", {"solver": "midpoint"}),
    ("midpoint-st", {"solver": "midpoint-st"}),
    ("rk4", {"solver": "rk4"}),
    ("rkck", {"solver": "rkck"}),
    ("rkdp", {"solver": "rkdp", "correction": "false"}),
    ("rkdp-corr", {"solver": "rkdp", "correction": "true"}),
    ("rkdverk", {"solver": "rkdverk"}),
    ("rkf", {"solver": "rkf"}),
    ("rkfeagin10", {"solver": "rkfeagin10"}),
    ("rkfeagin10-corr", {"solver": "rkfeagin10", "correction": "true"}),
    ("rkfeagin12", {"solver": "rkfeagin12"}),
    ("rkfeagin14", {"solver": "rkfeagin14"}),
    ("rkgl", {"solver": "rkgl"}),
    ("rklc", {"solver": "rklc"}),
    ("trapeze2", {"solver": "trapeze", "refine_steps_count": 2}),
]
BUTCHER = {"rkck", "rkdp", "rkdverk", "rkf", "rkfeagin10", "rkfeagin12", "rkfeagin14", "rkgl",
           "rklc"}


def _golden_param(param):
    """The golden test's settings (test/solver/test_nbody_solver.cpp:43-66):
    steps [1e-3, 3e-2]; Butcher solvers max_recursion 1, 2 substeps, one
    refinement sweep, error threshold 1e-5."""
    p = dict(param, min_step=1e-3, max_step=3e-2)
    if p["solver"] in BUTCHER:
        p.update(max_recursion=1, substep_subdivisions=2, refine_steps_count=1,
                 error_threshold=1e-5)
    return p


@pytest.mark.parametrize("golden,param", GOLDEN_CASES, ids=[c[0] for c in GOLDEN_CASES])
def test_reference_build_reproduces_its_goldens(ref, golden, param):
    """The reference build itself (solvers from its factory, 'simple'
    engine) reproduces the reference's golden end states at the test's
    1e-12: the shim build is the reference."""
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    y, t, _ = ref.solver_run(_golden_param(param), {"engine": "simple"}, d.to_state(), d.mass,
                             0.3)
    exp = NBodyData.load(str(GOLDEN / f"{golden}.txt"))
    assert abs(t - 0.3) < 1e-9
    assert np.max(np.abs(y - exp.to_state())) <= 1e-12


@pytest.mark.parametrize("name", ["euler", "rk4", "rkdp", "rkck", "rkf"])
def test_oracle_solvers_equal_reference(ref, oracle, name):
    """The oracle's solver restatement (orc_solver_run) equals the reference's
    solver on the reference's engine."""
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    p = _golden_param({"solver": name})
    y_ref, _, _ = ref.solver_run(p, {"engine": "simple"}, d.to_state(), d.mass, 0.3)
    y, _, _ = oracle.solver_run(name, d.to_state(), d.mass, 0.3, 1e-3, 3e-2, max_recursion=1,
                                substep_subdivisions=2, error_threshold=1e-5)
    assert np.max(np.abs(y - y_ref)) <= 1e-15 * max(1.0, np.max(np.abs(y_ref)))


def test_config1_rk4_equals_reference(ref, oracle):
    """The direct-sum parity configuration: N = 1024 uniform cube of side
    100, v ~ N(0, 0.1), m ~ U[0.5, 1.5] / N, rk4 with dt = 0.01 for 100 steps:
    the oracle (which the GPU FP64 engine is compared with at every step)
    against the reference's rk4 on its simple engine."""
    d = NBodyData.uniform_cube(1024, side=100.0, seed=1)
    y0 = d.to_state()
    y_ref, t, steps = ref.solver_run({"solver": "rk4", "min_step": 0.01, "max_step": 0.01},
                                     {"engine": "simple"}, y0, d.mass, 1.0 - 1e-9)
    assert steps == 100
    y, _, _ = oracle.solver_run("rk4", y0, d.mass, 1.0 - 1e-9, 0.01, 0.01)
    assert np.max(np.abs(y - y_ref) / np.maximum(np.abs(y_ref), 1e-300)) <= 1e-13


def test_statistics_equal_reference(ref, oracle):
    """print_statistics' conservation sums (nbody/nbody_data.cpp:57-145) of one
    state: momentum, angular momentum, mass centre and total energy."""
    d = NBodyData.make_universe(64)
    y, m = d.to_state(), d.mass
    r = ref.statistics(y, m)
    o = oracle.statistics(y, m)  # P[3], L[3], KE, PE, centre[3], mass
    assert np.allclose(o[:6], r[:6], rtol=1e-13, atol=1e-13 * np.abs(r[:6]).max())
    assert np.allclose(o[8:11], r[6:9], rtol=1e-13)
    assert abs((o[6] + o[7]) - r[9]) <= 1e-13 * abs(r[9])


def test_butcher_tables_equal_reference(ref):
    """The Butcher tables nbody_gb300/solvers.py runs (restated ones and the
    Feagin tables loaded from nbody_gb300/feagin_tables.json) equal the
    reference's tables (nbody_solver_rk_butcher::table) entry for entry."""
    from nbody_gb300.solvers import TABLES
    for name in sorted(BUTCHER):
        a, b1, b2, c, implicit, embedded = ref.butcher_table({"solver": name})
        t = TABLES[name]
        s = t.steps
        assert s == len(c), name
        ours = np.zeros((s, s))
        for i, row in enumerate(t.a):
            ours[i, :len(row)] = row
        assert np.array_equal(ours, a), name
        assert np.array_equal(np.array(t.b1), b1) and np.array_equal(np.array(t.b2), b2), name
        assert np.array_equal(np.array(t.c), c), name
        assert t.implicit == implicit and t.embedded == embedded, name


def test_stream_files_equal_reference(ref, tmp_path):
    """nbody_data_stream (nbody/nbody_data_stream.cpp:62-229): the oracle's
    restatement of the writer (which the GPU stream writer matches byte for
    byte) writes the same files as the reference, part rollover included."""
    from oracle.stream_oracle import OracleStream
    n, frames = 100, 6
    rng = np.random.default_rng(9)
    ys = rng.normal(size=(frames, 6 * n))
    mass = rng.uniform(0.5, 1.5, size=n)
    steps = np.arange(frames, dtype=np.uint64) * 3
    times = np.arange(frames) * 0.015
    base_r = str(tmp_path / "ref" / "st")
    base_o = str(tmp_path / "orc" / "st")
    ref.stream_write(base_r, 14000, ys, mass, steps, times)
    st = OracleStream(base_o, 14000)
    white = np.ones((n, 4), dtype=np.float32)  # the reference build's add_body colour
    for k in range(frames):
        y = ys[k]
        st.write(int(steps[k]), float(times[k]), y[:3 * n].reshape(3, n).T,
                 y[3 * n:].reshape(3, n).T, 0, white, mass)
    st.close()
    names = sorted(p.name for p in (tmp_path / "ref").iterdir())
    assert names == sorted(p.name for p in (tmp_path / "orc").iterdir())
    assert any(nm.endswith("1.dat") for nm in names)  # the part rolled over
    for nm in names:
        assert (tmp_path / "ref" / nm).read_bytes() == (tmp_path / "orc" / nm).read_bytes(), nm
