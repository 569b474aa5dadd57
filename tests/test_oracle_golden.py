"""The oracle against the reference's own known answers (CPU only).

* solver golden vectors: test/solver/test_nbody_solver.cpp:43-145 run each
  solver from test/data/initial_state.txt to t = 0.3 (steps [1e-3, 3e-2],
  max_recursion 1, substep_subdivisions 2, error_threshold 1e-5) on the
  'simple' engine and require the end state within 1e-12 absolute.
* heap index algebra: test/engine/test_nbody_engine.cpp:1071-1147.
* engine equalities the reference asserts: block == simple, BH at
  lambda = 1e8 == direct, heap == heap_stackless.
"""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from conftest import GOLDEN

SOLVERS = [("euler", "euler", False), ("rk4", "rk4", False), ("rkdp", "rkdp", False),
           ("rkdp-corr", "rkdp", True), ("rkck", "rkck", False), ("rkf", "rkf", False)]


@pytest.mark.parametrize("golden,solver,corr", SOLVERS)
def test_oracle_solver_goldens(oracle, golden, solver, corr):
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    y, t, _ = oracle.solver_run(solver, d.to_state(), d.mass, 0.3, 1e-3, 3e-2,
                                max_recursion=1, substep_subdivisions=2,
                                error_threshold=1e-5, correction=corr)
    d.from_state(y)
    expected = NBodyData.load(str(GOLDEN / f"{golden}.txt"))
    assert d.is_equal(expected, 1e-12)


def test_heap_index_known_answers(oracle):
    o = oracle
    assert o.next_down(8) == 9 and o.next_down(9) == 5
    assert [o.skip_idx(i) for i in (8, 9, 5, 11, 3, 7, 15)] == [9, 5, 3, 3, 1, 1, 1]
    assert o.next_up(1, 16) == 2 and o.next_up(8, 16) == 9
    assert o.next_up(9, 16) == 5 and o.next_up(15, 16) == 1
    for idx in range(1, 16):
        assert o.parent_idx(o.left_idx(idx)) == idx
        assert o.parent_idx(o.rght_idx(idx)) == idx
        assert o.left_idx(idx) + 1 == o.rght_idx(idx)

    def ffs_next_down(idx):  # the __ffs form of the CUDA build
        inv = ~idx & ((1 << 64) - 1)
        t = (inv & -inv).bit_length()
        return (idx >> (t - 1)) + 1
    for idx in range(1, 16):
        assert ffs_next_down(idx) == o.next_down(idx)


def test_block_equals_simple(oracle):
    d = NBodyData.make_universe(64)  # 128 bodies
    y = d.to_state()
    f0 = oracle.fcompute_simple(y, d.mass)
    f1 = oracle.fcompute_block(y, d.mass, nthreads=2)
    assert np.max(np.abs(f0 - f1)) < 1e-13


def test_make_universe_shape():
    d = NBodyData.make_universe(64)
    assert d.get_count() == 128
    assert abs(d.mass.sum() - 2000.0) < 1e-9
    assert d.box_size == 100


@pytest.mark.parametrize("layout,traverse", [(1, 0), (1, 1), (2, 0), (2, 1)])
def test_bh_exact_ratio_equals_direct(oracle, layout, traverse):
    # simple_bh at lambda = 1e8 vs simple, 1e-11 (test_nbody_engine.cpp:1358-1395)
    d = NBodyData.make_universe(64)
    y = d.to_state()
    f0 = oracle.fcompute_simple(y, d.mass)
    f1 = oracle.fcompute_bh(y, d.mass, 1e8, layout=layout, traverse=traverse)[0]
    assert np.max(np.abs(f0 - f1)) < 1e-11


@pytest.mark.parametrize("lam", [1e8, 3.1623])
def test_bh_heap_equals_stackless(oracle, lam):
    # heap vs heap_stackless at 1e-16 (test_nbody_engine.cpp:1457-1490)
    d = NBodyData.make_universe(512)  # 1024 bodies
    y = d.to_state()
    f0 = oracle.fcompute_bh(y, d.mass, lam, layout=1, traverse=1)[0]
    f1 = oracle.fcompute_bh(y, d.mass, lam, layout=2, traverse=1)[0]
    assert np.max(np.abs(f0 - f1)) <= 1e-16


def test_bh_refit_equals_build(oracle):
    # tree_build_rate 0 vs 2 at lambda 1e8, two steps with y *= 1.99
    d = NBodyData.make_universe(512)
    mut = lambda v: v + v * 0.99
    a = oracle.fcompute_bh(d.to_state(), d.mass, 1e8, steps=2, build_rate=0, mutate=mut)
    b = oracle.fcompute_bh(d.to_state(), d.mass, 1e8, steps=2, build_rate=2, mutate=mut)
    for fa, fb in zip(a, b):
        assert np.max(np.abs(fa - fb)) <= 1e-16


def test_bh_theta_error_is_bounded(oracle):
    # at lambda = 3.1623 the reference accepts 1e-2 absolute vs simple
    d = NBodyData.make_universe(64)
    y = d.to_state()
    f0 = oracle.fcompute_simple(y, d.mass)
    f1 = oracle.fcompute_bh(y, d.mass, 3.1623, layout=2, traverse=0)[0]
    assert np.max(np.abs(f0 - f1)) < 1e-2


def test_accel_rows_matches_block(oracle):
    d = NBodyData.uniform_cube(300, seed=3)
    y = d.to_state()
    acc = oracle.accel_rows(y, d.mass, 0.0, rows=np.arange(300), nthreads=2)
    f = oracle.fcompute_block(y, d.mass)
    a_ref = f[900:].reshape(3, 300).T
    assert np.max(np.abs(acc - a_ref)) <= 1e-12 * np.max(np.abs(a_ref))


def test_statistics_conserved_quantities(oracle):
    d = NBodyData.load(str(GOLDEN / "initial_state.txt"))
    st = oracle.statistics(d.to_state(), d.mass)
    P = (d.velocities * d.mass[:, None]).sum(axis=0)
    assert np.allclose(st[0:3], P, rtol=1e-12, atol=1e-12)
    ke = 0.5 * (d.mass * (d.velocities ** 2).sum(axis=1)).sum()
    assert abs(st[6] - ke) <= 1e-12 * abs(ke)
    assert st[7] < 0 and abs(st[11] - d.mass.sum()) < 1e-12
