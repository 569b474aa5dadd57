"""Barnes-Hut on the GPU against the oracle restatement of simple_bh.

FP64 mode reproduces the reference's cuda_bh / cuda_bh_tex vs simple_bh
comparisons (test/engine/test_nbody_engine.cpp:1255-1336): make_universe
N = 128 (and 1024), lambda in {3.1623, 1e8}, layouts heap / heap_stackless,
traversals cycle / nested_tree, tree_build_rate 0 and 2 (refit on odd steps),
two steps with y *= 1.99 between, 1e-13 absolute.  The mixed mode is judged
against the FP64 direct sum.
"""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData

pytestmark = pytest.mark.gpu


def _f(e, y):
    n6 = y.size
    my, mf = e.create_buffer(8 * n6), e.create_buffer(8 * n6)
    e.write_buffer(my, y)
    e.fill_buffer(mf, 1e10)
    e.fcompute(0.0, my, mf)
    out = np.zeros(n6)
    e.read_buffer(out, mf)
    e.free_buffer(my)
    e.free_buffer(mf)
    return out


LAYOUT = {"heap": 1, "heap_stackless": 2}
TRAV = {"cycle": 0, "nested_tree": 1}


@pytest.mark.parametrize("lam", [3.1623, 1e8])
@pytest.mark.parametrize("layout", ["heap", "heap_stackless"])
@pytest.mark.parametrize("trav", ["cycle", "nested_tree"])
@pytest.mark.parametrize("rate", [0, 2])
def test_bh_fp64_vs_simple_bh(make_engine, oracle, lam, layout, trav, rate):
    d = NBodyData.make_universe(64)  # 128 bodies
    e = make_engine(algo="bh", precision="fp64", distance_to_node_radius_ratio=lam,
                    tree_layout=layout, traverse_type=trav, tree_build_rate=rate)
    assert e.init(d)
    mut = lambda v: v + v * 0.99
    ref = oracle.fcompute_bh(d.to_state(), d.mass, lam, layout=LAYOUT[layout],
                             traverse=TRAV[trav], steps=2, build_rate=rate, mutate=mut)
    y = d.to_state()
    for step in range(2):
        e.set_step(step)
        f = _f(e, y)
        assert np.max(np.abs(f - ref[step])) <= 1e-13, f"step {step}"
        y = mut(y)


@pytest.mark.parametrize("n", [1, 2, 4, 8, 64, 1024, 4096])
def test_bh_fp64_sizes(make_engine, oracle, n):
    d = NBodyData.uniform_cube(n, side=10.0, seed=n)
    e = make_engine(algo="bh", precision="fp64", distance_to_node_radius_ratio=3.1623)
    assert e.init(d)
    f = _f(e, d.to_state())
    ref = oracle.fcompute_bh(d.to_state(), d.mass, 3.1623, layout=2, traverse=1)[0]
    assert np.max(np.abs(f - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_bh_fp64_large_exact_ratio(make_engine, oracle):
    # lambda = 1e8 opens every node: the walk is a direct sum in tree order
    d = NBodyData.make_universe(512)  # 1024 bodies
    e = make_engine(algo="bh", precision="fp64", distance_to_node_radius_ratio=1e8)
    assert e.init(d)
    f = _f(e, d.to_state())
    ref = oracle.fcompute_simple(d.to_state(), d.mass)
    assert np.max(np.abs(f - ref)) <= 1e-11


def test_bh_rejects_non_power_of_two(make_engine):
    d = NBodyData.uniform_cube(100, seed=1)
    e = make_engine(algo="bh", precision="fp64")
    assert not e.init(d)
    assert e.last_status == 6  # NBG_ERR_UNSUPPORTED


def _rel(a, a_ref):
    return np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)


@pytest.mark.parametrize("walk", [0, 1])
@pytest.mark.parametrize("lam", [2.0, 1.0 / 0.9])
def test_bh_mixed_error_vs_direct(make_engine, oracle, lam, walk):
    """Both FP32 walks (0: warp-coherent stackless, 1: group walk with
    interaction lists) are at least as accurate as the reference's own
    per-body FP64 walk (simple_bh heap_stackless) at the same ratio, all
    judged against the FP64 direct sum."""
    n = 16384
    d = NBodyData.plummer(n, seed=4)
    y = d.to_state()
    e = make_engine(algo="bh", precision="mixed", softening=0.0,
                    distance_to_node_radius_ratio=lam)
    e.tune_set("bh.walk", walk)
    assert e.init(d)
    f = _f(e, y)
    rows = np.random.default_rng(9).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 0.0, rows=rows)
    a = f[3 * n:].reshape(3, n).T[rows]
    f_bh = oracle.fcompute_bh(y, d.mass, lam, layout=2, traverse=0, nthreads=8)[0]
    a_bh = f_bh[3 * n:].reshape(3, n).T[rows]
    rel, rel_ref = _rel(a, a_ref), _rel(a_bh, a_ref)
    visits, inter = e.bh_counters()
    print(f"\nBH mixed walk={walk} lambda={lam:.3f}: p50 {np.median(rel):.2e} p99 {np.quantile(rel, 0.99):.2e}"
          f" (reference walk p50 {np.median(rel_ref):.2e} p99 {np.quantile(rel_ref, 0.99):.2e});"
          f" interactions/body {inter / n:.0f}, visits/warp {visits / (n / 32):.0f}")
    assert np.array_equal(f[:3 * n], y[3 * n:])
    assert np.quantile(rel, 0.99) <= np.quantile(rel_ref, 0.99)
    assert np.median(rel) <= np.median(rel_ref)


@pytest.mark.parametrize("n", [1, 2, 8, 16])
def test_bh_mixed_tiny(make_engine, oracle, n):
    """Below one warp group the mixed path walks per body (on the default
    Hilbert tree); at lambda 1e8 every node opens and the forces are the
    direct sum's."""
    d = NBodyData.plummer(n, seed=n + 3)
    y = d.to_state()
    e = make_engine(algo="bh", precision="mixed", softening=1e-3,
                    distance_to_node_radius_ratio=1e8)
    assert e.init(d)
    f = _f(e, y)
    assert np.array_equal(f[:3 * n], y[3 * n:])
    a_ref = oracle.accel_rows(y, d.mass, 1e-3, rows=np.arange(n))
    a = f[3 * n:].reshape(3, n).T
    scale = max(np.abs(a_ref).max(), 1e-30)
    assert np.all(np.abs(a - a_ref) <= 1e-5 * scale)


@pytest.mark.parametrize("n", [32, 64, 1024])
def test_bh_group_walk_small(make_engine, oracle, n):
    """Group walk on one or a few warps.  One warp (n = 32) opens the whole
    tree down to its leaves and is a direct sum; larger systems are at least
    as accurate as the reference's per-body walk at the same ratio."""
    d = NBodyData.plummer(n, seed=n)
    y = d.to_state()
    e = make_engine(algo="bh", precision="mixed", softening=0.0,
                    distance_to_node_radius_ratio=2.0)
    assert e.init(d)
    f = _f(e, y)
    a_ref = oracle.accel_rows(y, d.mass, 0.0, rows=np.arange(n))
    a = f[3 * n:].reshape(3, n).T
    rel = _rel(a, a_ref)
    assert np.array_equal(f[:3 * n], y[3 * n:])
    if n == 32:
        assert np.max(rel) < 1e-5
        return
    f_bh = oracle.fcompute_bh(y, d.mass, 2.0, layout=2, traverse=0)[0]
    rel_ref = _rel(f_bh[3 * n:].reshape(3, n).T, a_ref)
    assert np.quantile(rel, 0.99) <= np.quantile(rel_ref, 0.99)
    assert np.median(rel) <= np.median(rel_ref)


@pytest.mark.parametrize("eps", [1e-3, 0.0])
@pytest.mark.parametrize("lam", [2.0, 4.0])
def test_bh_quadrupole_walk(make_engine, oracle, lam, eps):
    """bh.order = 2 adds each accepted cell's quadrupole term: the same node
    tests and interactions as the monopole walk (both at one node test per
    lane and step: a group that reaches the test cap stops after a whole
    step, so its partial count depends on the step size), and a smaller
    error against the FP64 direct sum (cells' errors fall as (s/d)^3
    instead of (s/d)^2)."""
    n = 16384
    d = NBodyData.plummer(n, seed=8)
    y = d.to_state()
    rows = np.random.default_rng(2).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, eps, rows=rows)
    res = {}
    for order in (1, 2):
        e = make_engine(algo="bh", precision="mixed", softening=eps,
                        distance_to_node_radius_ratio=lam)
        e.tune_set("bh.order", order)
        e.tune_set("bh.walk_npl", 1)
        assert e.init(d)
        f = _f(e, y)
        assert np.array_equal(f[:3 * n], y[3 * n:])
        rel = _rel(f[3 * n:].reshape(3, n).T[rows], a_ref)
        res[order] = (rel, e.bh_counters())
    (r1, c1), (r2, c2) = res[1], res[2]
    print(f"\nlambda {lam}: monopole p50 {np.median(r1):.2e} p99 {np.quantile(r1, 0.99):.2e}; "
          f"quadrupole p50 {np.median(r2):.2e} p99 {np.quantile(r2, 0.99):.2e}")
    assert c1 == c2
    assert np.median(r2) < 0.5 * np.median(r1)
    assert np.quantile(r2, 0.99) < 0.7 * np.quantile(r1, 0.99)


@pytest.mark.parametrize("kind", ["plummer", "cube"])
@pytest.mark.parametrize("n", [1 << 21, 1 << 22])
def test_bh_group_walk_deep_trees(make_engine, oracle, n, kind):
    """Trees of 22 and 23 levels: the group walk's stack stays well inside
    its capacity (48 entries per level) and the forces keep their accuracy."""
    d = NBodyData.plummer(n, seed=21) if kind == "plummer" else \
        NBodyData.uniform_cube(n, side=2.0, seed=21)
    y = d.to_state()
    e = make_engine(algo="bh", precision="mixed", softening=1e-3,
                    distance_to_node_radius_ratio=2.0)
    assert e.init(d)
    f = _f(e, y)
    peak, cap = e.bh_stack_peak()
    rows = np.random.default_rng(4).choice(n, size=64, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 1e-3, rows=rows, nthreads=8)
    rel = _rel(f[3 * n:].reshape(3, n).T[rows], a_ref)
    print(f"\n{kind} N={n}: stack peak {peak} of {cap}; p50 {np.median(rel):.2e} max {rel.max():.2e}")
    assert 0 < peak < cap // 2
    assert np.all(np.isfinite(f)) and np.median(rel) < 1e-2


@pytest.mark.parametrize("lam", [2.0, 1.0 / 0.9])
def test_bh_curve_builds(make_engine, oracle, lam):
    """bh.build = 1 (Morton) and 2 (Hilbert): the leaves are the bodies in
    curve order (a permutation) and the walk over that tree keeps the
    accuracy of the reference's per-body walk on the kd tree at the same
    ratio (within 1.5x at p99)."""
    n = 16384
    d = NBodyData.plummer(n, seed=4)
    y = d.to_state()
    rows = np.random.default_rng(9).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 0.0, rows=rows)
    f_bh = oracle.fcompute_bh(y, d.mass, lam, layout=2, traverse=0, nthreads=8)[0]
    rel_ref = _rel(f_bh[3 * n:].reshape(3, n).T[rows], a_ref)
    res = {}
    for build in (0, 1, 2):
        e = make_engine(algo="bh", precision="mixed", softening=0.0,
                        distance_to_node_radius_ratio=lam)
        e.tune_set("bh.build", build)
        assert e.init(d)
        f = _f(e, y)
        assert np.array_equal(f[:3 * n], y[3 * n:])
        leaves = e.tree_leaves()
        assert sorted(leaves.tolist()) == list(range(n))
        res[build] = _rel(f[3 * n:].reshape(3, n).T[rows], a_ref)
        fb_first = e.bh_fallback_groups()
        e.bh_counters()
        # the test cap (3x the median of sampled groups' tests) depends on
        # the tree alone: a second call on the same state gives the same forces
        f2 = _f(e, y)
        fb_next = e.bh_fallback_groups()
        print(f"\nlambda {lam:.3f} build {build}: p50 {np.median(res[build]):.2e} "
              f"p99 {np.quantile(res[build], 0.99):.2e}; fallback groups {fb_first}, then {fb_next}")
        assert fb_next == fb_first <= n // 64 // 10
        assert np.array_equal(f, f2)
    print(f"reference walk p99 {np.quantile(rel_ref, 0.99):.2e}")
    for build in (1, 2):
        assert np.quantile(res[build], 0.99) <= 1.5 * np.quantile(rel_ref, 0.99)
        assert np.median(res[build]) <= 1.5 * np.median(res[0])


@pytest.mark.parametrize("kind", ["plummer", "cube"])
@pytest.mark.parametrize("build", [1, 2])
def test_bh_curve_leaf_order(make_engine, build, kind):
    """The Morton (1) and Hilbert (2) builds put the bodies in the leaves in
    exactly the order of the CPU restatement (tests/curve_order.py: box,
    21-bit cells, keys, stable sort on the key bits from 16 up), and a refit
    keeps that order."""
    from tests import curve_order as C
    n = 8192
    d = NBodyData.plummer(n, seed=12) if kind == "plummer" else \
        NBodyData.uniform_cube(n, side=3.0, seed=12)
    e = make_engine(algo="bh", precision="mixed", softening=1e-3,
                    distance_to_node_radius_ratio=2.0, tree_build_rate=2)
    e.tune_set("bh.build", build)
    assert e.init(d)
    y = d.to_state()
    e.set_step(0)
    _f(e, y)
    expect = C.leaf_order(d.vertices, hilbert=build == 2)
    assert np.array_equal(e.tree_leaves(), expect)
    e.set_step(1)  # refit: same leaves
    _f(e, y * 1.01)
    assert np.array_equal(e.tree_leaves(), expect)


def test_bh_hilbert_clustered_and_degenerate(make_engine, oracle):
    """The default mixed path on inputs that stress the curve order: two dense
    clusters far apart plus a sparse halo (groups that straddle the curve's
    jumps between them go to the per-body walk), and a system whose bodies
    all sit at one point.  Forces stay finite and, for the clusters, at
    least as accurate as the reference's per-body walk at the same ratio."""
    n = 16384
    rng = np.random.default_rng(17)
    a = NBodyData.plummer(7936, seed=31, scale=0.01)
    b = NBodyData.plummer(7936, seed=32, scale=0.01)
    halo = rng.uniform(-20.0, 20.0, size=(n - 2 * 7936, 3))
    pos = np.concatenate([a.vertices + [5.0, 0, 0], b.vertices - [5.0, 0, 0], halo])
    vel = np.zeros_like(pos)
    d = NBodyData(vertices=pos, velocities=vel, mass=np.full(n, 1.0 / n))
    y = d.to_state()
    e = make_engine(algo="bh", precision="mixed", softening=0.0, distance_to_node_radius_ratio=2.0)
    assert e.init(d)
    f = _f(e, y)
    fb = e.bh_fallback_groups()
    assert np.all(np.isfinite(f)) and np.array_equal(f[:3 * n], y[3 * n:])
    rows = np.random.default_rng(5).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 0.0, rows=rows)
    rel = _rel(f[3 * n:].reshape(3, n).T[rows], a_ref)
    f_bh = oracle.fcompute_bh(y, d.mass, 2.0, layout=2, traverse=0, nthreads=8)[0]
    rel_ref = _rel(f_bh[3 * n:].reshape(3, n).T[rows], a_ref)
    print(f"\nclusters + halo: fallback groups {fb}; p50 {np.median(rel):.2e} "
          f"p99 {np.quantile(rel, 0.99):.2e} (reference walk p99 {np.quantile(rel_ref, 0.99):.2e})")
    assert np.quantile(rel, 0.99) <= np.quantile(rel_ref, 0.99)
    # every body at one point: no direction, zero force
    n = 1024
    d = NBodyData(vertices=np.ones((n, 3)), velocities=np.zeros((n, 3)), mass=np.full(n, 1.0 / n))
    e = make_engine(algo="bh", precision="mixed", softening=0.0, distance_to_node_radius_ratio=2.0)
    assert e.init(d)
    f = _f(e, d.to_state())
    assert np.all(f[3 * n:] == 0.0)


@pytest.mark.parametrize("group,order", [(64, 1), (64, 2), (32, 1), (32, 2), (128, 1)])
def test_bh_body_walk_fallback(make_engine, oracle, group, order):
    """A group walk that exceeds bh.test_cap node tests hands its bodies to
    the per-body walk.  With a cap of one test every group does: the forces
    are then the reference's per-body walk on the same kd tree in FP32
    records (against the oracle's FP64 walk: equal but for the few bodies
    where an acceptance test falls the other way in FP32), and with the
    quadrupole term they are well below that walk's error."""
    n = 16384
    lam = 2.0
    d = NBodyData.plummer(n, seed=6)
    y = d.to_state()
    rows = np.random.default_rng(3).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 0.0, rows=rows)
    res = {}
    for cap in (0, 1):
        e = make_engine(algo="bh", precision="mixed", softening=0.0,
                        distance_to_node_radius_ratio=lam)
        e.tune_set("bh.group", group)
        e.tune_set("bh.order", order)
        e.tune_set("bh.build", 0)  # the reference's tree, as the oracle builds it
        if cap:
            e.tune_set("bh.test_cap", cap)
        assert e.init(d)
        f = _f(e, y)
        assert np.array_equal(f[:3 * n], y[3 * n:])
        assert e.bh_fallback_groups() == (n // group if cap else 0)
        res[cap] = f
    a_fb = res[1][3 * n:].reshape(3, n).T
    rel = _rel(a_fb[rows], a_ref)
    rel_gw = _rel(res[0][3 * n:].reshape(3, n).T[rows], a_ref)
    print(f"\ngroup {group} order {order}: fallback p50 {np.median(rel):.2e} p99 "
          f"{np.quantile(rel, 0.99):.2e}; group walk p50 {np.median(rel_gw):.2e} "
          f"p99 {np.quantile(rel_gw, 0.99):.2e}")
    f_bh = oracle.fcompute_bh(y, d.mass, lam, layout=2, traverse=0, nthreads=8)[0]
    a_bh = f_bh[3 * n:].reshape(3, n).T
    if order == 1:
        diff = _rel(a_fb, a_bh)
        assert np.median(diff) < 1e-5
        assert np.mean(diff > 1e-4) < 0.02
    else:
        rel_bh = _rel(a_bh[rows], a_ref)
        assert np.median(rel) < 0.5 * np.median(rel_bh)
        assert np.quantile(rel, 0.99) < 0.7 * np.quantile(rel_bh, 0.99)


def test_bh_mixed_refit_path(make_engine):
    n = 4096
    d = NBodyData.plummer(n, seed=5)
    e = make_engine(algo="bh", precision="mixed", softening=1e-3,
                    distance_to_node_radius_ratio=2.0, tree_build_rate=2)
    assert e.init(d)
    y = d.to_state()
    e.set_step(0)
    f0 = _f(e, y)
    e.set_step(1)  # refit: same bodies per leaf, same positions -> same forces
    f1 = _f(e, y)
    assert np.max(np.abs(f0 - f1)) == 0.0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_bh_refit_within_step(make_engine, precision):
    """tree_refit_within_step: a full build at the first fcompute of an engine
    step, refits of that topology for the step's other fcomputes.  Within a
    step the forces equal the reference rule's refit path (tree_build_rate 2,
    an odd step refits the even step's tree) on the same positions; at the
    next step they equal a fresh build."""
    n = 1 << 13
    d = NBodyData.plummer(n, seed=12)
    y0 = d.to_state()
    y1 = y0.copy()
    y1[:3 * n] += 2e-3 * y0[3 * n:]  # bodies moved along their velocities
    kw = dict(algo="bh", precision=precision, softening=1e-3, distance_to_node_radius_ratio=2.0)
    # each engine its own data: the data object holds the step counter
    a = make_engine(tree_refit_within_step=True, **kw)
    assert a.init(NBodyData.plummer(n, seed=12))
    b = make_engine(tree_build_rate=2, **kw)
    assert b.init(NBodyData.plummer(n, seed=12))
    c = make_engine(**kw)
    assert c.init(NBodyData.plummer(n, seed=12))
    a.set_step(4)
    b.set_step(4)
    assert np.array_equal(_f(a, y0), _f(b, y0))   # both build on y0
    b.set_step(5)
    f_refit = _f(a, y1)                           # same step: refit to y1
    assert np.array_equal(f_refit, _f(b, y1))     # rate 2, odd step: refit to y1
    f_build = _f(c, y1)
    assert not np.array_equal(f_refit, f_build)   # a rebuilt tree differs
    a.set_step(5)
    assert np.array_equal(_f(a, y1), f_build)     # new step: a fresh build


def test_bh_freeze_within_step(make_engine, oracle):
    """tree_freeze_within_step: at the step's build the frozen walk accepts
    the plain walk's cells (the same interaction count) and agrees with it to
    FP32 rounding (its pair differences add the leaves' FP32 residuals); at a
    later stage of the same step, with the bodies moved, every body meets
    exactly the cells of the build, while an unfrozen refit changes the
    accepted sets, and the forces stay as accurate as the plain walk's
    against the FP64 direct sum.  The next step builds afresh."""
    n = 1 << 15
    d = NBodyData.plummer(n, seed=13)
    y0 = d.to_state()
    y1 = y0.copy()
    y1[:3 * n] += 5e-3 * y0[3 * n:]
    kw = dict(algo="bh", precision="mixed", softening=1e-3, distance_to_node_radius_ratio=2.0)
    fz = make_engine(tree_freeze_within_step=True, **kw)
    rf = make_engine(tree_refit_within_step=True, **kw)
    pl = make_engine(**kw)
    for e in (fz, rf, pl):  # each engine its own data (it holds the step)
        assert e.init(NBodyData.plummer(n, seed=13))
        e.set_step(7)

    def close(f, g):
        a, b = f[3 * n:].reshape(3, n).T, g[3 * n:].reshape(3, n).T
        rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
        return np.sqrt(np.mean(rel ** 2)) < 1e-6 and rel.max() < 1e-4

    f0 = _f(fz, y0)
    _, i_build = fz.bh_counters()
    f0p = _f(pl, y0)
    _, i_plain = pl.bh_counters()
    assert i_build == i_plain and close(f0, f0p)
    _f(rf, y0)
    rf.bh_counters()
    f1 = _f(fz, y1)                  # same step: refit, acceptance frozen
    _, i_frozen = fz.bh_counters()
    _f(rf, y1)
    _, i_refit = rf.bh_counters()
    assert i_frozen == i_build
    assert i_refit != i_build
    assert np.all(np.isfinite(f1)) and not np.array_equal(f1, f0)
    rows = np.random.default_rng(2).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y1, d.mass, 1e-3, rows=rows)
    f1p = _f(pl, y1)
    pl.bh_counters()  # reset: the counters add up over calls
    err = [np.quantile(np.linalg.norm(f[3 * n:].reshape(3, n).T[rows] - a_ref, axis=1)
                       / np.linalg.norm(a_ref, axis=1), 0.99) for f in (f1, f1p)]
    assert err[0] < 1.5 * err[1]
    fz.set_step(8)
    f2 = _f(fz, y1)                  # new step: a fresh build
    _, i2 = fz.bh_counters()
    _f(pl, y1)
    _, i2p = pl.bh_counters()
    assert i2 == i2p and close(f2, f1p)


@pytest.mark.parametrize("n", [128, 4096, 1 << 16])
def test_bh_group128_as_accurate_as_group64(make_engine, oracle, n):
    """128-body groups (bh.group = 128) accept a refinement of every body's
    per-body set, like 64-body groups: on the default Hilbert tree the error
    against the FP64 direct sum is at most the 64-body walk's (their larger
    boxes open more cells), and a full tree of one group is a direct sum."""
    d = NBodyData.plummer(n, seed=17)
    y = d.to_state()
    rows = np.arange(n) if n <= 4096 else np.random.default_rng(5).choice(n, 1024, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 1e-3, rows=rows)
    errs = {}
    for g in (64, 128):
        e = make_engine(algo="bh", precision="mixed", softening=1e-3,
                        distance_to_node_radius_ratio=2.0)
        e.tune_set("bh.group", g)
        assert e.init(d)
        f = _f(e, y)
        assert np.array_equal(f[:3 * n], y[3 * n:])
        errs[g] = _rel(f[3 * n:].reshape(3, n).T[rows], a_ref)
    if n == 128:
        assert errs[128].max() < 1e-5
    assert np.quantile(errs[128], 0.99) <= 1.05 * np.quantile(errs[64], 0.99)
    assert np.median(errs[128]) <= 1.05 * np.median(errs[64])
