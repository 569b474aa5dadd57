"""Direct-sum parity on the GPU against the oracle.

* FP64 mode, the reference configuration N = 1024 uniform cube (side 100,
  v ~ N(0, 0.1), m ~ U[0.5, 1.5]/N, G = 1, reference clamp): rk4 with
  dt = 0.01 for 100 steps, state compared with the oracle every step within
  1e-10 relative; P/L/E/V drift of both reported.
* mixed mode (FP32 pairs, compensated sums, FP64 state), Plummer sphere with
  softening 1e-3: RMS relative force error <= 1e-6 against the FP64 oracle.
* ragged sizes (1 .. 1000, not multiples of any tile) for both modes.
* full size N = 131072: sampled rows against the oracle and the momentum
  balance sum_i m_i a_i = 0.
"""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from nbody_gb300.solvers import create_solver

pytestmark = pytest.mark.gpu


def _f_gpu(e, y):
    n6 = y.size
    my, mf = e.create_buffer(8 * n6), e.create_buffer(8 * n6)
    e.write_buffer(my, y)
    e.fill_buffer(mf, 1e10)
    e.fcompute(0.0, my, mf)
    f = np.zeros(n6)
    e.read_buffer(f, mf)
    e.free_buffer(my)
    e.free_buffer(mf)
    return f


def _rel_err(a, a_ref):
    num = np.linalg.norm(a - a_ref, axis=1)
    den = np.linalg.norm(a_ref, axis=1)
    return num / den


def test_config1_fp64_rk4_100_steps(make_engine, oracle):
    n, dt = 1024, 0.01
    d = NBodyData.uniform_cube(n, side=100.0, seed=20240101)
    e = make_engine(precision="fp64")
    assert e.init(d)
    s = create_solver({"solver": "rk4"})
    s.set_time_step(dt, dt)
    s.set_engine(e)
    y_ref = d.to_state()
    t_ref = 0.0
    st0 = oracle.statistics(y_ref, d.mass)
    worst = 0.0
    y = np.zeros(6 * n)
    for step in range(100):
        s.advise(dt)
        y_ref, t_ref, _ = oracle.solver_run("rk4", y_ref, d.mass, t_ref + 0.5 * dt, dt, dt,
                                            t0=t_ref)
        e.read_buffer(y, e.get_y())
        rel = np.max(np.abs(y - y_ref)) / np.max(np.abs(y_ref))
        worst = max(worst, rel)
        assert rel <= 1e-10, f"step {step}: {rel}"
    # P, L, E, V drift over the run: the GPU's own FP64 conservation sums on
    # the GPU state, the oracle's on the reference state
    st_gpu0, st_gpu = None, e.statistics()
    e2 = make_engine(precision="fp64")
    assert e2.init(d)
    st_gpu0 = e2.statistics()
    st_ref = oracle.statistics(y_ref, d.mass)

    def drifts(a, b):
        p = np.linalg.norm(b[0:3] - a[0:3])
        l = np.linalg.norm(b[3:6] - a[3:6]) / np.linalg.norm(a[3:6])
        en = abs((b[6] + b[7] - a[6] - a[7]) / (a[6] + a[7]))
        v = np.linalg.norm(b[8:11] - a[8:11])
        return np.array([p, l, en, v])

    dg, dr = drifts(st_gpu0, st_gpu), drifts(st0, st_ref)
    print(f"\nconfig1: worst per-step rel diff {worst:.3e}; drift P/L/E/V gpu "
          f"{' '.join(f'{x:.3e}' for x in dg)} ref {' '.join(f'{x:.3e}' for x in dr)}")
    assert np.allclose(st_gpu0, st0, rtol=1e-12, atol=1e-12)
    # equal drift: the two runs differ by rounding only
    assert np.allclose(dg, dr, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("sym", [0, 1, 2])
def test_mixed_plummer_force_error(make_engine, oracle, sym):
    """The mixed kernels (0: one-sided, 1: each unordered pair once, with the
    uniform-mass kernel the equal masses select; 2: the same with the
    general, mass-weighted kernel) on every row against the FP64 direct sum."""
    n = 16384
    d = NBodyData.plummer(n, seed=7)
    e = make_engine(precision="mixed", softening=1e-3)
    e.tune_set("direct.symmetric", min(sym, 1))
    if sym == 2:
        e.tune_set("direct.uniform_mass", 0)
    assert e.init(d)
    y = d.to_state()
    f = _f_gpu(e, y)
    a = f[3 * n:].reshape(3, n).T
    a_ref = oracle.accel_rows(y, d.mass, 1e-3)
    rel = _rel_err(a, a_ref)
    rms, p99 = float(np.sqrt(np.mean(rel ** 2))), float(np.quantile(rel, 0.99))
    print(f"\nmixed sym={sym} N={n}: rms {rms:.3e} p99 {p99:.3e} max {rel.max():.3e}")
    assert rms <= 1e-6
    assert np.array_equal(f[:3 * n], y[3 * n:])


@pytest.mark.parametrize("n", [1, 2, 15, 63, 65, 127, 129, 513, 1000, 1025, 2047, 5000])
@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed-onesided", "mixed-g3"])
def test_ragged_sizes(make_engine, oracle, n, prec):
    """Sizes around the tile (128) and range (1024) boundaries; above 1024
    bodies the symmetric kernel has pairs of ranges."""
    d = NBodyData.uniform_cube(n, side=10.0, seed=n)
    e = make_engine(precision=prec.split("-")[0])
    if prec == "mixed-onesided":
        e.tune_set("direct.symmetric", 0)
    if prec == "mixed-g3":  # symmetric kernel with 768-body ranges
        e.tune_set("direct.sym_g", 3)
    assert e.init(d)
    y = d.to_state()
    f = _f_gpu(e, y)
    f_ref = oracle.fcompute_simple(y, d.mass)
    assert np.array_equal(f[:3 * n], f_ref[:3 * n])
    if prec == "fp64":
        assert np.max(np.abs(f - f_ref)) <= 1e-13 * max(1.0, np.max(np.abs(f_ref)))
    elif n > 1:
        rel = _rel_err(f[3 * n:].reshape(3, n).T, f_ref[3 * n:].reshape(3, n).T)
        assert np.sqrt(np.mean(rel ** 2)) < 1e-5
    else:
        assert np.all(f[3:] == 0.0)


@pytest.mark.parametrize("sym", [0, 1, 3])
def test_full_size_sampled_and_momentum(make_engine, oracle, sym):
    n = 131072
    d = NBodyData.plummer(n, seed=11)
    e = make_engine(precision="mixed", softening=1e-3)
    e.tune_set("direct.symmetric", min(sym, 1))
    if sym == 3:
        e.tune_set("direct.sym_g", 3)
    assert e.init(d)
    y = d.to_state()
    f = _f_gpu(e, y)
    a = f[3 * n:].reshape(3, n).T
    rows = np.random.default_rng(3).choice(n, size=256, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, 1e-3, rows=rows)
    rel = _rel_err(a[rows], a_ref)
    rms = float(np.sqrt(np.mean(rel ** 2)))
    print(f"\nmixed sym={sym} N={n} sampled: rms {rms:.3e} p99 {np.quantile(rel, 0.99):.3e}")
    assert rms <= 1e-6
    # Newton's third law: sum m a = 0 up to rounding of the sum of |m a|
    net = np.abs((d.mass[:, None] * a).sum(axis=0))
    scale = (d.mass[:, None] * np.abs(a)).sum(axis=0)
    assert np.all(net <= 1e-5 * scale)


@pytest.mark.parametrize("n,g", [(8192, 4), (5000, 4), (16384, 3), (1000, 3), (1, 4)])
def test_uniform_mass_kernel_equals_general(make_engine, oracle, n, g):
    """Equal masses: the kernel that scales the pair sums by the mass once
    agrees with the mass-weighted kernel (both FP32 pairs, two-sum tiles) to
    FP32 rounding and with the FP64 direct sum, also when the last range is
    padded (n not a multiple of the 256 g-body range: the padding must add
    nothing), and unequal masses never select it."""
    d = NBodyData.plummer(n, seed=21)
    assert np.all(d.mass == d.mass[0])
    out = []
    for uni in (1, 0):
        e = make_engine(precision="mixed", softening=1e-3)
        e.tune_set("direct.uniform_mass", uni)
        e.tune_set("direct.sym_g", g)
        assert e.init(d)
        out.append(_f_gpu(e, d.to_state()))
    if n == 1:
        assert np.all(out[0][3:] == 0.0) and np.all(out[1][3:] == 0.0)
        return
    a_u, a_g = (o[3 * n:].reshape(3, n).T for o in out)
    rel = _rel_err(a_u, a_g)
    assert np.sqrt(np.mean(rel ** 2)) < 5e-7 and rel.max() < 1e-4
    a_ref = oracle.accel_rows(d.to_state(), d.mass, 1e-3)
    assert np.sqrt(np.mean(_rel_err(a_u, a_ref) ** 2)) <= 1e-6
    if n != 8192 or g != 4:
        return
    # a single differing mass switches the specialisation off: same result
    # as the general kernel, bit for bit except for atomic ordering
    d2 = NBodyData.plummer(n, seed=21)
    d2.mass = d2.mass.copy()
    d2.mass[17] *= 1.5
    e1 = make_engine(precision="mixed", softening=1e-3)
    assert e1.init(d2)
    e2 = make_engine(precision="mixed", softening=1e-3)
    e2.tune_set("direct.uniform_mass", 0)
    assert e2.init(d2)
    f1, f2 = _f_gpu(e1, d2.to_state()), _f_gpu(e2, d2.to_state())
    assert np.max(np.abs(f1 - f2)) <= 1e-12 * np.max(np.abs(f2))
