"""Batched ensemble: per-system forces against the oracle, one fixed-step
rkdp step against the oracle's restatement of the reference Butcher driver,
graph replay equal to direct launches, and adaptive runs that conserve
energy."""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from nbody_gb300.ensemble import Ensemble

pytestmark = pytest.mark.gpu

SIZES = [1, 33, 64, 100, 257, 1000, 4096]


def _systems(sizes, seed=0, kind="plummer"):
    out = []
    for i, n in enumerate(sizes):
        if kind == "plummer" and n > 1:
            out.append(NBodyData.plummer(n, seed=seed + i))
        else:
            out.append(NBodyData.uniform_cube(n, side=2.0, seed=seed + i))
    return out


@pytest.mark.parametrize("eps", [1e-3, 0.0])
def test_ensemble_forces_vs_oracle(gpulib, oracle, eps):
    sy = _systems(SIZES, seed=3)
    ens = Ensemble(softening=eps)
    ens.init(sy)
    f = ens.fcompute()
    B = sum(SIZES)
    a = f[3 * B:].reshape(3, B).T
    off = 0
    for d in sy:
        n = d.get_count()
        ref = oracle.accel_rows(d.to_state(), d.mass, eps)
        got = a[off:off + n]
        assert np.array_equal(f[off:off + n], d.velocities[:, 0])
        if n > 1:
            rel = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
            assert np.sqrt(np.mean(rel ** 2)) < 1e-5, (n, rel.max())
        else:
            assert np.all(got == 0.0)
        off += n
    ens.close()


@pytest.mark.parametrize("sizes", [[64, 200, 1000], [3000]], ids=["three", "one"])
def test_fixed_step_matches_oracle_rkdp(gpulib, oracle, sizes):
    """dt_min = dt_max: every attempt is accepted with y += dt sum b2 k; the
    oracle's rkdp with max_recursion 0 does the same step (reference clamp,
    no softening).  One system is the engine-owned fused RK step: the whole
    Dormand-Prince step of a single system on the device, one graph."""
    dt = 1e-3
    sy = _systems(sizes, seed=5)
    ens = Ensemble(softening=0.0, tolerance=1e-30, dt_initial=dt, dt_min=dt, dt_max=dt)
    ens.init(sy)
    ens.step(1)
    v, u = ens.get_state()
    off = 0
    for d in sy:
        n = d.get_count()
        yref, _, _ = oracle.solver_run("rkdp", d.to_state(), d.mass, 0.5 * dt, dt, dt,
                                       max_recursion=0)
        pos = yref[:3 * n].reshape(3, n).T
        vel = yref[3 * n:].reshape(3, n).T
        # FP32 pair math: the step's change agrees to ~1e-5 of its size
        dv = np.max(np.abs(vel - d.velocities))
        dx = np.max(np.abs(pos - d.vertices))
        assert np.max(np.abs(u[off:off + n] - vel)) <= 2e-4 * dv
        assert np.max(np.abs(v[off:off + n] - pos)) <= 2e-4 * dx
        off += n
    t, dts, acc, rej = ens.status()
    assert np.all(acc == 1) and np.all(rej == 0) and np.allclose(t, dt)
    ens.close()


def test_graph_equals_direct_launches(gpulib):
    sy = _systems([64, 300, 1500], seed=8)
    res = []
    for use_graph in (True, False):
        ens = Ensemble(tolerance=1e-8, use_graph=use_graph)
        ens.init(sy)
        ens.step(5)
        res.append(ens.get_state())
        res.append(ens.status())
        ens.close()
    assert np.array_equal(res[0][0], res[2][0]) and np.array_equal(res[0][1], res[2][1])
    for a, b in zip(res[1], res[3]):
        assert np.array_equal(a, b)


def test_adaptive_energy_drift(gpulib, oracle):
    rng = np.random.default_rng(2)
    sizes = rng.integers(64, 2049, size=24).tolist()
    sy = _systems(sizes, seed=11)
    ens = Ensemble(tolerance=1e-8)
    ens.init(sy)
    st0 = ens.statistics()
    ens.step(20)
    st1 = ens.statistics()
    t, dt, acc, rej = ens.status()
    e0, e1 = st0[:, 6] + st0[:, 7], st1[:, 6] + st1[:, 7]
    drift = np.abs((e1 - e0) / e0)
    print(f"\nensemble: accepted {acc.sum()} rejected {rej.sum()} max drift {drift.max():.2e} "
          f"median t {np.median(t):.3f}")
    assert np.all(acc + rej == 20)
    assert np.all(acc > 0)
    assert drift.max() < 1e-5
    ens.close()


def test_step_control_variants(gpulib):
    """The three step controllers on the same systems: without the hold
    after a rejection, with it (the default), and PI control; each keeps the
    energy drift small and PI control rejects fewer steps."""
    rng = np.random.default_rng(5)
    sizes = rng.integers(64, 1025, size=32).tolist()
    sy = _systems(sizes, seed=13)
    res = {}
    for name, hold, pi in (("free", 0, 0), ("hold", 1, 0), ("pi", 1, 1)):
        ens = Ensemble(tolerance=1e-8)
        ens.tune_set("ensemble.hold_after_reject", hold)
        ens.tune_set("ensemble.pi_control", pi)
        ens.init(sy)
        st0 = ens.statistics()
        ens.step(30)
        st1 = ens.statistics()
        t, dt, acc, rej = ens.status()
        e0, e1 = st0[:, 6] + st0[:, 7], st1[:, 6] + st1[:, 7]
        res[name] = (acc.sum(), rej.sum(), float(np.abs((e1 - e0) / e0).max()), float(t.sum()))
        ens.close()
    print("\n" + "; ".join(f"{k}: accepted {a} rejected {r} drift {d:.1e} sum t {tt:.3f}"
                           for k, (a, r, d, tt) in res.items()))
    for a, r, d, _ in res.values():
        assert a + r == 30 * 32 and d < 1e-5
    assert res["pi"][1] < res["hold"][1]


def test_ensemble_statistics_unsoftened_match_oracle(gpulib, oracle):
    sy = _systems([64, 500, 1200], seed=13)
    ens = Ensemble(softening=0.0)
    ens.init(sy)
    st = ens.statistics()
    for k, d in enumerate(sy):
        ref = oracle.statistics(d.to_state(), d.mass)
        assert np.allclose(st[k], ref, rtol=1e-10, atol=1e-13)
    ens.close()


@pytest.mark.parametrize("kind,eps", [("plummer", 1e-3), ("cube", 1e-3), ("plummer", 0.0)],
                         ids=["equal-mass", "unequal-mass", "clamp"])
@pytest.mark.parametrize("g", [1, 2])
def test_symmetric_kernel_matches_one_sided(gpulib, oracle, g, kind, eps):
    """The symmetric kernel (every unordered pair of a system once; the B
    sums through per-range FP32 partials and a fixed-order FP64 reduce)
    against the one-sided kernel on the same systems, sizes around the
    256 G-body ranges: FP32 rounding apart, both within the oracle's bound,
    and two evaluations equal bit for bit."""
    sizes = [1, 33, 255, 256, 257, 513, 700, 4096]
    sy = _systems(sizes, seed=12, kind=kind)
    out = {}
    for sym in (1, 0):
        ens = Ensemble(softening=eps)
        ens.tune_set("ensemble.symmetric", sym)
        ens.tune_set("ensemble.pairs_per_lane", g)
        ens.init(sy)
        out[sym] = ens.fcompute()
        if sym:
            assert np.array_equal(out[sym], ens.fcompute())
        ens.close()
    B = sum(sizes)
    assert np.array_equal(out[1][:3 * B], out[0][:3 * B])
    a_s, a_o = (out[k][3 * B:].reshape(3, B).T for k in (1, 0))
    off = 0
    for d in sy:
        n = d.get_count()
        if n == 1:
            assert np.all(a_s[off] == 0.0)
        else:
            ref = oracle.accel_rows(d.to_state(), d.mass, eps)
            nr = np.linalg.norm(ref, axis=1)
            rel_so = np.linalg.norm(a_s[off:off + n] - a_o[off:off + n], axis=1) / nr
            rel_s = np.linalg.norm(a_s[off:off + n] - ref, axis=1) / nr
            print(f"n={n} g={g} {kind} eps={eps}: sym vs one-sided rms {np.sqrt(np.mean(rel_so ** 2)):.2e}, "
                  f"sym vs oracle rms {np.sqrt(np.mean(rel_s ** 2)):.2e}")
            assert np.sqrt(np.mean(rel_so ** 2)) < 1e-6
            assert np.sqrt(np.mean(rel_s ** 2)) < 1e-5
        off += n


def test_ensemble_uniform_mass_kernel(gpulib, oracle):
    """Equal masses in every system select the kernel that scales each
    system's sums by its mass once; it agrees with the mass-weighted kernel to
    FP32 rounding.  One system with unequal masses keeps the general kernel
    for all (results against the oracle)."""
    sizes = [64, 300, 1000, 2048]
    sy = _systems(sizes, seed=9)
    out = []
    for uni in (1, 0):
        ens = Ensemble(softening=1e-3)
        ens.tune_set("ensemble.uniform_mass", uni)
        ens.init(sy)
        out.append(ens.fcompute())
        ens.close()
    B = sum(sizes)
    a_u, a_g = (o[3 * B:].reshape(3, B).T for o in out)
    rel = np.linalg.norm(a_u - a_g, axis=1) / np.linalg.norm(a_g, axis=1)
    assert np.sqrt(np.mean(rel ** 2)) < 5e-7 and rel.max() < 1e-4
    mixed = sy[:2] + _systems([500], seed=4, kind="cube")
    ens = Ensemble(softening=1e-3)
    ens.init(mixed)
    f = ens.fcompute()
    ens.close()
    Bm = sum(d.get_count() for d in mixed)
    a = f[3 * Bm:].reshape(3, Bm).T
    off = 0
    for d in mixed:
        n = d.get_count()
        ref = oracle.accel_rows(d.to_state(), d.mass, 1e-3)
        r = np.linalg.norm(a[off:off + n] - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert np.sqrt(np.mean(r ** 2)) < 1e-5
        off += n
