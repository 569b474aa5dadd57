"""The autotuner: cache logic on the CPU (a stand-in engine records what is
applied), and on the GPU the native search through the C ABI: every
candidate timed, the fastest kept, results unchanged in accuracy."""
import json

import numpy as np
import pytest

from nbody_gb300.autotune import TuneCache, cache_key, size_bucket, tune
from nbody_gb300.data import NBodyData


class _FakeEngine:
    device = 0

    def __init__(self, n):
        self.n = n
        self.applied = {}
        self.timed = 0

    def problem_size(self):
        return 6 * self.n

    def tune_variant(self):
        return "direct/mixed/soft"

    def tune_set(self, k, v):
        self.applied[k] = v

    def autotune(self, reps):
        self.timed += 1
        best = {"direct.symmetric": 1, "direct.blocks_per_sm": 3}
        self.applied.update(best)
        return {"scope": "direct", "n": self.n, "reps": reps,
                "candidates": [{"keys": best, "ms": 1.0}], "best": best}


def _ident(_device):
    return ("Test GPU", 152)


def test_size_bucket_and_key():
    assert [size_bucket(n) for n in (0, 1, 2, 3, 1000, 1024, 1025)] == [1, 1, 2, 4, 1024, 1024, 2048]
    assert cache_key("G", 152, "direct/mixed/soft", 131072) == "G|152|direct/mixed/soft|131072"


def test_cache_roundtrip_and_hit(tmp_path):
    path = tmp_path / "tune.json"
    e = _FakeEngine(100000)
    r1 = tune(e, cache=TuneCache(path), identity=_ident)
    assert r1["source"] == "measured" and e.timed == 1
    stored = json.loads(path.read_text())
    assert r1["key"] in stored and stored[r1["key"]]["best"] == r1["best"]
    # a new engine of a size in the same bucket gets the stored winners untimed
    e2 = _FakeEngine(120000)
    r2 = tune(e2, cache=TuneCache(path), identity=_ident)
    assert r2["source"] == "cache" and e2.timed == 0 and e2.applied == r1["best"]
    # force re-measures; another size bucket misses
    assert tune(e2, cache=TuneCache(path), identity=_ident, force=True)["source"] == "measured"
    e3 = _FakeEngine(300000)
    assert tune(e3, cache=TuneCache(path), identity=_ident)["source"] == "measured"
    assert len(TuneCache(path)) == 2


def test_corrupt_cache_is_ignored(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    assert len(TuneCache(path)) == 0
    assert tune(_FakeEngine(10), cache=TuneCache(path), identity=_ident)["source"] == "measured"


@pytest.mark.gpu
def test_engine_autotune_direct(make_engine, oracle, tmp_path):
    n = 16384
    d = NBodyData.plummer(n, seed=21)
    e = make_engine(precision="mixed", softening=1e-3)
    assert e.init(d)
    res = tune(e, reps=2, cache=TuneCache(tmp_path / "t.json"))
    rep = res["report"]
    ms = [c["ms"] for c in rep["candidates"]]
    print("\n" + json.dumps(rep))
    assert len(ms) >= 6 and all(np.isfinite(ms)) and min(ms) > 0
    best = rep["candidates"][int(np.argmin(ms))]["keys"]
    assert rep["best"] == best
    assert all(e.tune_get(k) == v for k, v in best.items())
    # the tuned engine still computes the same forces
    y = d.to_state()
    f = e.create_buffer(8 * 6 * n)
    e.fcompute(0.0, e.get_y(), f)
    out = np.zeros(6 * n)
    e.read_buffer(out, f)
    rows = np.arange(0, n, 64)
    a_ref = oracle.accel_rows(y, d.mass, 1e-3, rows=rows)
    a = out[3 * n:].reshape(3, n).T[rows]
    rel = np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    assert np.sqrt(np.mean(rel ** 2)) <= 1e-6


@pytest.mark.gpu
def test_engine_autotune_bh(make_engine):
    d = NBodyData.plummer(1 << 14, seed=22)
    e = make_engine(algo="bh", precision="mixed", softening=1e-3, distance_to_node_radius_ratio=2.0)
    assert e.init(d)
    rep = e.autotune(2)
    keys = [c["keys"] for c in rep["candidates"]]
    g64 = {"bh.walk": 1, "bh.group": 64}
    assert keys[:2] == [dict(g64, **{"bh.walk_blocks": b, "bh.acc_smem": 1}) for b in (5, 4)]
    assert keys[2:4] == [dict(g64, **{"bh.walk_blocks": 5, "bh.acc_smem": 1, "bh.eval_unroll": u})
                         for u in (1, 4)]
    assert keys[4:6] == [dict(g64, **{"bh.walk_blocks": b, "bh.acc_smem": 0}) for b in (4, 5)]
    assert keys[6:8] == [dict(g64, **{"bh.walk_blocks": 4, "bh.acc_smem": 0, "bh.eval_unroll": u})
                         for u in (1, 4)]
    assert keys[8:] == [{"bh.walk": 1, "bh.group": 32, "bh.walk_blocks": b} for b in (6, 8)] + \
        [{"bh.walk": 1, "bh.group": 128}, {"bh.walk": 0}]
    assert e.tune_get("bh.walk") == rep["best"]["bh.walk"]


@pytest.mark.gpu
def test_engine_autotune_bh_quadrupole(make_engine):
    """With quadrupole cells only the group walks, which add the term, are
    candidates; every candidate gives forces of the same accuracy."""
    d = NBodyData.plummer(1 << 14, seed=22)
    e = make_engine(algo="bh", precision="mixed", softening=1e-3, distance_to_node_radius_ratio=2.0)
    e.tune_set("bh.order", 2)
    assert e.init(d)
    y = e.get_y()
    f = e.create_buffer(8 * 6 * (1 << 14))
    e.fcompute(0.0, y, f)
    f0 = np.zeros(6 * (1 << 14))
    e.read_buffer(f0, f)
    rep = e.autotune(2)
    keys = [c["keys"] for c in rep["candidates"]]
    assert keys == [{"bh.walk": 1, "bh.group": 64, "bh.walk_blocks": b} for b in (3, 4)] + \
        [{"bh.walk": 1, "bh.group": 32}]
    e.fcompute(0.0, y, f)
    f1 = np.zeros(6 * (1 << 14))
    e.read_buffer(f1, f)
    if rep["best"]["bh.group"] == 64:  # same walk, another register budget: the same sums
        assert np.array_equal(f0, f1)
    else:
        n = 1 << 14
        a0, a1 = f0[3 * n:].reshape(3, n).T, f1[3 * n:].reshape(3, n).T
        rel = np.linalg.norm(a1 - a0, axis=1) / np.linalg.norm(a0, axis=1)
        assert np.median(rel) < 1e-2


@pytest.mark.gpu
def test_ensemble_autotune_keeps_results():
    from nbody_gb300.ensemble import Ensemble
    rng = np.random.default_rng(3)
    systems = [NBodyData.plummer(int(k), seed=100 + i) for i, k in enumerate(rng.integers(64, 600, 40))]
    ens = Ensemble(softening=1e-3, tolerance=1e-8)
    ens.init(systems)
    f0 = ens.fcompute()
    rep = ens.autotune(2)
    keys = [c["keys"] for c in rep["candidates"]]
    assert len(keys) == 12 and rep["best"] in keys
    # the symmetric kernel (G = 1, 2) first, then the one-sided shapes
    assert [k["ensemble.symmetric"] for k in keys] == [1, 1] + [0] * 10
    f1 = ens.fcompute()
    # another tile shape sums in another order: FP32 rounding only
    scale = np.abs(f0).max()
    assert np.max(np.abs(f1 - f0)) <= 1e-5 * scale
    ens.step(3)  # the step graph is captured again for the new shape
    ens.synchronize()
    t, dt, acc, rej = ens.status()
    assert np.all(acc + rej == 3) and np.all(np.isfinite(t))
    ens.close()
