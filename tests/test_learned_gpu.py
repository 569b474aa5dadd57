"""The learned monopole correction: sample generation, BF16 tensor-core
training kernels (gradients against an FP64 restatement), the inference
routine against the FP64 forward pass, and the measured change of the force
error that the trained network brings over plain Barnes-Hut at theta = 0.9."""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

EPS = 1e-3


def _bh_engine(make_engine, lam, learned=False, tight=2.0):
    return make_engine(algo="bh", precision="mixed", softening=EPS,
                       distance_to_node_radius_ratio=lam, learned=learned,
                       learned_tight_ratio=tight)


def test_param_count(gpulib):
    assert gpulib.nbg_learn_param_count() == M.N_PARAMS == 5443


def test_gradient_matches_fp64_restatement(make_engine):
    """Forward/backward of the training kernels vs FP64 numpy on the same
    (BF16-representable) weights and inputs."""
    e = _bh_engine(make_engine, 1.0 / 0.9)
    d = NBodyData.plummer(1024, seed=2)
    assert e.init(d)
    rng = np.random.default_rng(3)
    w = M.bf16(rng.normal(0, 0.3, size=M.N_PARAMS)).astype(np.float32)
    e.learn_set_weights(w)
    x = M.bf16(rng.normal(0, 1.0, size=(96, 16))).astype(np.float32)
    t = np.zeros((96, 4), dtype=np.float32)
    t[:, :3] = rng.normal(0, 0.5, size=(96, 3))
    loss_gpu, g_gpu = e.learn_loss_grad(x, t)
    loss_ref, g_ref = M.loss_grad(w, x, t)
    assert abs(loss_gpu - loss_ref) <= 2e-2 * loss_ref
    # BF16 activations between layers: compare the gradient as a vector
    err = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    cos = g_gpu @ g_ref / (np.linalg.norm(g_gpu) * np.linalg.norm(g_ref))
    print(f"\ngrad check: rel err {err:.3e}, cosine {cos:.6f}, loss {loss_gpu:.4e} vs {loss_ref:.4e}")
    assert err < 3e-2 and cos > 0.999
    # every parameter block carries gradient
    for a, b in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
                 (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.N_PARAMS)):
        blk = np.linalg.norm(g_gpu[a:b] - g_ref[a:b]) / np.linalg.norm(g_ref[a:b])
        assert blk < 5e-2, (a, b, blk)


def _subtree(leaves, n, node):
    k = n.bit_length() - 1
    lv = node.bit_length() - 1
    span = 1 << (k - lv)
    first = (node << (k - lv)) - n
    return leaves[first:first + span]


def test_samples_match_cpu_recomputation(make_engine):
    """Targets and features of generated samples recomputed on the CPU from
    the tree's leaf order: exact subtree sum minus monopole, scaled s^2/m."""
    n = 4096
    lam = 1.0 / 0.9
    d = NBodyData.plummer(n, seed=6)
    e = _bh_engine(make_engine, lam)
    assert e.init(d)
    got = e.learn_generate(20000, seed=2)
    assert got > 1000
    leaves = e.tree_leaves()
    assert sorted(leaves.tolist()) == list(range(n))
    x, t, meta = e.learn_read_samples(0, got)
    pos, mass = d.vertices, d.mass
    rng = np.random.default_rng(0)
    for k in rng.choice(got, size=60, replace=False):
        b, node = int(meta[k, 0]), int(meta[k, 1])
        bodies = _subtree(leaves, n, node)
        assert b not in set(bodies.tolist())
        m = mass[bodies].sum()
        com = (pos[bodies] * mass[bodies, None]).sum(axis=0) / m
        bmin, bmax = pos[bodies].min(axis=0), pos[bodies].max(axis=0)
        s = np.linalg.norm(bmax - bmin) * 0.5 + np.linalg.norm((bmax + bmin) / 2 - com)
        dr = pos[bodies] - pos[b]
        r2 = (dr * dr).sum(axis=1) + EPS * EPS
        exact = (dr * (mass[bodies] / (r2 * np.sqrt(r2)))[:, None]).sum(axis=0)
        dc = com - pos[b]
        rc2 = dc @ dc + EPS * EPS
        mono = dc * m / (rc2 * np.sqrt(rc2))
        target = (exact - mono) * s * s / m
        scale = max(np.abs(target).max(), 1e-3)
        assert np.allclose(t[k, :3], target, atol=2e-4 * scale + 1e-6), (k, t[k, :3], target)
        u = (pos[b] - com) / s
        assert np.allclose(x[k, :3], u, rtol=1e-4, atol=1e-4)
        q = np.einsum("k,ka,kb->ab", mass[bodies], pos[bodies] - com, pos[bodies] - com) / (m * s * s)
        qv = [q[0, 0], q[1, 1], q[2, 2], q[0, 1], q[0, 2], q[1, 2]]
        assert np.allclose(x[k, 3:9], qv, rtol=1e-3, atol=1e-5)
        assert np.allclose(x[k, 9:12], (bmax - bmin) / (2 * s), rtol=1e-4, atol=1e-5)
        assert np.isclose(x[k, 12], 1 / np.linalg.norm(u), rtol=1e-4)
        assert np.allclose(x[k, 13:16], (com - (bmax + bmin) / 2) / s, rtol=1e-3, atol=1e-5)
        # inside the band: accepted at lam, opened at the tight ratio 2
        dist = np.linalg.norm(dc)
        assert lam * s < dist * (1 + 1e-4) and dist <= 2.0 * s * (1 + 1e-4)


def _trained_weights(make_engine, epochs=8):
    """About 6e6 samples from Plummer and uniform-cube snapshots of 2^14 to
    2^18 bodies (the generalisation needs many snapshots and sizes)."""
    e = _bh_engine(make_engine, 1.0 / 0.9)
    total = 0
    sizes = [(1 << k, kind) for k in (14, 16, 18) for kind in ("plummer", "cube")]
    for i, (n, kind) in enumerate(sizes):
        d = NBodyData.plummer(n, seed=10 + i) if kind == "plummer" else \
            NBodyData.uniform_cube(n, side=2.0, seed=10 + i)
        assert e.init(d)
        total += e.learn_generate(1_000_000, seed=20 + i)
    x, t, _ = e.learn_read_samples(0, min(total, 200000))
    var0 = float((t[:, :3].astype(np.float64) ** 2).mean())
    tr, va = e.learn_train(epochs, batch=8192, lr=3e-3, seed=5)
    print(f"\nsamples {total}, target mean square {var0:.3e}, train MSE {tr:.3e}, val MSE {va:.3e}")
    return e.learn_get_weights(), var0, tr, va


@pytest.fixture(scope="module")
def trained(request):
    from nbody_gb300.engine import create_engine
    made = []

    def mk(**param):
        param.setdefault("engine", "gb300")
        eng = create_engine(param)
        made.append(eng)
        return eng
    res = _trained_weights(mk)
    for eng in made:
        eng.close()
    return res


def test_samples_and_training_repeat_bit_for_bit(make_engine):
    """Sample generation (pairs compacted in sampled-leaf order) and training
    (per-warp gradient sums added in warp and block order, no atomics) give
    the same samples and the same weights on every run with the same seeds."""
    runs = []
    for _ in range(2):
        e = _bh_engine(make_engine, 1.0 / 0.9)
        total = 0
        for i, kind in enumerate(("plummer", "cube")):
            d = NBodyData.plummer(1 << 14, seed=60 + i) if kind == "plummer" else \
                NBodyData.uniform_cube(1 << 14, side=2.0, seed=60 + i)
            assert e.init(d)
            total += e.learn_generate(200_000, seed=70 + i)
        x, t, meta = e.learn_read_samples(0, total)
        tr, va = e.learn_train(2, batch=4096, lr=3e-3, seed=9)
        runs.append((total, x, t, meta, tr, va, e.learn_get_weights()))
    (n0, x0, t0, m0, tr0, va0, w0), (n1, x1, t1, m1, tr1, va1, w1) = runs
    assert n0 == n1 and n0 > 10_000
    assert np.array_equal(m0, m1) and np.array_equal(x0, x1) and np.array_equal(t0, t1)
    assert tr0 == tr1 and va0 == va1
    assert np.array_equal(w0, w1)


def test_training_fits_the_residual(trained):
    w, var0, tr, va = trained
    assert np.all(np.isfinite(w))
    # An FP32 fit of the same network plateaus near 70 % explained mean
    # square on these features (the residual at 1.1 < d/s <= 2 is dominated
    # by multipoles above the quadrupole); require at least 55 %.
    assert va < 0.45 * var0


def test_inference_path_matches_fp64_forward(make_engine, trained):
    """The walk's tensor-core inference routine against the FP64 forward pass
    on the same weights."""
    w = trained[0]
    e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
    d = NBodyData.plummer(1024, seed=1)
    assert e.init(d)
    e.learn_set_weights(w)
    rng = np.random.default_rng(8)
    x = rng.normal(0, 0.7, size=(1000, 16)).astype(np.float32)
    x[:, 12] = np.abs(x[:, 12])
    got = e.learn_predict(x)
    ref = M.forward(M.bf16(w), M.bf16(x))
    assert np.linalg.norm(got - ref) <= 3e-2 * np.linalg.norm(ref)


# ---------------------------------------------------------------------------
# inference on the tcgen05 tensor cores ("learned.walk" = 1, the default)
# ---------------------------------------------------------------------------
def _random_weights(seed, scale=0.3):
    return np.random.default_rng(seed).normal(0, scale, M.N_PARAMS).astype(np.float32)


def _features(count, seed):
    x = np.random.default_rng(seed).normal(0, 0.7, size=(count, 16)).astype(np.float32)
    x[:, 12] = np.abs(x[:, 12])
    return x


def test_tensor_core_layouts(make_engine):
    """The tcgen05 operand, instruction-descriptor and tensor-memory layouts,
    layer by layer, on random weights with nonzero biases: the accumulators
    D1 = X W1 + b1, D2 = GELU(D1) W2 + b2 and D3 = GELU(D2) W3 + b3
    (columns past 3 zero; each bias enters as three BF16 terms through a
    K = 16 MMA against a block of ones, exact to FP32).  D1 is a sum of 16
    exact BF16 products and the bias in FP32; the next layers are checked
    from the GPU's own previous accumulators (whose GELU rounds to BF16 the
    same way)."""
    e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
    assert e.init(NBodyData.plummer(1024, seed=1))
    w = _random_weights(3)
    e.learn_set_weights(w)
    W1, _, W2, _, W3, _ = M.unpack(M.bf16(w))
    b1, b2, b3 = M.unpack(w)[1], M.unpack(w)[3], M.unpack(w)[5]  # biases stay FP32
    for count in (1, 200, 4096):
        x = _features(count, 11 + count)
        acc = e.learn_tc_accumulators(x).astype(np.float64)
        d1, d2, d3 = acc[:, 0:64], acc[:, 64:128], acc[:, 128:144]
        xb = M.bf16(x)
        err1 = np.abs(d1 - (xb @ W1 + b1)) / (np.abs(xb) @ np.abs(W1) + np.abs(b1) + 1e-30)
        z2 = M.bf16(M.gelu(d1)) @ W2 + b2
        err2 = np.linalg.norm(d2 - z2) / np.linalg.norm(z2)
        z3 = M.bf16(M.gelu(d2)) @ W3 + b3
        err3 = np.linalg.norm(d3[:, :3] - z3) / np.linalg.norm(z3)
        print(f"\ncount {count}: D1 max err / bound {err1.max():.2e}, D2 rel err {err2:.2e}, "
              f"D3 rel err {err3:.2e}")
        assert err1.max() < 1e-5
        assert err2 < 1e-2
        assert err3 < 1e-2
        assert np.all(d3[:, 3:] == 0.0)


@pytest.mark.parametrize("count", [1, 127, 128, 1000, 70001])
def test_tensor_core_inference_matches_mma_sync(make_engine, count):
    """The tcgen05 inference against the walk's mma.sync routine and the FP64
    forward pass on the same BF16 weights and inputs, for counts that are
    and are not multiples of the 128-row tile.  Both round the activations
    to BF16; their FP32 sums run in different orders, so an activation can
    round to the neighbouring BF16 value."""
    e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
    assert e.init(NBodyData.plummer(1024, seed=1))
    w = _random_weights(4)
    e.learn_set_weights(w)
    x = _features(count, 5 + count)
    tc = e.learn_predict_tc(x).astype(np.float64)
    ms = e.learn_predict(x).astype(np.float64)
    ref = M.forward(M.bf16(w), M.bf16(x))
    assert np.all(np.isfinite(tc))
    d_ms = np.linalg.norm(tc - ms) / np.linalg.norm(ms)
    d_ref = np.linalg.norm(tc - ref) / np.linalg.norm(ref)
    print(f"\ncount {count}: |tc - mma.sync| / |mma.sync| {d_ms:.2e}, "
          f"|tc - fp64| / |fp64| {d_ref:.2e}")
    assert d_ms < 1e-2
    assert d_ref < 3e-2


@pytest.mark.parametrize("n", [64, 128, 1 << 15])
def test_tensor_core_walk_with_zero_network_is_the_group_walk(make_engine, n):
    """Zero weights make every correction exactly zero, so the tensor-core
    learned walk equals the plain group walk at the loose ratio on the same
    tree (FP64 nodes) bit for bit -- with the group walk's band-cell records
    in place, and with every group handed to the per-body learned walk
    (bh.test_cap = 1); one group (N = 64), two, and many."""
    d = NBodyData.plummer(n, seed=41)
    for cap in (0, 1):
        plain = _bh_engine(make_engine, 1.0 / 0.9)
        plain.tune_set("bh.fp64_nodes", 1)
        plain.tune_set("bh.test_cap", cap)
        assert plain.init(d)
        f_plain = _forces(plain, n)
        e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
        e.tune_set("learned.judge", 0)
        e.tune_set("bh.test_cap", cap)
        assert e.init(d)
        e.learn_set_weights(np.zeros(M.N_PARAMS, dtype=np.float32))
        f = _forces(e, n)
        rows = e.learn_band_rows()
        print(f"\nn {n} test_cap {cap}: band rows per body {rows / n:.1f}")
        assert rows > 0 or n < 1024
        assert np.array_equal(f, f_plain)


@pytest.mark.parametrize("tune", [{"bh.group": 32}, {"bh.order": 2},
                                  {"bh.freeze_within_step": 1}],
                         ids=["group32", "quadrupole", "frozen"])
def test_other_walk_settings_take_the_per_body_learned_walk(make_engine, tune):
    """The tensor-core path needs the default group walk; with other walk
    settings the learned engine takes the per-body (warp-coherent) learned
    walk, the same forces as learned.walk = 0 bit for bit."""
    n = 1 << 13
    d = NBodyData.plummer(n, seed=43)
    w = _random_weights(6, scale=0.05)
    out = []
    for walk in (1, 0):
        e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
        e.tune_set("learned.judge", 0)
        e.tune_set("learned.walk", walk)
        for k, v in tune.items():
            e.tune_set(k, v)
        assert e.init(d)
        e.learn_set_weights(w)
        out.append(_forces(e, n))
    assert np.all(np.isfinite(out[0]))
    assert np.array_equal(out[0], out[1])


def test_tensor_core_walk_vs_plain(make_engine, oracle, trained):
    """The trained network on the tensor-core group walk at theta = 0.9,
    judged by the FP64 direct sum on a snapshot the network never saw: a
    lower p99 than the plain group walk at theta = 0.9 on the same tree and
    a median no higher; equal inputs give equal forces (the per-body sums run
    in a fixed order).  Training is not bitwise repeatable (atomic gradient
    sums): over runs the p99 falls 29 - 37 % and the median moves by -10 to
    +1 % (the group walk's refined cells leave the median little to gain)."""
    w = trained[0]
    n = 1 << 15
    d = NBodyData.plummer(n, seed=77)
    y = d.to_state()
    rows = np.random.default_rng(4).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, EPS, rows=rows)

    def rel(out):
        a = out[3 * n:].reshape(3, n).T[rows]
        return np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)

    plain = _bh_engine(make_engine, 1.0 / 0.9)
    plain.tune_set("bh.fp64_nodes", 1)
    assert plain.init(d)
    r_plain = rel(_forces(plain, n))
    e = _bh_engine(make_engine, 1.0 / 0.9, learned=True)
    e.tune_set("learned.judge", 0)
    assert e.init(d)
    e.learn_set_weights(w)
    f1 = _forces(e, n)
    f2 = _forces(e, n)
    assert np.all(np.isfinite(f1))
    assert np.array_equal(f1, f2)
    assert np.array_equal(f1[:3 * n], y[3 * n:])
    r = rel(f1)
    q = lambda v: f"p50 {np.median(v):.3e} p99 {np.quantile(v, 0.99):.3e}"
    print(f"\ngroup walk theta0.9: plain {q(r_plain)} | learned (tcgen05) {q(r)}")
    assert np.quantile(r, 0.99) < 0.85 * np.quantile(r_plain, 0.99)
    assert np.median(r) < 1.05 * np.median(r_plain)


@pytest.mark.parametrize("group", [0, 1])
def test_learned_walk_vs_plain(make_engine, oracle, trained, group):
    """What the trained network changes in the force at theta = 0.9, judged by
    the FP64 direct sum on a snapshot the network never saw, with theta = 0.5
    beside it.  Per-body inference (group 0) must lower the median and p99
    errors of plain theta = 0.9; the warp-centroid mode (group 1) is recorded.
    Both: finite forces, velocity rows copied exactly, and the learned walk
    visiting the same nodes as the plain walk at the same ratio."""
    w = trained[0]
    n = 1 << 15
    d = NBodyData.plummer(n, seed=77)
    y = d.to_state()
    rows = np.random.default_rng(4).choice(n, size=512, replace=False)
    a_ref = oracle.accel_rows(y, d.mass, EPS, rows=rows)

    def run(lam, learned):
        e = _bh_engine(make_engine, lam, learned=learned)
        e.tune_set("bh.walk", 0)  # the walk the learned path extends,
        e.tune_set("bh.fp64_nodes", 1)  # with the FP64 node update it uses
        assert e.init(d)
        if learned:
            e.learn_set_weights(w)
            e.tune_set("learned.group", group)
            e.tune_set("learned.judge", 0)  # the learned walk itself, never the fallback
        f = e.create_buffer(8 * 6 * n)
        e.fcompute(0.0, e.get_y(), f)
        out = np.zeros(6 * n)
        e.read_buffer(out, f)
        assert np.all(np.isfinite(out))
        assert np.array_equal(out[:3 * n], y[3 * n:])
        a = out[3 * n:].reshape(3, n).T[rows]
        return np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1), e.bh_counters()

    (plain09, c0), (learn09, c1), (plain05, _) = run(1 / 0.9, False), run(1 / 0.9, True), run(2.0, False)
    q = lambda r: f"p50 {np.median(r):.3e} p99 {np.quantile(r, 0.99):.3e}"
    print(f"\ngroup={group}: plain theta0.9 {q(plain09)} | learned theta0.9 {q(learn09)} | "
          f"plain theta0.5 {q(plain05)}")
    assert c0 == c1  # same walk: the correction adds work, never changes the visit sequence
    if group == 0:
        # training is not bitwise repeatable (atomic gradient sums): over runs
        # the median falls 13-23 % and the p99 4-17 %
        assert np.median(learn09) < 0.95 * np.median(plain09)
        assert np.quantile(learn09, 0.99) < np.quantile(plain09, 0.99)
    else:
        assert np.median(learn09) < 10 * np.median(plain09)


# ---------------------------------------------------------------------------
# the per-step judge and the plain fallback
# ---------------------------------------------------------------------------
def _splitmix64(x):
    m = (1 << 64) - 1
    x = (x + 0x9E3779B97F4A7C15) & m
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
    return x ^ (x >> 31)


def _judge_leaves(n, step, samples=4096, seed=1):
    """The judge's sampled leaves: S = samples rounded down to a power of two
    (at most n), leaf k (n / S) + off, off from (seed, step)."""
    s = 1
    while 2 * s <= min(samples, n, 4096):
        s *= 2
    stride = n // s
    off = _splitmix64(((seed * 0x100000001B3) & ((1 << 64) - 1)) ^ step) % stride
    return np.arange(s) * stride + off


def _forces(e, n):
    f = e.create_buffer(8 * 6 * n)
    e.fcompute(0.0, e.get_y(), f)
    out = np.zeros(6 * n)
    e.read_buffer(out, f)
    e.free_buffer(f)
    return out


def test_judge_trips_on_bad_weights_and_falls_back_bit_for_bit(make_engine):
    """All-ones weights make the correction nonsense: the judge sees a learned
    p99 above the plain theta = 0.5 walk's, and the fcompute -- and every
    further fcompute of the same step -- equals the engine's plain theta = 0.5
    path bit for bit (the same Hilbert tree with FP64 nodes, the same group
    walk).  The next step is judged again."""
    n = 1 << 15
    d = NBodyData.plummer(n, seed=31)
    plain = _bh_engine(make_engine, 2.0)
    plain.tune_set("bh.fp64_nodes", 1)
    assert plain.init(d)
    f_plain = _forces(plain, n)

    e = _bh_engine(make_engine, 1.0 / 0.9, learned=True, tight=2.0)
    assert e.init(d)
    e.learn_set_weights(np.ones(e.learn_param_count(), dtype=np.float32))
    assert e.learn_judge_stats()["judged_steps"] == 0
    f1 = _forces(e, n)
    st = e.learn_judge_stats()
    print(f"\nbad weights: {st}")
    assert st["judged_steps"] == 1 and st["fallback_steps"] == 1 and st["used_plain"]
    assert st["samples"] == 4096 and st["step"] == 0
    assert not (st["p99_learned"] <= st["p99_plain"])  # larger, or not finite
    assert 0.0 < st["p99_plain"] < 0.1
    assert np.array_equal(f1, f_plain)
    f2 = _forces(e, n)  # same step: plain again, not judged again
    assert np.array_equal(f2, f_plain)
    assert e.learn_judge_stats()["judged_steps"] == 1
    e.set_step(1)
    f3 = _forces(e, n)
    st = e.learn_judge_stats()
    assert st["judged_steps"] == 2 and st["fallback_steps"] == 2 and st["step"] == 1
    assert np.array_equal(f3, f_plain)


def test_judge_figures_and_decision(make_engine, oracle):
    """With a correction that changes nothing (zero weights) the learned walk
    is the group walk at the loose ratio.  The judge's learned p50
    and p99 equal a host recomputation on the same sampled bodies (the
    learned walk's forces against the FP64 direct sum); its plain figures
    equal the per-body walk at the tight ratio (the group walk forced to its
    per-body fallback for every group) on the same bodies; and the output is
    the learned walk's when the learned p99 is the smaller, the plain
    path's otherwise."""
    n = 1 << 14
    lam_l, lam_t = 1.6, 2.0
    d = NBodyData.plummer(n, seed=32)
    y = d.to_state()
    w = np.zeros(M.N_PARAMS, dtype=np.float32)

    raw = _bh_engine(make_engine, lam_l, learned=True, tight=lam_t)
    raw.tune_set("learned.judge", 0)
    assert raw.init(d)
    raw.learn_set_weights(w)
    f_learned = _forces(raw, n)
    leaves = raw.tree_leaves()

    e = _bh_engine(make_engine, lam_l, learned=True, tight=lam_t)
    assert e.init(d)
    e.learn_set_weights(w)
    out = _forces(e, n)
    st = e.learn_judge_stats()
    print(f"\nzero weights: {st}")

    bodies = leaves[_judge_leaves(n, 0)]
    a_ref = oracle.accel_rows(y, d.mass, EPS, rows=bodies)

    def rel(f):
        a = f[3 * n:].reshape(3, n).T[bodies]
        return np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    r_l = rel(f_learned)
    assert st["samples"] == bodies.size
    assert np.isclose(st["p50_learned"], np.quantile(r_l, 0.5), rtol=2e-3)
    assert np.isclose(st["p99_learned"], np.quantile(r_l, 0.99), rtol=2e-3)
    assert np.isclose(st["rms_learned"], np.sqrt(np.mean(r_l ** 2)), rtol=2e-3)

    body = _bh_engine(make_engine, lam_t)
    body.tune_set("bh.fp64_nodes", 1)
    body.tune_set("bh.test_cap", 1)  # every group handed to the per-body walk
    assert body.init(d)
    r_p = rel(_forces(body, n))
    assert np.isclose(st["p50_plain"], np.quantile(r_p, 0.5), rtol=1e-2)
    assert np.isclose(st["p99_plain"], np.quantile(r_p, 0.99), rtol=1e-2)

    assert st["used_plain"] == (st["p99_learned"] > st["p99_plain"])
    if st["used_plain"]:
        plain = _bh_engine(make_engine, lam_t)
        plain.tune_set("bh.fp64_nodes", 1)
        assert plain.init(d)
        assert np.array_equal(out, _forces(plain, n))
    else:
        assert np.array_equal(out, f_learned)
