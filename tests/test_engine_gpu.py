"""The reference's engine battery (test/engine/test_nbody_engine.cpp:10-1010)
run on the GB300 engine through the C ABI, FP64 and mixed modes.

Same data (make_universe with box 100, N = 128 / 1024), same operations,
same tolerances: machine epsilon for the integer-valued buffer algebra,
1e-13 absolute for FP64 fcompute against the 'simple' engine (here the oracle
restatement of it), poison fill of f with +-1e10 before each fcompute.
"""
import numpy as np
import pytest

from nbody_gb300.data import NBodyData

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps
MODES = [dict(precision="fp64"), dict(precision="mixed")]


@pytest.fixture(params=MODES, ids=["fp64", "mixed"])
def eng(request, make_engine):
    e = make_engine(**request.param)
    d = NBodyData.make_universe(64)
    assert e.init(d)
    e._data_obj = d
    return e


def _rand(rng, n):
    return rng.integers(0, 10000, size=n).astype(np.float64)


def test_mem(eng):
    m = eng.create_buffer(1024)
    assert m is not None
    eng.free_buffer(m)


def test_memcpy(eng):
    data = np.arange(8, dtype=np.float64)
    x = np.zeros(8)
    mem = eng.create_buffer(64)
    sub = eng.create_buffer(32)
    eng.write_buffer(mem, data)
    eng.read_buffer(x, mem)
    assert np.array_equal(data, x)
    eng.free_buffer(mem)
    eng.free_buffer(sub)


def test_copy_buffer(eng):
    n = eng.problem_size()
    d1 = np.arange(n, dtype=np.float64)
    d2 = np.zeros(n)
    m1, m2 = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    eng.write_buffer(m1, d1)
    eng.copy_buffer(m2, m1)
    eng.read_buffer(d2, m2)
    assert np.array_equal(d1, d2)


def test_fill_buffer(eng):
    m = eng.create_buffer(33 * 8)
    eng.fill_buffer(m, 777.0)
    out = np.zeros(33)
    eng.read_buffer(out, m)
    assert np.all(np.abs(out - 777.0) <= np.finfo(np.float64).tiny)


def test_fmadd_inplace(eng):
    rng = np.random.default_rng(1)
    n = eng.problem_size()
    a, b = _rand(rng, n), _rand(rng, n)
    ma, mb = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    eng.write_buffer(ma, a)
    eng.write_buffer(mb, b)
    eng.fmadd_inplace(ma, mb, 5.0)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    assert np.all(np.abs((a + 5.0 * b) - res) <= EPS)


def test_fmadd(eng):
    rng = np.random.default_rng(2)
    n = eng.problem_size()
    a, b, c = _rand(rng, n), _rand(rng, n), _rand(rng, n)
    ma, mb, mc = (eng.create_buffer(8 * n) for _ in range(3))
    for m, v in ((ma, a), (mb, b), (mc, c)):
        eng.write_buffer(m, v)
    eng.fmadd(ma, mb, mc, 5.0)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    assert np.all(np.abs((b + c * 5.0) - res) <= EPS)


# 35 terms: the stage count of the reference's rkfeagin14 table
@pytest.mark.parametrize("csize", [1, 3, 7, 20, 35])
def test_fmaddn_inplace(eng, csize):
    rng = np.random.default_rng(3 + csize)
    n = eng.problem_size()
    a = _rand(rng, n)
    b = _rand(rng, n * csize).reshape(csize, n)
    c = _rand(rng, csize)
    if csize > 1:
        c[0] = 0.0
        c[csize // 2] = 0.0
    ma = eng.create_buffer(8 * n)
    mb = eng.create_buffers(8 * n, csize)
    eng.write_buffer(ma, a)
    for k in range(csize):
        eng.write_buffer(mb[k], b[k].copy())
    eng.fmaddn_inplace(ma, mb, c, csize)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    assert np.all(np.abs((a + (b * c[:, None]).sum(axis=0)) - res) <= EPS)


@pytest.mark.parametrize("dsize", [1, 3, 7, 20, 35])
@pytest.mark.parametrize("null_b", [False, True])
def test_fmaddn(eng, dsize, null_b):
    rng = np.random.default_rng(11 + dsize)
    n = eng.problem_size()
    a, b = _rand(rng, n), _rand(rng, n)
    c = _rand(rng, n * dsize).reshape(dsize, n)
    d = _rand(rng, dsize)
    if dsize > 1:
        d[0] = 0.0
        d[dsize // 2] = 0.0
    ma, mb = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    mc = eng.create_buffers(8 * n, dsize)
    eng.write_buffer(ma, a)
    eng.write_buffer(mb, b)
    for k in range(dsize):
        eng.write_buffer(mc[k], c[k].copy())
    eng.fmaddn(ma, None if null_b else mb, mc, d, dsize)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    s = (c * d[:, None]).sum(axis=0)
    expect = s if null_b else b + s
    assert np.all(np.abs(expect - res) <= EPS)


def test_fmaddn_all_zero_keeps_a(eng):
    # b given and every coefficient zero: a is left untouched (nbody_engine.cpp:97-112)
    n = eng.problem_size()
    ma, mb = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    eng.fill_buffer(ma, 3.0)
    eng.fill_buffer(mb, 7.0)
    mc = eng.create_buffers(8 * n, 2)
    eng.fmaddn(ma, mb, mc, [0.0, 0.0], 2)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    assert np.all(res == 3.0)


def test_fmaddn_corr(eng):
    n = eng.problem_size()
    csize = 10
    factor = EPS / 2.0
    ma, mcorr = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    mb = eng.create_buffers(8 * n, csize)
    eng.write_buffer(ma, np.ones(n))
    eng.fill_buffer(mcorr, 0.0)
    for m in mb:
        eng.write_buffer(m, np.ones(n))
    eng.fmaddn_corr(ma, mcorr, mb, [factor] * csize, csize)
    res = np.zeros(n)
    eng.read_buffer(res, ma)
    assert np.all(np.abs((1.0 + csize * factor) - res) <= EPS)


def test_fmaxabs(eng):
    rng = np.random.default_rng(5)
    n = eng.problem_size()
    a = rng.integers(0, 10000, size=n).astype(np.float64) - 9000
    ma = eng.create_buffer(8 * n)
    eng.write_buffer(ma, a)
    assert abs(eng.fmaxabs(ma) - np.max(np.abs(a))) <= EPS
    empty = eng.create_buffer(0)
    assert eng.fmaxabs(empty) == 0.0


def _fcompute(eng, y, poison):
    n = eng.problem_size()
    my, mf = eng.create_buffer(8 * n), eng.create_buffer(8 * n)
    eng.write_buffer(my, y)
    eng.fill_buffer(mf, poison)
    eng.fcompute(0.0, my, mf)
    f = np.zeros(n)
    eng.read_buffer(f, mf)
    eng.free_buffer(my)
    eng.free_buffer(mf)
    return f


def test_fcompute_vs_simple(eng, oracle):
    d = eng._data_obj
    y = d.to_state()
    for step in range(2):  # test_fcompute's two passes with y *= 1.99 between
        f_ref = oracle.fcompute_simple(y, d.mass)
        eng.set_step(step)
        f = _fcompute(eng, y, -1e10)
        n = d.get_count()
        assert np.array_equal(f[:3 * n], f_ref[:3 * n])  # velocity copy is exact
        if eng._params.precision == 0:
            assert np.max(np.abs(f - f_ref)) <= 1e-13
        else:
            a, ar = f[3 * n:], f_ref[3 * n:]
            rel = np.abs(a - ar).reshape(3, n).T
            rel = np.linalg.norm(rel, axis=1) / np.linalg.norm(ar.reshape(3, n).T, axis=1)
            assert np.sqrt(np.mean(rel ** 2)) < 1e-5
        y = y + y * 0.99


def test_clamp(eng):
    n = eng.problem_size()
    a = np.where(np.arange(n) & 1, 4.0, -4.0)
    m = eng.create_buffer(8 * n)
    eng.write_buffer(m, a)
    eng.clamp(m, 1.0)
    b = np.zeros(n)
    eng.read_buffer(b, m)
    half = n // 2
    assert np.all(b[:half] == np.where(np.arange(half) & 1, 2.0, -2.0))
    assert np.all(b[half:] == a[half:])


class _Fake:
    """A memory object that is not the engine's (nbody_engine_memory_fake)."""

    def size(self):
        return 0


def test_negative_branches(eng):
    """test_nbody_engine.cpp:761-1010: every call with a foreign or NULL
    argument returns without effect and without crashing."""
    ps = eng.problem_size()
    fake = _Fake()
    real = eng.create_buffer(ps)
    arr = eng.create_buffers(ps, 1)
    eng.fcompute(0, fake, real)
    eng.fcompute(0, real, fake)
    eng.read_buffer(None, fake)
    eng.write_buffer(fake, None)
    eng.copy_buffer(fake, real)
    eng.copy_buffer(real, fake)
    eng.fmadd_inplace(fake, real, 1)
    eng.fmadd_inplace(real, fake, 1)
    eng.fmadd(fake, real, real, 0)
    eng.fmadd(real, real, fake, 0)
    eng.fmadd(real, fake, real, 0)
    eng.fmaddn_inplace(fake, arr, [0.0], 1)
    eng.fmaddn_inplace(real, arr, None, 1)
    eng.fmaddn_inplace(real, [fake], [0.0], 1)
    eng.fmaddn_inplace(real, arr, [0.0], 100)
    eng.fmaddn_inplace(real, [None], [1.0], 1)
    eng.fmaddn_corr(None, real, arr, [0.0], 1)
    eng.fmaddn_corr(real, None, arr, [0.0], 1)
    eng.fmaddn_corr(real, real, [None], [0.0], 1)
    eng.fmaddn_corr(real, real, arr, None, 1)
    eng.fmaddn_corr(real, real, arr, [0.0], 100)
    eng.fmaddn_corr(real, real, [None], [1.0], 1)
    eng.fmaddn(fake, real, arr, [0.0], 200000)
    eng.fmaddn(fake, real, arr, [0.0], 1)
    eng.fmaddn(fake, None, arr, [0.0], 1)
    eng.fmaddn(real, real, arr, None, 1)
    eng.fmaddn(real, None, arr, None, 1)
    eng.fmaddn(real, real, [fake], [0.0], 1)
    eng.fmaddn(real, None, [fake], [0.0], 1)
    eng.fmaddn(real, fake, arr, [0.0], 1)
    eng.fmaddn(real, real, [None], [1.0], 1)
    assert eng.fmaxabs(fake) == 0.0
    # a buffer of another engine is foreign too
    eng.synchronize()


def test_foreign_engine_buffer_rejected_by_library(make_engine, gpulib):
    import ctypes as C
    e1 = make_engine(precision="fp64")
    e2 = make_engine(precision="fp64")
    d = NBodyData.make_universe(64)
    assert e1.init(d) and e2.init(d)
    m2 = e2.create_buffer(8 * e2.problem_size())
    # straight through the C ABI: engine 1 must refuse engine 2's handle
    st = gpulib.nbg_fill_buffer(e1.handle, m2.handle, 1.0)
    assert st == 2
    assert b"not gb300 memory" in gpulib.nbg_last_error(e1.handle)
    st = gpulib.nbg_fcompute(e1.handle, 0.0, 0, e1.get_y().handle, m2.handle)
    assert st == 2


def test_invalid_device_rejected(gpulib):
    from nbody_gb300.engine import create_engine
    for dev in ("-1", "9999"):
        assert create_engine({"engine": "gb300", "device": dev}) is None


def test_init_rejects_empty_and_bh_ragged(make_engine):
    """No bodies is an error (status, message, no state); Barnes-Hut needs a
    power-of-two body count (the heap's leaves are [N, 2N))."""
    e = make_engine(precision="fp64")
    assert not e.init(NBodyData())
    assert e.last_status == 1  # NBG_ERR_INVALID_ARG
    b = make_engine(algo="bh", precision="mixed", softening=1e-3)
    assert not b.init(NBodyData.plummer(1000, seed=1))
    assert b.last_status == 6  # NBG_ERR_UNSUPPORTED
    assert b.init(NBodyData.plummer(1024, seed=1))
