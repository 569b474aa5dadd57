"""CPU checks of the curve-order restatement the GPU tree build is tested
against (tests/curve_order.py), and of the quadrupole term the mixed walks
evaluate."""
import numpy as np

from tests import curve_order as C


def test_hilbert_keys_are_a_curve():
    """On a 16^3 grid the keys are a bijection onto [0, 4096) and cells with
    consecutive keys are face neighbours: the Hilbert curve's defining
    property, which the Morton order lacks."""
    C._self_check(4)


def test_morton_keys_interleave():
    q = np.array([[1], [0], [0]], dtype=np.uint64)
    assert C.morton_keys(q)[0] == 1
    q = np.array([[0], [1], [0]], dtype=np.uint64)
    assert C.morton_keys(q)[0] == 2
    q = np.array([[0], [0], [1]], dtype=np.uint64)
    assert C.morton_keys(q)[0] == 4
    q = np.array([[(1 << 21) - 1]] * 3, dtype=np.uint64)
    assert C.morton_keys(q)[0] == (1 << 63) - 1


def test_quantize_spans_the_grid():
    rng = np.random.default_rng(1)
    pos = rng.normal(size=(1000, 3))
    q = C.quantize(pos)
    assert q.min(axis=1).tolist() == [0, 0, 0]
    assert all(v >= (1 << 21) - 2 for v in q.max(axis=1).tolist())  # FP64 rounding of the top
    order = C.leaf_order(pos, hilbert=True)
    assert sorted(order.tolist()) == list(range(1000))


def _quad_term(d, m, S):
    """The walk's monopole + quadrupole term of a cell (nbg_bh.cu, quad_pair)
    with the stored moments S = -3 M: a = d (m / r^3 + k / r^5) + S d / r^5,
    k = tr S / 2 - 2.5 d.S.d / r^2, d = cell mass centre - body."""
    r2 = d @ d
    inv5 = r2 ** -2.5
    k = 0.5 * np.trace(S) - 2.5 * (d @ S @ d) / r2
    return d * (m * r2 ** -1.5 + k * inv5) + (S @ d) * inv5


def test_quadrupole_term_converges_at_third_order():
    """Against the exact sum over a small cluster, the monopole error falls as
    (s/d)^2 and the walk's quadrupole term's as (s/d)^3 with the distance d."""
    rng = np.random.default_rng(5)
    pts = rng.normal(scale=0.3, size=(40, 3)) * np.array([1.0, 0.6, 0.3])
    w = rng.uniform(0.5, 1.5, 40)
    m = w.sum()
    c = (w[:, None] * pts).sum(0) / m
    off = pts - c
    M = (w[:, None, None] * off[:, :, None] * off[:, None, :]).sum(0)
    direction = np.array([0.48, 0.6, 0.64])
    err_mono, err_quad = [], []
    for dist in (4.0, 8.0, 16.0):
        x = c - dist * direction  # the body
        diff = pts - x
        exact = (w[:, None] * diff / (np.linalg.norm(diff, axis=1) ** 3)[:, None]).sum(0)
        d = c - x
        mono = m * d / np.linalg.norm(d) ** 3
        quad = _quad_term(d, m, -3.0 * M)
        err_mono.append(np.linalg.norm(mono - exact) / np.linalg.norm(exact))
        err_quad.append(np.linalg.norm(quad - exact) / np.linalg.norm(exact))
    for k in range(2):
        assert 3.0 < err_mono[k] / err_mono[k + 1] < 5.5   # ~ 2^2 per doubling
        assert 6.0 < err_quad[k] / err_quad[k + 1] < 11.0  # ~ 2^3 per doubling
    assert err_quad[-1] < 0.1 * err_mono[-1]
