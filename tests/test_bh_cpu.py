"""CPU checks of the curve-order restatement the GPU tree build is tested
against (tests/curve_order.py)."""
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
