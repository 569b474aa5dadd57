"""CPU restatement of the mixed path's space-filling-curve leaf order
(nbody_gb300/csrc/nbg_tree.cu: bbox_kernel, morton_keys_kernel, hilbert_key,
radix_sort from its third pass): the test checks the GPU build against it
leaf for leaf.  The Hilbert index follows J. Skilling, "Programming the
Hilbert curve", AIP Conf. Proc. 707 (2004): axes to the transposed index,
Gray decoding, then the bits interleaved from the most significant, axis 0
first."""
import numpy as np

BITS = 21
QMAX = float((1 << BITS) - 1)


def quantize(pos: np.ndarray) -> np.ndarray:
    """(n, 3) FP64 positions -> (3, n) uint64 cells of the 2^21-per-axis grid
    over the bounding box, by the kernel's FP64 operations."""
    lo = pos.min(axis=0)
    ext = pos.max(axis=0) - lo
    scale = np.where(ext > 0, QMAX / np.where(ext > 0, ext, 1.0), 0.0)
    v = (pos - lo) * scale
    return np.minimum(np.maximum(v, 0.0), QMAX).astype(np.uint64).T.copy()


def _spread3(v: np.ndarray) -> np.ndarray:
    out = np.zeros_like(v)
    for j in range(BITS):
        out |= ((v >> np.uint64(j)) & np.uint64(1)) << np.uint64(3 * j)
    return out


def hilbert_keys(q: np.ndarray) -> np.ndarray:
    X = [q[0].copy(), q[1].copy(), q[2].copy()]
    Q = 1 << (BITS - 1)
    while Q > 1:
        P = np.uint64(Q - 1)
        Qu = np.uint64(Q)
        for i in range(3):
            has = (X[i] & Qu) != 0
            t = (X[0] ^ X[i]) & P
            X0 = np.where(has, X[0] ^ P, X[0] ^ t)
            if i != 0:
                X[i] = np.where(has, X[i], X[i] ^ t)
            X[0] = X0
        Q >>= 1
    X[1] ^= X[0]
    X[2] ^= X[1]
    t = np.zeros_like(X[0])
    Q = 1 << (BITS - 1)
    while Q > 1:
        t = np.where((X[2] & np.uint64(Q)) != 0, t ^ np.uint64(Q - 1), t)
        Q >>= 1
    X = [x ^ t for x in X]
    return (_spread3(X[0]) << np.uint64(2)) | (_spread3(X[1]) << np.uint64(1)) | _spread3(X[2])


def morton_keys(q: np.ndarray) -> np.ndarray:
    return _spread3(q[0]) | (_spread3(q[1]) << np.uint64(1)) | (_spread3(q[2]) << np.uint64(2))


def leaf_order(pos: np.ndarray, hilbert: bool) -> np.ndarray:
    """Bodies in leaf order: a stable sort by the key bits from 16 up."""
    q = quantize(pos)
    keys = hilbert_keys(q) if hilbert else morton_keys(q)
    return np.argsort(keys >> np.uint64(16), kind="stable")


def _self_check(b: int = 4) -> None:
    """The curve property on a 2^b grid: the keys are a bijection and cells
    with consecutive keys are face neighbours."""
    global BITS
    saved, BITS = BITS, b
    try:
        g = np.arange(1 << b, dtype=np.uint64)
        x, y, z = np.meshgrid(g, g, g, indexing="ij")
        q = np.stack([x.ravel(), y.ravel(), z.ravel()])
        keys = hilbert_keys(q)
        assert np.array_equal(np.sort(keys), np.arange(1 << (3 * b), dtype=np.uint64))
        order = np.argsort(keys)
        steps = np.abs(np.diff(q[:, order].astype(np.int64), axis=1)).sum(axis=0)
        assert np.all(steps == 1)
    finally:
        BITS = saved
