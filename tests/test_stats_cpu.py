"""CPU model of the FP64 1/sqrt(x) refinement in the potential-energy sums
(nbody_gb300/csrc/nbg_stats.cu, rsqrt_fp64): an FP32 estimate y0, then
y = y0 + y0 e (1/2 + 3e/8) with e = 1 - x y0^2, the second-order step of the
series (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 + ...  The GPU kernel's sums are
checked against the oracle by tests/test_stats_gpu.py; this pins the step's
accuracy for estimates as far off as the hardware's, and the kernel's tile
schedule (each unordered pair once) for every block count."""
import numpy as np
import pytest


def _refine(x, y0):
    e = 1.0 - (x * y0) * y0
    return y0 * e * (e * 0.375 + 0.5) + y0


def test_second_order_step_is_within_a_few_ulp():
    if np.finfo(np.longdouble).nmant < 60:
        pytest.skip("needs an extended long double to judge FP64 results")
    rng = np.random.default_rng(11)
    x = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 100_000))
    y0 = (1.0 / np.sqrt(x.astype(np.float32))).astype(np.float64)
    y0 *= 1.0 + rng.uniform(-1.0, 1.0, x.size) * 2.0 ** -21  # worst FP32 estimate
    y = _refine(x, y0)
    exact = 1.0 / np.sqrt(x.astype(np.longdouble))
    rel = np.abs((y.astype(np.longdouble) - exact) / exact).astype(np.float64)
    assert rel.max() < 4 * 2.0 ** -53


def test_one_newton_step_would_not_be():
    """The plain Newton step y0 (3 - x y0^2) / 2 leaves an error of order e^2,
    far above FP64 rounding: the second-order term is needed."""
    if np.finfo(np.longdouble).nmant < 60:
        pytest.skip("needs an extended long double to judge FP64 results")
    x = np.array([2.0, 3.0, 7.0])
    y0 = (1.0 / np.sqrt(x)) * (1.0 + 2.0 ** -21)
    newton = y0 * (1.5 - 0.5 * x * y0 * y0)
    exact = 1.0 / np.sqrt(x.astype(np.longdouble))
    rel = np.abs((newton.astype(np.longdouble) - exact) / exact).astype(np.float64)
    assert rel.min() > 1e3 * 2.0 ** -53


@pytest.mark.parametrize("nb", list(range(1, 18)) + [32, 33, 512])
def test_cyclic_tile_schedule_counts_each_pair_once(nb):
    """The potential kernel's schedule (stats_potential_kernel): block b takes
    tiles (b + t) mod nb for t = 0 .. last, last = nb/2 - 1 for the upper half
    of an even nb and nb/2 otherwise; its own tile counts both orders of each
    pair (weight 1), the others one order (weight 2).  Every unordered tile
    pair must then carry weight 2 in total, and the blocks' loads differ by at
    most one tile."""
    weight = np.zeros((nb, nb))
    loads = []
    for b in range(nb):
        last = nb // 2 - 1 if (nb % 2 == 0 and b >= nb // 2) else nb // 2
        loads.append(last + 1)
        for t in range(last + 1):
            j = (b + t) % nb
            if t == 0:
                weight[b, b] += 2  # both orders of each pair inside the tile
            else:
                weight[min(b, j), max(b, j)] += 2
    assert np.all(weight[np.triu_indices(nb)] == 2)
    assert max(loads) - min(loads) <= 1
