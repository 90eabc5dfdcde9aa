"""The radiation network (core.radiation, native lpg_radiation_network)
against its Python definition, bit for bit, on the CPU."""

import numpy as np
import pytest

from laser_polio_gb300.core import _radiation_py
from laser_polio_gb300.core import radiation


@pytest.mark.parametrize("n,seed,ties", [(1, 0, False), (2, 1, False), (37, 2, False), (120, 3, True), (300, 4, False)])
def test_native_radiation_equals_the_python_definition(n, seed, ties):
    rng = np.random.default_rng(seed)
    pops = rng.lognormal(np.log(5e4), 0.8, n)
    if ties:  # equal distances and equal populations: the stable order decides
        xy = rng.integers(0, 5, (n, 2)).astype(np.float64)
        pops[: n // 2] = 1000.0
    else:
        xy = rng.uniform(0, 500, (n, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    for k, home in ((1.0, False), (0.3, True)):
        np.testing.assert_array_equal(radiation(pops, dist, k, include_home=home),
                                      _radiation_py(pops, dist, k, include_home=home))


def test_radiation_rejects_bad_shapes():
    with pytest.raises(ValueError, match="shape"):
        radiation(np.ones(3), np.zeros((2, 2)), 1.0)
    with pytest.raises(ValueError, match="NaN"):
        radiation(np.ones(2), np.array([[0.0, np.nan], [1.0, 0.0]]), 1.0)


def test_gravity_and_row_normalizer_on_the_references_example():
    """scripts/sandbox/debug_row_normalizer.py:7-32: three nodes (populations
    99510, 595855, 263884 scaled by 1e-3; distances 4, 66, 827), k = 100,
    a = b = 1, c = 2: gravity is k p_i p_j / d_ij^2 off the diagonal (the
    script's own comment), and rows summing above 0.3 are scaled to 0.3, as
    the script's manual restatement does.  Expected values computed here
    element by element."""
    from laser_polio_gb300.core import gravity, row_normalizer

    pops = np.array([99510, 595855, 263884]) / 1e3
    dist = np.array([[0, 4, 66], [4, 0, 827], [66, 827, 0]])
    want = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            if i != j:
                want[i, j] = 100 * pops[i] * pops[j] / float(dist[i, j]) ** 2
    got = gravity(pops, dist, 100, 1, 1, 2.0)
    np.testing.assert_allclose(got, want, rtol=1e-15)
    norm = row_normalizer(got, 0.3)
    for i in range(3):
        s = want[i].sum()
        np.testing.assert_allclose(norm[i], want[i] * (0.3 / s) if s > 0.3 else want[i], rtol=1e-15)
    # the script's integer network, promoted to float as its fix does
    net = row_normalizer(np.array([[0, 6, 2], [10, 0, 13], [15, 10, 0]], dtype=float), 0.3)
    np.testing.assert_allclose(net.sum(axis=1), [0.3, 0.3, 0.3], rtol=1e-15)
