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
