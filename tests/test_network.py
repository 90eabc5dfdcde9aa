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
    for k in (1.0, 0.3):
        np.testing.assert_array_equal(radiation(pops, dist, k), _radiation_py(pops, dist, k))


def test_radiation_ties_do_not_depend_on_node_order():
    """Nodes at equal distances (duplicate coordinates, and a node on top of
    i): s_ij counts only the strictly closer ones, so relabelling the nodes
    permutes the network and changes no value; checked against a direct sum
    of the definition."""
    rng = np.random.default_rng(7)
    n = 40
    xy = rng.integers(0, 4, (n, 2)).astype(np.float64)  # many duplicate coordinates
    pops = rng.lognormal(np.log(2e4), 0.6, n)
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    net = radiation(pops, dist, 1.0)
    for i in range(n):
        for j in range(n):
            if i == j:
                assert net[i, j] == 0.0
                continue
            inside = [m for m in range(n) if m not in (i, j) and dist[i, m] < dist[i, j]]
            s = float(np.sum(pops[inside])) if inside else 0.0
            want = pops[i] * pops[j] / ((pops[i] + s) * (pops[i] + pops[j] + s))
            assert abs(net[i, j] - want) <= 1e-12 * want, (i, j)
    perm = rng.permutation(n)
    net_p = radiation(pops[perm], dist[np.ix_(perm, perm)], 1.0)
    np.testing.assert_allclose(net_p, net[np.ix_(perm, perm)], rtol=1e-12, atol=0)


def test_radiation_rejects_include_home():
    with pytest.raises(ValueError, match="include_home"):
        radiation(np.ones(3), np.ones((3, 3)) - np.eye(3), 1.0, include_home=True)
    with pytest.raises(ValueError, match="include_home"):
        _radiation_py(np.ones(3), np.ones((3, 3)) - np.eye(3), 1.0, include_home=True)


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
