"""The draw hook and deterministic math shared by oracle and engine."""

import math

import numpy as np
from scipy import stats

from oracle import oracle as O


def test_philox_matches_numpy_philox():
    # numpy's Philox increments the counter before each block
    for key, ctr in [((0, 0), (0, 0, 0, 0)), ((0x12345678, 0x9ABCDEF0), (5, 0, 0, 0)), ((2**64 - 1, 3), (2**63, 7, 9, 11))]:
        bg = np.random.Philox(key=np.array(key, dtype=np.uint64), counter=np.array(ctr, dtype=np.uint64))
        want = [int(x) for x in bg.random_raw(4)]
        c = list(ctr)
        c[0] = (c[0] + 1) % 2**64
        assert O.philox(c, key) == want


def test_exp_log_expm1_within_few_ulp():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-700, 700, 3000), rng.uniform(-1, 1, 3000), rng.uniform(-1e-9, 1e-9, 300)])
    for x in xs:
        b = math.exp(x)
        assert abs(O.det_exp(x) - b) <= 2 * np.spacing(b)
    for x in xs[3000:]:
        b = math.expm1(x)
        if b != 0:
            assert abs(O.det_expm1(x) - b) <= 4 * abs(np.spacing(b))
    ys = np.concatenate([np.exp(rng.uniform(-700, 700, 3000)), rng.uniform(0.5, 2, 3000), [5e-324, 1e-310]])
    for y in ys:
        b = math.log(y)
        if b != 0:
            assert abs(O.det_log(y) - b) <= 3 * abs(np.spacing(b))
    for k in [0, 1, 2, 10, 19, 20, 21, 50, 1000, 10**6]:
        assert abs(O.det_lfact(k) - math.lgamma(k + 1)) <= 1e-12 * max(1.0, math.lgamma(k + 1))


def test_poisson_sampler_moments():
    for lam in [0.3, 3.0, 9.9, 10.0, 57.0, 2500.0]:
        x = O.poisson_many(17, lam, 40000)
        assert abs(x.mean() - lam) < 5 * math.sqrt(lam / len(x)) + 1e-9
        assert abs(x.var() / lam - 1) < 0.05
    x = O.poisson_many(5, 4.0, 40000)
    obs = np.bincount(x, minlength=20)[:12]
    exp = stats.poisson.pmf(np.arange(12), 4.0) * len(x)
    assert stats.chisquare(obs, exp * obs.sum() / exp.sum()).pvalue > 1e-4


def test_poisson_inversion_from_mode_and_ptrs_distribution():
    # the three samplers: inversion from 0 (< 10), from the mode (10 - 200), PTRS (>= 200)
    for seed, lam in [(21, 9.5), (22, 10.0), (23, 30.0), (24, 150.7), (25, 199.9), (26, 200.0), (27, 640.0)]:
        x = O.poisson_many(seed, lam, 200000)
        lo, hi = int(lam - 4 * math.sqrt(lam)), int(lam + 4 * math.sqrt(lam)) + 1
        lo = max(lo, 0)
        edges = np.arange(lo, hi + 1)
        obs = np.array([np.count_nonzero(x < lo)] + [np.count_nonzero(x == k) for k in edges[:-1]]
                       + [np.count_nonzero(x >= hi)])
        cdf = stats.poisson.cdf
        exp = np.array([cdf(lo - 1, lam)] + list(stats.poisson.pmf(edges[:-1], lam)) + [1 - cdf(hi - 1, lam)])
        exp = exp * len(x)
        keep = exp > 5
        assert stats.chisquare(obs[keep], exp[keep] * obs[keep].sum() / exp[keep].sum()).pvalue > 1e-4, lam
        assert abs(x.mean() - lam) < 5 * math.sqrt(lam / len(x))


def test_gamma_and_negbinom_moments():
    for a in [0.5, 1.0, 4.0, 1000.0]:
        g = O.gamma_many(3, a, 40000)
        assert abs(g.mean() - a) < 5 * math.sqrt(a / len(g))
    r, p = 5.0, 0.3
    nb = O.negbinom_many(9, r, p, 40000)
    mean = r * (1 - p) / p
    assert abs(nb.mean() - mean) < 5 * math.sqrt(r * (1 - p) / p**2 / len(nb))


def test_distribution_kinds():
    n = 20000
    assert np.all(O.dist_many(1, 0, 7.0, 0.0, 10) == 7.0)
    e = O.dist_many(1, 1, 2.0, 0.0, n)
    assert abs(e.mean() - 2.0) < 0.1
    ln = O.dist_many(1, 3, 12.5, 3.5, n)
    assert abs(ln.mean() - 12.5) < 0.2 and abs(ln.std() - 3.5) < 0.2
    u = O.dist_many(1, 6, 2.0, 10.0, n)
    assert u.min() == 2 and u.max() == 9 and np.all(u == np.floor(u))


def test_km_newborn_lifespans_follow_table():
    cum = np.array([100, 150, 180, 200, 1000])
    days = np.array([O.km_newborn(cum, 100, 7, 3, s) for s in range(20000)])
    years = days // 365
    freq = np.bincount(years, minlength=5) / len(years)
    want = np.diff(np.concatenate([[0], cum])) / cum[-1]
    assert np.allclose(freq, want, atol=0.02)


def test_fix_risk_integer_and_single_forms_equal_double_definition():
    from oracle.oracle import fix_risk_many

    rng = np.random.default_rng(3)
    bits = rng.integers(0, 2**32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    r = bits.view(np.float32)
    special = np.array([0.0, -0.0, 1.0, 0.5, 1.5, 2.5, 2**-24, 1.5 * 2**-24, 2**-25, 3 * 2**-25, 2**-126,
                        np.inf, -np.inf, np.nan, 2.0**38, 2.0**39, 3.4e38, 1e-45, 0.999999940395,
                        1.00000011920929], dtype=np.float32)
    # every float whose product with 2^24 lies near a half-integer
    m = np.arange(1, 1 << 12, dtype=np.float64)
    halves = ((m + 0.5) / 2.0**24).astype(np.float32)
    r = np.concatenate([r, special, halves, np.nextafter(halves, np.float32(1)), np.nextafter(halves, np.float32(0))])
    a, b, c = fix_risk_many(r)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
