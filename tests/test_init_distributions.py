"""The initialisation against the reference's own, in distribution.

tests/golden/reference_init.npz holds statistics of 16 runs (seeds 1..16)
of the reference's unmodified initialisation: SEIR_ABM(pars) and the five
component constructors (model.py:101-175, 561-713, 816-866, 1548-1611,
1887-1894), imported by tests/golden/make_reference_fixtures.py --init, on
14 nodes of about 1500 agents with every initialisation parameter in play
(per-node immunity, initial infections as counts and as a fraction, a
missed fraction, the default timer distributions, correlated heterogeneity,
the reference's age pyramid, births).

This package fills the same table on the device (init.fill ->
lpg_init_columns) with its own draws; on a machine without a GPU the oracle's
restatement, which makes the same draws, stands in (tests/conftest.py).  For
16 seeds of its own:
  - exactly equal: the capacity, the number of missed agents, the infected
    per node, the alive per node, and the defaults of the other columns;
  - the recovered per node (the immune less those then infected): mean over
    the runs within 5 standard errors of the reference's;
  - the histograms of the three timers (every slot), of the ages in years,
    of the ages at death and of the RI day offsets: chi-square homogeneity,
    each at alpha 1e-3 / 6;
  - risk and infectivity: two-sample Kolmogorov-Smirnov on 32000 pairs each,
    alpha 1e-3, and their Spearman correlation within 0.03.
The GPU test also requires the device's table to equal the oracle's bit for
bit.
"""

import sys
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

import laser_polio_gb300 as lp
from laser_polio_gb300.core import PropertySet

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import replay_cases  # noqa: E402

FIXTURE = HERE / "golden" / "reference_init.npz"
SEEDS = range(101, 117)


def _ours():
    with np.load(FIXTURE) as z:
        ref = {k: z[k] for k in z.files}
    runs = []
    for seed in SEEDS:
        pars = replay_cases.make_pars("init", lp, PropertySet)
        pars.seed = seed
        pars.age_pyramid_path = ref["pyramid"]
        sim = lp.SEIR_ABM(pars)
        sim.components = replay_cases.components(lp)
        runs.append((replay_cases.init_statistics(sim.people, sim.people.count, sim.people.capacity),
                     sim.people.capacity, sim))
    return ref, runs


def _chi2(a, b):
    keep = (a + b) > 0
    table = np.stack([a[keep], b[keep]])
    return stats.chi2_contingency(table)[1]


def check(ref, runs):
    assert all(cap == int(ref["capacity"][0]) for _, cap, _ in runs)
    ours = {k: [r[0][k] for r in runs] for k in runs[0][0]}
    assert np.all(np.stack(ours["missed"]) == ref["missed"][0])
    sbn = np.stack(ours["state_by_node"])  # [runs, 4 states, nodes]
    rsbn = ref["state_by_node"]
    assert np.all(sbn[:, 2] == rsbn[0, 2])  # infected per node
    assert np.all(sbn[:, 1] == 0)
    assert np.all(sbn.sum(axis=1) == rsbn[0].sum(axis=0))  # alive per node
    m_o, m_r = sbn[:, 3].mean(0), rsbn[:, 3].mean(0)
    se = np.sqrt((sbn[:, 3].var(0) + rsbn[:, 3].var(0)) / len(runs)) + 0.5
    assert np.all(np.abs(m_o - m_r) <= 5 * se), (m_o, m_r)
    assert np.all(np.sum(ours["defaults"], axis=0) == ref["defaults"])
    ps = {k: _chi2(np.sum(ours[k], axis=0), ref[k]) for k in ("et", "it", "pt", "age_years", "death_age_years",
                                                                 "ri_offset")}
    assert min(ps.values()) > 1e-3 / len(ps), ps
    ri = np.concatenate(ours["risk_inf"], axis=1)
    rr = ref["risk_inf"]
    p_risk = stats.ks_2samp(ri[0], rr[0]).pvalue
    p_inf = stats.ks_2samp(ri[1], rr[1]).pvalue
    assert p_risk > 1e-3 and p_inf > 1e-3, (p_risk, p_inf)
    rho_o, rho_r = stats.spearmanr(ri[0], ri[1])[0], stats.spearmanr(rr[0], rr[1])[0]
    assert abs(rho_o - rho_r) < 0.03, (rho_o, rho_r)
    return ps, p_risk, p_inf, rho_o, rho_r


def test_initialisation_matches_the_references():
    ref, runs = _ours()
    check(ref, runs)


@pytest.mark.gpu
def test_gpu_initialisation_matches_the_references_and_the_oracle():
    from laser_polio_gb300 import init as dinit
    from oracle_backend import oracle_fill

    ref, runs = _ours()
    check(ref, runs)
    # the device's table equals the oracle's restatement bit for bit
    sim = runs[0][2]
    dev = {k: np.asarray(getattr(sim.people, k)).copy() for k in replay_cases.INIT_COLUMNS}
    pars = replay_cases.make_pars("init", lp, PropertySet)
    pars.seed = SEEDS[0]
    pars.age_pyramid_path = ref["pyramid"]
    saved = dinit.fill
    dinit.fill = oracle_fill
    try:
        host = lp.SEIR_ABM(pars)
        host.components = replay_cases.components(lp)
    finally:
        dinit.fill = saved
    for k, v in dev.items():
        np.testing.assert_array_equal(v, np.asarray(getattr(host.people, k)), err_msg=k)
