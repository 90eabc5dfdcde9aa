"""Per-node force of infection against an FP64 oracle.

The transmission step (model.py:1315-1363) mixes each node's summed
infectivity over the network, scales it by seasonality and the node's R0
scalar, divides by the node's population and turns the rate into a
probability; the expected new exposures of a node are its susceptibles'
summed risk times the summed probabilities.  The engine and the C oracle
evaluate this from exact fixed-point sums (risk in units of 2^-24,
infectivity in units of 2^-32, the network in units of 2^-62).  The bound
checked here is the one stated for the step: every node's expected exposures
within 1e-6 relative of an FP64 evaluation from the unquantised float32
columns (sums in FP64, the FP64 network, the probability as -expm1(-rate),
the exact value that the reference's 1 - exp(-rate) rounds), on every
transmission tick and every node where the FP64 value is not zero, and zero
where it is.
"""

import numpy as np
import pytest

from laser_polio_gb300 import synthetic
from laser_polio_gb300.engine import make_desc

REL = 1e-6


def _fp64_exposures(params, agg64, pop):
    """lam[t, n] from FP64 sums: srisk [nt, n], beta [nt, n, ns] (strain
    scalars applied) and pop [nt, n]."""
    N = np.asarray(params["network"], np.float64)
    r0s = np.asarray(params["r0_scalars"], np.float64)
    seas = np.asarray(params["seasonality"], np.float64)
    keep = 1.0 - N.sum(1)
    lam = np.zeros_like(agg64["srisk"])
    for t in range(1, lam.shape[0]):
        beta = agg64["beta"][t]
        u = beta * keep[:, None] + N.T @ beta
        rate = u * seas[t] * r0s[:, None] / np.maximum(pop[t], 1.0)[:, None]
        lam[t] = agg64["srisk"][t] * (-np.expm1(-rate)).sum(1)
    return lam


def _check(lam, lam64, what):
    ticks = slice(1, lam.shape[0])
    got, want = lam[ticks], lam64[ticks]
    zero = want == 0
    assert np.all(got[zero] == 0), f"{what}: nonzero where the FP64 value is zero"
    rel = np.abs(got[~zero] - want[~zero]) / want[~zero]
    assert rel.size > 0
    worst = float(rel.max())
    assert worst <= REL, f"{what}: worst per-node relative difference {worst:.3g} > {REL}"
    return worst


def _oracle_run(params, cols):
    from oracle.oracle import OracleSim

    desc, keep = make_desc(params)
    o = OracleSim(desc, keepalive=keep)
    o.record_aggregates()
    o.bind_columns({k: v.copy() for k, v in cols.items()})
    o.start()
    o.step(params["nt"] - 1)
    agg, agg64 = o.read_aggregates(), o.read_aggregates_fp64()
    o.close()
    return agg, agg64


def test_oracle_node_exposures_within_1e6_of_fp64():
    """The oracle's fixed-point step against FP64 sums of the same columns,
    per node and tick, over an outbreak in 30 nodes with three strains."""
    params, cols = synthetic.bundle(kind="nigeria", n_agents=300_000, n_nodes=30, dur=150, seed=7)
    agg, agg64 = _oracle_run(params, cols)
    assert agg["lam"][1:].sum() > 0
    lam64 = _fp64_exposures(params, agg64, agg["pop"])
    _check(agg["lam"], lam64, "oracle")


@pytest.mark.gpu
def test_gpu_node_exposures_equal_the_oracle_and_are_within_1e6_of_fp64():
    """The engine's recorded per-node expected exposures (lpg_record_aggregates)
    equal the oracle's bit for bit and so meet the FP64 bound, at the
    Nigeria-like shape (774 nodes, three strains, SIA and RI) over 400 ticks."""
    from laser_polio_gb300._lib import Handle

    params, cols = synthetic.bundle(kind="nigeria", n_agents=2_000_000, n_nodes=774, dur=400, seed=11)
    agg_o, agg64 = _oracle_run(params, cols)
    desc, _keep = make_desc(params)
    h = Handle([desc])
    try:
        h.record_aggregates(0)
        h.bind_columns(0, {k: v.copy() for k, v in cols.items()})
        h.start()
        h.step(params["nt"] - 1)
        h.sync()
        agg_g = h.read_aggregates(0, params["nt"], params["n_nodes"], params["n_strains"])
    finally:
        h.close()
    for k in ("srisk", "beta", "pop", "lam"):
        np.testing.assert_array_equal(agg_g[k], agg_o[k], err_msg=k)
    assert agg_g["lam"][1:].sum() > 0
    _check(agg_g["lam"], _fp64_exposures(params, agg64, agg_o["pop"]), "engine")
