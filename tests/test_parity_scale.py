"""Bit-exact parity of the engine with the oracle at the benchmark
configurations' own shapes.

  - the Zamfara-like configuration in full: 14 nodes, 1e6 agents, 365 ticks;
  - the Nigeria-scale shape over its whole 2555-tick run at reduced agents
    (774 nodes, 2e6 agents): every SIA day (14), every RI tick (182), every
    birth tick (365) and the chunk-list rebuilds they cause;
  - the continental shape (4000 nodes, 5000 km gravity network) at 4e6
    agents over 40 ticks;
  - a 64-replicate calibration batch with the batch configuration's node
    counts ({14, 44, 120, 300}), per-replicate R0, seasonality and gravity k
    and 730 ticks, at 1/50 of its agents, in one handle.

Every result array and every agent column must be identical (the oracle and
the engine consume the same counter-based draws; see test_parity_gpu).
"""

import numpy as np
import pytest

from laser_polio_gb300 import synthetic
from laser_polio_gb300.engine import make_desc
from oracle_backend import assert_same
from oracle_backend import run_spec_gpu
from oracle_backend import run_spec_oracle
from oracle_backend import snapshot

pytestmark = pytest.mark.gpu


def _parity_sim(sim):
    spec, cols_o, res_o = snapshot(sim)
    _, cols_g, res_g = snapshot(sim)
    so = run_spec_oracle(spec, cols_o, res_o, sim.nt - 1)
    sg = run_spec_gpu(spec, cols_g, res_g, sim.nt - 1)
    assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error)
    assert_same(res_o, res_g, "result")
    assert_same(cols_o, cols_g, "column", count=so.count)
    return res_o, so


def test_parity_zamfara_full_size():
    """14 nodes, 1e6 agents, 365 ticks, all five components."""
    sim = synthetic.zamfara_like()
    assert sim.people.count == 1_000_000 and sim.nt == 366
    res, st = _parity_sim(sim)
    assert st.t == 366
    assert res["new_exposed"].sum() > 1000
    assert res["births"].sum() > 0 and res["ri_vaccinated"].sum() > 0


def test_parity_nigeria_shape_whole_run():
    """774 nodes, 2e6 agents, all 2555 ticks: 14 SIA days, 182 RI ticks and
    365 birth ticks."""
    sim = synthetic.nigeria_like(n_agents=2_000_000, n_nodes=774, dur=2555, seed=42)
    res, st = _parity_sim(sim)
    assert st.t == 2556
    sia_days = np.flatnonzero(res["sia_vaccinated"].sum(1))
    assert len(sia_days) == 14
    # newborns keep ri_timer = -1 (the RI membership test at model.py:1731
    # looks at classes), so RI doses reach the initial 42-98-day-olds only
    assert len(np.flatnonzero(res["ri_vaccinated"].sum(1))) >= 5
    assert len(np.flatnonzero(res["births"].sum(1))) > 300
    assert res["new_exposed"].sum() > 0


def test_parity_continental_shape():
    """The continental workload's node layout (4000 nodes, populations
    lognormal(ln 2.5e5, 0.9), dense gravity network over a 5000 km square,
    RI and births) at 4e6 agents over 40 ticks: network rows of 4000 sources
    in the per-node mixing form, nodes of a few dozen to ten thousand agents."""
    from laser_polio_gb300._lib import Handle
    from oracle.oracle import OracleSim

    p, cols = synthetic.bundle("continental", n_agents=4_000_000, dur=40, seed=7)
    assert p["n_nodes"] == 4000 and p["count"] == 4_000_000 and p["network"].shape == (4000, 4000)
    d, keep = make_desc(p)
    o = OracleSim(d, keepalive=keep)
    c_o = {k: v.copy() for k, v in cols.items()}
    o.bind_columns(c_o)
    o.start()
    o.step(p["nt"] - 1)
    res_o = _results(p)
    o.read_results(res_o)
    o.read_columns(c_o)
    so = o.state()
    o.close()
    h = Handle([d])
    try:
        c_g = {k: v.copy() for k, v in cols.items()}
        h.bind_columns(0, c_g)
        h.start()
        h.step(p["nt"] - 1)
        h.sync()
        sg = h.state(0)
        assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error)
        res_g = _results(p)
        h.read_results(0, res_g)
        h.read_columns(0, c_g)
    finally:
        h.close()
    assert_same(res_o, res_g, "result")
    assert_same(c_o, c_g, "column", count=so.count)
    assert res_o["new_exposed"].sum() > 1000 and res_o["births"].sum() > 0 and res_o["ri_vaccinated"].sum() > 0


def test_parity_64_replicates_of_the_batch_shapes():
    """64 replicates (nodes from {14, 44, 120, 300}, per-replicate R0,
    seasonality and gravity k, 730 ticks) in one handle, each equal to its
    own oracle run."""
    from laser_polio_gb300._lib import Handle

    specs = synthetic.replicate_specs(64, seed=42, dur=730)
    for sp in specs:
        sp["n_agents"] = max(20_000, sp["n_agents"] // 50)
    bundles = [synthetic.bundle(**sp) for sp in specs]
    assert {p["n_nodes"] for p, _ in bundles} == {14, 44, 120, 300}
    descs = [make_desc(p) for p, _ in bundles]
    outs_o = []
    for (p, cols), (d, keep) in zip(bundles, descs):
        from oracle.oracle import OracleSim

        o = OracleSim(d, keepalive=keep)
        c = {k: v.copy() for k, v in cols.items()}
        o.bind_columns(c)
        o.start()
        o.step(p["nt"] - 1)
        res = _results(p)
        o.read_results(res)
        o.read_columns(c)
        outs_o.append((o.state(), res, c))
        o.close()
    h = Handle([d for d, _ in descs])
    try:
        cols_g = [{k: v.copy() for k, v in cols.items()} for _, cols in bundles]
        for i, c in enumerate(cols_g):
            h.bind_columns(i, c)
        h.start()
        h.step(730)
        h.sync()
        exposed = 0
        for i, ((p, _), (so, res_o, c_o)) in enumerate(zip(bundles, outs_o)):
            sg = h.state(i)
            assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error), i
            res_g = _results(p)
            h.read_results(i, res_g)
            h.read_columns(i, cols_g[i])
            assert_same(res_o, res_g, f"replicate {i} result")
            assert_same(c_o, cols_g[i], f"replicate {i} column", count=so.count)
            exposed += int(res_o["new_exposed"].sum())
        assert exposed > 0
    finally:
        h.close()


def _results(params):
    from laser_polio_gb300 import _abi

    nt, n, ns = params["nt"], params["n_nodes"], params["n_strains"]
    return {name: np.zeros((nt, n, ns) if wide else (nt, n), np.int32) for name, wide in _abi.RESULT_FIELDS}
