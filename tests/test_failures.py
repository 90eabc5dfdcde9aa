"""Failure handling in the forms a shared GPU allows: nothing here faults,
traps or hangs the device.

  - Bad parameters are rejected on the host before any device work
    (lpg_check_desc / lpg_create), with the reference's ValueError.
  - A bounded device wait that runs out: the staged RI/SIA sweep's consumers
    wait on an mbarrier with an iteration limit.  The test hook
    lpg_test_stall_sweep makes the producer withhold its stages and cuts the
    limit, so the wait runs out as it would if a copy never landed; the kernel
    records LPG_ERR_TIMEOUT against the simulation it was sweeping, drains
    the copies it did issue and returns, and the context stays usable.
  - The same for the grid barrier of the first selection round
    (lpg_test_stall_round0): one CTA held back, the others' bounded wait runs
    out, every running simulation records LPG_ERR_TIMEOUT.
"""

import numpy as np
import pytest

from laser_polio_gb300 import _lib
from laser_polio_gb300 import synthetic
from laser_polio_gb300.engine import make_desc


def _results(params):
    from laser_polio_gb300 import _abi

    nt, n, ns = params["nt"], params["n_nodes"], params["n_strains"]
    return {name: np.zeros((nt, n, ns) if wide else (nt, n), np.int32) for name, wide in _abi.RESULT_FIELDS}


@pytest.mark.parametrize("field,value,match", [
    ("r0_scalars", np.nan, "r0_scalars"),
    ("network", -0.1, "network"),
    ("vx_prob_ri", 1.5, "vx_prob_ri"),
    ("birth_rate", np.inf, "birth_rate"),
    ("seasonality", np.nan, "seasonality"),
])
def test_bad_parameters_are_rejected_on_the_host(field, value, match):
    params, _ = synthetic.bundle(kind="zamfara", n_agents=20_000, n_nodes=6, dur=30, seed=1)
    a = np.array(params[field], dtype=np.float64, copy=True)
    a.flat[min(3, a.size - 1)] = value
    params[field] = a
    desc, _keep = make_desc(params)
    with pytest.raises(ValueError, match=match):
        _lib.check_desc(desc)


def test_a_good_description_passes_the_host_check():
    params, _ = synthetic.bundle(kind="nigeria", n_agents=50_000, n_nodes=12, dur=200, seed=2)
    desc, _keep = make_desc(params)
    _lib.check_desc(desc)


@pytest.mark.gpu
def test_gpu_a_wait_that_runs_out_reports_timeout_on_its_simulation():
    """Two simulations in one handle; only the second has an SIA campaign
    (tick 180), which is what the staged sweep serves.  With every stage
    withheld and the consumers' limit at 4096 iterations, the second ends
    with LPG_ERR_TIMEOUT on tick 180 while the first runs to its end
    bit-exact with its oracle run; then a fresh handle on the same device
    runs a simulation bit-exact."""
    from oracle_backend import assert_same
    from oracle.oracle import OracleSim

    plain, plain_cols = synthetic.bundle(kind="zamfara", n_agents=100_000, n_nodes=8, dur=200, seed=3)
    sia, sia_cols = synthetic.bundle(kind="nigeria", n_agents=200_000, n_nodes=20, dur=200, seed=4)
    assert not plain["sia"] and sia["sia"][0][0] == 180
    d0, k0 = make_desc(plain)
    d1, k1 = make_desc(sia)

    def oracle_run(params, cols, desc, keep):
        o = OracleSim(desc, keepalive=keep)
        c = {k: v.copy() for k, v in cols.items()}
        o.bind_columns(c)
        o.start()
        o.step(params["nt"] - 1)
        res = _results(params)
        o.read_results(res)
        o.read_columns(c)
        st = o.state()
        o.close()
        return st, res, c

    so, res_o, cols_o = oracle_run(plain, plain_cols, d0, k0)
    h = _lib.Handle([d0, d1])
    try:
        h.test_stall_sweep(0, 4096)
        cols_g = {k: v.copy() for k, v in plain_cols.items()}
        h.bind_columns(0, cols_g)
        h.bind_columns(1, {k: v.copy() for k, v in sia_cols.items()})
        h.start()
        h.step(200)
        statuses = h.sync_statuses()
        assert statuses == [0, -4], statuses
        s1 = h.state(1, check=False)
        assert s1.error == -4 and s1.t == 181  # stopped after the SIA day
        sg = h.state(0, check=False)
        assert (sg.t, sg.count, sg.error) == (so.t, so.count, 0)
        res_g = _results(plain)
        h.read_results(0, res_g)
        h.read_columns(0, cols_g)
        assert_same(res_o, res_g, "result")
        assert_same(cols_o, cols_g, "column", count=so.count)
    finally:
        h.close()
    # the context is still usable
    so2, res_o2, cols_o2 = oracle_run(sia, sia_cols, d1, k1)
    h = _lib.Handle([d1])
    try:
        cols_g = {k: v.copy() for k, v in sia_cols.items()}
        h.bind_columns(0, cols_g)
        h.start()
        h.step(200)
        assert h.sync_statuses() == [0]
        res_g = _results(sia)
        h.read_results(0, res_g)
        h.read_columns(0, cols_g)
        assert_same(res_o2, res_g, "result")
        assert_same(cols_o2, cols_g, "column", count=so2.count)
        assert res_g["sia_vaccinated"][180].sum() > 0
    finally:
        h.close()


@pytest.mark.gpu
def test_gpu_a_round0_barrier_that_runs_out_stops_the_run_and_leaves_the_context_usable():
    """The first selection round is one cooperative launch whose CTAs meet
    at a grid barrier with a bounded wait.  With CTA 0 held back from the
    barrier (lpg_test_stall_round0) and the limit at 4096 polls, the other
    CTAs give up: every running simulation records LPG_ERR_TIMEOUT on the
    first tick with transmission demand and stops there; a fresh handle on
    the same device then runs bit-exact with the oracle."""
    from oracle_backend import assert_same
    from oracle.oracle import OracleSim

    params, cols = synthetic.bundle(kind="zamfara", n_agents=100_000, n_nodes=8, dur=60, seed=3)
    d, keep = make_desc(params)
    h = _lib.Handle([d, d])
    try:
        h.test_stall_round0(True, 4096)
        h.bind_columns(0, {k: v.copy() for k, v in cols.items()})
        h.bind_columns(1, {k: v.copy() for k, v in cols.items()})
        h.start()
        h.step(params["nt"] - 1)
        assert h.sync_statuses() == [-4, -4]
        s0, s1 = h.state(0, check=False), h.state(1, check=False)
        assert s0.error == s1.error == -4 and s0.t == s1.t and 1 < s0.t < params["nt"]
    finally:
        h.close()
    o = OracleSim(d, keepalive=keep)
    c_o = {k: v.copy() for k, v in cols.items()}
    o.bind_columns(c_o)
    o.start()
    o.step(params["nt"] - 1)
    res_o = _results(params)
    o.read_results(res_o)
    o.read_columns(c_o)
    so = o.state()
    o.close()
    h = _lib.Handle([d])
    try:
        c_g = {k: v.copy() for k, v in cols.items()}
        h.bind_columns(0, c_g)
        h.start()
        h.step(params["nt"] - 1)
        assert h.sync_statuses() == [0]
        res_g = _results(params)
        h.read_results(0, res_g)
        h.read_columns(0, c_g)
        assert_same(res_o, res_g, "result")
        assert_same(c_o, c_g, "column", count=so.count)
    finally:
        h.close()
