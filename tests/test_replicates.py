"""run_replicates: several SEIR_ABM in one handle (the calibration replicate
loop, calib/objective.py:47-70, as one batch).  The batched device path is
checked against the oracle replicate by replicate on the GPU
(test_parity_batched_replicates); here, on the CPU, a stand-in handle checks
the host side: one handle for all sims, binding in order, one step call to
the longest run, and every sim's own arrays, count, t and should_stop filled
from its own replicate."""

import types

import numpy as np
import pytest

from laser_polio_gb300 import engine
from laser_polio_gb300 import synthetic


class _FakeHandle:
    made = []

    def __init__(self, descs, device=0):
        self.descs = list(descs)
        self.calls = []
        self.closed = False
        _FakeHandle.made.append(self)

    def bind_columns(self, i, cols):
        self.calls.append(("bind", i))

    def start(self):
        self.calls.append(("start",))

    def step(self, n):
        self.calls.append(("step", n))
        if getattr(self, "fail_on_step", False):
            raise RuntimeError("device error")

    def sync(self):
        self.calls.append(("sync",))

    def sync_statuses(self):
        self.calls.append(("sync",))
        return list(getattr(self, "statuses", [0] * len(self.descs)))

    def read_results(self, i, res):
        for a in res.values():
            a[...] = 100 + i

    def read_columns(self, i, cols):
        self.calls.append(("columns", i))

    def state(self, i, check=True):
        return types.SimpleNamespace(t=int(self.descs[i].nt), count=int(self.descs[i].count) + 10 + i,
                                     stopped=i == 1, error=0)

    def close(self):
        self.closed = True


def test_one_handle_for_all_sims_and_results_back_in_each(monkeypatch):
    monkeypatch.setattr(engine._lib, "Handle", _FakeHandle)
    _FakeHandle.made.clear()
    sims = [synthetic.zamfara_like(n_agents=4_000, dur=8, seed=1),
            synthetic.zamfara_like(n_agents=6_000, dur=12, seed=2, n_nodes=5)]
    counts = [s.people.count for s in sims]
    assert engine.run_replicates(sims) == [None, None]
    (h,) = _FakeHandle.made
    assert len(h.descs) == 2 and h.closed
    assert h.calls[:3] == [("bind", 0), ("bind", 1), ("start",)]
    assert ("step", max(s.nt for s in sims) - 1) in h.calls
    for i, s in enumerate(sims):
        assert np.all(s.results.S == 100 + i) and np.all(s.results.new_exposed == 100 + i)
        assert s.people.count == counts[i] + 10 + i and s.t == s.nt
    assert sims[1].should_stop and not sims[0].should_stop


def test_handle_is_closed_when_a_step_fails(monkeypatch):
    class Failing(_FakeHandle):
        fail_on_step = True

    monkeypatch.setattr(engine._lib, "Handle", Failing)
    _FakeHandle.made.clear()
    with pytest.raises(RuntimeError, match="device error"):
        engine.run_replicates([synthetic.zamfara_like(n_agents=3_000, dur=5, seed=3)])
    assert _FakeHandle.made[0].closed
    engine.run_replicates([])  # nothing to run


def test_bad_replicates_fail_alone(monkeypatch):
    """A replicate with bad parameters (a NaN R0 scalar), node ids out of
    range, or a device failure (births beyond its capacity) gets its own
    error; the handle runs the others, which end as their own runs would
    (the reference's replicate loop catches each replicate's exception and
    goes on, calib/objective.py:47-70)."""
    monkeypatch.setattr(engine._lib, "Handle", _FakeHandle)
    _FakeHandle.made.clear()
    sims = [synthetic.zamfara_like(n_agents=4_000, dur=8, seed=s) for s in range(5)]
    sims[1].pars.r0_scalars = np.array(sims[1].pars.r0_scalars, dtype=float)
    sims[1].pars.r0_scalars[2] = np.nan
    sims[3].people.node_id[7] = 99
    counts = [s.people.count for s in sims]
    _FakeHandle.statuses = [0, 0, -2]  # the third sim of the batch (sims[4]) outgrows its capacity
    try:
        errors = engine.run_replicates(sims)
    finally:
        del _FakeHandle.statuses
    (h,) = _FakeHandle.made
    assert len(h.descs) == 3 and h.closed
    assert errors[0] is None and errors[2] is None
    assert isinstance(errors[1], ValueError) and "r0_scalars[2]" in str(errors[1])
    assert isinstance(errors[3], ValueError) and "node_id" in str(errors[3])
    assert isinstance(errors[4], ValueError)
    for i, j in ((0, 0), (2, 1), (4, 2)):
        assert np.all(sims[i].results.S == 100 + j) and sims[i].people.count == counts[i] + 10 + j
    assert sims[1].t == 0 and sims[3].t == 0


@pytest.mark.gpu
def test_gpu_a_replicate_that_outgrows_its_capacity_fails_alone():
    """On the device: one replicate's births exceed its capacity; it stops
    with LPG_ERR_CAPACITY at that tick while the others run to their end,
    bit-exact with their own oracle runs."""
    from oracle_backend import assert_same
    from oracle_backend import run_spec_oracle
    from oracle_backend import snapshot

    sims = [synthetic.zamfara_like(n_agents=40_000, dur=60, seed=s) for s in (11, 12, 13)]
    small = sims[1].people
    small._capacity = small.count + 50  # a few weeks of births
    for name in ("disease_state", "strain", "exposure_timer", "infection_timer", "paralysis_timer",
                 "potentially_paralyzed", "paralyzed", "ipv_protected", "chronically_missed", "node_id",
                 "ri_timer", "acq_risk_multiplier", "daily_infectivity", "date_of_birth", "date_of_death"):
        setattr(small, name, np.ascontiguousarray(getattr(small, name)[: small.capacity]))
    snaps = {i: snapshot(sims[i]) for i in (0, 2)}
    states = {i: run_spec_oracle(spec, cols, res, sims[i].nt - 1) for i, (spec, cols, res) in snaps.items()}
    errors = engine.run_replicates(sims)
    assert errors[0] is None and errors[2] is None
    assert isinstance(errors[1], ValueError)
    assert 1 < sims[1].t < sims[1].nt
    for i, (_, cols_o, res_o) in snaps.items():
        so = states[i]
        s = sims[i]
        assert (s.people.count, s.t) == (so.count, so.t), i
        assert_same(res_o, {k: getattr(s.results, k) for k in res_o}, f"replicate {i} result")
        assert_same(cols_o, {k: getattr(s.people, k) for k in cols_o}, f"replicate {i} column", count=so.count)


@pytest.mark.gpu
def test_gpu_run_replicates_equals_each_oracle_run():
    """Through run_replicates on the device, each sim ends bit-exact with
    its own oracle run (results, columns, count, t, stop)."""
    from oracle_backend import assert_same
    from oracle_backend import run_spec_oracle
    from oracle_backend import snapshot

    sims = [synthetic.zamfara_like(n_agents=40_000, dur=60, seed=5),
            synthetic.nigeria_like(n_agents=90_000, n_nodes=20, dur=45, seed=6)]
    snaps = [snapshot(s) for s in sims]
    states = [run_spec_oracle(spec, cols, res, s.nt - 1) for s, (spec, cols, res) in zip(sims, snaps)]
    engine.run_replicates(sims)
    for i, (s, (_, cols_o, res_o), so) in enumerate(zip(sims, snaps, states)):
        assert (s.people.count, s.t, s.should_stop) == (so.count, so.t, bool(so.stopped)), i
        res_g = {k: getattr(s.results, k) for k in res_o}
        cols_g = {k: getattr(s.people, k) for k in cols_o}
        assert_same(res_o, res_g, f"replicate {i} result")
        assert_same(cols_o, cols_g, f"replicate {i} column", count=so.count)


def test_replicate_objective_reports_failures_and_averages_the_rest(monkeypatch):
    """calibrate.replicate_objective, the reference's objective loop
    (calib/objective.py:47-82) as one batch: every buildable replicate goes
    to one run_replicates call; a replicate that cannot be built, whose run
    fails or whose scoring fails is reported and left out; the value is the
    mean of the others' scores."""
    from laser_polio_gb300 import calibrate

    batches = []

    def fake_run(sims, autotune=False):
        batches.append((list(sims), autotune))
        return [None if s.rep != 3 else RuntimeError("device error") for s in sims]

    monkeypatch.setattr(engine, "run_replicates", fake_run)

    def make_sim(params, rep):
        if rep == 1:
            raise ValueError("bad parameters")
        return types.SimpleNamespace(rep=rep, r0=params["r0"], pars=types.SimpleNamespace(seed=100 + rep))

    def score(sim):
        if sim.rep == 4:
            raise KeyError("no target")
        return -float(sim.rep) * sim.r0

    logged = []
    out = calibrate.replicate_objective(make_sim, {"r0": 2.0}, score, n_replicates=6, autotune=True,
                                        log=logged.append)
    assert len(batches) == 1 and [s.rep for s in batches[0][0]] == [0, 2, 3, 4, 5] and batches[0][1] is True
    assert out["scores"] == [0.0, -4.0, -10.0] and out["seeds"] == [100, 102, 105]
    assert out["value"] == pytest.approx(-14.0 / 3)
    assert [r for r, _ in out["errors"]] == [1, 3, 4] and len(logged) == 3
    none = calibrate.replicate_objective(lambda p, r: (_ for _ in ()).throw(ValueError("x")), {}, score,
                                         n_replicates=2, log=logged.append)
    assert np.isnan(none["value"]) and none["scores"] == [] and len(none["errors"]) == 2


@pytest.mark.gpu
def test_gpu_replicate_objective_scores_each_replicate_as_its_own_run():
    """Scores of a batched trial equal those of the same replicates run one
    by one with sim.run() (the batch changes the time, not the results)."""
    from laser_polio_gb300 import calibrate

    def make_sim(params, rep):
        return synthetic.zamfara_like(n_agents=30_000, dur=50, seed=40 + rep)

    def score(sim):
        return float(np.log1p(np.asarray(sim.results.new_exposed, np.float64)).sum())

    out = calibrate.replicate_objective(make_sim, {}, score, n_replicates=3, log=lambda m: None)
    alone = []
    for rep in range(3):
        s = make_sim({}, rep)
        s.run()
        alone.append(score(s))
    assert out["errors"] == [] and out["scores"] == alone
    assert out["value"] == pytest.approx(float(np.mean(alone)))
