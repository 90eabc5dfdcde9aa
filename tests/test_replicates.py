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

    def read_results(self, i, res):
        for a in res.values():
            a[...] = 100 + i

    def read_columns(self, i, cols):
        self.calls.append(("columns", i))

    def state(self, i):
        return types.SimpleNamespace(t=int(self.descs[i].nt), count=1000 + i, stopped=i == 1, error=0)

    def close(self):
        self.closed = True


def test_one_handle_for_all_sims_and_results_back_in_each(monkeypatch):
    monkeypatch.setattr(engine._lib, "Handle", _FakeHandle)
    _FakeHandle.made.clear()
    sims = [synthetic.zamfara_like(n_agents=4_000, dur=8, seed=1),
            synthetic.zamfara_like(n_agents=6_000, dur=12, seed=2, n_nodes=5)]
    engine.run_replicates(sims)
    (h,) = _FakeHandle.made
    assert len(h.descs) == 2 and h.closed
    assert h.calls[:3] == [("bind", 0), ("bind", 1), ("start",)]
    assert ("step", max(s.nt for s in sims) - 1) in h.calls
    for i, s in enumerate(sims):
        assert np.all(s.results.S == 100 + i) and np.all(s.results.new_exposed == 100 + i)
        assert s.people.count == 1000 + i and s.t == s.nt
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
