"""Run an SEIR_ABM built with laser_polio_gb300 on the CPU oracle.

Test-only: it hands the same C-ABI description the engine would get
(engine.build_sim_spec) to the oracle and copies the outcome back into the
sim's host arrays, exactly where the engine's finish step would put it.
"""

from __future__ import annotations

import numpy as np

from laser_polio_gb300.engine import _advance_count
from laser_polio_gb300.engine import build_sim_spec
from laser_polio_gb300.engine import host_columns
from oracle.oracle import OracleSim


def run_with_oracle(sim, n_ticks=None):
    spec = build_sim_spec(sim)
    cols = {k: getattr(sim.people, k) for k in spec.columns}  # host arrays (device columns copied over once)
    o = OracleSim(spec.desc, keepalive=spec)
    o.bind_columns(cols)
    o.start()
    o.step(sim.nt - 1 if n_ticks is None else n_ticks)
    st = o.state()
    o.read_results(spec.results)
    o.read_columns(cols)
    _advance_count(sim.people, st.count)
    sim.t = st.t
    sim.should_stop = bool(st.stopped)
    o.close()
    return sim


def snapshot(sim):
    """Copies of the spec's columns (on the host, wherever they live) and
    results, for parity comparisons."""
    spec = build_sim_spec(sim)
    cols = host_columns(spec)
    res = {k: v.copy() for k, v in spec.results.items()}
    return spec, cols, res


def run_spec_oracle(spec, cols, res, n_ticks):
    o = OracleSim(spec.desc, keepalive=spec)
    o.bind_columns(cols)
    o.start()
    o.step(n_ticks)
    st = o.state()
    o.read_results(res)
    o.read_columns(cols)
    o.close()
    return st


def run_spec_gpu(spec, cols, res, n_ticks, graphs=True, check=False):
    from laser_polio_gb300._lib import Handle

    h = Handle([spec.desc])
    h.set_graphs(graphs)
    h.bind_columns(0, cols)
    h.start()
    if check:
        for _ in range(n_ticks):
            h.step(1)
            h.check_invariants()
    else:
        h.step(n_ticks)
    h.sync()
    st = h.state(0)
    h.read_results(0, res)
    h.read_columns(0, cols)
    h.close()
    return st


def assert_same(a: dict, b: dict, what: str, count=None):
    for k in a:
        x, y = a[k], b[k]
        if count is not None and x.ndim == 1:
            x, y = x[:count], y[:count]
        if not np.array_equal(x, y):
            idx = np.argwhere(x != y)
            raise AssertionError(f"{what} '{k}' differs at {len(idx)} entries, first {idx[:5].tolist()}: "
                                 f"{x[tuple(idx[0])]} vs {y[tuple(idx[0])]}")


class OracleHandle:
    """The engine handle's interface (laser_polio_gb300._lib.Handle) over the
    oracle, one simulation per handle: lets a CPU test drive the drop-in
    components' whole host path (GpuTick, run_replicates) with the oracle in
    place of the device."""

    made = []

    def __init__(self, descs, device=0):
        descs = list(descs)
        assert len(descs) == 1, "one simulation per oracle handle"
        self.o = OracleSim(descs[0])
        OracleHandle.made.append(self)

    def bind_columns(self, sim, cols):
        self.o.bind_columns(cols)

    def start(self):
        self.o.start()

    def step(self, n):
        self.o.step(n)

    def sync(self):
        pass

    def sync_statuses(self):
        return [int(self.o.state().error)]

    def state(self, sim=0, check=True):
        return self.o.state()

    def read_results(self, sim, res):
        self.o.read_results(res)

    def read_columns(self, sim, cols):
        self.o.read_columns(cols)

    def close(self):
        self.o.close()


def oracle_fill(people, spec, parts):
    """laser_polio_gb300.init.fill with the oracle's restatement of the
    device initialisation (lpo_init_columns, the same draws): host numpy
    columns, for tests on a machine without a GPU."""
    from laser_polio_gb300 import init as dinit
    from oracle.oracle import init_columns

    cols = {}
    for name in dinit.part_columns(parts):
        if not people.has_column(name):
            people.add_scalar_property(name, dtype=dinit.COLUMN_DTYPES[name], default=0)
        cols[name] = getattr(people, name)
    desc, _keep = spec.desc()
    init_columns(desc, parts, cols)
