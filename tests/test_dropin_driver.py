"""The drop-in components under a driver that is not this package's.

The reference's SEIR_ABM (model.py:209-289) only knows the component
protocol: its components setter filters and orders the given classes by
``__name__`` in ``default_run_order`` and keeps one instance of each; its
run() logs tick 0, then on every later tick calls every instance's step()
and then every instance's log(t), and stops early when ``should_stop`` is
set.  It creates no engine and never touches the people's count except
through LaserFrame's own methods.  ``ForeignDriver`` below is that driver,
written from the protocol alone, around a population built by this
package's SEIR_ABM constructor.  The components must find or create their
engine themselves and leave results, columns, count, t and should_stop as
this package's own run() does.

The CPU test runs the components' whole host path with the oracle in place
of the device (oracle_backend.OracleHandle); the GPU test runs the engine.
"""

import numpy as np
import pytest

import laser_polio_gb300 as lp
from laser_polio_gb300 import engine
from laser_polio_gb300.core import PropertySet
from oracle_backend import OracleHandle
from oracle_backend import assert_same
from oracle_backend import run_with_oracle

RUN_ORDER = ["VitalDynamics_ABM", "DiseaseState_ABM", "RI_ABM", "SIA_ABM", "Transmission_ABM"]


class ForeignDriver:
    """The tick loop and component registration of the reference's SEIR_ABM
    (model.py:209-289), nothing else."""

    def __init__(self, built):
        for name in ("pars", "people", "results", "nodes", "nt", "datevec", "perf_stats", "verbose"):
            setattr(self, name, getattr(built, name))
        self.t = 0
        self.should_stop = False
        self._components = []
        self.instances = []

    @property
    def components(self):
        return self._components

    @components.setter
    def components(self, classes):
        lookup = {cls.__name__: cls for cls in classes}
        self._components = [lookup[name] for name in RUN_ORDER if name in lookup]
        self.instances = [cls(self) for cls in self._components]

    def log_results(self, t):
        for c in self.instances:
            c.log(t)

    def run(self):
        for tick in range(self.nt):
            if tick == 0:
                self.log_results(tick)
                self.t += 1
            else:
                for c in self.instances:
                    c.step()
                self.log_results(tick)
                self.t += 1
                if self.should_stop:
                    break


def _pars(seed, stop):
    return PropertySet({
        "seed": seed, "start_date": lp.date("2019-01-01"), "dur": 90,
        "init_pop": np.array([20000, 12000, 8000]), "cbr": np.array([30.0, 30.0, 30.0]),
        "init_immun": [0.2, 0.4, 0.1], "init_prev": [15, 0, 4], "r0": 14,
        "r0_scalars": np.array([1.0, 0.8, 1.2]),
        "distances": np.array([[0, 30, 60], [30, 0, 40], [60, 40, 0]]),
        "migration_method": "gravity", "gravity_k": 0.5, "max_migr_frac": 0.2,
        "vx_prob_ri": [0.5, 0.6, 0.4], "vx_prob_ipv": [0.2, 0.0, 0.3], "missed_frac": 0.05,
        "sia_schedule": [{"date": "2019-02-01", "nodes": [0, 2], "age_range": (0, 5 * 365), "vaccinetype": "nOPV2"}],
        "vx_prob_sia": [0.8, 0.7, 0.9], "stop_if_no_cases": stop, "verbose": 0,
    })


def _classes():
    # given out of order: registration orders them by name
    return [lp.Transmission_ABM, lp.SIA_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.VitalDynamics_ABM]


def _run_both(seed, stop):
    want = lp.SEIR_ABM(_pars(seed, stop))
    want.components = _classes()
    run_with_oracle(want)
    drv = ForeignDriver(lp.SEIR_ABM(_pars(seed, stop)))
    drv.components = _classes()
    assert [type(c).__name__ for c in drv.instances] == RUN_ORDER
    assert not hasattr(drv, "_engine")
    drv.run()
    return want, drv


def _same_outcome(want, drv):
    assert (drv.t, drv.should_stop, drv.people.count) == (want.t, want.should_stop, want.people.count)
    names = [k for k in vars(want.results) if isinstance(getattr(want.results, k), np.ndarray)]
    assert "new_exposed" in names and "sia_vaccinated" in names
    assert_same({k: getattr(want.results, k) for k in names}, {k: getattr(drv.results, k) for k in names}, "result")
    cols = ["disease_state", "strain", "node_id", "exposure_timer", "infection_timer", "ri_timer", "date_of_death"]
    assert_same({k: getattr(want.people, k) for k in cols}, {k: getattr(drv.people, k) for k in cols}, "column",
                count=want.people.count)


@pytest.mark.parametrize("seed,stop", [(3, False), (4, True)])
def test_components_under_a_foreign_driver_with_the_oracle(monkeypatch, seed, stop):
    monkeypatch.setattr(engine._lib, "Handle", OracleHandle)
    want, drv = _run_both(seed, stop)
    _same_outcome(want, drv)
    assert drv.results.new_exposed.sum() > 0 and drv.results.births.sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("seed,stop", [(3, False), (4, True)])
def test_gpu_components_under_a_foreign_driver(seed, stop):
    want, drv = _run_both(seed, stop)
    _same_outcome(want, drv)
