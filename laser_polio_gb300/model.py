"""SEIR_ABM driver and the five drop-in components.

Each class carries the reference's name, takes the reference's ``pars`` and
fills the reference's ``sim.results`` arrays; the names matter because the
components setter orders and filters classes by ``__name__``
(laser_polio/model.py:226-237).  Initialisation (timers, immunity, seeding,
ages, lifespans, heterogeneity, network) runs on the host with numpy exactly
as in the reference, because it is once per run and its random draws are
not part of the replayed stream.  Every per-tick ``step()`` and ``log()``
goes to the shared ``GpuTick`` engine (engine.py), which runs the whole tick
on the GPU through the C ABI in include/lpg.h.
"""

from __future__ import annotations

import numbers
import time
from collections import defaultdict
from copy import deepcopy
from datetime import datetime

import numpy as np
import scipy.stats as stats

from . import pars as _pars
from . import utils as lpu
from .core import AliasedDistribution
from .core import KaplanMeierEstimator
from .core import LaserFrame
from .core import PropertySet
from .core import calc_capacity
from .core import distance
from .core import gravity
from .core import radiation
from .core import resolve_pyramid
from .core import row_normalizer

__all__ = ["RI_ABM", "SEIR_ABM", "SIA_ABM", "DiseaseState_ABM", "Transmission_ABM", "VitalDynamics_ABM"]


class TimingStats:
    """Accumulated wall time per label, in ns (the keys the reference's
    TimingStats uses, laser_polio/utils.py:819-945)."""

    def __init__(self):
        self.stats = defaultdict(int)

    class _Watch:
        def __init__(self, owner, label):
            self.owner, self.label = owner, label

        def __enter__(self):
            self.t0 = time.perf_counter_ns()
            return self

        def __exit__(self, *exc):
            self.owner.stats[self.label] += time.perf_counter_ns() - self.t0
            return False

    def start(self, label):
        return TimingStats._Watch(self, label)


class SEIR_ABM:
    """Agent-based SEIR polio model (laser_polio/model.py:51-342).

    Disease state codes: -1 dead/inactive, 0 S, 1 E, 2 I, 3 R.
    """

    def common_init(self, pars, verbose):
        self.perf_stats = TimingStats()
        self.pars = deepcopy(_pars.default_pars)
        if pars is not None:
            unexpected = set(pars.to_dict().keys()) - set(self.pars.to_dict().keys())
            if unexpected:
                print(f"Warning: ignoring unexpected parameters: {list(unexpected)}")
                filtered = {k: v for k, v in pars.items() if k in self.pars}
                self.pars <<= filtered
            else:
                self.pars <<= pars
        pars = self.pars
        self.verbose = pars["verbose"] if "verbose" in pars else 1
        if pars.seed is None:
            now = datetime.now()  # noqa: DTZ005
            pars.seed = now.microsecond ^ int(now.timestamp())
            if self.verbose >= 1:
                print(f"No seed provided. Using random seed of {pars.seed}.")
        np.random.seed(int(pars.seed) & 0xFFFFFFFF)
        self.t = 0
        self.nt = pars.dur + 1
        self.datevec = lpu.daterange(self.pars["start_date"], days=self.nt)
        self.should_stop = False

    def __init__(self, pars: PropertySet = None, verbose=1):
        self.common_init(pars, verbose)
        pars = self.pars
        pars.init_pop = np.atleast_1d(pars.init_pop).astype(int)
        if pars.init_sus_by_age is not None:
            raise NotImplementedError("init_sus_by_age (real-data initialisation through run_sim) is not supported")
        total_pop = int(np.sum(pars.init_pop))
        # capacity estimate with the reference's fudge factor (model.py:124-137)
        expected_births = 0
        if (pars.cbr is not None) and (len(np.atleast_1d(pars.cbr)) == 1):
            expected_births = calc_capacity(pars.init_pop.sum(), pars.dur + 100, np.atleast_1d(pars.cbr)[0]) - pars.init_pop.sum()
        elif (pars.cbr is not None) and (len(pars.cbr) > 1):
            expected_births = calc_capacity(pars.init_pop.sum(), pars.dur + 100, np.mean(pars.cbr)) - pars.init_pop.sum()
        fudge = 1 + 4 / np.sqrt(expected_births) if expected_births > 0 else 1
        capacity = int(fudge * (total_pop + expected_births))
        self.people = LaserFrame(capacity=capacity, initial_count=total_pop)

        p = self.people
        p.add_scalar_property("disease_state", dtype=np.int8, default=-1)
        p.disease_state[: p.count] = 0
        p.add_scalar_property("potentially_paralyzed", dtype=np.int8, default=-1)
        p.add_scalar_property("paralyzed", dtype=np.int8, default=0)
        p.add_scalar_property("ipv_protected", dtype=np.int8, default=0)
        self.results = LaserFrame(capacity=1)
        p.add_scalar_property("strain", dtype=np.int8, default=0)
        p.add_scalar_property("chronically_missed", dtype=np.uint8, default=0)
        n_missed = int(pars.missed_frac * p.count)
        missed_ids = np.random.choice(p.count, size=n_missed, replace=False)
        p.chronically_missed[missed_ids] = 1

        p.add_scalar_property("node_id", dtype=np.int16, default=-1)
        self.nodes = np.arange(len(pars.init_pop))
        pop_by_node = pars.init_pop
        if np.any(pop_by_node <= 0) or np.any(np.isnan(pop_by_node)):
            raise ValueError("pop_by_node must be positive & non-nan")
        p.node_id[:total_pop] = np.repeat(np.arange(len(pop_by_node)), pop_by_node).astype(np.int16)
        self._components = []
        self.instances = []

    @property
    def components(self) -> list:
        return self._components

    @components.setter
    def components(self, components: list) -> None:
        lookup = {cls.__name__: cls for cls in components}
        ordered = [lookup[name] for name in _pars.default_run_order if name in lookup]
        self._components = ordered
        self.instances = []
        for cls in ordered:
            with self.perf_stats.start(cls.__name__ + ".__init__()"):
                self.instances.append(cls(self))
        self._engine = None

    def run(self):
        """SEIR_ABM.run (model.py:246-282).  With GPU components the whole
        loop runs on the device in one call; the result is the same as the
        per-tick loop below, which is kept for component sets that mix in
        host classes."""
        if self.instances and all(isinstance(c, _GpuComponent) for c in self.instances):
            with self.perf_stats.start("GpuTick.run()"):
                _engine_of(self).run_all()
            if self.should_stop and self.verbose >= 1:
                print(f"[SEIR_ABM] Early stopping at t={self.t}: no E/I and no future seed_schedule events.")
            return
        for tick in range(self.nt):
            if tick == 0:
                self.log_results(tick)
                self.t += 1
                continue
            for component in self.instances:
                with self.perf_stats.start(component.__class__.__name__ + ".step()"):
                    component.step()
            self.log_results(tick)
            self.t += 1
            if self.should_stop:
                if self.verbose >= 1:
                    print(f"[SEIR_ABM] Early stopping at t={self.t}: no E/I and no future seed_schedule events.")
                break

    def log_results(self, t):
        for component in self.instances:
            with self.perf_stats.start(component.__class__.__name__ + ".log()"):
                component.log(t)


def _engine_of(sim):
    """The sim's GpuTick, created on first use.  The reference's own
    SEIR_ABM (model.py:209-289) knows nothing of an engine: its components
    setter only instantiates the classes and its run() only calls step() and
    log(t), so the first call from any drop-in component creates it."""
    eng = getattr(sim, "_engine", None)
    if eng is None:
        from .engine import GpuTick

        eng = GpuTick(sim)
        sim._engine = eng
    return eng


class _GpuComponent:
    """Base of the drop-in components: step()/log() go to the shared engine."""

    def step(self):
        _engine_of(self.sim).step(self)

    def log(self, t):
        _engine_of(self.sim).log(self, t)

    def plot(self, save=False, results_path=None):
        pass


# ---------------------------------------------------------------------------
class DiseaseState_ABM(_GpuComponent):
    """Timers, immunity and seeding at init (model.py:561-713); per tick the
    E->I->R progression, paralysis, seed schedule and stop rule
    (model.py:715-795) run in the engine's sweep."""

    def _common_init(self, sim):
        self.sim = sim
        self.people = sim.people
        self.pars = sim.pars
        self.nodes = sim.nodes
        self.results = sim.results
        self.verbose = self.pars["verbose"] if "verbose" in self.pars else 1
        self.seed_schedule = defaultdict(list)
        if self.pars.seed_schedule is not None:
            for entry in self.pars.seed_schedule:
                if "date" in entry and "dot_name" in entry:
                    d = lpu.date(entry["date"])
                    t = (d - lpu.date(self.pars.start_date)).days
                    lookup = self.pars.node_lookup or {}
                    node_id = next((nid for nid, info in lookup.items() if info["dot_name"] == entry["dot_name"]), None)
                    if node_id is not None:
                        self.seed_schedule[t].append((node_id, entry["prevalence"]))
                elif "timestep" in entry and "node_id" in entry:
                    self.seed_schedule[entry["timestep"]].append((entry["node_id"], entry["prevalence"]))

    def _initialize_results_arrays(self):
        nt, nn, ns = self.sim.nt, len(self.nodes), len(self.sim.pars.strain_ids)
        r = self.results
        for name in ("S", "E", "I", "R"):
            r.add_array_property(name, shape=(nt, nn), dtype=np.int32)
        r.add_array_property("E_by_strain", shape=(nt, nn, ns), dtype=np.int32)
        r.add_array_property("I_by_strain", shape=(nt, nn, ns), dtype=np.int32)
        for name in ("potentially_paralyzed", "paralyzed", "new_potentially_paralyzed", "new_paralyzed", "pop"):
            r.add_array_property(name, shape=(nt, nn), dtype=np.int32)
        r.pop[0] = self.sim.pars.init_pop

    def __init__(self, sim):
        self._common_init(sim)
        self._initialize_results_arrays()
        pars = self.pars
        p = sim.people
        p.add_scalar_property("exposure_timer", dtype=np.int8, default=0)
        p.add_scalar_property("infection_timer", dtype=np.int8, default=0)
        p.add_scalar_property("paralysis_timer", dtype=np.int8, default=0)
        p.exposure_timer[:] = np.clip(pars.dur_exp(p.capacity), 0, 127)
        p.infection_timer[:] = np.clip(pars.dur_inf(p.capacity), 0, 127)
        raw = pars.t_to_paralysis(p.capacity) - p.exposure_timer
        upper = np.minimum(p.infection_timer, 127)
        p.paralysis_timer[:] = np.clip(raw, 0, upper).astype(np.int8)

        # immunity (model.py:590-618)
        if isinstance(pars.init_immun, float):
            immun = np.full_like(pars.init_pop, fill_value=pars.init_immun, dtype=np.float32)
        elif isinstance(pars.init_immun, list):
            immun = np.asarray(pars.init_immun, dtype=np.float32)
        elif isinstance(pars.init_immun, np.ndarray):
            immun = pars.init_immun
        else:
            raise ValueError(f"Unsupported init_immun type: {type(pars.init_immun)}")
        for nid, (frac, node_pop) in enumerate(zip(immun, pars.init_pop, strict=False)):
            assert 0.0 <= frac <= 1.0, f"Invalid immunity fraction: {frac} for node {nid}"
            n_rec = int(frac * node_pop)
            if n_rec > 0:
                idx = np.where(p.node_id == nid)[0]
                p.disease_state[np.random.choice(idx, size=n_rec, replace=False)] = 3

        # initial infections (model.py:670-713)
        infected = []
        total = int(np.sum(pars.init_pop))
        if isinstance(pars.init_prev, float):
            infected = np.random.choice(total, size=int(total * pars.init_prev), replace=False)
        elif isinstance(pars.init_prev, (int, np.integer)) and not isinstance(pars.init_prev, bool):
            infected = np.random.choice(total, size=min(int(pars.init_prev), total), replace=False)
        elif isinstance(pars.init_prev, (list, np.ndarray)):
            if len(pars.init_prev) != len(pars.init_pop):
                raise ValueError(
                    f"Length mismatch: init_prev has {len(pars.init_prev)} entries, expected {len(pars.init_pop)} nodes."
                )
            node_ids = p.node_id[: p.count]
            states = p.disease_state[: p.count]
            infected = []
            for node, prev in enumerate(pars.init_prev):
                if not isinstance(prev, numbers.Real):
                    raise ValueError(f"Unsupported value in init_prev list at node {node}: {prev}")
                n_inf = int(pars.init_pop[node] * prev) if 0 < prev < 1 else min(int(prev), pars.init_pop[node])
                alive = np.where((node_ids == node) & (states >= 0))[0]
                k = min(n_inf, len(alive))
                infected.extend(np.random.choice(alive, size=k, replace=False))
        else:
            raise ValueError(f"Unsupported init_prev type: {type(pars.init_prev)}")
        p.disease_state[np.asarray(infected, dtype=np.int64)] = 2


# ---------------------------------------------------------------------------
def populate_heterogeneous_values(start, end, acq_risk_out, infectivity_out, pars):
    """Correlated lognormal acquisition risk and gamma infectivity through a
    Gaussian copula (model.py:816-866)."""
    mean_ln = 1
    var_ln = pars.risk_mult_var
    mu_ln = np.log(mean_ln**2 / np.sqrt(var_ln + mean_ln**2))
    sigma_ln = np.sqrt(np.log(var_ln / mean_ln**2 + 1))
    mean_gamma = pars.r0 / np.mean(pars.dur_inf(1000))
    shape_gamma = 1
    scale_gamma = max(mean_gamma / shape_gamma, 1e-10)
    rho = 2.0 * np.sin(np.pi * pars.corr_risk_inf / 6)
    L = np.linalg.cholesky(np.array([[1, rho], [rho, 1]]))
    batch = 1_000_000
    for b0 in range(start, end, batch):
        b1 = min(b0 + batch, end)
        z = np.random.normal(size=(b1 - b0, 2)) @ L.T
        if pars.individual_heterogeneity:
            acq_risk_out[b0:b1] = np.exp(mu_ln + sigma_ln * z[:, 0])
            infectivity_out[b0:b1] = stats.gamma.ppf(stats.norm.cdf(z[:, 1]), a=shape_gamma, scale=scale_gamma)
        else:
            acq_risk_out[b0:b1] = 1.0
            infectivity_out[b0:b1] = mean_gamma


class Transmission_ABM(_GpuComponent):
    """Heterogeneity and the mixing network at init (model.py:1153-1279);
    per tick the infectivity reduce, mixing, draws and weighted selection
    (model.py:1281-1459) and the SEIR counts of log() (model.py:1461-1487)
    run in the engine."""

    def __init__(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = np.arange(len(sim.pars.init_pop))
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1
        self.r0_scalars = np.array(self.pars.r0_scalars)
        self._initialize_people_fields()
        self._initialize_common()

    def _initialize_people_fields(self):
        count = self.people.capacity
        self.people.add_scalar_property("acq_risk_multiplier", dtype=np.float32, default=1.0)
        self.people.add_scalar_property("daily_infectivity", dtype=np.float32, default=1.0)
        populate_heterogeneous_values(0, count, self.people.acq_risk_multiplier, self.people.daily_infectivity, self.pars)

    def _initialize_common(self):
        self.sim.results.add_vector_property("network", length=len(self.sim.nodes), dtype=np.float32)
        init_pops = self.sim.pars.init_pop
        if self.sim.pars.distances is not None:
            dist = np.asarray(self.sim.pars.distances, dtype=np.float64)
        else:
            lookup = self.sim.pars.node_lookup
            ids = sorted(lookup.keys())
            lats = np.array([lookup[i]["lat"] for i in ids])
            lons = np.array([lookup[i]["lon"] for i in ids])
            n = len(self.sim.nodes)
            dist = np.zeros((n, n))
            for i in range(n):
                for j in range(i + 1, n):
                    d = distance(lats[i], lons[i], lats[j], lons[j]) or 1
                    dist[i, j] = dist[j, i] = d
        method = self.pars.migration_method.lower()
        if method == "gravity":
            k = self.pars.gravity_k * 10 ** (self.pars.gravity_k_exponent)
            a, b, c = self.pars.gravity_a, self.pars.gravity_b, self.pars.gravity_c
            net = gravity(init_pops, dist, k, a, b, c)
            net /= np.power(init_pops.sum(), c)
        elif method == "radiation":
            net = radiation(init_pops, dist, 10**self.pars.radiation_k_log10, include_home=False)
        else:
            raise ValueError(f"Unknown migration method: {self.pars.migration_method}")
        self.network = row_normalizer(net, self.pars.max_migr_frac)
        nt, nn, ns = self.sim.nt, len(self.nodes), len(self.pars.strain_ids)
        self.sim.results.add_array_property("new_exposed", shape=(nt, nn), dtype=np.int32)
        self.sim.results.add_array_property("new_exposed_by_strain", shape=(nt, nn, ns), dtype=np.int32)


# ---------------------------------------------------------------------------
class VitalDynamics_ABM(_GpuComponent):
    """Ages, lifespans and birth rates at init (model.py:1522-1687); per tick
    deaths and births (model.py:1689-1757) run in the engine."""

    def __init__(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = sim.nodes
        self.results = sim.results
        self.pars = sim.pars
        self.step_size = self.pars.step_size_VitalDynamics_ABM
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1
        self._initialize_ages_and_births()
        self._initialize_deaths()
        self._initialize_birth_rates()

    def _initialize_ages_and_births(self):
        pars = self.pars
        p = self.people
        p.add_scalar_property("date_of_birth", dtype=np.int32, default=-1)
        pyramid = resolve_pyramid(pars.age_pyramid_path)
        sampler = AliasedDistribution(pyramid[:, 2] + pyramid[:, 3])
        samples = sampler.sample(p.count)
        lo = np.maximum(pyramid[:, 0] * 365, 1)
        hi = (pyramid[:, 1] + 1) * 365
        ages = np.zeros(p.count, dtype=np.int32)
        for i in range(len(pyramid)):
            mask = samples == i
            ages[mask] = np.random.randint(lo[i], hi[i], mask.sum())
        ages[ages == 0] = 1
        p.date_of_birth[: p.count] = -ages

    def _initialize_deaths(self):
        pars = self.pars
        if pars.cbr is None:
            return
        nt, nn = self.sim.nt, len(self.nodes)
        self.results.add_array_property("births", shape=(nt, nn), dtype=np.int32)
        self.results.add_array_property("deaths", shape=(nt, nn), dtype=np.int32)
        self.people.add_scalar_property("date_of_death", dtype=np.int32, default=0)
        cum = lpu.create_cumulative_deaths(np.sum(pars.init_pop), max_age_years=100)
        self.death_estimator = KaplanMeierEstimator(cum)
        ages = -self.people.date_of_birth[: self.people.count]
        lifespans = self.death_estimator.predict_age_at_death(ages, max_year=100)
        self.people.date_of_death[: self.people.count] = lifespans - ages

    def _initialize_birth_rates(self):
        pars = self.pars
        self.birth_rate = np.zeros(len(self.nodes))
        if pars.cbr is not None:
            cbr = np.atleast_1d(pars.cbr)
            if len(cbr) == 1:
                self.birth_rate[:] = cbr[0] / (365 * 1000)
            else:
                self.birth_rate[:] = np.array(cbr) / (365 * 1000)


# ---------------------------------------------------------------------------
class RI_ABM(_GpuComponent):
    """RI timers at init (model.py:1887-1894); per tick the OPV/IPV dosing of
    fast_ri (model.py:1784-1855, 1920-1985) runs in the engine."""

    def __init__(self, sim):
        self.sim = sim
        self.step_size = sim.pars.step_size_RI_ABM
        self.people = sim.people
        self.nodes = sim.nodes
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = self.pars["verbose"] if "verbose" in self.pars else 1
        self.people.add_scalar_property("ri_timer", dtype=np.int16, default=-1)
        dob = self.people.date_of_birth[: self.people.count]
        days = np.random.uniform(42, 98, self.people.count)
        self.people.ri_timer[: self.people.count] = (dob + days).astype(np.int32)
        nt, nn, ns = self.sim.nt, len(self.sim.nodes), len(self.pars.strain_ids)
        r = self.sim.results
        r.add_array_property("ri_vaccinated", shape=(nt, nn), dtype=np.int32)
        r.add_array_property("ri_protected", shape=(nt, nn), dtype=np.int32)
        r.add_array_property("ri_new_exposed_by_strain", shape=(nt, nn, ns), dtype=np.int32)
        r.add_array_property("ipv_vaccinated", shape=(nt, nn), dtype=np.int32)


# ---------------------------------------------------------------------------
class SIA_ABM(_GpuComponent):
    """Campaign schedule at init (model.py:2064-2097); per tick the dosing of
    fast_sia (model.py:1994-2060, 2099-2156) runs in the engine."""

    def __init__(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = sim.nodes
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1
        nt, nn, ns = self.sim.nt, len(self.nodes), len(self.pars.strain_ids)
        self.results.add_array_property("sia_vaccinated", shape=(nt, nn), dtype=np.int32)
        self.results.add_array_property("sia_protected", shape=(nt, nn), dtype=np.int32)
        self.results.add_array_property("sia_new_exposed_by_strain", shape=(nt, nn, ns), dtype=np.int32)
        sched = self.pars["sia_schedule"] if "sia_schedule" in self.pars else None
        self.sia_schedule = [] if sched is None else sched
        for event in self.sia_schedule:
            event["date"] = lpu.date(event["date"])
