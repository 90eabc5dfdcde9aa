"""SEIR_ABM and the five drop-in components.

Each class has the reference's name, takes the reference's ``pars`` and
fills the reference's ``sim.results`` arrays; the names matter because the
components setter keeps and orders classes by ``__name__``
(laser_polio/model.py:226-237).

Construction.  SEIR_ABM and each component describe what their slice of the
agent table holds (an init.InitSpec: population per node, how many agents
are missed, immune, infected, the timer and heterogeneity distributions,
the age pyramid, the lifespan table) and the device fills it
(init.fill -> lpg_init_columns): the columns are device-resident from the
start, and reading one by attribute brings it to the host.  Small per-run
state (results arrays, the network, schedules, birth rates) is built on the
host.

Running.  Every per-tick ``step()`` and ``log()`` goes to the sim's GpuTick
engine (engine.py), created on first use, which runs the whole tick on the
GPU through the C ABI of include/lpg.h.
"""

from __future__ import annotations

import time
from collections import defaultdict
from copy import deepcopy
from datetime import datetime

import numpy as np

from . import _abi
from . import init as _init
from . import pars as _pars
from . import utils as lpu
from .core import KaplanMeierEstimator
from .core import LaserFrame
from .core import PropertySet
from .core import calc_capacity
from .core import distance
from .core import gravity
from .core import radiation
from .core import resolve_pyramid
from .core import row_normalizer

__all__ = ["RI_ABM", "SEIR_ABM", "SIA_ABM", "DiseaseState_ABM", "Transmission_ABM", "VitalDynamics_ABM",
           "populate_heterogeneous_values"]


class TimingStats:
    """Wall time per label, in ns, under the labels the reference uses
    (laser_polio/utils.py:819-945)."""

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


def capacity_for(total, pars) -> int:
    """Agent slots for a run: everyone present at the start and everyone born
    within the run's duration plus 100 days at the (mean) crude birth rate,
    times a margin 1 + 4/sqrt(births) that narrows as births grow; without
    births, just the starting population (model.py:118-137)."""
    if pars.cbr is None:
        return int(total)
    rate = float(np.mean(np.atleast_1d(pars.cbr)))
    births = calc_capacity(total, pars.dur + 100, rate) - total
    if births <= 0:
        return int(total)
    return int((1.0 + 4.0 / np.sqrt(births)) * (total + births))


def _spec_of(sim) -> _init.InitSpec:
    """The sim's initialisation description, created from its pars and
    people when the sim was not built by this package's SEIR_ABM."""
    spec = getattr(sim, "_init", None)
    if spec is None:
        pops = np.atleast_1d(sim.pars.init_pop).astype(np.int64)
        spec = _init.InitSpec(sim.pars.seed if sim.pars.seed is not None else 0, pops, sim.people.count,
                              sim.people.capacity)
        sim._init = spec
    return spec


class SEIR_ABM:
    """Agent-based SEIR polio model (laser_polio/model.py:51-342).

    Disease state codes: -1 dead or not yet born, 0 S, 1 E, 2 I, 3 R.
    """

    def common_init(self, pars, verbose):
        """Parameters (defaults overridden by ``pars``; unknown keys dropped
        with a warning), the seed, and the time axis."""
        self.perf_stats = TimingStats()
        merged = deepcopy(_pars.default_pars)
        if pars is not None:
            given = pars.to_dict() if isinstance(pars, PropertySet) else dict(pars)
            unknown = sorted(set(given) - set(merged.keys()))
            if unknown:
                print(f"Warning: ignoring unexpected parameters: {unknown}")
                given = {k: v for k, v in given.items() if k in merged}
            merged <<= given
        self.pars = merged
        self.verbose = merged["verbose"] if "verbose" in merged else verbose
        if merged.seed is None:
            stamp = datetime.now()  # noqa: DTZ005  (a seed from the clock, as the reference does)
            merged.seed = stamp.microsecond ^ int(stamp.timestamp())
            if self.verbose >= 1:
                print(f"No seed provided. Using random seed of {merged.seed}.")
        self.t = 0
        self.nt = merged.dur + 1
        self.datevec = lpu.daterange(merged["start_date"], days=self.nt)
        self.should_stop = False

    def __init__(self, pars: PropertySet = None, verbose=1):
        self.common_init(pars, verbose)
        p = self.pars
        p.init_pop = np.atleast_1d(p.init_pop).astype(int)
        if p.init_sus_by_age is not None:
            raise NotImplementedError("init_sus_by_age (real-data initialisation through run_sim) is not supported")
        pops = p.init_pop
        if np.any(pops <= 0) or np.any(np.isnan(pops)):
            raise ValueError("pop_by_node must be positive & non-nan")
        total = int(pops.sum())
        self.people = LaserFrame(capacity=capacity_for(total, p), initial_count=total)
        self.results = LaserFrame(capacity=1)
        self.nodes = np.arange(len(pops))
        self._init = _init.InitSpec(p.seed, pops, total, self.people.capacity)
        self._init.missed_k = _init.missed_count(p.missed_frac, total)
        _init.fill(self.people, self._init, _abi.INIT_BASE | _abi.INIT_MISSED)
        self._components = []
        self.instances = []
        self._engine = None

    @classmethod
    def init_from_file(cls, people: LaserFrame, pars: PropertySet = None):
        """A model around an agent table loaded from a snapshot
        (model.py:177-195): the people as they are, the nodes they live in,
        empty results and no components yet."""
        model = cls.__new__(cls)
        model.common_init(pars, verbose=2)
        model.people = people
        model.nodes = np.unique(people.node_id[: people.count])
        model.results = LaserFrame(capacity=1)
        model._engine = None
        model.components = []
        return model

    @property
    def components(self) -> list:
        return self._components

    @components.setter
    def components(self, components: list) -> None:
        by_name = {cls.__name__: cls for cls in components}
        self._components = [by_name[name] for name in _pars.default_run_order if name in by_name]
        self.instances = []
        for cls in self._components:
            with self.perf_stats.start(cls.__name__ + ".__init__()"):
                self.instances.append(cls(self))
        self._engine = None

    def run(self):
        """SEIR_ABM.run (model.py:246-282).  With drop-in components only,
        the whole loop runs on the device in one call, with the same result
        as the per-tick loop below (kept for component sets that mix in host
        classes)."""
        if self.instances and all(isinstance(c, _GpuComponent) for c in self.instances):
            with self.perf_stats.start("GpuTick.run()"):
                _engine_of(self).run_all()
            if self.should_stop and self.verbose >= 1:
                print(f"[SEIR_ABM] Early stopping at t={self.t}: no E/I and no future seed_schedule events.")
            return
        for tick in range(self.nt):
            if tick > 0:
                for component in self.instances:
                    with self.perf_stats.start(component.__class__.__name__ + ".step()"):
                        component.step()
            self.log_results(tick)
            self.t += 1
            if tick > 0 and self.should_stop:
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


def _results(sim, names, wide=False):
    nt, nn, ns = sim.nt, len(sim.nodes), len(sim.pars.strain_ids)
    for name in names:
        sim.results.add_array_property(name, shape=(nt, nn, ns) if wide else (nt, nn), dtype=np.int32)


# ---------------------------------------------------------------------------
class DiseaseState_ABM(_GpuComponent):
    """E -> I -> R progression, paralysis, the seed schedule and the stop
    rule (model.py:505-812).  At construction: the results arrays, the
    timers of every slot, the immune and the initially infected agents
    (filled on the device)."""

    def _common_init(self, sim):
        self.sim = sim
        self.people = sim.people
        self.pars = sim.pars
        self.nodes = sim.nodes
        self.results = sim.results
        self.verbose = self.pars["verbose"] if "verbose" in self.pars else 1
        # tick -> [(node, prevalence)]; entries by date name their node by dot_name
        self.seed_schedule = defaultdict(list)
        lookup = self.pars.node_lookup or {}
        start = lpu.date(self.pars.start_date)
        for entry in self.pars.seed_schedule or []:
            if "date" in entry and "dot_name" in entry:
                node = next((nid for nid, info in lookup.items() if info["dot_name"] == entry["dot_name"]), None)
                if node is not None:
                    self.seed_schedule[(lpu.date(entry["date"]) - start).days].append((node, entry["prevalence"]))
            elif "timestep" in entry and "node_id" in entry:
                self.seed_schedule[entry["timestep"]].append((entry["node_id"], entry["prevalence"]))

    def _initialize_results_arrays(self):
        _results(self.sim, ("S", "E", "I", "R", "potentially_paralyzed", "paralyzed", "new_potentially_paralyzed",
                            "new_paralyzed", "pop"))
        _results(self.sim, ("E_by_strain", "I_by_strain"), wide=True)
        self.results.pop[0] = self.sim.pars.init_pop

    def __init__(self, sim):
        self._common_init(sim)
        self._initialize_results_arrays()
        pars = self.pars
        spec = _spec_of(sim)
        spec.dur_exp, spec.dur_inf, spec.t_to_paralysis = (pars.dur_exp.spec(), pars.dur_inf.spec(),
                                                           pars.t_to_paralysis.spec())
        spec.immune_k = _init.immune_counts(pars.init_immun, pars.init_pop)
        spec.prev_per_node, spec.prev_k = _init.prevalence_counts(pars.init_prev, pars.init_pop)
        _init.fill(sim.people, spec, _abi.INIT_TIMERS | _abi.INIT_IMMUNITY | _abi.INIT_PREVALENCE)

    @classmethod
    def init_from_file(cls, sim):
        """For a loaded agent table (model.py:506-524): results arrays, and
        for the unborn slots fresh timers and heterogeneity, with their
        paralysis and IPV flags at -1 as the reference leaves them."""
        self = cls.__new__(cls)
        self._common_init(sim)
        self._initialize_results_arrays()
        p = sim.people
        count, cap = p.count, getattr(p, "true_capacity", p.capacity)
        populate_heterogeneous_values(count, cap, p.acq_risk_multiplier, p.daily_infectivity, self.pars)
        et, it, pt = _unborn_timers(sim, count, cap)
        p.exposure_timer[count:cap], p.infection_timer[count:cap], p.paralysis_timer[count:cap] = et, it, pt
        p.potentially_paralyzed[count:cap] = -1
        p.paralyzed[count:cap] = -1
        p.ipv_protected[count:cap] = -1
        return self


def _slice_of_fresh_init(pars, capacity, parts, start, end, **fields):
    """Columns of a fresh initialisation over [start, end): the draws are
    keyed by slot, so these are the values those slots get in a table of
    ``end`` slots."""
    people = LaserFrame(capacity=end, initial_count=0)
    spec = _init.InitSpec(pars.seed if pars.seed is not None else 0, np.zeros(1, np.int64), 0, end)
    for k, v in fields.items():
        setattr(spec, k, v)
    _init.fill(people, spec, parts)
    return {name: np.asarray(getattr(people, name))[start:end] for name in _init.part_columns(parts)}


def _unborn_timers(sim, start, end):
    pars = sim.pars
    cols = _slice_of_fresh_init(pars, end, _abi.INIT_TIMERS, start, end, dur_exp=pars.dur_exp.spec(),
                                dur_inf=pars.dur_inf.spec(), t_to_paralysis=pars.t_to_paralysis.spec())
    return cols["exposure_timer"], cols["infection_timer"], cols["paralysis_timer"]


def populate_heterogeneous_values(start, end, acq_risk_out, infectivity_out, pars):
    """Acquisition risk and daily infectivity of slots [start, end)
    (model.py:816-866), correlated lognormal risk and exponential
    infectivity, drawn on the device as the initialisation draws them."""
    cols = _slice_of_fresh_init(pars, end, _abi.INIT_HETEROGENEITY, start, end,
                                heterogeneity=pars.individual_heterogeneity, risk_mult_var=pars.risk_mult_var,
                                corr_risk_inf=pars.corr_risk_inf, r0=pars.r0, dur_inf=pars.dur_inf.spec())
    acq_risk_out[start:end] = cols["acq_risk_multiplier"]
    infectivity_out[start:end] = cols["daily_infectivity"]


# ---------------------------------------------------------------------------
class Transmission_ABM(_GpuComponent):
    """Mixing, draws and weighted selection of the exposed, and the SEIR
    counts (model.py:1152-1491).  At construction: the migration network,
    the results arrays and every slot's acquisition risk and daily
    infectivity (filled on the device)."""

    def _bind(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = np.arange(len(sim.pars.init_pop))
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1
        self.r0_scalars = np.array(self.pars.r0_scalars)

    def __init__(self, sim):
        self._bind(sim)
        spec = _spec_of(sim)
        p = self.pars
        spec.heterogeneity = p.individual_heterogeneity
        spec.risk_mult_var, spec.corr_risk_inf, spec.r0 = p.risk_mult_var, p.corr_risk_inf, p.r0
        spec.dur_inf = p.dur_inf.spec()
        _init.fill(sim.people, spec, _abi.INIT_HETEROGENEITY)
        self._initialize_common()

    @classmethod
    def init_from_file(cls, sim):
        """For a loaded agent table (model.py:1169-1188): infectivity scaled
        by r0 / old_r0 when the run's R0 differs from the stored one."""
        self = cls.__new__(cls)
        self._bind(sim)
        old = sim.pars["old_r0"] if "old_r0" in sim.pars else sim.pars.r0
        if sim.pars.r0 != old:
            sim.people.daily_infectivity *= sim.pars.r0 / old
        self._initialize_common()
        return self

    def _distances(self):
        if self.sim.pars.distances is not None:
            return np.asarray(self.sim.pars.distances, dtype=np.float64)
        lookup = self.sim.pars.node_lookup
        ids = sorted(lookup.keys())
        lat = np.array([lookup[i]["lat"] for i in ids])
        lon = np.array([lookup[i]["lon"] for i in ids])
        n = len(self.sim.nodes)
        d = np.zeros((n, n))
        for i in range(n):
            for j in range(i + 1, n):
                d[i, j] = d[j, i] = distance(lat[i], lon[i], lat[j], lon[j]) or 1.0  # a zero distance counts as 1
        return d

    def _initialize_common(self):
        """The network (model.py:1213-1258): gravity scaled by the total
        population to the power c, or radiation; then rows capped at
        max_migr_frac."""
        self.sim.results.add_vector_property("network", length=len(self.sim.nodes), dtype=np.float32)
        pops = self.sim.pars.init_pop
        dist = self._distances()
        method = self.pars.migration_method.lower()
        if method == "gravity":
            p = self.pars
            k = p.gravity_k * 10 ** p.gravity_k_exponent
            net = gravity(pops, dist, k, p.gravity_a, p.gravity_b, p.gravity_c) / np.power(pops.sum(), p.gravity_c)
        elif method == "radiation":
            net = radiation(pops, dist, 10 ** self.pars.radiation_k_log10, include_home=False)
        else:
            raise ValueError(f"Unknown migration method: {self.pars.migration_method}")
        self.network = row_normalizer(net, self.pars.max_migr_frac)
        _results(self.sim, ("new_exposed",))
        _results(self.sim, ("new_exposed_by_strain",), wide=True)


# ---------------------------------------------------------------------------
class VitalDynamics_ABM(_GpuComponent):
    """Births and deaths (model.py:1521-1765).  At construction: the results
    arrays, birth rates, the lifespan table, and every initial agent's date
    of birth and of death (filled on the device)."""

    def _bind(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = sim.nodes
        self.results = sim.results
        self.pars = sim.pars
        self.step_size = self.pars.step_size_VitalDynamics_ABM
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1

    def __init__(self, sim):
        self._bind(sim)
        spec = _spec_of(sim)
        spec.age_lo, spec.age_hi, spec.age_weight = _init.age_bins(resolve_pyramid(self.pars.age_pyramid_path))
        parts = _abi.INIT_AGES
        self.death_estimator = None
        if self.pars.cbr is not None:
            _results(sim, ("births", "deaths"))
            cum = lpu.create_cumulative_deaths(np.sum(self.pars.init_pop), max_age_years=100)
            self.death_estimator = KaplanMeierEstimator(cum)
            spec.km, spec.km_max_year = np.asarray(cum, np.int64), 100
            parts |= _abi.INIT_DEATHS
        _init.fill(sim.people, spec, parts)
        self._initialize_birth_rates()

    @classmethod
    def init_from_file(cls, sim):
        """For a loaded agent table (model.py:1528-1537): results arrays if
        missing, birth rates and the lifespan table."""
        self = cls.__new__(cls)
        self._bind(sim)
        for name in ("births", "deaths"):
            if not isinstance(getattr(sim.results, name, None), np.ndarray):
                _results(sim, (name,))
        self._initialize_birth_rates()
        self.death_estimator = KaplanMeierEstimator(lpu.create_cumulative_deaths(np.sum(self.pars.init_pop), 100))
        return self

    def _initialize_birth_rates(self):
        """Per-node daily births per person: cbr / (365 * 1000)."""
        self.birth_rate = np.zeros(len(self.nodes))
        if self.pars.cbr is not None:
            cbr = np.atleast_1d(np.asarray(self.pars.cbr, dtype=np.float64))
            self.birth_rate[:] = (cbr[0] if len(cbr) == 1 else cbr) / (365 * 1000)


# ---------------------------------------------------------------------------
class RI_ABM(_GpuComponent):
    """Routine immunisation (model.py:1858-1992).  At construction: the
    results arrays and every initial agent's RI date (filled on the
    device)."""

    def _bind(self, sim):
        self.sim = sim
        self.step_size = sim.pars.step_size_RI_ABM
        self.people = sim.people
        self.nodes = sim.nodes
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = self.pars["verbose"] if "verbose" in self.pars else 1
        _results(sim, ("ri_vaccinated", "ri_protected", "ipv_vaccinated"))
        _results(sim, ("ri_new_exposed_by_strain",), wide=True)

    def __init__(self, sim):
        self._bind(sim)
        if not sim.people.has_column("date_of_birth"):
            raise AttributeError("RI_ABM needs people.date_of_birth (VitalDynamics_ABM sets it)")
        _init.fill(sim.people, _spec_of(sim), _abi.INIT_RI)

    @classmethod
    def init_from_file(cls, sim):
        """For a loaded agent table (model.py:1872-1885): the RI dates are
        kept; only the results arrays."""
        self = cls.__new__(cls)
        self._bind(sim)
        return self


# ---------------------------------------------------------------------------
class SIA_ABM(_GpuComponent):
    """Campaigns (model.py:2063-2163).  At construction: the results arrays
    and the schedule with its dates parsed."""

    def __init__(self, sim):
        self.sim = sim
        self.people = sim.people
        self.nodes = sim.nodes
        self.pars = sim.pars
        self.results = sim.results
        self.verbose = sim.pars["verbose"] if "verbose" in sim.pars else 1
        _results(sim, ("sia_vaccinated", "sia_protected"))
        _results(sim, ("sia_new_exposed_by_strain",), wide=True)
        schedule = self.pars["sia_schedule"] if "sia_schedule" in self.pars else None
        self.sia_schedule = [] if schedule is None else schedule
        for event in self.sia_schedule:
            event["date"] = lpu.date(event["date"])

    @classmethod
    def init_from_file(cls, sim):
        return cls(sim)
