"""GpuTick: the device engine behind the drop-in components.

One ``GpuTick`` per SEIR_ABM.  On the first ``step()`` or ``log()`` it turns
``sim.pars``/``sim.people``/``sim.results`` into the plain C structures of
include/lpg.h (``build_sim_spec``), uploads the agent columns, and from then
on runs each tick on the GPU.  The host copies of the columns and results
are refreshed when the run ends (last tick or early stop), which is when the
reference's callers read them.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from . import _lib
from . import utils as lpu


class SimSpec:
    """An lpg_sim_desc plus the numpy arrays its pointers refer to."""

    def __init__(self, desc, keep, columns, results):
        self.desc = desc
        self._keep = keep
        self.columns = columns  # name -> numpy column (reference slot order)
        self.results = results  # name -> numpy result array present in sim.results


def _vaccine_strain(vaccinetype: str) -> int:
    # model.py:1934-1940 and 2115-2120
    if "nOPV" in vaccinetype:
        return 2
    if any(v in vaccinetype for v in ["mOPV", "tOPV", "topv"]):
        return 1
    return 1


def _node_vector(value, n, dtype):
    arr = np.asarray(value, dtype=dtype)
    if arr.ndim == 0:
        arr = np.full(n, arr, dtype=dtype)
    return np.ascontiguousarray(np.broadcast_to(arr, (n,)), dtype=dtype)


def build_sim_spec(sim) -> SimSpec:
    """Describe ``sim`` (an SEIR_ABM with drop-in components) for the C ABI."""
    pars = sim.pars
    names = {c.__name__ if isinstance(c, type) else type(c).__name__ for c in sim.components}
    mask = 0
    for name, bit in _abi.COMPONENT_BITS.items():
        if name in names:
            mask |= bit
    inst = {type(c).__name__: c for c in sim.instances}
    n = len(sim.nodes)
    ns = len(pars.strain_ids)
    if ns > _abi.LPG_MAX_STRAINS:
        raise ValueError(f"at most {_abi.LPG_MAX_STRAINS} strains are supported, got {ns}")
    keep = []

    def arr(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a

    d = _abi.lpg_sim_desc()
    d.n_nodes = n
    d.n_strains = ns
    d.nt = sim.nt
    d.count = sim.people.count
    d.capacity = sim.people.capacity
    d.seed = int(pars.seed) & 0xFFFFFFFFFFFFFFFF
    d.components = mask
    d.stop_if_no_cases = int(bool(pars["stop_if_no_cases"]) and "DiseaseState_ABM" in inst)

    vd = inst.get("VitalDynamics_ABM")
    d.vd_step = int(pars.step_size_VitalDynamics_ABM)
    d.birth_rate = _abi.ptr(arr(vd.birth_rate if vd is not None else np.zeros(n), np.float64), _abi.P_f64)
    if vd is not None and getattr(vd, "death_estimator", None) is not None:
        km = arr(vd.death_estimator.cumulative_deaths, np.int64)
    else:
        km = arr(lpu.create_cumulative_deaths(int(np.sum(pars.init_pop)), 100), np.int64)
    d.km_cumdeaths = _abi.ptr(km, _abi.P_i64)
    d.km_len = len(km)
    d.km_max_year = 100

    d.p_paralysis = float(np.float32(pars.p_paralysis))
    seeds = []
    ds = inst.get("DiseaseState_ABM")
    if ds is not None:
        for t, entries in ds.seed_schedule.items():
            for node, value in entries:
                if isinstance(value, float):
                    seeds.append((int(t), int(node), 0, float(value)))
                elif isinstance(value, (int, np.integer)):
                    seeds.append((int(t), int(node), 1, float(value)))
                else:
                    raise ValueError(f"Unsupported seed value type: {type(value)}")
    seed_arr = (_abi.lpg_seed_event * max(1, len(seeds)))()
    for i, (t, node, is_count, value) in enumerate(seeds):
        seed_arr[i].tick, seed_arr[i].node, seed_arr[i].is_count, seed_arr[i].value = t, node, is_count, value
    keep.append(seed_arr)
    d.seeds = C.cast(seed_arr, C.POINTER(_abi.lpg_seed_event))
    d.n_seeds = len(seeds)
    kind, p1, p2 = pars.dur_inf.spec()
    d.dur_inf = _abi.lpg_dist(kind, p1, p2)

    d.ri_step = int(pars.step_size_RI_ABM)
    d.ri_enabled = int(pars["vx_prob_ri"] is not None and "RI_ABM" in inst)
    d.ri_strain = _vaccine_strain(getattr(pars, "ri_vaccine_type", "tOPV") if "ri_vaccine_type" in pars else "tOPV")
    d.vx_prob_ri = _abi.ptr(arr(_node_vector(pars["vx_prob_ri"] if pars["vx_prob_ri"] is not None else 0.0, n, np.float64), np.float64), _abi.P_f64)
    ipv = pars["vx_prob_ipv"] if pars["vx_prob_ipv"] is not None else 0.0
    d.vx_prob_ipv = _abi.ptr(arr(_node_vector(ipv, n, np.float64), np.float64), _abi.P_f64)

    sia = inst.get("SIA_ABM")
    events = []
    if sia is not None and pars.vx_prob_sia is not None:
        start = lpu.date(pars.start_date)
        for ev in sia.sia_schedule:
            t = (lpu.date(ev["date"]) - start).days
            if t < 1 or t >= sim.nt:
                continue
            node_mask = np.zeros(n, np.uint8)
            node_mask[ev["nodes"]] = 1
            min_age, max_age = ev["age_range"]
            vt = ev["vaccinetype"]
            events.append((t, _vaccine_strain(vt), int(min_age), int(max_age), float(pars["vx_efficacy"][vt]), arr(node_mask, np.uint8)))
    sia_arr = (_abi.lpg_sia_event * max(1, len(events)))()
    for i, (t, st, lo, hi, eff, m) in enumerate(events):
        e = sia_arr[i]
        e.tick, e.strain, e.min_age, e.max_age, e.efficacy = t, st, lo, hi, eff
        e.node_mask = _abi.ptr(m, _abi.P_u8)
    keep.append(sia_arr)
    d.sia = C.cast(sia_arr, C.POINTER(_abi.lpg_sia_event))
    d.n_sia = len(events)
    if events:
        counts_per_tick = np.bincount([e[0] for e in events])
        if counts_per_tick.max() > _abi.LPG_MAX_SIA_PER_DAY:
            raise ValueError(f"at most {_abi.LPG_MAX_SIA_PER_DAY} SIA events on one day are supported")
    vps = pars.vx_prob_sia if pars.vx_prob_sia is not None else np.zeros(n)
    d.vx_prob_sia = _abi.ptr(arr(_node_vector(np.asarray(vps, dtype=np.float32), n, np.float32), np.float32), _abi.P_f32)

    tx = inst.get("Transmission_ABM")
    d.strain_r0_scalars = _abi.ptr(arr(np.array(list(pars.strain_r0_scalars.values()), dtype=np.float64)[:ns], np.float64), _abi.P_f64)
    net = tx.network if tx is not None else np.zeros((n, n))
    d.network = _abi.ptr(arr(net, np.float64), _abi.P_f64)
    d.r0_scalars = _abi.ptr(arr(_node_vector(np.asarray(pars.r0_scalars, dtype=np.float64), n, np.float64), np.float64), _abi.P_f64)
    d.seasonality = _abi.ptr(arr(lpu.seasonality_table(sim.datevec, pars["seasonal_amplitude"], pars["seasonal_peak_doy"]), np.float64), _abi.P_f64)
    d.zero_inflation = float(pars.node_seeding_zero_inflation)
    d.nb_r = int(max(1, int(np.round(pars.node_seeding_dispersion))))

    results = {}
    for name, _ in _abi.RESULT_FIELDS:
        a = getattr(sim.results, name, None)
        if isinstance(a, np.ndarray) and a.dtype == np.int32:
            results[name] = a
    pop = results.get("pop")
    pop0 = arr(pop[0] if pop is not None else np.asarray(pars.init_pop), np.int32)
    d.pop0 = _abi.ptr(pop0, _abi.P_i32)
    Rres = results.get("R")
    if Rres is not None and np.any(Rres):
        d.R_preseed = _abi.ptr(arr(Rres, np.int32), _abi.P_i32)
    else:
        d.R_preseed = None

    columns = {}
    for name, _, dtype in _abi.COLUMN_FIELDS:
        a = getattr(sim.people, name, None)
        if isinstance(a, np.ndarray):
            if a.dtype != dtype or not a.flags["C_CONTIGUOUS"]:
                raise TypeError(f"people.{name} must be a contiguous {np.dtype(dtype).name} array")
            columns[name] = a
    return SimSpec(d, keep, columns, results)


class GpuTick:
    """Runs the components' per-tick work of one SEIR_ABM on the GPU."""

    def __init__(self, sim):
        self.sim = sim
        self.handle = None
        self.spec = None
        self._tick_done = -1
        self._log_done = -1
        self._finished = False

    # -- lifecycle -----------------------------------------------------------
    def _ensure_started(self):
        if self.handle is not None:
            return
        self.spec = build_sim_spec(self.sim)
        self.handle = _lib.Handle([self.spec.desc])
        self.handle.bind_columns(0, self.spec.columns)
        self.handle.start()

    def _finish(self):
        """Copy device results and columns back into the host arrays."""
        if self._finished:
            return
        self.handle.sync()
        self.handle.read_results(0, self.spec.results)
        self.handle.read_columns(0, self.spec.columns)
        st = self.handle.state(0)
        self.sim.people._set_count(st.count)
        self._finished = True

    # -- per-tick interface used by the components ----------------------------
    def step(self, component):
        self._ensure_started()
        t = self.sim.t
        if t == self._tick_done:
            return
        st = self.handle.state(0)
        if st.t != t:
            raise RuntimeError(f"engine is at tick {st.t} but the model is at tick {t}")
        self.handle.step(1)
        self._tick_done = t
        if self.spec.desc.stop_if_no_cases:
            st = self.handle.state(0)
            if st.stopped:
                self.sim.should_stop = True

    def log(self, component, t):
        self._ensure_started()
        if t == self._log_done:
            return
        self._log_done = t
        if t >= self.sim.nt - 1 or self.sim.should_stop:
            self._finish()

    def run_all(self):
        """All ticks on the device, then one copy back."""
        self._ensure_started()
        self.handle.step(self.sim.nt - 1)
        self.handle.sync()
        st = self.handle.state(0)
        self.sim.t = st.t
        self.sim.should_stop = bool(st.stopped)
        self._finish()

    def close(self):
        if self.handle is not None:
            self.handle.close()
            self.handle = None
