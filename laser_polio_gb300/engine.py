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


def make_desc(p: dict):
    """An lpg_sim_desc from plain parameters.

    Keys: n_nodes, n_strains, nt, count, capacity, seed, components (mask),
    stop_if_no_cases, vd_step, birth_rate[n], km_cumdeaths, km_max_year,
    p_paralysis, seeds [(tick, node, is_count, value)], dur_inf (kind, p1, p2),
    ri_step, ri_enabled, ri_strain, vx_prob_ri[n], vx_prob_ipv[n],
    sia [(tick, strain, min_age, max_age, efficacy, node_mask[n])],
    vx_prob_sia[n], strain_r0_scalars[ns], network[n, n], r0_scalars[n],
    seasonality[nt], zero_inflation, nb_r, pop0[n], R_preseed[nt, n] or None.
    Returns (desc, keepalive list).
    """
    keep = []

    def arr(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a

    n = int(p["n_nodes"])
    d = _abi.lpg_sim_desc()
    d.n_nodes = n
    d.n_strains = int(p["n_strains"])
    d.nt = int(p["nt"])
    d.count = int(p["count"])
    d.capacity = int(p["capacity"])
    d.seed = int(p["seed"]) & 0xFFFFFFFFFFFFFFFF
    d.components = int(p["components"])
    d.stop_if_no_cases = int(p.get("stop_if_no_cases", 0))
    d.vd_step = int(p.get("vd_step", 7))
    d.birth_rate = _abi.ptr(arr(_node_vector(p.get("birth_rate", 0.0), n, np.float64), np.float64), _abi.P_f64)
    km = arr(p["km_cumdeaths"], np.int64)
    d.km_cumdeaths = _abi.ptr(km, _abi.P_i64)
    d.km_len = len(km)
    d.km_max_year = int(p.get("km_max_year", 100))
    d.p_paralysis = float(np.float32(p.get("p_paralysis", 1 / 2000)))
    seeds = list(p.get("seeds", []))
    seed_arr = (_abi.lpg_seed_event * max(1, len(seeds)))()
    for i, (t, node, is_count, value) in enumerate(seeds):
        seed_arr[i].tick, seed_arr[i].node, seed_arr[i].is_count, seed_arr[i].value = int(t), int(node), int(is_count), float(value)
    keep.append(seed_arr)
    d.seeds = C.cast(seed_arr, C.POINTER(_abi.lpg_seed_event))
    d.n_seeds = len(seeds)
    kind, p1, p2 = p.get("dur_inf", (0, 1.0, 0.0))
    d.dur_inf = _abi.lpg_dist(int(kind), float(p1), float(p2))
    d.ri_step = int(p.get("ri_step", 14))
    d.ri_enabled = int(p.get("ri_enabled", 0))
    d.ri_strain = int(p.get("ri_strain", 1))
    d.vx_prob_ri = _abi.ptr(arr(_node_vector(p.get("vx_prob_ri", 0.0), n, np.float64), np.float64), _abi.P_f64)
    d.vx_prob_ipv = _abi.ptr(arr(_node_vector(p.get("vx_prob_ipv", 0.0), n, np.float64), np.float64), _abi.P_f64)
    events = list(p.get("sia", []))
    sia_arr = (_abi.lpg_sia_event * max(1, len(events)))()
    for i, (t, st, lo, hi, eff, mask) in enumerate(events):
        e = sia_arr[i]
        e.tick, e.strain, e.min_age, e.max_age, e.efficacy = int(t), int(st), int(lo), int(hi), float(eff)
        e.node_mask = _abi.ptr(arr(mask, np.uint8), _abi.P_u8)
    keep.append(sia_arr)
    d.sia = C.cast(sia_arr, C.POINTER(_abi.lpg_sia_event))
    d.n_sia = len(events)
    if events:
        per_tick = np.bincount([int(e[0]) for e in events])
        if per_tick.max() > _abi.LPG_MAX_SIA_PER_DAY:
            raise ValueError(f"at most {_abi.LPG_MAX_SIA_PER_DAY} SIA events on one day are supported")
    d.vx_prob_sia = _abi.ptr(arr(_node_vector(np.asarray(p.get("vx_prob_sia", 0.0), dtype=np.float32), n, np.float32), np.float32), _abi.P_f32)
    d.strain_r0_scalars = _abi.ptr(arr(p["strain_r0_scalars"], np.float64), _abi.P_f64)
    d.network = _abi.ptr(arr(p["network"], np.float64), _abi.P_f64)
    d.r0_scalars = _abi.ptr(arr(_node_vector(np.asarray(p.get("r0_scalars", 1.0), dtype=np.float64), n, np.float64), np.float64), _abi.P_f64)
    d.seasonality = _abi.ptr(arr(p["seasonality"], np.float64), _abi.P_f64)
    d.zero_inflation = float(p.get("zero_inflation", 0.0))
    d.nb_r = int(p.get("nb_r", 1000))
    d.pop0 = _abi.ptr(arr(p["pop0"], np.int32), _abi.P_i32)
    rp = p.get("R_preseed")
    d.R_preseed = _abi.ptr(arr(rp, np.int32), _abi.P_i32) if rp is not None else None
    return d, keep


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
    p = {"n_nodes": n, "n_strains": ns, "nt": sim.nt, "count": sim.people.count, "capacity": sim.people.capacity,
         "seed": int(pars.seed), "components": mask,
         "stop_if_no_cases": int(bool(pars["stop_if_no_cases"]) and "DiseaseState_ABM" in inst)}

    vd = inst.get("VitalDynamics_ABM")
    p["vd_step"] = int(pars.step_size_VitalDynamics_ABM)
    p["birth_rate"] = vd.birth_rate if vd is not None else np.zeros(n)
    if vd is not None and getattr(vd, "death_estimator", None) is not None:
        p["km_cumdeaths"] = vd.death_estimator.cumulative_deaths
    else:
        p["km_cumdeaths"] = lpu.create_cumulative_deaths(int(np.sum(pars.init_pop)), 100)
    p["km_max_year"] = 100

    p["p_paralysis"] = pars.p_paralysis
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
    p["seeds"] = seeds
    p["dur_inf"] = pars.dur_inf.spec()

    p["ri_step"] = int(pars.step_size_RI_ABM)
    p["ri_enabled"] = int(pars["vx_prob_ri"] is not None and "RI_ABM" in inst)
    p["ri_strain"] = _vaccine_strain(pars["ri_vaccine_type"] if "ri_vaccine_type" in pars else "tOPV")
    p["vx_prob_ri"] = pars["vx_prob_ri"] if pars["vx_prob_ri"] is not None else 0.0
    p["vx_prob_ipv"] = pars["vx_prob_ipv"] if pars["vx_prob_ipv"] is not None else 0.0

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
            events.append((t, _vaccine_strain(vt), int(min_age), int(max_age), float(pars["vx_efficacy"][vt]), node_mask))
    p["sia"] = events
    p["vx_prob_sia"] = pars.vx_prob_sia if pars.vx_prob_sia is not None else 0.0

    tx = inst.get("Transmission_ABM")
    p["strain_r0_scalars"] = np.array(list(pars.strain_r0_scalars.values()), dtype=np.float64)[:ns]
    p["network"] = tx.network if tx is not None else np.zeros((n, n))
    p["r0_scalars"] = np.asarray(pars.r0_scalars, dtype=np.float64)
    p["seasonality"] = lpu.seasonality_table(sim.datevec, pars["seasonal_amplitude"], pars["seasonal_peak_doy"])
    p["zero_inflation"] = float(pars.node_seeding_zero_inflation)
    p["nb_r"] = int(max(1, int(np.round(pars.node_seeding_dispersion))))

    results = {}
    for name, _ in _abi.RESULT_FIELDS:
        a = getattr(sim.results, name, None)
        if isinstance(a, np.ndarray) and a.dtype == np.int32:
            results[name] = a
    pop = results.get("pop")
    p["pop0"] = pop[0] if pop is not None else np.asarray(pars.init_pop)
    Rres = results.get("R")
    p["R_preseed"] = Rres if (Rres is not None and np.any(Rres)) else None
    d, keep = make_desc(p)

    # each column as it lives: a device-resident tensor, or the host array
    people = sim.people
    if hasattr(people, "engine_columns"):
        columns = people.engine_columns([name for name, _, _ in _abi.COLUMN_FIELDS])
    else:  # a LaserFrame of another package: host arrays
        columns = {name: getattr(people, name) for name, _, _ in _abi.COLUMN_FIELDS
                   if isinstance(getattr(people, name, None), np.ndarray)}
    for name, _, dtype in _abi.COLUMN_FIELDS:
        a = columns.get(name)
        if isinstance(a, np.ndarray) and (a.dtype != dtype or not a.flags["C_CONTIGUOUS"]):
            raise TypeError(f"people.{name} must be a contiguous {np.dtype(dtype).name} array")
    return SimSpec(d, keep, columns, results)


def _advance_count(people, count: int) -> None:
    """Bring people.count to the engine's count through LaserFrame's public
    add(n), as laser_core's LaserFrame advances it (births only grow it)."""
    n = int(count) - int(people.count)
    if n < 0:
        raise RuntimeError(f"engine count {count} is below people.count {people.count}")
    if n:
        people.add(n)


def _check_node_ids(spec) -> None:
    """node_id of the first count slots within [0, n_nodes) (lpg_start
    checks the same on the device for the whole handle); a device-resident
    column is checked where it lives."""
    n, count = spec.desc.n_nodes, spec.desc.count
    node = spec.columns.get("node_id")
    if node is not None and count and (int(node[:count].min()) < 0 or int(node[:count].max()) >= n):
        raise ValueError(f"LPG_ERR_NODE: node_id outside [0, {n}) among the first {count} slots")


def host_columns(spec) -> dict:
    """Copies of a spec's columns on the host (numpy), wherever they live."""
    return {k: (v.copy() if isinstance(v, np.ndarray) else v.cpu().numpy().copy()) for k, v in spec.columns.items()}


def _autotune_key(handle_sims, sims):
    import torch

    from . import autotune

    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    nodes = sum(len(s.nodes) for s in sims)
    agents = sum(int(s.people.count) for s in sims)
    return autotune.workload_key(props.name, props.multi_processor_count, len(sims), nodes, agents), \
        props.multi_processor_count


def run_replicates(sims, autotune=False) -> list:
    """Run several SEIR_ABM (drop-in GPU components) as one batch: one
    handle, one launch sequence per tick for all of them.  The reference's
    calibration runs its replicates one after another, each in its own
    try/except, so that a failing replicate is reported and the others go on
    (calib/objective.py:47-70).  The same holds here:
      - each sim's description and node ids are checked on the host first
        (lpg_check_desc); a sim that fails is left out of the batch;
      - on the device a sim that fails (births beyond its capacity, a
        timed-out wait) stops at that tick while the others run to their end.
    The sims may differ in nodes, agents, durations and components; each
    stops at its own last tick or stop rule.  With ``autotune`` the tick
    kernels' grid sizes are picked on the run's first ticks, or taken from
    the on-disk cache for the same kind of batch (autotune.py); the results
    are the same either way.  Every sim that ran holds what
    its own run() would have left (results, people columns and count, t and
    should_stop; a failed one as far as it got).  Returns one entry per sim:
    None, or the exception its run raised (ValueError for bad parameters,
    node ids and capacity, as the reference; LpgError otherwise).  A failure
    of the whole device (a CUDA error) raises."""
    sims = list(sims)
    errors = [None] * len(sims)
    if not sims:
        return errors
    ok, specs = [], []
    for i, s in enumerate(sims):
        try:
            sp = build_sim_spec(s)
            _lib.check_desc(sp.desc)
            _check_node_ids(sp)
        except (ValueError, TypeError, _lib.LpgError) as exc:
            errors[i] = exc
            continue
        ok.append(i)
        specs.append(sp)
    if not ok:
        return errors
    handle = _lib.Handle([sp.desc for sp in specs])
    try:
        for j, sp in enumerate(specs):
            handle.bind_columns(j, sp.columns)
        handle.start()
        remaining = max(int(sims[i].nt) for i in ok) - 1
        if autotune and remaining > 0:
            from . import autotune as _tune

            key, sm_count = _autotune_key(specs, [sims[i] for i in ok])
            _, stepped = _tune.tune(handle, key, sm_count)
            remaining -= stepped
        if remaining > 0:
            handle.step(remaining)
        statuses = handle.sync_statuses()
        for j, (i, sp) in enumerate(zip(ok, specs)):
            sim = sims[i]
            handle.read_results(j, sp.results)
            handle.read_columns(j, sp.columns)
            st = handle.state(j, check=False)
            _advance_count(sim.people, st.count)
            sim.t = st.t
            sim.should_stop = bool(st.stopped)
            if statuses[j]:
                errors[i] = _lib.error_for(statuses[j], f"replicate {i}: device error at tick {st.t}")
    finally:
        handle.close()
    return errors


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
        _advance_count(self.sim.people, st.count)
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
