"""Seeded synthetic populations with the shapes of the benchmark workloads.

The reference is quoted on real Nigerian data (node lookup, age pyramid,
immunity tables) that does not ship with it; these generators stand in for
that data with seeded numpy draws of the stated shapes, sizes and
distributions:

  zamfara_like   14 nodes, 1e6 agents: node pops lognormal(ln 7e4, 0.6)
                 rescaled to the total; exponential age pyramid (mean 20 y,
                 0-80 y); everyone over 15 y recovered and 80% of under-15s;
                 10 infections in each of 2 random nodes; gravity network
                 (k 0.5, a 1, b 1, c 2) on coordinates uniform in a 200 km
                 square, max export 0.2; R0 14, seasonal amplitude 0.4 peaking
                 on day 180, r0_scalars lognormal(0, 0.3); exposure gamma(mean
                 3 d, shape 3), infection gamma(mean 24 d, shape 4); risk and
                 infectivity correlated lognormals (sigma 0.8, rho 0.8); CBR 35,
                 RI coverage 50%; 365 ticks; seed 42.
  nigeria_like   the same recipe at 774 nodes / 2.2e8 agents with node pops
                 lognormal(ln 2.8e5, 0.7), under-15 immunity U(0.4, 0.9) per
                 node, three strains, RI coverage beta(6, 4), an SIA every
                 180 d over 30% of nodes (ages 0-5 y, coverage beta(8, 3),
                 efficacy 0.6), CBR 37, 2555 ticks.

Both return a fully initialised SEIR_ABM with the five drop-in components.
For the full sizes, ``bundle`` builds the same recipe directly as
reference-ordered column arrays (no SEIR_ABM, no per-agent Python), in
parallel chunks on the host; ``replicate_specs`` draws the per-replicate
settings of a calibration batch (64 replicates of 1e6-2e7 agents, 730 ticks).
"""

from __future__ import annotations

import numpy as np

from . import model as M
from .core import PropertySet
from .distributions import gamma
from .utils import date


def _node_pops(rng, n_nodes, mu, sigma, total):
    raw = rng.lognormal(mu, sigma, n_nodes)
    pops = np.maximum(np.round(raw / raw.sum() * total).astype(np.int64), 1)
    pops[np.argmax(pops)] += int(total) - int(pops.sum())
    return pops


def _gravity_distances(rng, n_nodes, side_km):
    xy = rng.uniform(0, side_km, size=(n_nodes, 2))
    d = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    d[d == 0] = 1.0
    np.fill_diagonal(d, 0.0)
    return d


def _base_pars(rng, n_nodes, pops, dur, seed, cbr, side_km, amp, peak, r0):
    return {
        "seed": seed,
        "start_date": date("2019-01-01"),
        "dur": dur,
        "init_pop": pops,
        "init_immun": 0.0,
        "init_prev": np.zeros(n_nodes),
        "cbr": np.full(n_nodes, float(cbr)),
        "r0": r0,
        "r0_scalars": rng.lognormal(0.0, 0.3, n_nodes),
        "seasonal_amplitude": amp,
        "seasonal_peak_doy": peak,
        "risk_mult_var": float(np.exp(0.8**2) - 1.0),
        "corr_risk_inf": 0.8,
        "dur_exp": gamma(shape=3, scale=1.0),
        "dur_inf": gamma(shape=4, scale=6.0),
        "distances": _gravity_distances(rng, n_nodes, side_km),
        "migration_method": "gravity",
        "gravity_k": 0.5,
        "gravity_k_exponent": 0.0,
        "gravity_a": 1,
        "gravity_b": 1,
        "gravity_c": 2.0,
        "max_migr_frac": 0.2,
        "stop_if_no_cases": False,
        "verbose": 0,
    }


def _age_immunity(sim, rng, under15_immunity):
    """Recovered over 15 y; a node-specific fraction of under-15s recovered."""
    p = sim.people
    n = p.count
    age = -p.date_of_birth[:n].astype(np.int64)
    node = p.node_id[:n]
    state = p.disease_state[:n]
    state[age > 15 * 365] = 3
    young = age <= 15 * 365
    frac = np.asarray(under15_immunity)[node]
    state[young & (rng.random(n) < frac)] = 3


def _seed_infections(sim, rng, n_seed_nodes, per_node):
    p = sim.people
    n = p.count
    nodes = rng.choice(len(sim.nodes), size=n_seed_nodes, replace=False)
    for nd in nodes:
        idx = np.flatnonzero(p.node_id[:n] == nd)
        pick = rng.choice(idx, size=min(per_node, len(idx)), replace=False)
        p.disease_state[pick] = 2
        p.strain[pick] = 0


def zamfara_like(n_agents=1_000_000, dur=365, seed=42, n_nodes=14):
    rng = np.random.default_rng(seed)
    pops = _node_pops(rng, n_nodes, np.log(7e4), 0.6, n_agents)
    pars = _base_pars(rng, n_nodes, pops, dur, seed, 35, 200.0, 0.4, 180, 14)
    pars.update({"vx_prob_ri": 0.5, "vx_prob_ipv": 0.0})
    sim = M.SEIR_ABM(PropertySet(pars))
    sim.components = [M.VitalDynamics_ABM, M.DiseaseState_ABM, M.RI_ABM, M.SIA_ABM, M.Transmission_ABM]
    _age_immunity(sim, rng, np.full(n_nodes, 0.8))
    _seed_infections(sim, rng, 2, 10)
    return sim


def nigeria_like_pars(n_agents=220_000_000, n_nodes=774, dur=2555, seed=42, mu=np.log(2.8e5), sigma=0.7,
                      side_km=1000.0):
    """Parameters (no agents) of the Nigeria-scale workload: node
    populations lognormal(mu, sigma) summing to n_agents, coordinates in a
    side_km square, CBR 37, R0 14 with amplitude 0.4 peaking on day 180, RI
    coverage beta(6, 4), an SIA on a random 30% of nodes every 180 days
    (ages 0-5 y, coverage beta(8, 3), efficacy 0.6), three strains; under-15
    immunity uniform(0.4, 0.9) per node (returned beside the parameters)."""
    rng = np.random.default_rng(seed)
    pops = _node_pops(rng, n_nodes, mu, sigma, n_agents)
    pars = _base_pars(rng, n_nodes, pops, dur, seed, 37, side_km, 0.4, 180, 14)
    sia = []
    for k, t in enumerate(range(180, dur + 1, 180)):
        nodes = np.sort(rng.choice(n_nodes, size=max(1, int(0.3 * n_nodes)), replace=False))
        d = date("2019-01-01")
        import datetime as dt

        sia.append({"date": (d + dt.timedelta(days=t)).isoformat(), "nodes": nodes.tolist(),
                    "age_range": (0, 5 * 365), "vaccinetype": "mOPV2" if k % 2 == 0 else "nOPV2"})
    pars.update({
        "vx_prob_ri": rng.beta(6, 4, n_nodes),
        "vx_prob_ipv": np.zeros(n_nodes),
        "vx_prob_sia": rng.beta(8, 3, n_nodes),
        "sia_schedule": sia,
        "vx_efficacy": {"mOPV2": 0.6, "nOPV2": 0.6},
        "strain_r0_scalars": {0: 1.0, 1: 0.25, 2: 0.125},
    })
    immun = rng.uniform(0.4, 0.9, n_nodes)
    return pars, immun, rng


def continental_pars(n_agents=1_000_000_000, n_nodes=4000, dur=365, seed=42):
    """Parameters (no agents) of the continental workload: 4000 nodes,
    1e9 agents with node populations lognormal(ln 2.5e5, 0.9), a dense
    gravity network from coordinates in a 5000 km square, 365 ticks; RI, SIA
    schedule, strains and the rest as the Nigeria-scale workload."""
    return nigeria_like_pars(n_agents, n_nodes, dur, seed, mu=np.log(2.5e5), sigma=0.9, side_km=5000.0)


def nigeria_like(n_agents=2_000_000, n_nodes=774, dur=2555, seed=42):
    """Host-initialised Nigeria-like sim (moderate sizes; tests and CPU runs)."""
    return _host_sim(*nigeria_like_pars(n_agents, n_nodes, dur, seed))


def continental_like(n_agents=4_000_000, n_nodes=4000, dur=365, seed=42):
    """Host-initialised sim of the continental workload's shape (4000 nodes,
    lognormal(ln 2.5e5, 0.9) node populations, 5000 km square) at moderate
    agent counts (tests and CPU runs)."""
    return _host_sim(*continental_pars(n_agents, n_nodes, dur, seed))


def _host_sim(pars, immun, rng):
    sim = M.SEIR_ABM(PropertySet(pars))
    sim.components = [M.VitalDynamics_ABM, M.DiseaseState_ABM, M.RI_ABM, M.SIA_ABM, M.Transmission_ABM]
    _age_immunity(sim, rng, immun)
    _seed_infections(sim, rng, 2, 10)
    return sim


# ---------------------------------------------------------------------------
# Full-size bundles: reference-ordered columns built directly (no per-agent
# Python), in parallel chunks, optionally into caller-provided (e.g. pinned)
# host buffers.  Same recipe as nigeria_like / zamfara_like.

COLUMN_DTYPES = {
    "disease_state": np.int8,
    "strain": np.int8,
    "exposure_timer": np.int8,
    "infection_timer": np.int8,
    "paralysis_timer": np.int8,
    "potentially_paralyzed": np.int8,
    "paralyzed": np.int8,
    "ipv_protected": np.int8,
    "chronically_missed": np.uint8,
    "node_id": np.int16,
    "ri_timer": np.int16,
    "acq_risk_multiplier": np.float32,
    "daily_infectivity": np.float32,
    "date_of_birth": np.int32,
    "date_of_death": np.int32,
}


def _km_ages(rng, cum, ages_days, max_year=100):
    """Vectorised KM age at death (same rule as core.KaplanMeierEstimator)."""
    top = min(int(max_year), len(cum) - 1)
    years = np.minimum(ages_days // 365, top)
    lower = np.where(years > 0, cum[np.maximum(years - 1, 0)], 0)
    total = cum[top]
    span = np.maximum(total - lower, 0)
    draw = lower + np.floor(rng.random(len(ages_days)) * span).astype(np.int64)
    y = np.searchsorted(cum[: top + 1], draw, side="right")
    y = np.where(span > 0, np.maximum(y, years), top)
    y = np.minimum(y, top)
    lo = np.where(y == years, ages_days, y * 365)
    hi = np.maximum((y + 1) * 365, lo + 1)
    return (lo + np.floor(rng.random(len(ages_days)) * (hi - lo)).astype(np.int64)).astype(np.int32)


def bundle(kind="nigeria", n_agents=None, n_nodes=None, dur=None, seed=42, capacity_factor=1.3, threads=None,
           alloc=None, r0=14.0, amp=0.4, peak=180, gravity_k=0.5):
    """(make_desc parameters, reference-ordered columns) of a synthetic run.

    kind 'nigeria' (defaults 2.2e8 agents, 774 nodes, 2555 ticks),
    'continental' (1e9 agents, 4000 nodes, 365 ticks; node populations
    lognormal(ln 2.5e5, 0.9), 5000 km square, otherwise as 'nigeria') or
    'zamfara' (1e6 agents, 14 nodes, 365 ticks).  ``alloc(name, n, dtype)``
    may supply the column buffers (pinned host memory for the end-to-end
    measurement).  r0, amp, peak and gravity_k are the replicate-level
    parameters a calibration varies (R0, seasonal amplitude and peak day,
    gravity k).  params["distances"] is the node distance matrix the gravity
    network was built from (make_desc ignores it).
    """
    import concurrent.futures as cf
    import datetime as dt

    from scipy.special import ndtr

    from .core import gravity
    from .core import row_normalizer
    from .engine import _vaccine_strain
    from .utils import create_cumulative_deaths
    from .utils import seasonality_table

    if kind == "nigeria":
        n_agents = int(2.2e8 if n_agents is None else n_agents)
        n_nodes = 774 if n_nodes is None else n_nodes
        dur = 2555 if dur is None else dur
        mu, sg, side, cbr = np.log(2.8e5), 0.7, 1000.0, 37
    elif kind == "continental":
        n_agents = int(1e9 if n_agents is None else n_agents)
        n_nodes = 4000 if n_nodes is None else n_nodes
        dur = 365 if dur is None else dur
        mu, sg, side, cbr = np.log(2.5e5), 0.9, 5000.0, 37
    else:
        n_agents = int(1e6 if n_agents is None else n_agents)
        n_nodes = 14 if n_nodes is None else n_nodes
        dur = 365 if dur is None else dur
        mu, sg, side, cbr = np.log(7e4), 0.6, 200.0, 35
    rng = np.random.default_rng(seed)
    pops = _node_pops(rng, n_nodes, mu, sg, n_agents)
    count = int(pops.sum())
    capacity = int(count * capacity_factor)
    nt = dur + 1
    r0 = float(r0)
    if kind in ("nigeria", "continental"):
        immun = rng.uniform(0.4, 0.9, n_nodes)
        p_ri = rng.beta(6, 4, n_nodes)
        p_sia = rng.beta(8, 3, n_nodes)
        sia = []
        for k, t in enumerate(range(180, dur + 1, 180)):
            mask = np.zeros(n_nodes, np.uint8)
            mask[rng.choice(n_nodes, size=max(1, int(0.3 * n_nodes)), replace=False)] = 1
            sia.append((t, _vaccine_strain("mOPV2" if k % 2 == 0 else "nOPV2"), 0, 5 * 365, 0.6, mask))
    else:
        immun = np.full(n_nodes, 0.8)
        p_ri = np.full(n_nodes, 0.5)
        p_sia = np.zeros(n_nodes)
        sia = []
    r0s = rng.lognormal(0.0, 0.3, n_nodes)
    xy = rng.uniform(0, side, size=(n_nodes, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    dist[dist == 0] = 1.0
    np.fill_diagonal(dist, 0.0)
    net = row_normalizer(gravity(pops, dist, float(gravity_k), 1, 1, 2.0) / np.power(float(pops.sum()), 2.0), 0.2)
    start = dt.date(2019, 1, 1)
    datevec = [start + dt.timedelta(days=i) for i in range(nt)]
    cum = create_cumulative_deaths(count, 100).astype(np.int64)
    seed_nodes = rng.choice(n_nodes, size=2, replace=False)
    params = {
        "n_nodes": n_nodes, "n_strains": 3, "nt": nt, "count": count, "capacity": capacity, "seed": seed,
        "components": 31, "stop_if_no_cases": 0, "vd_step": 7, "birth_rate": np.full(n_nodes, cbr / 365000.0),
        "km_cumdeaths": cum, "km_max_year": 100, "p_paralysis": 1 / 2000, "seeds": [], "dur_inf": (2, 4.0, 6.0),
        "ri_step": 14, "ri_enabled": 1, "ri_strain": 1, "vx_prob_ri": p_ri, "vx_prob_ipv": np.zeros(n_nodes),
        "sia": sia, "vx_prob_sia": p_sia.astype(np.float32), "strain_r0_scalars": np.array([1.0, 0.25, 0.125]),
        "network": net, "r0_scalars": r0s, "seasonality": seasonality_table(datevec, float(amp), int(peak)),
        "zero_inflation": 0.0, "nb_r": 1000, "pop0": pops.astype(np.int32), "R_preseed": None,
        "distances": dist,
    }

    alloc = alloc or (lambda name, n, dtype: np.empty(n, dtype=dtype))
    cols = {name: alloc(name, capacity, dt_) for name, dt_ in COLUMN_DTYPES.items()}
    node_start = np.concatenate([[0], np.cumsum(pops)])
    var = float(np.exp(0.8**2) - 1.0)
    mu_ln = np.log(1.0 / np.sqrt(var + 1.0))
    sigma_ln = np.sqrt(np.log(var + 1.0))
    rho = 2.0 * np.sin(np.pi * 0.8 / 6)
    scale_inf = r0 / 24.0
    m_par, s_par = 12.5, 3.5
    mu_p = np.log(m_par**2 / np.sqrt(s_par**2 + m_par**2))
    sg_p = np.sqrt(np.log(s_par**2 / m_par**2 + 1))
    trunc = 1.0 - np.exp(-80.0 / 20.0)
    chunk = 1 << 22
    spans = [(a, min(a + chunk, capacity)) for a in range(0, capacity, chunk)]
    seqs = np.random.SeedSequence(seed).spawn(len(spans))

    def fill(i):
        a, b = spans[i]
        g = np.random.default_rng(seqs[i])
        n = b - a
        et = np.clip(-np.log(g.random((3, n))).sum(0), 0, 127)
        it = np.clip(-6.0 * np.log(g.random((4, n))).sum(0), 0, 127)
        et8 = et.astype(np.int8)
        it8 = it.astype(np.int8)
        raw = np.exp(mu_p + sg_p * g.standard_normal(n)) - et8
        cols["exposure_timer"][a:b] = et8
        cols["infection_timer"][a:b] = it8
        cols["paralysis_timer"][a:b] = np.clip(raw, 0, np.minimum(it8, 127)).astype(np.int8)
        z1 = g.standard_normal(n)
        z2 = rho * z1 + np.sqrt(1 - rho * rho) * g.standard_normal(n)
        cols["acq_risk_multiplier"][a:b] = np.exp(mu_ln + sigma_ln * z1)
        cols["daily_infectivity"][a:b] = -scale_inf * np.log(np.maximum(ndtr(-z2), 1e-300))
        cols["strain"][a:b] = 0
        cols["potentially_paralyzed"][a:b] = -1
        cols["paralyzed"][a:b] = 0
        cols["ipv_protected"][a:b] = 0
        cols["chronically_missed"][a:b] = 0
        live = max(0, min(b, count) - a)
        ds = cols["disease_state"]
        ds[a:b] = -1
        cols["node_id"][a:b] = -1
        cols["ri_timer"][a:b] = -1
        cols["date_of_birth"][a:b] = -1
        cols["date_of_death"][a:b] = 0
        if live:
            idx = np.arange(a, a + live)
            node = (np.searchsorted(node_start, idx, side="right") - 1).astype(np.int16)
            cols["node_id"][a : a + live] = node
            age_y = -20.0 * np.log(1.0 - g.random(live) * trunc)
            age = np.maximum(1, (age_y * 365.0).astype(np.int64))
            cols["date_of_birth"][a : a + live] = -age
            st = np.zeros(live, np.int8)
            st[age > 15 * 365] = 3
            young = age <= 15 * 365
            st[young & (g.random(live) < immun[node])] = 3
            ds[a : a + live] = st
            cols["ri_timer"][a : a + live] = (-age + g.uniform(42, 98, live)).astype(np.int32).astype(np.int16)
            cols["date_of_death"][a : a + live] = _km_ages(g, cum, age) - age

    with cf.ThreadPoolExecutor(max_workers=threads or min(32, (os_cpu() or 4))) as ex:
        list(ex.map(fill, range(len(spans))))
    for nd in seed_nodes:
        lo, hi = node_start[nd], node_start[nd + 1]
        pick = rng.choice(np.arange(lo, hi), size=min(10, hi - lo), replace=False)
        cols["disease_state"][pick] = 2
        cols["strain"][pick] = 0
    return params, cols


def incidence_inputs(T=365, n_nodes=774, n_strains=3, n_agents=2.2e8, seed=42, mu=np.log(2.8e5), sigma=0.7,
                     side_km=1000.0):
    """Node-level aggregates of a replayed Nigeria-scale run, for the
    expected-incidence map and its adjoint (laser_polio_gb300.ops.
    expected_incidence): node populations lognormal(mu, sigma), by default
    (ln 2.8e5, 0.7), summing to n_agents on a side_km (1000 km) square, growing at CBR 37 minus a flat 10 per
    1000; susceptibles 5-30% of a node carrying unit mean risk; infectivity
    by strain (1, 0.25, 0.125 of the VDPV2 level) of about 0.6 per infected
    agent-day from a few hundred infected agents, zero in 30% of node-ticks;
    ticks from 2019-01-01 with their day of year and year length; the
    gravity network k=0.5, a=b=1, c=2, max export fraction 0.2; R0 over the
    recorded R0 = 1, seasonal amplitude 0.4 peaking on day 180, r0_scalars
    lognormal(0, 0.3).  Returns the dict expected_incidence takes."""
    import datetime as dt

    rng = np.random.default_rng(seed)
    pops = _node_pops(rng, n_nodes, mu, sigma, n_agents).astype(np.float64)
    dist = _gravity_distances(rng, n_nodes, side_km)
    growth = (37.0 - 10.0) / 365000.0
    pop = pops[None, :] * (1.0 + growth) ** np.arange(T)[:, None]
    sus = rng.uniform(0.05, 0.3, n_nodes)
    srisk = pop * sus[None, :] * rng.lognormal(-0.005, 0.1, (T, n_nodes))
    scal = np.array([1.0, 0.25, 0.125, 0.0625])[:n_strains]
    infected = rng.gamma(2.0, 150.0, (T, n_nodes, n_strains)) * (rng.uniform(size=(T, n_nodes, n_strains)) > 0.3)
    beta = 0.6 * infected * scal[None, None, :]
    dates = [dt.date(2019, 1, 1) + dt.timedelta(days=i) for i in range(T)]
    doy = np.array([d.timetuple().tm_yday for d in dates], np.float64)
    year = np.array([366.0 if (d.year % 4 == 0 and (d.year % 100 != 0 or d.year % 400 == 0)) else 365.0
                     for d in dates])
    return dict(srisk=srisk, beta=beta, pop=pop, doy=doy, year=year, r0s=rng.lognormal(0.0, 0.3, n_nodes), R=1.0,
                amp=0.4, peak=180.0, pops=pops, dist=dist, k=0.5, a=1.0, b=1.0, c=2.0, max_frac=0.2)


def replicate_specs(n=64, seed=42, dur=730):
    """Per-replicate settings of a calibration batch: node counts from
    {14, 44, 120, 300}, agents log-uniform in [1e6, 2e7] (about 4e8 in total
    for 64), R0 ~ U(8, 20), seasonal amplitude ~ U(0.1, 0.6), peak day
    ~ U(0, 364), gravity k ~ lognormal(ln 0.5, 0.5), seeds seed + r."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n):
        out.append({
            "kind": "zamfara",
            "n_nodes": int(rng.choice([14, 44, 120, 300])),
            "n_agents": int(np.exp(rng.uniform(np.log(1e6), np.log(2e7)))),
            "dur": dur,
            "seed": seed + r,
            "r0": float(rng.uniform(8, 20)),
            "amp": float(rng.uniform(0.1, 0.6)),
            "peak": int(rng.integers(0, 365)),
            "gravity_k": float(rng.lognormal(np.log(0.5), 0.5)),
        })
    return out


def os_cpu():
    import os

    return os.cpu_count()
