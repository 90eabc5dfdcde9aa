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
                 efficacy 0.6), CBR 37, 2555 ticks.  Its columns are built on
                 the host for moderate sizes and by ``device_columns`` on the
                 GPU for the full size.

Both return a fully initialised SEIR_ABM with the five drop-in components.
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


def nigeria_like_pars(n_agents=220_000_000, n_nodes=774, dur=2555, seed=42):
    """Parameters (no agents) of the Nigeria-scale workload."""
    rng = np.random.default_rng(seed)
    pops = _node_pops(rng, n_nodes, np.log(2.8e5), 0.7, n_agents)
    pars = _base_pars(rng, n_nodes, pops, dur, seed, 37, 1000.0, 0.4, 180, 14)
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


def nigeria_like(n_agents=2_000_000, n_nodes=774, dur=2555, seed=42):
    """Host-initialised Nigeria-like sim (moderate sizes; tests and CPU runs)."""
    pars, immun, rng = nigeria_like_pars(n_agents, n_nodes, dur, seed)
    sim = M.SEIR_ABM(PropertySet(pars))
    sim.components = [M.VitalDynamics_ABM, M.DiseaseState_ABM, M.RI_ABM, M.SIA_ABM, M.Transmission_ABM]
    _age_immunity(sim, rng, immun)
    _seed_infections(sim, rng, 2, 10)
    return sim
