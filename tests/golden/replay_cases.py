"""Replay cases: small simulations that the reference's own code and this
project's oracle and engine run from the same initial agent table with the
same counter-based draws (see reference_harness.py).

Each case is a parameter set in the reference's ``pars`` vocabulary plus a
seeded recipe for the initial columns.  The reference builds its SEIR_ABM
from the parameters (its own init), then the recipe's columns overwrite the
agent table, as the reference's own tests poke columns before run().  The
cases between them use every component and every draw of the per-tick step:
births and deaths, E/I/R progression with paralysis and IPV, the seed
schedule (counts and prevalences, two entries for one node on one tick),
RI (OPV and IPV), SIA (two campaigns on one day), transmission with
gravity and radiation networks, Poisson and zero-inflated negative binomial
counts, heavy selection collisions, three strains and the early stop.
"""

from __future__ import annotations

import numpy as np

CASES = ("busy", "zamfara", "collisions", "stop")


def make_pars(name, lp, property_set, pyramid_path=None):
    """The case's parameters as a property_set, with lp's date and
    Distribution helpers (the reference's module or this package's)."""
    p = {"start_date": lp.date("2019-01-01"), "verbose": 0}
    if pyramid_path is not None:
        p["age_pyramid_path"] = str(pyramid_path)
    if name == "busy":
        p.update(
            seed=5, dur=150, init_pop=np.array([6000, 4000, 3000, 1500]), cbr=np.array([300.0, 150.0, 300.0, 40.0]),
            init_immun=[0.3, 0.5, 0.1, 0.0], init_prev=[0, 0, 0, 0], r0=12,
            r0_scalars=np.array([1.0, 0.8, 1.3, 0.5]),
            distances=np.array([[0, 30, 60, 90], [30, 0, 40, 70], [60, 40, 0, 20], [90, 70, 20, 0]]),
            migration_method="gravity", gravity_k=0.5, max_migr_frac=0.2,
            sia_schedule=[
                {"date": "2019-01-10", "nodes": [0, 2], "age_range": (0, 5 * 365), "vaccinetype": "nOPV2"},
                {"date": "2019-01-10", "nodes": [1, 2], "age_range": (30, 3 * 365), "vaccinetype": "mOPV2"},
                {"date": "2019-03-01", "nodes": [0, 1, 2, 3], "age_range": (0, 10 * 365), "vaccinetype": "topv"},
            ],
            vx_prob_sia=[0.8, 0.7, 0.9, 0.5], vx_prob_ri=[0.6, 0.5, 0.4, 0.9], vx_prob_ipv=[0.3, 0.0, 0.5, 0.2],
            missed_frac=0.05, node_seeding_zero_inflation=0.4, node_seeding_dispersion=2,
            seed_schedule=[{"timestep": 5, "node_id": 3, "prevalence": 25},
                           {"timestep": 5, "node_id": 3, "prevalence": 0.01},
                           {"timestep": 40, "node_id": 1, "prevalence": 0.002}],
            p_paralysis=0.05, stop_if_no_cases=False, dur_inf=lp.gamma(shape=4, scale=6.0),
        )
    elif name == "zamfara":
        rng = np.random.default_rng(14)
        xy = rng.uniform(0, 200, (14, 2))
        d = np.sqrt(((xy[:, None] - xy[None]) ** 2).sum(-1))
        p.update(
            seed=42, dur=365, init_pop=np.round(rng.lognormal(np.log(1400), 0.5, 14)).astype(int),
            cbr=np.full(14, 35.0), init_immun=0.0, init_prev=0, r0=14, r0_scalars=rng.lognormal(0, 0.3, 14),
            seasonal_amplitude=0.4, seasonal_peak_doy=180, distances=d, migration_method="radiation",
            radiation_k_log10=-0.3, max_migr_frac=0.2, vx_prob_ri=0.5, vx_prob_ipv=0.1,
            stop_if_no_cases=False, p_paralysis=1 / 2000, dur_inf=lp.gamma(shape=4, scale=6.0),
        )
    elif name == "native":  # the zamfara case's first 120 ticks: an outbreak growing in 14 nodes
        p = dict(make_pars("zamfara", lp, dict, pyramid_path))
        p.update(dur=120)
        return property_set(p)
    elif name == "init":  # the reference's own initialisation: every init parameter exercised
        rng = np.random.default_rng(21)
        p.update(
            seed=1, dur=30, init_pop=np.round(rng.lognormal(np.log(1500), 0.5, 14)).astype(int),
            cbr=np.full(14, 37.0), init_immun=list(rng.uniform(0.2, 0.9, 14)),
            init_prev=[10, 0, 0.01, 0, 3, 0, 0, 0, 0, 0, 0, 0, 0, 25], missed_frac=0.1,
            r0=14, r0_scalars=np.ones(14), distances=np.ones((14, 14)) - np.eye(14), migration_method="gravity",
            vx_prob_ri=0.5,
        )
    elif name == "collisions":
        p.update(
            seed=77, dur=40, init_pop=np.array([3000, 1500, 800]), cbr=np.array([30.0, 30.0, 30.0]),
            init_immun=[0.0, 0.0, 0.0], init_prev=[0, 0, 0], r0=200, r0_scalars=np.array([1.0, 1.5, 0.7]),
            distances=np.array([[0, 10, 30], [10, 0, 15], [30, 15, 0]]), migration_method="gravity",
            gravity_k=0.5, max_migr_frac=0.3, stop_if_no_cases=False,
        )
    elif name == "stop":
        p.update(
            seed=13, dur=300, init_pop=np.array([3000, 2000, 1000]), cbr=np.array([35.0, 35.0, 35.0]),
            init_immun=[0.0, 0.0, 0.0], init_prev=[0, 0, 0], r0=0.8, r0_scalars=np.array([1.0, 0.9, 1.1]),
            distances=np.array([[0, 50, 80], [50, 0, 40], [80, 40, 0]]), migration_method="gravity",
            gravity_k=0.2, max_migr_frac=0.1, stop_if_no_cases=True,
            seed_schedule=[{"timestep": 20, "node_id": 2, "prevalence": 3}],
        )
    else:
        raise KeyError(name)
    return property_set(p)


def components(lp):
    return [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.SIA_ABM, lp.Transmission_ABM]


def initial_columns(name, count, capacity, init_pop, seed):
    """The agent table the case starts from (reference slot order, length
    capacity): a mix of S, E, I and R with timers, strains, paralysis and IPV
    flags, chronically-missed agents, ages with RI dates and dates of death
    inside the run; slots past count as the reference leaves unborn slots
    (timers, risk and infectivity drawn, the rest at the defaults)."""
    rng = np.random.default_rng(seed)
    n = count
    cap = capacity
    cols = {}
    node = np.repeat(np.arange(len(init_pop)), init_pop).astype(np.int16)
    if name == "busy":
        rng.shuffle(node)  # slots of the nodes interleaved, as after births
    state = rng.choice(np.array([0, 1, 2, 3], np.int8), n,
                       p={"busy": [0.55, 0.03, 0.04, 0.38], "zamfara": [0.35, 0.0, 0.002, 0.648],
                          "native": [0.35, 0.0, 0.002, 0.648],
                          "collisions": [0.97, 0.0, 0.03, 0.0], "stop": [0.6, 0.0, 0.001, 0.399]}[name])
    strain = np.where(rng.random(n) < 0.8, 0, rng.integers(1, 3, n)).astype(np.int8)
    strain[(state != 1) & (state != 2)] = 0
    age = np.where(rng.random(n) < 0.3, rng.integers(1, 5 * 365, n), rng.integers(1, 80 * 365, n))
    dod = np.where(rng.random(n) < 0.02, rng.integers(1, 200, n), rng.integers(400, 30000, n))

    def full(v, dtype):
        return np.full(cap, v, dtype=dtype)

    cols["disease_state"] = full(-1, np.int8)
    cols["disease_state"][:n] = state
    cols["strain"] = full(0, np.int8)
    cols["strain"][:n] = strain
    cols["exposure_timer"] = rng.integers(0, 6, cap).astype(np.int8)
    cols["infection_timer"] = rng.integers(0, 31, cap).astype(np.int8)
    cols["paralysis_timer"] = rng.integers(0, 16, cap).astype(np.int8)
    pp = full(-1, np.int8)
    pp[:n] = np.where(rng.random(n) < 0.05, rng.integers(0, 2, n), -1).astype(np.int8)
    cols["potentially_paralyzed"] = pp
    cols["paralyzed"] = full(0, np.int8)
    cols["paralyzed"][:n] = ((pp[:n] == 1) & (rng.random(n) < 0.1)).astype(np.int8)
    cols["ipv_protected"] = full(0, np.int8)
    cols["ipv_protected"][:n] = (rng.random(n) < 0.1).astype(np.int8)
    cols["chronically_missed"] = full(0, np.uint8)
    cols["chronically_missed"][:n] = (rng.random(n) < 0.05).astype(np.uint8)
    cols["node_id"] = full(-1, np.int16)
    cols["node_id"][:n] = node
    cols["date_of_birth"] = full(-1, np.int32)
    cols["date_of_birth"][:n] = -age
    cols["date_of_death"] = full(0, np.int32)
    cols["date_of_death"][:n] = dod
    cols["ri_timer"] = full(-1, np.int16)
    cols["ri_timer"][:n] = (-age + rng.uniform(42, 98, n)).astype(np.int32).astype(np.int16)
    # risks at or above 0.5: whole multiples of 2^-24 (the selection's weight units)
    cols["acq_risk_multiplier"] = np.maximum(0.5, rng.lognormal(0.0, 0.5, cap)).astype(np.float32)
    cols["daily_infectivity"] = rng.exponential(0.5, cap).astype(np.float32)
    return cols


INIT_COLUMNS = ("disease_state", "chronically_missed", "node_id", "exposure_timer", "infection_timer",
                "paralysis_timer", "acq_risk_multiplier", "daily_infectivity", "date_of_birth", "date_of_death",
                "ri_timer", "strain", "potentially_paralyzed", "paralyzed", "ipv_protected")


def init_statistics(people, count, capacity):
    """Summaries of an initial agent table that a test can compare with
    another: exact counts, histograms of the integer columns and a sample of
    the (risk, infectivity) pairs."""
    c = {k: np.asarray(getattr(people, k)) for k in INIT_COLUMNS}
    live = slice(0, count)
    n_nodes = int(c["node_id"][live].max()) + 1
    out = {
        "state_by_node": np.stack([np.bincount(c["node_id"][live][c["disease_state"][live] == s],
                                               minlength=n_nodes) for s in range(4)]),
        "missed": np.array([int(c["chronically_missed"][live].sum())]),
        "et": np.bincount(c["exposure_timer"].astype(np.int64) + 128, minlength=256),
        "it": np.bincount(c["infection_timer"].astype(np.int64) + 128, minlength=256),
        "pt": np.bincount(c["paralysis_timer"].astype(np.int64) + 128, minlength=256),
        "age_years": np.bincount(-c["date_of_birth"][live] // 365, minlength=101)[:101],
        "death_age_years": np.bincount(np.minimum((c["date_of_death"][live] - c["date_of_birth"][live]) // 365,
                                                  150), minlength=151),
        "ri_offset": np.bincount((c["ri_timer"][live].astype(np.int64) - c["date_of_birth"][live]) % 65536,
                                 minlength=65536)[:200],
        "risk_inf": np.stack([c["acq_risk_multiplier"][:2000], c["daily_infectivity"][:2000]]).astype(np.float32),
        "defaults": np.array([int((c["strain"][live] != 0).sum()), int((c["potentially_paralyzed"] != -1).sum()),
                              int((c["paralyzed"] != 0).sum()), int((c["ipv_protected"] != 0).sum()),
                              int((c["disease_state"][count:] != -1).sum())]),
    }
    return out


