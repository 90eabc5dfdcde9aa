"""Bit-exact parity of the CUDA engine with the CPU oracle.

Every test builds a simulation, hands identical copies of its C-ABI
description and columns to the oracle and to the engine (through the C ABI),
runs both, and requires every result array and every agent column to be
identical.  Integer state must match exactly (the oracle and the engine
consume the same counter-based draws); there is no floating-point tolerance
because every floating-point quantity that feeds an integer decision is
computed with the same operations in the same order on both sides.
"""

import numpy as np
import pytest

import laser_polio_gb300 as lp
from laser_polio_gb300 import synthetic
from laser_polio_gb300.core import PropertySet
from oracle_backend import assert_same
from oracle_backend import run_spec_gpu
from oracle_backend import run_spec_oracle
from oracle_backend import snapshot

pytestmark = pytest.mark.gpu


def parity(sim, n_ticks=None, graphs=True, check=False):
    spec, cols_o, res_o = snapshot(sim)
    _, cols_g, res_g = snapshot(sim)
    n = sim.nt - 1 if n_ticks is None else n_ticks
    so = run_spec_oracle(spec, cols_o, res_o, n)
    sg = run_spec_gpu(spec, cols_g, res_g, n, graphs=graphs, check=check)
    assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error)
    assert_same(res_o, res_g, "result")
    assert_same(cols_o, cols_g, "column", count=so.count)
    return res_o, so


def test_parity_zamfara_like_small():
    sim = synthetic.zamfara_like(n_agents=200_000, dur=120, seed=42)
    res, st = parity(sim, check=False)
    assert res["new_exposed"].sum() > 0


def test_parity_with_invariant_checks():
    sim = synthetic.zamfara_like(n_agents=50_000, dur=60, seed=3)
    parity(sim, check=True, graphs=False)


def test_parity_nigeria_like_small():
    sim = synthetic.nigeria_like(n_agents=400_000, n_nodes=60, dur=400, seed=9)
    res, st = parity(sim)
    assert res["sia_vaccinated"].sum() > 0
    assert res["ri_vaccinated"].sum() > 0
    assert res["births"].sum() > 0


def _busy_sim(seed=5, dur=200, zi=0.0, disp=1000, stop=False, seeds=None, cbr=300):
    sia = [
        {"date": "2019-01-10", "nodes": [0, 2], "age_range": (0, 5 * 365), "vaccinetype": "nOPV2"},
        {"date": "2019-01-10", "nodes": [1, 2], "age_range": (30, 3 * 365), "vaccinetype": "mOPV2"},
        {"date": "2019-03-01", "nodes": [0, 1, 2, 3], "age_range": (0, 10 * 365), "vaccinetype": "topv"},
    ]
    pars = PropertySet(
        {
            "seed": seed,
            "start_date": lp.date("2019-01-01"),
            "dur": dur,
            "init_pop": np.array([30000, 20000, 15000, 5000]),
            "cbr": np.array([cbr, cbr / 2, cbr, 40]),
            "init_immun": [0.3, 0.5, 0.1, 0.0],
            "init_prev": [20, 0, 5, 0],
            "r0": 12,
            "r0_scalars": np.array([1.0, 0.8, 1.3, 0.5]),
            "distances": np.array([[0, 30, 60, 90], [30, 0, 40, 70], [60, 40, 0, 20], [90, 70, 20, 0]]),
            "migration_method": "gravity",
            "gravity_k": 0.5,
            "max_migr_frac": 0.2,
            "sia_schedule": sia,
            "vx_prob_sia": [0.8, 0.7, 0.9, 0.5],
            "vx_prob_ri": [0.6, 0.5, 0.4, 0.9],
            "vx_prob_ipv": [0.3, 0.0, 0.5, 0.2],
            "missed_frac": 0.05,
            "node_seeding_zero_inflation": zi,
            "node_seeding_dispersion": disp,
            "stop_if_no_cases": stop,
            "seed_schedule": seeds,
            "p_paralysis": 0.05,
            "verbose": 0,
        }
    )
    sim = lp.SEIR_ABM(pars)
    sim.components = [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.SIA_ABM, lp.Transmission_ABM]
    return sim


def test_parity_all_components_busy():
    res, st = parity(_busy_sim())
    assert res["births"].sum() > 1000
    assert res["sia_protected"].sum() > 0
    assert res["new_paralyzed"].sum() > 0


def test_parity_zero_inflated_seeding():
    res, st = parity(_busy_sim(seed=8, zi=0.4, disp=2))
    assert res["new_exposed"].sum() > 0


def test_parity_seed_schedule_and_stop():
    seeds = [
        {"timestep": 5, "node_id": 3, "prevalence": 25},
        {"timestep": 5, "node_id": 3, "prevalence": 0.01},
        {"timestep": 40, "node_id": 1, "prevalence": 0.002},
        {"timestep": 41, "node_id": 0, "prevalence": 10},
    ]
    res, st = parity(_busy_sim(seed=12, seeds=seeds))
    res, st = parity(_busy_sim(seed=13, stop=True, dur=300))


def test_parity_unsorted_nodes_and_per_tick_driver():
    sim = _busy_sim(seed=21, dur=80)
    rng = np.random.default_rng(0)
    n = sim.people.count
    perm = rng.permutation(n)
    for name in ("disease_state", "node_id", "date_of_birth", "date_of_death", "ri_timer"):
        col = getattr(sim.people, name)
        col[:n] = col[:n][perm]
    parity(sim, graphs=False)


def test_per_tick_driver_matches_run_all():
    a = _busy_sim(seed=31, dur=60, stop=True)
    b = _busy_sim(seed=31, dur=60, stop=True)
    a.run()
    eng = b._engine
    for tick in range(b.nt):
        if tick == 0:
            b.log_results(0)
            b.t += 1
            continue
        for c in b.instances:
            c.step()
        b.log_results(tick)
        b.t += 1
        if b.should_stop:
            break
    del eng
    assert a.t == b.t
    for name in ("S", "E", "I", "R", "new_exposed", "births", "deaths", "ri_vaccinated", "sia_vaccinated"):
        assert np.array_equal(getattr(a.results, name), getattr(b.results, name)), name
    assert np.array_equal(a.people.disease_state, b.people.disease_state)


def test_capacity_error_is_raised():
    sim = _busy_sim(seed=4, dur=120, cbr=4000)
    sim.people._capacity = sim.people.count + 10
    for name in ("disease_state", "strain", "exposure_timer", "infection_timer", "paralysis_timer",
                 "potentially_paralyzed", "paralyzed", "ipv_protected", "chronically_missed", "node_id",
                 "ri_timer", "acq_risk_multiplier", "daily_infectivity", "date_of_birth", "date_of_death"):
        setattr(sim.people, name, np.ascontiguousarray(getattr(sim.people, name)[: sim.people.capacity]))
    with pytest.raises(ValueError):
        sim.run()


def test_parity_heavy_collisions():
    """Demand close to the susceptible count: many selection rounds per node."""
    pars = PropertySet(
        {
            "seed": 77,
            "start_date": lp.date("2019-01-01"),
            "dur": 40,
            "init_pop": np.array([3000, 1500, 800]),
            "cbr": np.array([30, 30, 30]),
            "init_immun": [0.0, 0.2, 0.0],
            "init_prev": [30, 10, 5],
            "r0": 200,
            "risk_mult_var": 9.0,
            "r0_scalars": np.array([1.0, 1.5, 0.7]),
            "distances": np.array([[0, 10, 30], [10, 0, 15], [30, 15, 0]]),
            "migration_method": "gravity",
            "gravity_k": 0.5,
            "max_migr_frac": 0.3,
            "stop_if_no_cases": False,
            "verbose": 0,
        }
    )
    sim = lp.SEIR_ABM(pars)
    sim.components = [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.Transmission_ABM]
    res, st = parity(sim, check=True, graphs=False)
    assert res["new_exposed"].sum() > 2000


def test_parity_batched_replicates():
    """Replicates of different sizes, node counts, durations and components
    in one handle: each equals its own oracle run."""
    from laser_polio_gb300._lib import Handle

    sims = [
        synthetic.zamfara_like(n_agents=80_000, dur=90, seed=1),
        synthetic.nigeria_like(n_agents=150_000, n_nodes=44, dur=120, seed=2),
        _busy_sim(seed=8, dur=70, stop=True),
        synthetic.zamfara_like(n_agents=30_000, dur=150, seed=3, n_nodes=5),
    ]
    snaps_o = [snapshot(s) for s in sims]
    snaps_g = [snapshot(s) for s in sims]
    states_o = [run_spec_oracle(spec, cols, res, s.nt - 1) for s, (spec, cols, res) in zip(sims, snaps_o)]
    h = Handle([spec.desc for spec, _, _ in snaps_g])
    for i, (_, cols, _) in enumerate(snaps_g):
        h.bind_columns(i, cols)
    h.start()
    h.step(max(s.nt for s in sims) - 1)
    h.sync()
    for i, ((_, cols_o, res_o), (_, cols_g, res_g), so) in enumerate(zip(snaps_o, snaps_g, states_o)):
        sg = h.state(i)
        assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error), i
        h.read_results(i, res_g)
        h.read_columns(i, cols_g)
        assert_same(res_o, res_g, f"replicate {i} result")
        assert_same(cols_o, cols_g, f"replicate {i} column", count=so.count)
    h.close()


def test_parity_batch_of_many_small_nodes():
    """A batch whose nodes outnumber one wave of the per-node kernels (more
    than six a GB300 SM: 912): the node steps run in their batch forms (the
    one-warp mixing, the lane-per-node draws), and each replicate still
    equals its own oracle run."""
    from laser_polio_gb300._lib import Handle

    sims = [synthetic.nigeria_like(n_agents=60_000, n_nodes=120, dur=60, seed=20 + k) for k in range(8)]
    sims.append(synthetic.zamfara_like(n_agents=40_000, dur=60, seed=29))
    snaps_o = [snapshot(s) for s in sims]
    snaps_g = [snapshot(s) for s in sims]
    assert sum(spec.desc.n_nodes for spec, _, _ in snaps_g) > 912
    states_o = [run_spec_oracle(spec, cols, res, s.nt - 1) for s, (spec, cols, res) in zip(sims, snaps_o)]
    h = Handle([spec.desc for spec, _, _ in snaps_g])
    for i, (_, cols, _) in enumerate(snaps_g):
        h.bind_columns(i, cols)
    h.start()
    h.step(max(s.nt for s in sims) - 1)
    h.sync()
    for i, ((_, cols_o, res_o), (_, cols_g, res_g), so) in enumerate(zip(snaps_o, snaps_g, states_o)):
        sg = h.state(i)
        assert (sg.t, sg.stopped, sg.count, sg.error) == (so.t, so.stopped, so.count, so.error), i
        h.read_results(i, res_g)
        h.read_columns(i, cols_g)
        assert_same(res_o, res_g, f"replicate {i} result")
        assert_same(cols_o, cols_g, f"replicate {i} column", count=so.count)
    assert sum(res_o["new_exposed"].sum() for _, _, res_o in snaps_o) > 0
    h.close()


def test_work_counters_are_consistent():
    """The device work counters (lpg_read_counters) start at zero, are reset
    by turning profiling on, and agree with the results they stand behind."""
    from laser_polio_gb300._lib import Handle

    sim = _busy_sim(seed=11, dur=150)
    spec, cols, res = snapshot(sim)
    h = Handle([spec.desc])
    h.bind_columns(0, cols)
    h.start()
    assert all(v == 0 for v in h.counters().values())
    h.step(40)
    h.sync()
    h.set_profiling(True)
    assert all(v == 0 for v in h.counters().values())
    h.step(sim.nt - 41)
    h.sync()
    c = h.counters()
    h.read_results(0, res)
    h.close()
    assert 0 < c["sweep_due"] <= c["sweep_index"]
    assert c["sweep_evt_due"] <= c["sweep_due"] and c["sweep_dod_due"] <= c["sweep_due"]
    assert c["sweep_evt_due"] + c["sweep_dod_due"] >= c["sweep_due"]
    assert c["queue_ds"] >= int(res["deaths"][41:].sum())
    assert c["queue_rs"] > 0
    assert 0 < c["ri_due"] <= c["ri_index"]
    if res["new_exposed"][41:].sum() > 0:
        assert c["sel_targets"] > 0


def test_parity_ri_timers_extremes_and_mid_run_reads():
    """RI timers over the whole int16 range (wrap-around, zero, the first RI
    tick's wider window), deaths and births, with the columns read back in
    the middle of the run and at its end."""
    from laser_polio_gb300._lib import Handle
    from oracle.oracle import OracleSim

    sim = _busy_sim(seed=17, dur=130, cbr=600)
    n = sim.people.count
    rng = np.random.default_rng(3)
    edge = np.array([-32768, -32767, -32760, -15, -14, -13, -1, 0, 1, 13, 14, 15, 28, 29, 32760, 32766, 32767])
    ri = rng.integers(-32768, 32768, n)
    ri[: n // 3] = rng.choice(edge, n // 3)
    ri[n // 3 : n // 2] = rng.integers(-30, 200, n // 2 - n // 3)
    sim.people.ri_timer[:n] = ri.astype(np.int16)
    spec, cols_o, res_o = snapshot(sim)
    _, cols_g, res_g = snapshot(sim)
    o = OracleSim(spec.desc, keepalive=spec)
    o.bind_columns(cols_o)
    o.start()
    h = Handle([spec.desc])
    h.bind_columns(0, cols_g)
    h.start()
    for n_ticks in (29, 41, sim.nt - 71):
        o.step(n_ticks)
        h.step(n_ticks)
        h.sync()
        o.read_columns(cols_o)
        h.read_columns(0, cols_g)
        so, sg = o.state(), h.state(0)
        assert (sg.t, sg.count) == (so.t, so.count)
        assert_same(cols_o, cols_g, "column", count=so.count)
    h.check_invariants()
    o.read_results(res_o)
    h.read_results(0, res_g)
    o.close()
    h.close()
    assert_same(res_o, res_g, "result")
    assert res_o["ri_vaccinated"].sum() > 0
