"""Known-answer tests of the reference's model initialisation, restated
against this package (host numpy init; no device needed).

tests/test_seir_abm_init.py:22-50 and tests/test_diseasestate_abm.py:38-62,
486-494: population size, capacity, node ids, the disease-state columns and
initial counts, and the time-to-paralysis timers."""

import numpy as np

import laser_polio_gb300 as lp
from laser_polio_gb300.core import PropertySet


def _seir_sim():
    pars = PropertySet({"start_date": lp.date("2020-01-01"), "dur": 10, "init_pop": np.array([1000, 500]),
                        "cbr": np.array([30, 25]), "seed": 3})
    return lp.SEIR_ABM(pars), pars


def _ds_sim():
    pars = PropertySet(
        {
            "start_date": lp.date("2020-01-01"),
            "dur": 30,
            "init_pop": np.array([1000, 500]),
            "cbr": np.array([30, 25]),
            "r0_scalars": np.array([0.5, 2.0]),
            "init_immun": 0.2,
            "init_prev": 0.05,
            "dur_exp": lp.normal(mean=3, std=1),
            "dur_inf": lp.gamma(shape=4.51, scale=5.32),
            "p_paralysis": 1 / 2000,
            "stop_if_no_cases": False,
            "seed": 4,
        }
    )
    sim = lp.SEIR_ABM(pars)
    sim.components = [lp.DiseaseState_ABM]
    return sim


def test_total_pop_capacity_and_nodes():
    """tests/test_seir_abm_init.py:22-50."""
    sim, pars = _seir_sim()
    assert sim.people.count == np.sum(sim.pars.init_pop) == len(sim.people) == pars.init_pop.sum()
    assert sim.people.capacity > sim.people.count
    node_ids = sim.people.node_id[: sim.people.count]
    assert set(np.unique(node_ids)) == set(range(len(pars.init_pop)))
    np.testing.assert_array_equal(np.bincount(node_ids), pars.init_pop)


def test_disease_state_columns_and_initial_counts():
    """tests/test_diseasestate_abm.py:38-62: the columns exist; no one is
    exposed, init_prev of the population is infected, and the immune share
    is recovered less those whom the infections overrode."""
    sim = _ds_sim()
    for name in ("disease_state", "paralyzed", "exposure_timer", "infection_timer"):
        assert hasattr(sim.people, name)
    total = int(np.sum(sim.pars.init_pop))
    rec, inf = int(sim.pars.init_immun * total), int(sim.pars.init_prev * total)
    ds = sim.people.disease_state
    assert total - rec - inf <= np.sum(ds == 0) <= total - rec
    assert np.sum(ds == 1) == 0
    assert np.sum(ds == 2) == inf
    assert rec - inf <= np.sum(ds == 3) <= rec


def test_time_to_paralysis():
    """tests/test_diseasestate_abm.py:486-494: t_to_paralysis has mean 12.5
    and sd 3.5 (within 3), and the paralysis timers plus the exposure timers
    have that mean."""
    sim = _ds_sim()
    dist = sim.pars.t_to_paralysis(1000)
    e_timer, p_timer = sim.people.exposure_timer, sim.people.paralysis_timer
    assert np.isclose(dist.mean(), 12.5, atol=3) and np.isclose(dist.std(), 3.5, atol=3)
    assert np.isclose(p_timer.mean() + e_timer.mean(), 12.5, atol=3)
    assert np.isclose(p_timer.std(), 3.5, atol=3)


def test_component_columns_and_result_arrays():
    """tests/test_vital_dynamics.py:27-34, tests/test_interventions.py:41-46,
    tests/test_strain_transmission.py:58-83: the columns and result arrays
    the components add, the strain result shapes and the strain ids."""
    from oracle_backend import run_with_oracle

    pars = PropertySet({"start_date": lp.date("2019-01-01"), "dur": 10, "init_pop": np.array([10000, 10000]),
                        "cbr": np.array([30, 25]), "init_prev": np.array([0.001, 0.0]), "stop_if_no_cases": False,
                        "seed": 5})
    sim = lp.SEIR_ABM(pars)
    sim.components = [lp.VitalDynamics_ABM, lp.DiseaseState_ABM, lp.RI_ABM, lp.SIA_ABM, lp.Transmission_ABM]
    for name in ("date_of_birth", "date_of_death", "ri_timer"):
        assert hasattr(sim.people, name), name
    for name in ("births", "deaths", "ri_vaccinated"):
        assert hasattr(sim.results, name), name
    run_with_oracle(sim)
    nt, nn, ns = sim.results.I_by_strain.shape
    assert (nt, nn, ns) == (sim.pars.dur + 1, len(sim.pars.init_pop), len(sim.pars.strain_ids))
    assert sim.results.E_by_strain.shape == sim.results.I_by_strain.shape
    assert sim.pars.strain_ids["VDPV2"] == 0 and sim.pars.strain_ids["Sabin2"] == 1 and sim.pars.strain_ids["nOPV2"] == 2
