"""Default parameters and component run order (laser_polio/pars.py:10-99).

The values and keys are the reference's; this is the parameter contract the
drop-in components honour.
"""

import datetime

import numpy as np

from . import distributions as _d
from .core import PropertySet

__all__ = ["default_pars", "default_run_order"]

default_pars = PropertySet(
    {
        "seed": None,
        "start_date": datetime.date(2019, 1, 1),
        "dur": 30,
        "init_pop": [15000, 10000],
        "init_immun": [0.0, 0.0],
        "init_sus_by_age": None,
        "age_pyramid_path": "data/Nigeria_age_pyramid_2024.csv",
        "cbr": [37, 41],
        "strain_ids": {"VDPV2": 0, "Sabin2": 1, "nOPV2": 2},
        "strain_r0_scalars": {0: 1.0, 1: 0.25, 2: 0.125},
        "init_prev": [0.0, 0.0],
        "seed_schedule": None,
        "r0": 14,
        "r0_scalars": [0.8, 1.2],
        "seasonal_amplitude": 0.125,
        "seasonal_peak_doy": 180,
        "individual_heterogeneity": True,
        "risk_mult_var": 4.0,
        "corr_risk_inf": 0.8,
        "dur_exp": _d.poisson(lam=3),
        "dur_inf": _d.gamma(shape=4.51, scale=5.32),
        "t_to_paralysis": _d.lognormal(mean=12.5, sigma=3.5),
        "p_paralysis": 1 / 2000,
        "shp": None,
        "node_lookup": None,
        "distances": np.array([[0, 100], [100, 0]]),
        "node_seeding_dispersion": 1000,
        "node_seeding_zero_inflation": 0.0,
        "migration_method": "radiation",
        "radiation_k_log10": -0.3,
        "gravity_k": 1.0,
        "gravity_k_exponent": 0.0,
        "gravity_a": 1,
        "gravity_b": 1,
        "gravity_c": 2.0,
        "max_migr_frac": 0.1,
        "vx_prob_ri": None,
        "vx_prob_ipv": None,
        "ipv_start_year": 2015,
        "sia_schedule": None,
        "vx_prob_sia": None,
        "missed_frac": 0.0,
        "vx_efficacy": {
            "perfect": 1.0,
            "bOPV": 0,
            "f-IPV": 0,
            "IPV": 0,
            "IPV + bOPV": 0,
            "mOPV2": 0.7,
            "nOPV2": 0.7 * 0.8,
            "nOPV2 + fIPV": 0.7 * 0.8,
            "topv": 0.5,
        },
        "step_size_VitalDynamics_ABM": 7,
        "step_size_DiseaseState_ABM": 1,
        "step_size_RI_ABM": 14,
        "step_size_SIA_ABM": 1,
        "step_size_Transmission_ABM": 1,
        "actual_data": None,
        "summary_config": None,
        "verbose": 1,
        "stop_if_no_cases": True,
    }
)

default_run_order = ["VitalDynamics_ABM", "DiseaseState_ABM", "RI_ABM", "SIA_ABM", "Transmission_ABM"]
