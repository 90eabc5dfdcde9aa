"""ctypes mirror of include/lpg.h.

These structures are the only thing that crosses the C boundary: plain
integers, doubles and pointers.  They are shared by the engine binding
(``engine.py``) and by anything else that speaks the same ABI.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

LPG_MAX_STRAINS = 4
LPG_MAX_SIA_PER_DAY = 8

LPG_OK = 0
STATUS_NAMES = {
    0: "LPG_OK",
    -1: "LPG_ERR_ARG",
    -2: "LPG_ERR_CAPACITY",
    -3: "LPG_ERR_NODE",
    -4: "LPG_ERR_TIMEOUT",
    -5: "LPG_ERR_CUDA",
    -6: "LPG_ERR_STATE",
    -7: "LPG_ERR_NOMEM",
    -8: "LPG_ERR_INTERNAL",
}

COMP_VD, COMP_DS, COMP_RI, COMP_SIA, COMP_TX = 1, 2, 4, 8, 16
COMPONENT_BITS = {
    "VitalDynamics_ABM": COMP_VD,
    "DiseaseState_ABM": COMP_DS,
    "RI_ABM": COMP_RI,
    "SIA_ABM": COMP_SIA,
    "Transmission_ABM": COMP_TX,
}

DIST_KINDS = {
    "constant": 0,
    "exponential": 1,
    "gamma": 2,
    "lognormal": 3,
    "normal": 4,
    "poisson": 5,
    "uniform": 6,
    "lognormal_int": 7,
}

P_i8 = C.POINTER(C.c_int8)
P_u8 = C.POINTER(C.c_uint8)
P_i16 = C.POINTER(C.c_int16)
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_f32 = C.POINTER(C.c_float)
P_f64 = C.POINTER(C.c_double)


class lpg_dist(C.Structure):
    _fields_ = [("kind", C.c_int32), ("p1", C.c_double), ("p2", C.c_double)]


class lpg_sia_event(C.Structure):
    _fields_ = [
        ("tick", C.c_int32),
        ("strain", C.c_int32),
        ("min_age", C.c_int32),
        ("max_age", C.c_int32),
        ("efficacy", C.c_double),
        ("node_mask", P_u8),
    ]


class lpg_seed_event(C.Structure):
    _fields_ = [("tick", C.c_int32), ("node", C.c_int32), ("is_count", C.c_int32), ("value", C.c_double)]


class lpg_sim_desc(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32),
        ("n_strains", C.c_int32),
        ("nt", C.c_int32),
        ("count", C.c_int64),
        ("capacity", C.c_int64),
        ("seed", C.c_uint64),
        ("components", C.c_uint32),
        ("stop_if_no_cases", C.c_int32),
        ("vd_step", C.c_int32),
        ("birth_rate", P_f64),
        ("km_cumdeaths", P_i64),
        ("km_len", C.c_int32),
        ("km_max_year", C.c_int32),
        ("p_paralysis", C.c_float),
        ("seeds", C.POINTER(lpg_seed_event)),
        ("n_seeds", C.c_int32),
        ("dur_inf", lpg_dist),
        ("ri_step", C.c_int32),
        ("ri_enabled", C.c_int32),
        ("ri_strain", C.c_int32),
        ("vx_prob_ri", P_f64),
        ("vx_prob_ipv", P_f64),
        ("sia", C.POINTER(lpg_sia_event)),
        ("n_sia", C.c_int32),
        ("vx_prob_sia", P_f32),
        ("strain_r0_scalars", P_f64),
        ("network", P_f64),
        ("r0_scalars", P_f64),
        ("seasonality", P_f64),
        ("zero_inflation", C.c_double),
        ("nb_r", C.c_int32),
        ("pop0", P_i32),
        ("R_preseed", P_i32),
    ]


COLUMN_FIELDS = [
    ("disease_state", P_i8, np.int8),
    ("strain", P_i8, np.int8),
    ("exposure_timer", P_i8, np.int8),
    ("infection_timer", P_i8, np.int8),
    ("paralysis_timer", P_i8, np.int8),
    ("potentially_paralyzed", P_i8, np.int8),
    ("paralyzed", P_i8, np.int8),
    ("ipv_protected", P_i8, np.int8),
    ("chronically_missed", P_u8, np.uint8),
    ("node_id", P_i16, np.int16),
    ("ri_timer", P_i16, np.int16),
    ("acq_risk_multiplier", P_f32, np.float32),
    ("daily_infectivity", P_f32, np.float32),
    ("date_of_birth", P_i32, np.int32),
    ("date_of_death", P_i32, np.int32),
]


class lpg_columns(C.Structure):
    _fields_ = [(name, ptype) for name, ptype, _ in COLUMN_FIELDS]


# lpg_set_launch's tick kernels: name -> (index, largest grid, the profile
# entries it times); None: the engine's default is the largest (the
# cooperative k_sel_round0, whose CTAs must all be resident at once)
LAUNCH = {
    "due": (0, 8192, ("k_due",)),
    "sweep_due": (1, 1024, ("k_sweep_a",)),
    "sweep_rs": (2, 1024, ("k_sweep_b",)),
    "evb": (3, 8192, ("k_evb",)),
    "select": (4, None, ("k_sel_round0",)),
    "rounds": (5, 1024, ("k_sel_rounds",)),
    "newborns": (6, 8192, ("k_newborns",)),
}

# lpg_init_columns' parts, in the order they run
INIT_BASE, INIT_MISSED, INIT_TIMERS, INIT_IMMUNITY, INIT_PREVALENCE = 1, 2, 4, 8, 16
INIT_HETEROGENEITY, INIT_AGES, INIT_DEATHS, INIT_RI = 32, 64, 128, 256


class lpg_init_desc(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32),
        ("prev_per_node", C.c_int32),
        ("count", C.c_int64),
        ("capacity", C.c_int64),
        ("seed", C.c_uint64),
        ("node_pop", P_i64),
        ("missed_k", C.c_int64),
        ("immune_k", P_i64),
        ("prev_k", P_i64),
        ("dur_exp", lpg_dist),
        ("dur_inf", lpg_dist),
        ("t_to_paralysis", lpg_dist),
        ("heterogeneity", C.c_int32),
        ("n_age_bins", C.c_int32),
        ("risk_mult_var", C.c_double),
        ("corr_risk_inf", C.c_double),
        ("r0", C.c_double),
        ("age_lo_days", P_i32),
        ("age_hi_days", P_i32),
        ("age_weight", P_i64),
        ("km_cumdeaths", P_i64),
        ("km_len", C.c_int32),
        ("km_max_year", C.c_int32),
    ]


RESULT_FIELDS = [
    ("S", False),
    ("E", False),
    ("I", False),
    ("R", False),
    ("E_by_strain", True),
    ("I_by_strain", True),
    ("potentially_paralyzed", False),
    ("paralyzed", False),
    ("new_potentially_paralyzed", False),
    ("new_paralyzed", False),
    ("pop", False),
    ("births", False),
    ("deaths", False),
    ("new_exposed", False),
    ("new_exposed_by_strain", True),
    ("ri_vaccinated", False),
    ("ri_protected", False),
    ("ri_new_exposed_by_strain", True),
    ("ipv_vaccinated", False),
    ("sia_vaccinated", False),
    ("sia_protected", False),
    ("sia_new_exposed_by_strain", True),
]


class lpg_results_view(C.Structure):
    _fields_ = [(name, P_i32) for name, _ in RESULT_FIELDS]


class lpg_sim_state(C.Structure):
    _fields_ = [("t", C.c_int32), ("stopped", C.c_int32), ("count", C.c_int64), ("error", C.c_int32)]


# lpg.h's LPG_CTR_* indices, in order
COUNTER_NAMES = ("sweep_index", "sweep_due", "sweep_evt_due", "sweep_dod_due", "queue_ds", "queue_rs",
                 "sel_targets", "sel_node_rounds", "ri_index", "ri_due")


class lpg_profile(C.Structure):
    _fields_ = [
        ("n_kernels", C.c_int32),
        ("names", C.c_char_p * 16),
        ("total_ms", C.c_double * 16),
        ("launches", C.c_int64 * 16),
    ]


class lpg_incidence_in(C.Structure):
    _fields_ = [
        ("T", C.c_int32),
        ("G", C.c_int32),
        ("S", C.c_int32),
        *[(name, C.POINTER(C.c_double)) for name in ("srisk", "beta", "pop", "doy", "year", "r0s", "pops", "dist")],
        *[(name, C.c_double) for name in ("R", "amp", "peak", "k", "a", "b", "c", "max_frac")],
    ]


INCIDENCE_SCALAR_GRADS = ("R", "amp", "peak", "k", "a", "b", "c")


class lpg_incidence_grad(C.Structure):
    _fields_ = [
        *[(name, C.c_double) for name in INCIDENCE_SCALAR_GRADS],
        ("r0s", C.POINTER(C.c_double)),
        ("network", C.POINTER(C.c_double)),
    ]


class lpg_incidence_params(C.Structure):
    _fields_ = [
        *[(name, C.c_double) for name in ("R", "amp", "peak", "k", "a", "b", "c", "max_frac")],
        ("r0s", C.POINTER(C.c_double)),
    ]


def ptr(arr, ctype):
    """Pointer to the first element of a contiguous numpy array (or NULL)."""
    if arr is None:
        return None
    assert arr.flags["C_CONTIGUOUS"], "arrays crossing the C ABI must be contiguous"
    return arr.ctypes.data_as(ctype)


def make_columns(cols: dict) -> lpg_columns:
    """Build an lpg_columns from a dict name -> column (missing = NULL): a
    numpy array, or a CUDA tensor (a device-resident column), of the
    reference's element type."""
    out = lpg_columns()
    for name, ptype, dtype in COLUMN_FIELDS:
        arr = cols.get(name)
        if arr is None:
            continue
        if isinstance(arr, np.ndarray):
            if arr.dtype != dtype:
                raise TypeError(f"column {name} must be {np.dtype(dtype).name}, got {arr.dtype}")
            setattr(out, name, ptr(arr, ptype))
        else:
            if str(arr.dtype).rsplit(".", 1)[-1] != np.dtype(dtype).name or not arr.is_contiguous():
                raise TypeError(f"column {name} must be a contiguous {np.dtype(dtype).name} tensor, got {arr.dtype}")
            setattr(out, name, C.cast(C.c_void_p(arr.data_ptr()), ptype))
    return out


def make_results_view(res: dict) -> lpg_results_view:
    out = lpg_results_view()
    for name, _ in RESULT_FIELDS:
        arr = res.get(name)
        if arr is not None:
            if arr.dtype != np.int32:
                raise TypeError(f"result {name} must be int32")
            setattr(out, name, ptr(arr, P_i32))
    return out
