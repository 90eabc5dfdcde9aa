"""The model's initialisation on the device.

The reference fills the agent table in SEIR_ABM.__init__ and in each
component's constructor with numpy draws over every slot (model.py:101-175,
561-713, 816-866, 1548-1611, 1887-1894), which takes minutes at the Nigeria
scale (the reference flags it slow at :852).  Here the same constructors
describe what to fill (``InitSpec``) and ``fill`` runs the matching parts of
lpg_init_columns (include/lpg.h) on the device, into CUDA tensors that
become the sim's device-resident columns (core.LaserFrame).  The numbers
that decide how many agents are chosen (missed, immune, initially infected)
are worked out here on the host exactly as the reference's expressions give
them; every per-agent draw is made on the device.

There is no CPU path: without a CUDA device ``fill`` raises.
"""

from __future__ import annotations

import ctypes as C
import numbers

import numpy as np

from . import _abi
from . import _lib

# the columns each part writes (and reads), by lpg_init_columns' part bits
PART_COLUMNS = {
    _abi.INIT_BASE: ("disease_state", "node_id", "strain", "potentially_paralyzed", "paralyzed", "ipv_protected",
                     "chronically_missed"),
    _abi.INIT_MISSED: ("chronically_missed",),
    _abi.INIT_TIMERS: ("exposure_timer", "infection_timer", "paralysis_timer"),
    _abi.INIT_IMMUNITY: ("disease_state",),
    _abi.INIT_PREVALENCE: ("disease_state",),
    _abi.INIT_HETEROGENEITY: ("acq_risk_multiplier", "daily_infectivity"),
    _abi.INIT_AGES: ("date_of_birth",),
    _abi.INIT_DEATHS: ("date_of_birth", "date_of_death"),
    _abi.INIT_RI: ("date_of_birth", "ri_timer"),
}
COLUMN_DTYPES = {name: dtype for name, _, dtype in _abi.COLUMN_FIELDS}


def part_columns(parts: int):
    names = []
    for bit, cols in PART_COLUMNS.items():
        if parts & bit:
            names += [c for c in cols if c not in names]
    return names


class InitSpec:
    """The fields of an lpg_init_desc, gathered by SEIR_ABM and its
    components as they are constructed."""

    def __init__(self, seed, node_pop, count, capacity):
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.node_pop = np.ascontiguousarray(node_pop, dtype=np.int64)
        self.count = int(count)
        self.capacity = int(capacity)
        self.missed_k = 0
        self.immune_k = None
        self.prev_k = None
        self.prev_per_node = 1
        self.dur_exp = self.dur_inf = self.t_to_paralysis = (0, 0.0, 0.0)
        self.heterogeneity = 1
        self.risk_mult_var = 0.0
        self.corr_risk_inf = 0.0
        self.r0 = 0.0
        self.age_lo = self.age_hi = self.age_weight = None
        self.km = None
        self.km_max_year = 100

    def desc(self):
        """(lpg_init_desc, arrays its pointers refer to)."""
        keep = []

        def p64(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int64)
            keep.append(a)
            return _abi.ptr(a, _abi.P_i64)

        def p32(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return _abi.ptr(a, _abi.P_i32)

        d = _abi.lpg_init_desc()
        d.n_nodes = len(self.node_pop)
        d.prev_per_node = int(self.prev_per_node)
        d.count, d.capacity, d.seed = self.count, self.capacity, self.seed
        d.node_pop = p64(self.node_pop)
        d.missed_k = int(self.missed_k)
        d.immune_k = p64(self.immune_k)
        d.prev_k = p64(self.prev_k)
        d.dur_exp = _abi.lpg_dist(*self.dur_exp)
        d.dur_inf = _abi.lpg_dist(*self.dur_inf)
        d.t_to_paralysis = _abi.lpg_dist(*self.t_to_paralysis)
        d.heterogeneity = int(bool(self.heterogeneity))
        d.risk_mult_var, d.corr_risk_inf, d.r0 = float(self.risk_mult_var), float(self.corr_risk_inf), float(self.r0)
        d.n_age_bins = 0 if self.age_weight is None else len(self.age_weight)
        d.age_lo_days, d.age_hi_days = p32(self.age_lo), p32(self.age_hi)
        d.age_weight = p64(self.age_weight)
        d.km_cumdeaths = p64(self.km)
        d.km_len = 0 if self.km is None else len(self.km)
        d.km_max_year = int(self.km_max_year)
        return d, keep


# -- the counts the reference's expressions give ------------------------------
def missed_count(missed_frac, count) -> int:
    """int(missed_frac * n) (model.py:155-158)."""
    return int(missed_frac * count)


def immune_counts(init_immun, init_pop) -> np.ndarray:
    """int(immun_frac * node_pop) per node (model.py:589-618): a float gives
    every node the same float32 fraction, a list is read as float32, an
    array is used as it is; a fraction outside [0, 1] is an error."""
    pop = np.asarray(init_pop)
    if isinstance(init_immun, float):
        fr = np.full_like(pop, fill_value=init_immun, dtype=np.float32)
    elif isinstance(init_immun, list):
        fr = np.asarray(init_immun, dtype=np.float32)
    elif isinstance(init_immun, np.ndarray):
        fr = init_immun
        if fr.shape != pop.shape:
            raise ValueError("init_immun must match init_pop shape")
    else:
        raise ValueError(f"Unsupported init_immun type: {type(init_immun)}")
    out = np.zeros(len(pop), np.int64)
    for nid, (f, n) in enumerate(zip(fr, pop, strict=False)):
        if not (0.0 <= f <= 1.0):
            raise ValueError(f"Invalid immunity fraction: {f} for node {nid}")
        out[nid] = max(int(f * n), 0)
    return out


def prevalence_counts(init_prev, init_pop):
    """(per_node, counts) of the initially infected (model.py:670-713): a
    float is a fraction of everyone, an int a count of everyone (at most
    all), a list or array one entry per node, each a fraction (0 < v < 1)
    or a count (at most the node)."""
    pop = np.asarray(init_pop)
    total = int(np.sum(pop))
    if isinstance(init_prev, float):
        return 0, np.array([int(total * init_prev)], np.int64)
    if isinstance(init_prev, (int, np.integer)) and not isinstance(init_prev, bool):
        return 0, np.array([min(int(init_prev), total)], np.int64)
    if isinstance(init_prev, (list, np.ndarray)):
        if len(init_prev) != len(pop):
            raise ValueError(f"Length mismatch: init_prev has {len(init_prev)} entries, expected {len(pop)} nodes.")
        k = np.zeros(len(pop), np.int64)
        for node, prev in enumerate(init_prev):
            if not isinstance(prev, numbers.Real):
                raise ValueError(f"Unsupported value in init_prev list at node {node}: {prev}")
            k[node] = int(pop[node] * prev) if 0 < prev < 1 else min(int(prev), int(pop[node]))
        return 1, k
    raise ValueError(f"Unsupported init_prev type: {type(init_prev)}")


def age_bins(pyramid):
    """Bins of an age pyramid [min_age, max_age, M, F] rows: [lo, hi) in days
    with lo = max(min * 365, 1), hi = (max + 1) * 365, weight M + F
    (model.py:1576-1583)."""
    pyr = np.asarray(pyramid, dtype=np.int64)
    lo = np.maximum(pyr[:, 0] * 365, 1)
    hi = (pyr[:, 1] + 1) * 365
    return lo.astype(np.int32), hi.astype(np.int32), (pyr[:, 2] + pyr[:, 3]).astype(np.int64)


# -- running the parts -----------------------------------------------------------
def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("laser_polio_gb300 initialises its agent table on a CUDA device and none is available "
                           "(there is no CPU path)")
    return torch


def fill(people, spec: InitSpec, parts: int) -> None:
    """Run ``parts`` of lpg_init_columns for ``people`` on the device.  The
    columns the parts write become device-resident; a column already on the
    host is uploaded first and written back into the same numpy array, so
    that references to it stay valid."""
    torch = _torch()
    names = part_columns(parts)
    tensors, host_back = {}, {}
    dev_cols = people.device_columns()
    for name in names:
        if name in dev_cols:
            tensors[name] = dev_cols[name]
        elif people.has_column(name):
            host = getattr(people, name)
            tensors[name] = torch.from_numpy(np.ascontiguousarray(host)).cuda()
            host_back[name] = host
        else:
            tdt = getattr(torch, np.dtype(COLUMN_DTYPES[name]).name)
            tensors[name] = torch.empty(spec.capacity, dtype=tdt, device="cuda")
    cols = _abi.lpg_columns()
    for name, t in tensors.items():
        setattr(cols, name, C.cast(C.c_void_p(t.data_ptr()), dict((n, p) for n, p, _ in _abi.COLUMN_FIELDS)[name]))
    desc, _keep = spec.desc()
    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.lpg_init_columns(C.byref(desc), int(parts), C.byref(cols), C.c_void_p(stream))
    if rc != 0:
        raise _lib.error_for(rc, lib.lpg_op_last_error().decode())
    for name, t in tensors.items():
        if name in host_back:
            host_back[name][...] = t.cpu().numpy()
        else:
            people.set_device_column(name, t)


def mean_infectivity(seed, r0, dur_inf) -> float:
    """r0 / mean of 1000 infectious durations, as the device initialisation
    draws them (lpg_init_mean_infectivity)."""
    return float(_lib.load().lpg_init_mean_infectivity(int(seed) & 0xFFFFFFFFFFFFFFFF, float(r0),
                                                       _abi.lpg_dist(*dur_inf)))
