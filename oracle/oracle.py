"""ctypes wrapper of the C oracle (lpg_oracle.c).

Test infrastructure (see oracle/__init__.py).  It takes exactly the same
lpg_sim_desc / lpg_columns / lpg_results_view structures as the CUDA engine,
so a test can hand one simulation description to both and compare.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from laser_polio_gb300 import _abi

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.lpo_create.restype = C.c_void_p
        L.lpo_create.argtypes = [C.POINTER(_abi.lpg_sim_desc)]
        L.lpo_destroy.argtypes = [C.c_void_p]
        L.lpo_bind_columns.argtypes = [C.c_void_p, C.POINTER(_abi.lpg_columns)]
        L.lpo_read_columns.argtypes = [C.c_void_p, C.POINTER(_abi.lpg_columns)]
        L.lpo_read_results.argtypes = [C.c_void_p, C.POINTER(_abi.lpg_results_view)]
        L.lpo_get_state.argtypes = [C.c_void_p, C.POINTER(_abi.lpg_sim_state)]
        L.lpo_start.argtypes = [C.c_void_p]
        L.lpo_step.argtypes = [C.c_void_p, C.c_int32]
        L.lpo_last_error.restype = C.c_char_p
        L.lpo_last_error.argtypes = [C.c_void_p]
        L.lpo_philox.argtypes = [C.POINTER(C.c_uint64), C.c_uint64, C.c_uint64]
        for name in ("lpo_exp", "lpo_expm1", "lpo_mlog"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = [C.c_double]
        L.lpo_lfact.restype = C.c_double
        L.lpo_lfact.argtypes = [C.c_int64]
        L.lpo_fix_risk_many.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
        L.lpo_poisson_many.argtypes = [C.c_uint64, C.c_double, C.c_int64, C.POINTER(C.c_int64)]
        L.lpo_gamma_many.argtypes = [C.c_uint64, C.c_double, C.c_int64, C.POINTER(C.c_double)]
        L.lpo_negbinom_many.argtypes = [C.c_uint64, C.c_double, C.c_double, C.c_int64, C.POINTER(C.c_int64)]
        L.lpo_dist_many.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_int64, C.POINTER(C.c_double)]
        L.lpo_km_newborn.restype = C.c_int32
        L.lpo_km_newborn.argtypes = [C.POINTER(C.c_int64), C.c_int32, C.c_int32, C.c_uint64, C.c_int32, C.c_uint64]
        L.lpo_num_threads.restype = C.c_int
        L.lpo_record_aggregates.argtypes = [C.c_void_p, C.c_int]
        L.lpo_read_aggregates.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
        L.lpo_read_aggregates_fp64.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 2
        for name, res in (("lpo_u01", C.c_double), ("lpo_u53", C.c_uint64), ("lpo_raw", C.c_uint64)):
            getattr(L, name).restype = res
            getattr(L, name).argtypes = [C.c_uint64, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_uint64]
        L.lpo_tx_u0.restype = C.c_double
        L.lpo_tx_u0.argtypes = [C.c_uint64, C.c_int32, C.c_uint64]
        L.lpo_tx_negbinom.restype = C.c_int64
        L.lpo_tx_negbinom.argtypes = [C.c_uint64, C.c_int32, C.c_uint64, C.c_double, C.c_double]
        L.lpo_tx_poisson.restype = C.c_int64
        L.lpo_tx_poisson.argtypes = [C.c_uint64, C.c_int32, C.c_uint64, C.c_double]
        L.lpo_init_columns.argtypes = [C.POINTER(_abi.lpg_init_desc), C.c_uint32, C.POINTER(_abi.lpg_columns)]
        L.lpo_init_mean_infectivity.restype = C.c_double
        L.lpo_init_mean_infectivity.argtypes = [C.c_uint64, C.c_double, _abi.lpg_dist]
        L.lpo_seed_timer.restype = C.c_double
        L.lpo_seed_timer.argtypes = [C.c_uint64, C.c_int32, C.c_uint64, C.c_uint64, C.c_int, C.c_double, C.c_double]
        _lib = L
    return _lib


class OracleSim:
    """One simulation run by the CPU oracle, driven like the engine handle."""

    def __init__(self, desc: _abi.lpg_sim_desc, keepalive=None):
        self._keep = keepalive
        self.desc = desc
        self.h = lib().lpo_create(C.byref(desc))

    def bind_columns(self, cols: dict):
        lib().lpo_bind_columns(self.h, C.byref(_abi.make_columns(cols)))

    def start(self):
        lib().lpo_start(self.h)

    def step(self, n_ticks: int):
        rc = lib().lpo_step(self.h, int(n_ticks))
        if rc != 0:
            raise RuntimeError(f"oracle: {_abi.STATUS_NAMES.get(rc, rc)}: {lib().lpo_last_error(self.h).decode()}")

    def state(self) -> _abi.lpg_sim_state:
        st = _abi.lpg_sim_state()
        lib().lpo_get_state(self.h, C.byref(st))
        return st

    def read_results(self, res: dict):
        lib().lpo_read_results(self.h, C.byref(_abi.make_results_view(res)))

    def read_columns(self, cols: dict):
        lib().lpo_read_columns(self.h, C.byref(_abi.make_columns(cols)))

    def record_aggregates(self, on: bool = True):
        """Record the expected-incidence map's inputs per transmission tick
        (as the engine's lpg_record_aggregates); before start()."""
        if lib().lpo_record_aggregates(self.h, int(bool(on))) != 0:
            raise RuntimeError("oracle: record_aggregates after start")

    def read_aggregates(self) -> dict:
        """srisk, pop, lam [nt, n_nodes] and beta [nt, n_nodes, n_strains]."""
        nt, n, ns = self.desc.nt, self.desc.n_nodes, self.desc.n_strains
        out = {"srisk": np.zeros((nt, n)), "beta": np.zeros((nt, n, ns)), "pop": np.zeros((nt, n)),
               "lam": np.zeros((nt, n))}
        dp = C.POINTER(C.c_double)
        if lib().lpo_read_aggregates(self.h, *[_abi.ptr(out[k], dp) for k in ("srisk", "beta", "pop", "lam")]) != 0:
            raise RuntimeError("oracle: aggregates were not recorded")
        return out

    def read_aggregates_fp64(self) -> dict:
        """srisk [nt, n_nodes] and beta [nt, n_nodes, n_strains] of the same
        ticks summed in FP64 straight from the float32 risk and infectivity
        columns, without the fixed-point units the step itself uses."""
        nt, n, ns = self.desc.nt, self.desc.n_nodes, self.desc.n_strains
        out = {"srisk": np.zeros((nt, n)), "beta": np.zeros((nt, n, ns))}
        dp = C.POINTER(C.c_double)
        if lib().lpo_read_aggregates_fp64(self.h, _abi.ptr(out["srisk"], dp), _abi.ptr(out["beta"], dp)) != 0:
            raise RuntimeError("oracle: aggregates were not recorded")
        return out

    def close(self):
        if self.h:
            lib().lpo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def philox(ctr, key):
    c = (C.c_uint64 * 4)(*[int(x) for x in ctr])
    lib().lpo_philox(c, int(key[0]), int(key[1]))
    return [int(x) for x in c]


def det_exp(x):
    return lib().lpo_exp(float(x))


def det_expm1(x):
    return lib().lpo_expm1(float(x))


def det_log(x):
    return lib().lpo_mlog(float(x))


def det_lfact(k):
    return lib().lpo_lfact(int(k))


def poisson_many(seed, lam, n):
    out = np.zeros(n, np.int64)
    lib().lpo_poisson_many(seed, lam, n, out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out


def gamma_many(seed, shape, n):
    out = np.zeros(n, np.float64)
    lib().lpo_gamma_many(seed, shape, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def negbinom_many(seed, r, p, n):
    out = np.zeros(n, np.int64)
    lib().lpo_negbinom_many(seed, r, p, n, out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out


def dist_many(seed, kind, p1, p2, n):
    out = np.zeros(n, np.float64)
    lib().lpo_dist_many(seed, kind, p1, p2, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def km_newborn(cum, max_year, seed, t, slot):
    cum = np.ascontiguousarray(cum, dtype=np.int64)
    return lib().lpo_km_newborn(cum.ctypes.data_as(C.POINTER(C.c_int64)), len(cum), max_year, seed, t, slot)


def num_threads():
    return lib().lpo_num_threads()


def count_seirp(node_id, disease_state, strain, potentially_paralyzed, paralyzed, n_nodes, n_strains, n_people):
    """count_SEIRP (laser_polio/model.py:869-899, kernel :902-929) in numpy.

    Returns (S, E, I, R, E_by_strain, I_by_strain, POTP, P, n_invalid).  The
    reference indexes out of bounds for a node id outside [0, n_nodes) or an
    E/I strain outside [0, n_strains); such slots are skipped here and
    counted in n_invalid.
    """
    n = int(n_people)
    nd = np.asarray(node_id[:n]).astype(np.int64)
    ds = np.asarray(disease_state[:n]).astype(np.int8)
    st = np.asarray(strain[:n]).astype(np.int64)
    pp = np.asarray(potentially_paralyzed[:n]).astype(np.int8)
    pa = np.asarray(paralyzed[:n]).astype(np.int8)
    G, ns = int(n_nodes), int(n_strains)
    alive = ds >= 0
    node_ok = (nd >= 0) & (nd < G)
    ei = (ds == 1) | (ds == 2)
    strain_ok = (st >= 0) & (st < ns)
    live = alive & node_ok
    n_invalid = int(np.count_nonzero(alive & ~node_ok) + np.count_nonzero(live & ei & ~strain_ok))

    def count(mask):
        return np.bincount(nd[live & mask], minlength=G).astype(np.int32)

    S = count(ds == 0)
    R = count(ds == 3)
    POTP = count(pp == 1)
    P = count(pa == 1)
    Ebs = np.zeros((G, ns), dtype=np.int32)
    Ibs = np.zeros((G, ns), dtype=np.int32)
    for k in range(ns):
        Ebs[:, k] = count((ds == 1) & (st == k))
        Ibs[:, k] = count((ds == 2) & (st == k))
    return S, Ebs.sum(axis=1).astype(np.int32), Ibs.sum(axis=1).astype(np.int32), R, Ebs, Ibs, POTP, P, n_invalid


def fix_risk_many(r):
    """(double-precision, integer-bits and single-precision fixed-point
    weights) of the float32 array r."""
    r = np.ascontiguousarray(r, dtype=np.float32)
    a = np.empty(len(r), np.uint64)
    b = np.empty(len(r), np.uint64)
    c = np.empty(len(r), np.uint64)
    lib().lpo_fix_risk_many(r.ctypes.data, len(r), a.ctypes.data, b.ctypes.data, c.ctypes.data)
    return a, b, c


def init_columns(desc, parts, cols):
    """The oracle's restatement of lpg_init_columns over host numpy columns
    (name -> array of length capacity)."""
    rc = lib().lpo_init_columns(C.byref(desc), int(parts), C.byref(_abi.make_columns(cols)))
    if rc != 0:
        raise ValueError(f"oracle: lpo_init_columns failed ({rc})")
