"""Loader and thin wrapper of the CUDA engine library (liblpg.so).

The library is built in-tree by ``laser_polio_gb300.build``.  There is no
fallback: if the library is missing or no CUDA device is present, creating
a handle raises.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import _abi

LIB_PATH = Path(__file__).resolve().parent / "_build" / "liblpg.so"
_lib = None

# the C entry points and their signatures, as declared in include/lpg.h
SIGNATURES = {
    "lpg_version": (C.c_int, []),
    "lpg_create": (C.c_int, [C.POINTER(_abi.lpg_sim_desc), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "lpg_bind_columns": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_abi.lpg_columns)]),
    "lpg_start": (C.c_int, [C.c_void_p]),
    "lpg_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "lpg_sync": (C.c_int, [C.c_void_p]),
    "lpg_get_state": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_abi.lpg_sim_state)]),
    "lpg_read_results": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_abi.lpg_results_view)]),
    "lpg_read_columns": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_abi.lpg_columns)]),
    "lpg_record_aggregates": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "lpg_read_aggregates": (C.c_int, [C.c_void_p, C.c_int32] + [C.POINTER(C.c_double)] * 4),
    "lpg_check_invariants": (C.c_int, [C.c_void_p]),
    "lpg_set_graphs": (C.c_int, [C.c_void_p, C.c_int32]),
    "lpg_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "lpg_read_profile": (C.c_int, [C.c_void_p, C.POINTER(_abi.lpg_profile)]),
    "lpg_read_counters": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int32]),
    "lpg_cuda_stream": (C.c_void_p, [C.c_void_p]),
    "lpg_kernel_launches": (C.c_int64, [C.c_void_p]),
    "lpg_last_error": (C.c_char_p, [C.c_void_p]),
    "lpg_destroy": (None, [C.c_void_p]),
    "lpg_count_seirp": (C.c_int, [C.c_void_p] * 5 + [C.c_int32, C.c_int32, C.c_int64] + [C.c_void_p] * 10),
    "lpg_count_seirp_static": (C.c_int, [C.c_void_p] * 5 + [C.c_int32, C.c_int32, C.c_int64] + [C.c_void_p] * 10),
    "lpg_expected_incidence": (C.c_int, [C.POINTER(_abi.lpg_incidence_in), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(_abi.lpg_incidence_grad), C.c_void_p]),
    "lpg_incidence_plan_create": (C.c_int, [C.POINTER(_abi.lpg_incidence_in), C.POINTER(C.c_double), C.c_void_p,
                                            C.POINTER(C.c_void_p)]),
    "lpg_incidence_plan_eval": (C.c_int, [C.c_void_p, C.POINTER(_abi.lpg_incidence_params), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.POINTER(_abi.lpg_incidence_grad)]),
    "lpg_incidence_plan_stream": (C.c_void_p, [C.c_void_p]),
    "lpg_incidence_plan_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "lpg_incidence_plan_read_profile": (C.c_int, [C.c_void_p, C.POINTER(_abi.lpg_profile)]),
    "lpg_incidence_plan_destroy": (None, [C.c_void_p]),
    "lpg_write_results_csv": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_char_p)]),
    "lpg_radiation_network": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32, C.c_double,
                                        C.c_int32, C.POINTER(C.c_double)]),
    "lpg_op_last_error": (C.c_char_p, []),
    "lpg_check_desc": (C.c_int, [C.POINTER(_abi.lpg_sim_desc)]),
    "lpg_init_columns": (C.c_int, [C.POINTER(_abi.lpg_init_desc), C.c_uint32, C.POINTER(_abi.lpg_columns),
                                   C.c_void_p]),
    "lpg_init_mean_infectivity": (C.c_double, [C.c_uint64, C.c_double, _abi.lpg_dist]),
    "lpg_test_stall_sweep": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64]),
    "lpg_test_stall_round0": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64]),
    "lpg_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "lpg_get_launch": (C.c_int, [C.c_void_p, C.c_int32]),
}


def load(path: os.PathLike | None = None):
    """Load liblpg.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if path is None:
        from . import build as _build

        try:
            _build.build()
        except (OSError, FileNotFoundError) as exc:  # nvcc absent: use a prebuilt library if there is one
            if not p.exists():
                raise RuntimeError(f"CUDA engine library {p} is missing and could not be built: {exc}") from exc
    if not p.exists():
        raise RuntimeError(f"CUDA engine library {p} is missing; run laser_polio_gb300.build")
    lib = C.CDLL(str(p))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    if path is None:
        _lib = lib
    return lib


class LpgError(RuntimeError):
    def __init__(self, code, msg):
        self.code = code
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")


def error_for(code: int, msg: str) -> Exception:
    """The exception a failed call raises: ValueError where the reference
    raises one (capacity exhausted, LaserFrame.add; bad parameters), else
    LpgError carrying the status."""
    if code in (-1, -2, -3):
        return ValueError(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}" if code != -2 else msg)
    return LpgError(code, msg)


def check_desc(desc) -> None:
    """Raise what lpg_create would for this one simulation description
    (lpg_check_desc: host only, needs no GPU)."""
    lib = load()
    rc = lib.lpg_check_desc(C.byref(desc))
    if rc != 0:
        raise error_for(rc, lib.lpg_op_last_error().decode())


class Handle:
    """One lpg_handle: simulations that advance together on one GPU."""

    def __init__(self, descs, device: int = 0):
        self.lib = load()
        arr = (_abi.lpg_sim_desc * len(descs))(*descs)
        self._descs = arr
        h = C.c_void_p()
        rc = self.lib.lpg_create(arr, len(descs), int(device), C.byref(h))
        self.h = h
        self._check(rc)

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.lpg_last_error(self.h).decode() if self.h else ""
            if rc == -2:
                raise ValueError(msg)
            raise LpgError(rc, msg)

    def bind_columns(self, sim: int, cols: dict):
        self._check(self.lib.lpg_bind_columns(self.h, sim, C.byref(_abi.make_columns(cols))))

    def start(self):
        self._check(self.lib.lpg_start(self.h))

    def step(self, n_ticks: int):
        self._check(self.lib.lpg_step(self.h, int(n_ticks)))

    def sync(self):
        self._check(self.lib.lpg_sync(self.h))

    def sync_statuses(self) -> list:
        """Wait for queued work and return each simulation's own status (0 or
        a negative lpg_status): a simulation that failed on the device (births
        beyond its capacity, a timed-out wait, an internal check) stops there
        while the others run on.  A failure of the whole handle (a CUDA
        error) raises."""
        rc = self.lib.lpg_sync(self.h)
        if rc == -5:  # LPG_ERR_CUDA
            self._check(rc)
        out = []
        for i in range(len(self._descs)):
            st = _abi.lpg_sim_state()
            self._check(self.lib.lpg_get_state(self.h, i, C.byref(st)))
            out.append(int(st.error))
        return out

    def state(self, sim: int = 0, check: bool = True) -> _abi.lpg_sim_state:
        st = _abi.lpg_sim_state()
        self._check(self.lib.lpg_get_state(self.h, sim, C.byref(st)))
        if st.error and check:
            self.sync()
        return st

    def set_launch(self, which: int, blocks: int):
        """Grid size of a tick kernel (lpg_set_launch; LAUNCH_* in _abi)."""
        self._check(self.lib.lpg_set_launch(self.h, int(which), int(blocks)))

    def get_launch(self, which: int) -> int:
        rc = self.lib.lpg_get_launch(self.h, int(which))
        if rc < 0:
            self._check(rc)
        return int(rc)

    def test_stall_sweep(self, stages: int, wait_spin: int = 0):
        """Test hook (lpg_test_stall_sweep): the staged RI/SIA sweep issues
        only `stages` stages and its consumers give up after `wait_spin`
        iterations, so that a test can make the bounded wait run out."""
        self._check(self.lib.lpg_test_stall_sweep(self.h, int(stages), int(wait_spin)))

    def test_stall_round0(self, skip: bool, wait_spin: int = 0):
        """Test hook (lpg_test_stall_round0): CTA 0 of the first selection
        round does not arrive at the round's grid barrier and the others give
        up after `wait_spin` polls, so that a test can make that bounded wait
        run out."""
        self._check(self.lib.lpg_test_stall_round0(self.h, int(bool(skip)), int(wait_spin)))

    def read_results(self, sim: int, res: dict):
        self._check(self.lib.lpg_read_results(self.h, sim, C.byref(_abi.make_results_view(res))))

    def read_columns(self, sim: int, cols: dict):
        self._check(self.lib.lpg_read_columns(self.h, sim, C.byref(_abi.make_columns(cols))))

    def record_aggregates(self, sim: int, on: bool = True):
        """Record the expected-incidence map's inputs on every transmission
        tick (lpg_record_aggregates); before start()."""
        self._check(self.lib.lpg_record_aggregates(self.h, sim, int(bool(on))))

    def read_aggregates(self, sim: int, nt: int, n_nodes: int, n_strains: int) -> dict:
        """srisk, pop, lam [nt, n_nodes] and beta [nt, n_nodes, n_strains] as
        recorded (lpg_read_aggregates); zero rows where transmission did not run."""
        import numpy as np

        out = {"srisk": np.zeros((nt, n_nodes)), "beta": np.zeros((nt, n_nodes, n_strains)),
               "pop": np.zeros((nt, n_nodes)), "lam": np.zeros((nt, n_nodes))}
        dp = C.POINTER(C.c_double)
        self._check(self.lib.lpg_read_aggregates(self.h, sim, *[_abi.ptr(out[k], dp)
                                                               for k in ("srisk", "beta", "pop", "lam")]))
        return out

    def check_invariants(self):
        self._check(self.lib.lpg_check_invariants(self.h))

    def set_graphs(self, on: bool):
        self._check(self.lib.lpg_set_graphs(self.h, int(bool(on))))

    def set_profiling(self, on: bool):
        self._check(self.lib.lpg_set_profiling(self.h, int(bool(on))))

    def profile(self) -> dict:
        p = _abi.lpg_profile()
        self._check(self.lib.lpg_read_profile(self.h, C.byref(p)))
        return {p.names[k].decode(): (p.total_ms[k], p.launches[k]) for k in range(p.n_kernels)}

    def counters(self) -> dict:
        """The device work counters (lpg_read_counters), by name."""
        buf = (C.c_uint64 * len(_abi.COUNTER_NAMES))()
        self._check(self.lib.lpg_read_counters(self.h, buf, len(buf)))
        return dict(zip(_abi.COUNTER_NAMES, (int(x) for x in buf)))

    def cuda_stream(self) -> int:
        return self.lib.lpg_cuda_stream(self.h) or 0

    def kernel_launches(self) -> int:
        return int(self.lib.lpg_kernel_launches(self.h))

    def close(self):
        if self.h:
            self.lib.lpg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
