"""Run the reference's own laser_polio code, unmodified, in this process.

Test infrastructure: make_reference_fixtures.py uses it to produce the
golden files in this directory.  Nothing else imports it, and nothing here
runs on a machine without the reference checkout (the path is given on the
command line).

The reference imports packages that are not installed here.  They are
replaced in sys.modules before the import:
  - numba: ``njit`` returns the function itself, ``prange`` is ``range``,
    one thread (``get_num_threads`` 1, ``get_thread_id`` 0), and the type
    objects cast (``nb.float32(x)``) or describe signatures (``nb.int8[:]``).
    The reference's numba kernels therefore run as plain Python over the
    same numpy arrays, in index order.
  - laser_core (laser-core ~= 0.6, pyproject.toml:45; not vendored):
    LaserFrame, PropertySet, gravity, radiation, row_normalizer, distance,
    calc_capacity, KaplanMeierEstimator, AliasedDistribution,
    load_pyramid_csv and seed, from this package's own restatement
    (laser_polio_gb300.core).
  - plotting, progress-bar, logging-timezone, table and CLI packages
    (matplotlib, cartopy, imageio_ffmpeg, sciris, alive_progress, pytz,
    pandas, geopandas, click, yaml): inert stand-ins; sciris' print helpers
    print, alive_bar is a context manager.

Replay: ``DrawHook`` takes the place of ``np.random`` inside the reference's
modules while its tick loop runs.  Every random call the per-tick step makes
is answered with the counter-based draw that the oracle and the CUDA engine
use for the same purpose, tick and slot or node (lpg_rng.h, through the
oracle's lpo_* exports).  Which draw a call is follows from where it is
made: the hook reads the calling frame (function name and its locals, e.g.
the slot ``i`` in a kernel loop, the node ``n`` in the transmission step).
A call from anywhere else raises, so that an unknown draw cannot pass
unnoticed.  What the reference then computes with those draws is its own
code's arithmetic: the float32 per-thread sums, ``1 - np.exp(-rate)``, the
float64 cumulative sums and searchsorted of the weighted selection.
"""

from __future__ import annotations

import ctypes as C
import importlib
import sys
import types

import numpy as np

# ---------------------------------------------------------------------------
# stand-in modules


class _Inert:
    """Anything: callable, subscriptable, an attribute source, a context
    manager, a base class."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Inert()

    def __getattr__(self, name):
        return _Inert()

    def __getitem__(self, k):
        return _Inert()

    def __setitem__(self, k, v):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def __iter__(self):
        return iter(())


class _InertMeta(type):
    """Inert classes: usable as types (isinstance) and as objects
    (subscripted, assigned into, attributes, iteration)."""

    def __getattr__(cls, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _InertMeta(name, (_Inert,), {})

    def __getitem__(cls, k):
        return _Inert()

    def __setitem__(cls, k, v):
        pass

    def __iter__(cls):
        return iter(())


class _InertModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _InertMeta(name, (_Inert,), {})


class _NbType:
    """numba scalar type: casts when called, describes an array when
    subscripted (signatures)."""

    def __init__(self, np_type):
        self.np_type = np_type

    def __call__(self, x):
        return self.np_type(x)

    def __getitem__(self, k):
        return self


def _njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


def _numba_module():
    nb = types.ModuleType("numba")
    nb.njit = _njit
    nb.jit = _njit
    nb.prange = range
    nb.get_num_threads = lambda: 1
    nb.get_thread_id = lambda: 0
    nb.set_num_threads = lambda n: None
    for name, t in (("int8", np.int8), ("int16", np.int16), ("int32", np.int32), ("int64", np.int64),
                    ("uint8", np.uint8), ("uint16", np.uint16), ("uint32", np.uint32), ("float32", np.float32),
                    ("float64", np.float64)):
        setattr(nb, name, _NbType(t))
    nb.boolean = np.bool_
    return nb


def _laser_core_modules():
    from laser_polio_gb300 import core

    def seed(s):
        np.random.seed(int(s) & 0xFFFFFFFF)

    mods = {}

    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        mods[name] = m
        return m

    mod("laser_core")
    mod("laser_core.laserframe", LaserFrame=core.LaserFrame)
    mod("laser_core.propertyset", PropertySet=core.PropertySet)
    mod("laser_core.migration", distance=core.distance, gravity=core.gravity, radiation=core.radiation,
        row_normalizer=core.row_normalizer)
    mod("laser_core.random", seed=seed)
    mod("laser_core.utils", calc_capacity=core.calc_capacity)
    mod("laser_core.demographics")
    mod("laser_core.demographics.kmestimator", KaplanMeierEstimator=core.KaplanMeierEstimator)
    mod("laser_core.demographics.pyramid", AliasedDistribution=core.AliasedDistribution,
        load_pyramid_csv=core.load_pyramid_csv)
    return mods


class _AliveBar:
    def __init__(self, *a, **k):
        pass

    def __enter__(self):
        return lambda *a, **k: None

    def __exit__(self, *exc):
        return False


INERT_PACKAGES = ("matplotlib", "cartopy", "imageio_ffmpeg", "pandas", "geopandas", "click", "yaml", "pytz",
                  "sciris", "alive_progress", "seaborn", "h5py", "optuna", "shapely")


class _InertFinder:
    """Import hook: any module of INERT_PACKAGES (and its submodules) is an
    inert package."""

    def find_spec(self, name, path=None, target=None):
        import importlib.machinery

        if name.split(".")[0] in INERT_PACKAGES:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = _InertModule(spec.name)
        m.__path__ = []
        return m

    def exec_module(self, module):
        pass


def install_standins():
    sys.modules["numba"] = _numba_module()
    sys.modules.update(_laser_core_modules())
    if not any(isinstance(f, _InertFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _InertFinder())
    import sciris  # noqa: F401  (inert)
    import alive_progress  # noqa: F401  (inert)

    import pytz  # noqa: F401  (inert, but for its one real use: a tzinfo for the log file's name)
    import zoneinfo

    sys.modules["pytz"].timezone = zoneinfo.ZoneInfo
    sc = sys.modules["sciris"]
    for fn in ("printred", "printgreen", "printcyan", "printyellow"):
        setattr(sc, fn, lambda *a, **k: None)
    sys.modules["alive_progress"].alive_bar = _AliveBar


def import_reference(src_dir):
    """laser_polio from ``src_dir`` (the checkout's src/), unmodified."""
    install_standins()
    if str(src_dir) not in sys.path:
        sys.path.insert(0, str(src_dir))
    lp = importlib.import_module("laser_polio")
    return lp


# ---------------------------------------------------------------------------
# the draw hook

P_PARALYSIS, P_RI, P_SIA, P_BIRTH, P_KM, P_TXCOUNT, P_SELECT, P_STRAIN, P_SEEDPICK, P_SEEDTIMER = range(1, 11)


class _NumpyWithHook(types.ModuleType):
    """numpy, except ``random``."""

    def __init__(self, hook):
        super().__init__("numpy")
        object.__setattr__(self, "_hook", hook)

    def __getattr__(self, name):
        if name == "random":
            return self._hook
        return getattr(np, name)


class DrawHook:
    """np.random for the reference's modules during replay (see the module
    docstring).  ``sim`` gives the tick (sim.t) and the seed (pars.seed)."""

    def __init__(self, sim, seed_events, dist_spec):
        from oracle import oracle as O

        self.L = O.lib()
        self.sim = sim
        self.seed = int(sim.pars.seed) & 0xFFFFFFFFFFFFFFFF
        self.seed_events = seed_events  # [(tick, node, value)] in the order the engine numbers them
        self.dist_spec = dist_spec      # (kind, p1, p2) of dur_inf
        self.rounds = {}                # (tick, node) -> selection rounds drawn
        self.calls = {}
        self._ri_k = {}                 # (tick, slot) -> RI draws made
        self._seed_used = set()         # (tick, position) of seed entries already drawn

    # bookkeeping --------------------------------------------------------------
    def _t(self):
        return int(self.sim.t)

    def _count(self, what):
        self.calls[what] = self.calls.get(what, 0) + 1

    @staticmethod
    def _frame(depth=2):
        return sys._getframe(depth)

    def _unknown(self, name, f):
        raise RuntimeError(f"draw hook: np.random.{name} from {f.f_code.co_name} "
                           f"({f.f_code.co_filename}:{f.f_lineno}) has no counterpart in the replayed stream")

    # the calls of the per-tick step ------------------------------------------
    def random(self, size=None):
        f = self._frame()
        if f.f_code.co_name == "disease_state_step_kernel" and size is None:
            self._count("paralysis")
            return self.L.lpo_u01(self.seed, P_PARALYSIS, self._t(), int(f.f_locals["i"]), 0, 0)
        self._unknown("random", f)

    def rand(self, *shape):
        f = self._frame()
        name = f.f_code.co_name
        t = self._t()
        if name == "fast_ri" and not shape:
            i = int(f.f_locals["i"])
            k = self._ri_k.get((t, i), 0)  # first draw OPV, second IPV
            self._ri_k[(t, i)] = k + 1
            self._count("ri")
            return self.L.lpo_u01(self.seed, P_RI, t, i, 0, k)
        if name == "fast_sia" and not shape:
            self._count("sia")
            return self.L.lpo_u01(self.seed, P_SIA, t, int(f.f_locals["i"]), 0, self._sia_k(f))
        if name == "step" and not shape and "node_seeding_zero_inflation" in f.f_locals:
            self._count("zero_inflation")
            return self.L.lpo_tx_u0(self.seed, t, int(f.f_locals["n"]))
        if name == "tx_infect_nb":
            node = int(f.f_locals["node"])
            if not shape:  # the strain of a selected agent
                self._count("strain")
                return self.L.lpo_u01(self.seed, P_STRAIN, t, int(f.f_locals["person_idx"]), 0, 0)
            (k,) = shape
            r = self.rounds.get((t, node), 0)
            self.rounds[(t, node)] = r + 1
            self._count("select")
            m = np.array([self.L.lpo_u53(self.seed, P_SELECT, t, node, r, q) for q in range(int(k))], np.uint64)
            return m.astype(np.float64) * 2.0**-53
        self._unknown("rand", f)

    def poisson(self, lam, size=None):
        f = self._frame()
        if f.f_code.co_name == "step" and "node_seeding_zero_inflation" in f.f_locals and size is None:
            self._count("poisson")
            return self.L.lpo_tx_poisson(self.seed, self._t(), int(f.f_locals["n"]), float(lam))
        self._unknown("poisson", f)

    def negative_binomial(self, r, p, size=None):
        f = self._frame()
        if f.f_code.co_name == "step" and "node_seeding_zero_inflation" in f.f_locals and size is None:
            self._count("negbinom")
            return self.L.lpo_tx_negbinom(self.seed, self._t(), int(f.f_locals["n"]), float(r), float(p))
        self._unknown("negative_binomial", f)

    def multinomial(self, n, pvals, size=None):
        # the split only fixes the total (tx_infect_nb sums it per node and
        # draws each agent's strain itself): any split of n will do
        f = self._frame()
        if f.f_code.co_name == "step" and "node_seeding_zero_inflation" in f.f_locals:
            out = np.zeros(len(pvals), np.int64)
            out[0] = n
            return out
        self._unknown("multinomial", f)

    def binomial(self, n, p, size=None):
        f = self._frame()
        if f.f_code.co_name == "step" and "birth_fraction" in f.f_locals and np.all(np.asarray(n) == 1):
            t = self._t()
            p = np.asarray(p, dtype=np.float64)
            u = np.array([self.L.lpo_u01(self.seed, P_BIRTH, t, nd, 0, 0) for nd in range(len(p))])
            self._count("births")
            return (u < p).astype(np.int64)
        self._unknown("binomial", f)

    def choice(self, a, size=None, replace=True, p=None):
        f = self._frame()
        if f.f_code.co_name == "step" and "candidates" in f.f_locals and not replace:
            t = self._t()
            e = self._seed_event(f, t)
            cand = np.asarray(a, dtype=np.int64)
            keys = np.array([self.L.lpo_raw(self.seed, P_SEEDPICK, t, int(i), e, 0) for i in cand], np.uint64)
            order = np.lexsort((cand, keys))
            self._count("seed_pick")
            self._seed_e = e
            return cand[order[: int(size)]]
        self._unknown("choice", f)

    def gamma(self, shape, scale=1.0, size=None):
        return self._seed_timer("gamma", size)

    def normal(self, loc=0.0, scale=1.0, size=None):
        return self._seed_timer("normal", size)

    def _seed_timer(self, name, size):
        # dur_inf(n) of the seed schedule (model.py:777) through Distribution.sample's
        # numba loop: the slot is the caller's inds_zero_timers[i]
        f = self._frame(3)
        loop = f
        g = f.f_back
        while g is not None and not (g.f_code.co_name == "step" and "inds_zero_timers" in g.f_locals):
            g = g.f_back
        if g is None or size is not None or "i" not in loop.f_locals:
            self._unknown(name, f)
        slot = int(g.f_locals["inds_zero_timers"][int(loop.f_locals["i"])])
        kind, p1, p2 = self.dist_spec
        self._count("seed_timer")
        return self.L.lpo_seed_timer(self.seed, self._t(), slot, self._seed_e, kind, p1, p2)

    # helpers -----------------------------------------------------------------
    def _sia_k(self, f):
        g = f.f_back  # SIA_ABM.step: which of the day's events this is
        ev = g.f_locals["event"]
        day = [e for e in g.f_locals["self"].sia_schedule if e["date"] == g.f_locals["self"].sim.datevec[self._t()]]
        return next(k for k, e in enumerate(day) if e is ev)

    def _seed_event(self, f, t):
        node, value = f.f_locals["node_id"], f.f_locals["value"]
        entries = f.f_locals["self"].seed_schedule[t]
        pos = next(k for k, e in enumerate(entries)
                   if e[0] == node and e[1] is value and (t, k) not in self._seed_used)
        self._seed_used.add((t, pos))
        # the engine numbers events in the order build_sim_spec lists them
        k = 0
        for e, (tt, nd, val) in enumerate(self.seed_events):
            if tt == t:
                if k == pos:
                    return e
                k += 1
        raise RuntimeError(f"draw hook: seed event {pos} of tick {t} not found")


def km_hook_factory(hook, cum, max_year):
    """predict_age_at_death for the newborns of VitalDynamics_ABM.step
    (model.py:1724-1725): the engine's Kaplan-Meier draw per slot."""
    L = hook.L
    cum = np.ascontiguousarray(cum, dtype=np.int64)

    def predict(ages_days, max_year=max_year, _orig=None):
        f = sys._getframe(1)
        if f.f_code.co_name == "step" and "start" in f.f_locals and "end" in f.f_locals:
            t = hook._t()
            start, end = int(f.f_locals["start"]), int(f.f_locals["end"])
            cp = cum.ctypes.data_as(C.POINTER(C.c_int64))
            hook._count("km")
            return np.array([L.lpo_km_newborn(cp, len(cum), int(max_year), hook.seed, t, s) for s in range(start, end)],
                            dtype=np.int32)
        raise RuntimeError("draw hook: predict_age_at_death outside the newborn step")

    return predict


def attach(lp_model_modules, hook):
    """np.random -> hook in the given reference modules."""
    proxy = _NumpyWithHook(hook)
    for m in lp_model_modules:
        m.np = proxy


def detach(lp_model_modules):
    for m in lp_model_modules:
        m.np = np
