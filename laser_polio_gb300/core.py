"""Host-side containers that the reference takes from laser_core.

laser_core (~=0.6, not vendored with the reference and not installed here)
provides ``PropertySet`` (the parameter bag), ``LaserFrame`` (the
structure-of-arrays agent table) and a handful of demographic and migration
helpers.  The reference uses them at these call sites:
laser_polio/model.py:13-23 (imports), :139 (LaserFrame), :1235-1258
(distance/gravity/radiation/row_normalizer), :1535-1536, :1605-1611
(KaplanMeierEstimator), :1558-1559, :1583-1584 (AliasedDistribution,
load_pyramid_csv), :129-131 (calc_capacity).  This module restates the
behaviour those call sites rely on; the semantics of the numerical helpers
come from their published descriptions and the reference's own comments
(scripts/sandbox/debug_row_normalizer.py:14-32), and are not pinned by any
reference test.
"""

from __future__ import annotations

import copy
import math
from pathlib import Path

import numpy as np


class PropertySet:
    """Attribute-and-item parameter bag (laser_core.propertyset.PropertySet).

    ``a <<= b`` overrides existing keys (the reference filters unknown keys
    before using it, model.py:62-72); ``a += b`` adds or overrides keys.
    """

    def __init__(self, *dicts, **kwargs):
        object.__setattr__(self, "_d", {})
        for d in dicts:
            self._d.update(d.to_dict() if isinstance(d, PropertySet) else dict(d))
        self._d.update(kwargs)

    def __getattr__(self, k):
        try:
            return self._d[k]
        except KeyError:
            raise AttributeError(k) from None

    def __setattr__(self, k, v):
        self._d[k] = v

    def __getitem__(self, k):
        return self._d[k]

    def __setitem__(self, k, v):
        self._d[k] = v

    def __contains__(self, k):
        return k in self._d

    def __iter__(self):
        return iter(self._d)

    def __len__(self):
        return len(self._d)

    def get(self, k, default=None):
        return self._d.get(k, default)

    def keys(self):
        return self._d.keys()

    def items(self):
        return self._d.items()

    def values(self):
        return self._d.values()

    def to_dict(self):
        return dict(self._d)

    def __ilshift__(self, other):
        other = other.to_dict() if isinstance(other, PropertySet) else dict(other)
        for k in other:
            if k not in self._d:
                raise KeyError(f"Key '{k}' not found in PropertySet")
        self._d.update(other)
        return self

    def __iadd__(self, other):
        other = other.to_dict() if isinstance(other, PropertySet) else dict(other)
        self._d.update(other)
        return self

    def __add__(self, other):
        out = PropertySet(self)
        out += other
        return out

    def __deepcopy__(self, memo):
        return PropertySet(copy.deepcopy(self._d, memo))

    def __repr__(self):
        return f"PropertySet({self._d!r})"


class LaserFrame:
    """Structure-of-arrays agent table (laser_core.laserframe.LaserFrame).

    Columns are arrays of length ``capacity``; ``count`` is the active
    prefix; ``add(n)`` appends n rows and returns (start, end).  There is no
    compaction: dead agents keep their slot.

    A column is either a host numpy array (an ordinary attribute, as in
    laser_core) or device-resident: a CUDA tensor that the device
    initialisation filled and the engine reads and writes in place.  Reading
    a device-resident column by attribute (``people.disease_state``) copies it
    to the host once; from then on the numpy array is the column, so callers
    may change it in place before a run, as the reference's tests do.  The
    engine takes each column from wherever it lives (``engine_columns``).
    """

    def __init__(self, capacity: int, initial_count: int = -1):
        self._capacity = int(capacity)
        self._count = self._capacity if initial_count < 0 else int(initial_count)
        self._dev = {}
        if self._count > self._capacity:
            raise ValueError(f"initial_count {initial_count} exceeds capacity {capacity}")

    def __getattr__(self, name):
        dev = self.__dict__.get("_dev")
        if dev is not None and name in dev:
            host = dev.pop(name).cpu().numpy()
            object.__setattr__(self, name, host)
            return host
        raise AttributeError(name)

    def has_column(self, name) -> bool:
        return name in self.__dict__.get("_dev", {}) or isinstance(self.__dict__.get(name), np.ndarray)

    def device_columns(self) -> dict:
        """The columns that live on the device, by name (CUDA tensors)."""
        return dict(self._dev)

    def set_device_column(self, name, tensor):
        """Make ``tensor`` (CUDA, length capacity) the column ``name``; a host
        copy of the column, if there was one, is dropped."""
        if int(tensor.shape[0]) != self._capacity:
            raise ValueError(f"column {name}: {tuple(tensor.shape)} elements for capacity {self._capacity}")
        self.__dict__.pop(name, None)
        self._dev[name] = tensor

    def engine_columns(self, names) -> dict:
        """name -> the column as it lives (CUDA tensor or numpy array) for
        the names present, without copying anything."""
        out = {}
        for name in names:
            if name in self._dev:
                out[name] = self._dev[name]
            elif isinstance(self.__dict__.get(name), np.ndarray):
                out[name] = self.__dict__[name]
        return out

    @property
    def capacity(self) -> int:
        return self._capacity

    @property
    def count(self) -> int:
        return self._count

    def _set_count(self, n: int):
        self._count = int(n)

    def __len__(self) -> int:
        """The active count, as laser_core's LaserFrame (len(sim.people) in
        tests/test_seir_abm_init.py:25)."""
        return self._count

    def add_scalar_property(self, name, dtype=np.uint32, default=0):
        self._dev.pop(name, None)
        setattr(self, name, np.full(self._capacity, default, dtype=dtype))

    def add_vector_property(self, name, length, dtype=np.uint32, default=0):
        setattr(self, name, np.full((length, self._capacity), default, dtype=dtype))

    def add_array_property(self, name, shape, dtype=np.uint32, default=0):
        setattr(self, name, np.full(shape, default, dtype=dtype))

    def add(self, count: int):
        if self._count + count > self._capacity:
            raise ValueError(f"Capacity exceeded: count {self._count} + {count} > capacity {self._capacity}")
        start = self._count
        self._count += int(count)
        return start, self._count


def calc_capacity(population, nticks, cbr):
    """Population after ``nticks`` days of growth at crude birth rate ``cbr``
    per 1000 per year (laser_core.utils.calc_capacity as used at
    model.py:129-131)."""
    growth = (1.0 + float(cbr) / 1000.0) ** (float(nticks) / 365.0)
    return int(math.ceil(float(population) * growth))


def distance(lat1, lon1, lat2, lon2):
    """Great-circle distance in km (haversine), laser_core.migration.distance."""
    r = 6371.0
    p1, p2 = np.radians(lat1), np.radians(lat2)
    dphi = p2 - p1
    dl = np.radians(lon2) - np.radians(lon1)
    a = np.sin(dphi / 2) ** 2 + np.cos(p1) * np.cos(p2) * np.sin(dl / 2) ** 2
    return 2 * r * np.arcsin(np.sqrt(a))


def gravity(pops, distances, k, a, b, c):
    """Gravity flows k * p_i^a * p_j^b / d_ij^c with a zero diagonal
    (scripts/sandbox/debug_row_normalizer.py:14)."""
    pops = np.asarray(pops, dtype=np.float64)
    d = np.asarray(distances, dtype=np.float64)
    n = len(pops)
    out = np.zeros((n, n), dtype=np.float64)
    off = ~np.eye(n, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        num = k * np.power(pops[:, None], a) * np.power(pops[None, :], b)
        val = num / np.power(d, c)
    out[off] = val[off]
    out[~np.isfinite(out)] = 0.0
    return out


def radiation(pops, distances, k, include_home=False):
    """Radiation-model flows (Simini et al., Nature 484, 2012):
    k * p_i * p_j / ((p_i + s_ij) (p_i + p_j + s_ij)), s_ij = population
    strictly closer to i than j, excluding i and j (nodes tied with j are
    outside).  Computed by the native lpg_radiation_network (host threads),
    equal bit for bit to the definition in _radiation_py.  include_home=True
    is rejected: the reference only builds include_home=False
    (model.py:1252-1254)."""
    import ctypes as C

    from . import _lib

    p = np.ascontiguousarray(np.asarray(pops, dtype=np.float64))
    d = np.ascontiguousarray(np.asarray(distances, dtype=np.float64))
    n = len(p)
    if d.shape != (n, n):
        raise ValueError(f"radiation: distances have shape {d.shape}, expected {(n, n)}")
    out = np.empty((n, n), dtype=np.float64)
    lib = _lib.load()
    dp = C.POINTER(C.c_double)
    rc = lib.lpg_radiation_network(p.ctypes.data_as(dp), d.ctypes.data_as(dp), n, float(k), int(bool(include_home)),
                                   out.ctypes.data_as(dp))
    if rc != 0:
        raise ValueError(lib.lpg_op_last_error().decode())
    return out


def _radiation_py(pops, distances, k, include_home=False):
    """radiation() as a Python loop: the definition the native builder
    follows operation for operation.  s_ij counts the nodes other than i and
    j strictly closer to i than j (ties with j are outside the circle)."""
    if include_home:
        raise ValueError("include_home=True is not supported (the reference builds its network with "
                         "include_home=False)")
    pops = np.asarray(pops, dtype=np.float64)
    d = np.asarray(distances, dtype=np.float64)
    n = len(pops)
    out = np.zeros((n, n), dtype=np.float64)
    for i in range(n):
        di = d[i]
        order = np.argsort(di, kind="stable")
        sorted_p = pops[order]
        cum = np.cumsum(sorted_p)
        before = np.concatenate([[0.0], cum[:-1]])  # populations of the ranks before each rank
        for rank in range(1, n):  # a tie starts no new sum: the nodes at j's distance are not inside
            if di[order[rank]] == di[order[rank - 1]]:
                before[rank] = before[rank - 1]
        for rank, j in enumerate(order):
            if j == i:
                continue
            s = before[rank] - (pops[i] if di[i] < di[j] else 0.0)
            out[i, j] = k * pops[i] * pops[j] / ((pops[i] + s) * (pops[i] + pops[j] + s))
    return out


def row_normalizer(network, max_rowsum):
    """Scale down rows whose sum exceeds ``max_rowsum`` to exactly that sum
    (scripts/sandbox/debug_row_normalizer.py:31-32)."""
    net = np.array(network, dtype=np.float64, copy=True)
    rs = net.sum(axis=1)
    big = rs > max_rowsum
    net[big] = net[big] * (max_rowsum / rs[big])[:, None]
    return net


class KaplanMeierEstimator:
    """Lifespans from a cumulative-deaths-by-age-year table
    (laser_core.demographics.kmestimator, used at model.py:1605-1611, 1725).

    predict_age_at_death(ages_days): year of death drawn as searchsorted
    (side='right') of a uniform integer between the deaths already behind the
    agent's current age-year and the total up to ``max_year``; the day is
    uniform within that year and not before the current age.
    """

    def __init__(self, cumulative_deaths):
        self.cumulative_deaths = np.asarray(cumulative_deaths, dtype=np.int64)

    def predict_age_at_death(self, ages_days, max_year=100):
        ages_days = np.asarray(ages_days, dtype=np.int64)
        cum = self.cumulative_deaths
        top = min(int(max_year), len(cum) - 1)
        years = np.minimum(ages_days // 365, top)
        lower = np.where(years > 0, cum[np.maximum(years - 1, 0)], 0)
        total = cum[top]
        span = np.maximum(total - lower, 0)
        draw = lower + np.floor(np.random.random(len(ages_days)) * span).astype(np.int64)
        y = np.searchsorted(cum[: top + 1], draw, side="right")
        y = np.where(span > 0, np.maximum(y, years), top)
        y = np.minimum(y, top)
        day_lo = np.where(y == years, ages_days, y * 365)
        day_hi = (y + 1) * 365
        day_hi = np.maximum(day_hi, day_lo + 1)
        return (day_lo + np.floor(np.random.random(len(ages_days)) * (day_hi - day_lo)).astype(np.int64)).astype(np.int32)


class AliasedDistribution:
    """Sampler of bin indices proportional to ``counts``
    (laser_core.demographics.pyramid.AliasedDistribution)."""

    def __init__(self, counts):
        c = np.asarray(counts, dtype=np.float64)
        self._cdf = np.cumsum(c) / c.sum()

    def sample(self, n):
        u = np.random.random(int(n))
        return np.searchsorted(self._cdf, u, side="right").astype(np.int32)


def load_pyramid_csv(path):
    """Read an age pyramid CSV with columns Age ("0-4", ..., "100+"), M, F into
    rows [min_age, max_age, M, F] (laser_core.demographics.pyramid)."""
    rows = []
    with open(path) as fh:
        header = fh.readline()
        del header
        for line in fh:
            parts = [p.strip() for p in line.strip().split(",")]
            if len(parts) < 3 or not parts[0]:
                continue
            age = parts[0]
            if age.endswith("+"):
                lo = int(age[:-1])
                hi = lo + 4
            else:
                lo, hi = (int(x) for x in age.split("-"))
            rows.append([lo, hi, int(float(parts[1])), int(float(parts[2]))])
    return np.array(rows, dtype=np.int64)


def exponential_pyramid(mean_years=20.0, max_years=80, bin_years=5, total=1_000_000):
    """Synthetic age pyramid: exponential ages (mean ``mean_years``) truncated
    to [0, max_years), in the [min, max, M, F] layout of load_pyramid_csv."""
    edges = np.arange(0, max_years + bin_years, bin_years)
    mass = np.exp(-edges[:-1] / mean_years) - np.exp(-edges[1:] / mean_years)
    counts = np.maximum(np.round(mass / mass.sum() * total), 1).astype(np.int64)
    half = counts // 2
    return np.stack([edges[:-1], edges[1:] - 1, half, counts - half], axis=1)


def resolve_pyramid(path_or_array):
    """Pyramid rows from a CSV path, an array, or the synthetic default when
    the path does not exist."""
    if path_or_array is None:
        return exponential_pyramid()
    if isinstance(path_or_array, np.ndarray):
        return path_or_array
    p = Path(path_or_array)
    if p.exists():
        return load_pyramid_csv(p)
    return exponential_pyramid()
