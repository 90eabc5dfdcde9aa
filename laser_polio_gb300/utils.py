"""Calendar and demographic helpers used on the per-tick path.

Restates laser_polio/utils.py:137-161 (date, daterange), :589-625 (get_doy,
get_seasonality) and :795-816 (create_cumulative_deaths).
"""

from __future__ import annotations

import calendar
import datetime as dt

import numpy as np


def date(value):
    """A datetime.date from 'YYYY-MM-DD' or a date (utils.py:137-143)."""
    if isinstance(value, dt.datetime):
        return value.date()
    if isinstance(value, dt.date):
        return value
    return dt.datetime.strptime(value, "%Y-%m-%d").date()


def daterange(start_date, days):
    """Array of ``days`` consecutive dates from ``start_date`` (utils.py:146-161)."""
    start_date = date(start_date)
    return np.array([start_date + dt.timedelta(days=i) for i in range(days)])


def get_doy(sim):
    """1-based day of year of the current tick (utils.py:589-613)."""
    return sim.datevec[sim.t].timetuple().tm_yday


def get_seasonality(sim):
    """1 + amplitude * cos(2 pi (doy - peak) / days_in_year), with a 366-day
    year in leap years (utils.py:616-625)."""
    doy = get_doy(sim)
    year = sim.datevec[sim.t].year
    days_in_year = 366 if calendar.isleap(year) else 365
    return 1 + sim.pars["seasonal_amplitude"] * np.cos(2 * np.pi * (doy - sim.pars["seasonal_peak_doy"]) / days_in_year)


def seasonality_table(datevec, amplitude, peak_doy):
    """get_seasonality evaluated at every tick of ``datevec`` (float64)."""
    out = np.empty(len(datevec), dtype=np.float64)
    for t, d in enumerate(datevec):
        days_in_year = 366 if calendar.isleap(d.year) else 365
        doy = d.timetuple().tm_yday
        out[t] = 1 + amplitude * np.cos(2 * np.pi * (doy - peak_doy) / days_in_year)
    return out


def create_cumulative_deaths(total_population, max_age_years):
    """Back-loaded cumulative deaths by age-year (utils.py:795-816)."""
    ages_years = np.arange(max_age_years + 1)
    base_mortality_rate = 0.0001
    growth_factor = 2
    mortality_rates = base_mortality_rate * (growth_factor ** (ages_years / 10))
    return np.cumsum(mortality_rates * total_population).astype(int)


# save_sim_results' result columns: (column name, sim.results attribute)
RESULT_TABLE_COLUMNS = (
    ("S", "S"),
    ("E", "E"),
    ("I", "I"),
    ("R", "R"),
    ("P", "paralyzed"),
    ("births", "births"),
    ("deaths", "deaths"),
    ("new_exposed", "new_exposed"),
    ("potentially_paralyzed", "potentially_paralyzed"),
    ("new_potentially_paralyzed", "new_potentially_paralyzed"),
    ("new_paralyzed", "new_paralyzed"),
)


def save_sim_results(sim, filename="simulation_results.h5", summary_config=None):
    """Save the results table of a run (utils.py:689-786): one row per
    (timestep, node), timestep-major, with the columns timestep, date, node,
    dot_name (from ``sim.pars.node_lookup``, "UNKNOWN" where missing), S, E,
    I, R, P, births, deaths, new_exposed, potentially_paralyzed,
    new_potentially_paralyzed and new_paralyzed.

    A ``.h5`` name is written as the reference does (pandas ``to_hdf``,
    key "results", table format, complevel 5), so it needs pandas with
    PyTables.  Any other name is written as CSV by native host code
    (``lpg_write_results_csv``), in the format of pandas'
    ``to_csv(index=False)``.  Returns the table: a pandas DataFrame when
    pandas is importable, else a dict of numpy columns.

    ``summary_config`` (the reference's temporal and regional groupings,
    utils.py:1040-1160) is not supported and raises NotImplementedError.
    """
    import ctypes as C
    from pathlib import Path

    from . import _lib

    if summary_config is not None:
        raise NotImplementedError("save_sim_results: summary_config groupings are not supported")
    nt, nodes = int(sim.nt), len(sim.nodes)
    try:
        lookup = sim.pars.node_lookup or {}
    except (AttributeError, KeyError):
        lookup = {}
    dot_names = [str(lookup.get(n, {}).get("dot_name", "UNKNOWN")) for n in range(nodes)]
    dates = [str(d) for d in list(sim.datevec)[:nt]]
    if len(dates) != nt:
        raise ValueError(f"save_sim_results: {len(dates)} dates for {nt} timesteps")
    fields = {}
    for col, attr in RESULT_TABLE_COLUMNS:
        a = np.ascontiguousarray(np.asarray(getattr(sim.results, attr)), dtype=np.int32)
        if a.shape != (nt, nodes):
            raise ValueError(f"save_sim_results: results.{attr} has shape {a.shape}, expected {(nt, nodes)}")
        fields[col] = a
    table = {
        "timestep": np.repeat(np.arange(nt), nodes),
        "date": np.repeat(np.asarray(list(sim.datevec)[:nt], dtype=object), nodes),
        "node": np.tile(np.arange(nodes), nt),
        "dot_name": np.tile(np.asarray(dot_names, dtype=object), nt),
        **{col: a.reshape(-1) for col, a in fields.items()},
    }
    try:
        import pandas as pd
    except ImportError:
        pd = None
    if Path(filename).suffix == ".h5":
        if pd is None:
            raise ImportError("save_sim_results: writing .h5 needs pandas (with PyTables)")
        df = pd.DataFrame(table)
        df["dot_name"] = df["dot_name"].astype("category")
        df["date"] = pd.to_datetime(df["date"])
        df.to_hdf(filename, key="results", mode="w", format="table", complevel=5)
        return df
    lib = _lib.load()
    enc = lambda xs: (C.c_char_p * len(xs))(*[x.encode() for x in xs])  # noqa: E731
    names = [col for col, _ in RESULT_TABLE_COLUMNS]
    ptrs = (C.c_void_p * len(names))(*[fields[c].ctypes.data for c in names])
    rc = lib.lpg_write_results_csv(str(filename).encode(), nt, nodes, enc(dates), enc(dot_names), len(names),
                                   enc(names), ptrs)
    if rc != 0:
        raise OSError(lib.lpg_op_last_error().decode())
    if pd is not None:
        df = pd.DataFrame(table)
        df["dot_name"] = df["dot_name"].astype("category")
        return df
    return table
