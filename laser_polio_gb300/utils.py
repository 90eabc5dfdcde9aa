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

GROUPING_LEVELS = ("adm0", "adm01", "dot_name")


def time_period_labels(dates, time_config):
    """The time_period label of each date (add_temporal_groupings,
    utils.py:1040-1073): bins [bins[i-1], bins[i]) closed on the left, the
    first open below and the last open above (pd.cut with right=False);
    len(labels) must be len(bins) + 1.  None when the config has no bins."""
    if "bins" not in time_config or "labels" not in time_config:
        return None
    edges = np.array([np.datetime64(date(b), "D") for b in time_config["bins"]])
    labels = [str(x) for x in time_config["labels"]]
    if len(labels) != len(edges) + 1:
        raise ValueError("time_periods: there must be one label more than bin edges")
    days = np.array([np.datetime64(date(d), "D") for d in dates])
    return [labels[k] for k in np.searchsorted(edges, days, side="right")]


def _pattern_hits(pattern, names):
    import re

    rx = re.compile(pattern, re.IGNORECASE)
    return np.array([bool(rx.search(n)) for n in names])


def regional_columns(dot_names, region_groupings=None, grouping_level="adm0", regions_yaml_path=None, regions=None):
    """adm0, adm1, adm01 and region of each dot name (add_regional_groupings,
    utils.py:1076-1160): adm0 and adm1 are the dot name's second and third
    ':' fields ("" where missing, pandas' NaN), adm01 = adm0 + ":" + adm1,
    and region the column named by grouping_level (adm0, adm01 or
    dot_name).  For each country in region_groupings, its nodes whose adm01
    equals a pattern with ':' (at the adm01 level) or whose dot name contains
    the pattern (a case-insensitive regular expression, as str.contains) take
    the group's name.  The groups come from ``regions`` (a dict as in
    data/regions.yaml) or from the YAML file; a file that cannot be read
    leaves the default regions, as the reference does."""
    if grouping_level not in GROUPING_LEVELS:
        raise ValueError(f"Invalid grouping_level: {grouping_level}. Must be one of 'adm0', 'adm01', or 'dot_name'.")
    parts = [n.split(":") for n in dot_names]
    adm0 = [p[1] if len(p) > 1 else "" for p in parts]
    adm1 = [p[2] if len(p) > 2 else "" for p in parts]
    adm01 = [f"{a}:{b}" if a != "" and b != "" else "" for a, b in zip(adm0, adm1)]
    cols = {"adm0": adm0, "adm1": adm1, "adm01": adm01, "dot_name": list(dot_names)}
    region = np.array(cols[grouping_level], dtype=object)
    if region_groupings:
        data = regions
        if data is None:
            try:
                import yaml

                from . import root

                with open(regions_yaml_path or root / "data" / "regions.yaml") as f:
                    data = yaml.safe_load(f)
            except (FileNotFoundError, ImportError, OSError):
                print(f"Warning: Could not load {regions_yaml_path}, using adm0 for all countries")
                data = None
        if data is not None:
            a0 = np.array(adm0, dtype=object)
            a01 = np.array(adm01, dtype=object)
            for country in region_groupings:
                upper = country.upper()
                if upper not in data:
                    print(f"Warning: Custom regions not found for {country} in regions.yaml, using adm0")
                    continue
                in_country = a0 == upper
                for group, patterns in data[upper].items():
                    hit = np.zeros(len(dot_names), dtype=bool)
                    for pat in patterns:
                        if grouping_level == "adm01" and ":" in pat:
                            hit |= a01 == pat
                        else:
                            hit |= _pattern_hits(pat, dot_names)
                    region[in_country & hit] = group
    return {"adm0": adm0, "adm1": adm1, "adm01": adm01, "region": [str(x) for x in region]}


def save_sim_results(sim, filename="simulation_results.h5", summary_config=None):
    """Save the results table of a run (utils.py:689-786): one row per
    (timestep, node), timestep-major, with the columns timestep, date, node,
    dot_name (from ``sim.pars.node_lookup``, "UNKNOWN" where missing), S, E,
    I, R, P, births, deaths, new_exposed, potentially_paralyzed,
    new_potentially_paralyzed and new_paralyzed.

    With a ``summary_config`` (run_sim always passes one), the reference's
    groupings follow: time_period from its "time_periods" (bins, labels),
    then adm0, adm1, adm01 and region from "region_groupings" and
    "grouping_level" (both given, or region_groupings alone at the adm0
    level, or grouping_level alone, or neither at the dot_name level).
    The custom regions come from data/regions.yaml under ``root`` (PyYAML),
    from "regions_yaml_path", or — an addition for hosts without PyYAML —
    from a "regions" dict of the same structure in the summary_config.

    A ``.h5`` name is written as the reference does (pandas ``to_hdf``,
    key "results", table format, complevel 5), so it needs pandas with
    PyTables.  Any other name is written as CSV by native host code
    (``lpg_write_results_csv``), in the format of pandas'
    ``to_csv(index=False)``.  Returns the table: a pandas DataFrame when
    pandas is importable, else a dict of numpy columns.
    """
    import ctypes as C
    from pathlib import Path

    from . import _lib

    nt, nodes = int(sim.nt), len(sim.nodes)
    try:
        lookup = sim.pars.node_lookup or {}
    except (AttributeError, KeyError):
        lookup = {}
    dot_names = [str(lookup.get(n, {}).get("dot_name", "UNKNOWN")) for n in range(nodes)]
    datevec = list(sim.datevec)[:nt]
    dates = [str(d) for d in datevec]
    if len(dates) != nt:
        raise ValueError(f"save_sim_results: {len(dates)} dates for {nt} timesteps")
    fields = {}
    for col, attr in RESULT_TABLE_COLUMNS:
        raw = np.asarray(getattr(sim.results, attr))
        if raw.dtype.kind not in "iub":
            raise TypeError(f"save_sim_results: results.{attr} is {raw.dtype}; the native writer takes integer "
                            "counts (the reference's results arrays are int32)")
        if raw.size and (int(raw.min()) < np.iinfo(np.int32).min or int(raw.max()) > np.iinfo(np.int32).max):
            raise ValueError(f"save_sim_results: results.{attr} holds values outside int32")
        a = np.ascontiguousarray(raw, dtype=np.int32)
        if a.shape != (nt, nodes):
            raise ValueError(f"save_sim_results: results.{attr} has shape {a.shape}, expected {(nt, nodes)}")
        fields[col] = a
    tick_cols, node_cols = {}, {}
    if summary_config is not None:
        if "time_periods" in summary_config:
            labels = time_period_labels(dates, summary_config["time_periods"])
            if labels is not None:
                tick_cols["time_period"] = labels
        groups = summary_config.get("region_groupings", None)
        level = summary_config.get("grouping_level", None)
        if groups is not None:
            node_cols = regional_columns(dot_names, groups, level if level is not None else "adm0",
                                         regions_yaml_path=summary_config.get("regions_yaml_path"),
                                         regions=summary_config.get("regions"))
        else:
            node_cols = regional_columns(dot_names, grouping_level=level if level is not None else "dot_name")
    table = {
        "timestep": np.repeat(np.arange(nt), nodes),
        "date": np.repeat(np.asarray(datevec, dtype=object), nodes),
        "node": np.tile(np.arange(nodes), nt),
        "dot_name": np.tile(np.asarray(dot_names, dtype=object), nt),
        **{col: a.reshape(-1) for col, a in fields.items()},
        **{col: np.repeat(np.asarray(v, dtype=object), nodes) for col, v in tick_cols.items()},
        **{col: np.tile(np.asarray(v, dtype=object), nt) for col, v in node_cols.items()},
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

    def enc(xs):
        return (C.c_char_p * max(1, len(xs)))(*[x.encode() for x in xs])

    names = [col for col, _ in RESULT_TABLE_COLUMNS]
    ptrs = (C.c_void_p * len(names))(*[fields[c].ctypes.data for c in names])
    tick_vals = [v for col in tick_cols for v in tick_cols[col]]
    node_vals = [v for col in node_cols for v in node_cols[col]]
    rc = lib.lpg_write_results_csv(str(filename).encode(), nt, nodes, enc(dates), enc(dot_names), len(names),
                                   enc(names), ptrs, len(tick_cols), enc(list(tick_cols)), enc(tick_vals),
                                   len(node_cols), enc(list(node_cols)), enc(node_vals))
    if rc != 0:
        raise OSError(lib.lpg_op_last_error().decode())
    if pd is not None:
        df = pd.DataFrame(table)
        df["dot_name"] = df["dot_name"].astype("category")
        return df
    return table
