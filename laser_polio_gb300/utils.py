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
