"""laser_polio_gb300 — the per-tick agent step of laser-polio on a GB300.

Drop-in replacements for laser_polio's SEIR_ABM components
(VitalDynamics_ABM, DiseaseState_ABM, RI_ABM, SIA_ABM, Transmission_ABM)
whose step() and log() run as hand-written sm_103a CUDA kernels behind the
C ABI in include/lpg.h.  The parameter contract (pars), the Distribution
objects and the sim.results arrays are the reference's.
"""

from pathlib import Path

__version__ = "0.1.0"

# the project root, as laser_polio.root (tests patch it to find data files)
root = Path(__file__).resolve().parents[1]

from .core import LaserFrame
from .core import PropertySet
from .distributions import Distribution
from .distributions import constant
from .distributions import exponential
from .distributions import gamma
from .distributions import lognormal
from .distributions import lognormal_int
from .distributions import normal
from .distributions import poisson
from .distributions import uniform
from .model import RI_ABM
from .model import SEIR_ABM
from .model import SIA_ABM
from .model import DiseaseState_ABM
from .model import Transmission_ABM
from .model import VitalDynamics_ABM
from .pars import default_pars
from .pars import default_run_order
from .utils import create_cumulative_deaths
from .utils import date
from .utils import daterange
from .utils import get_doy
from .utils import get_seasonality
from .utils import save_sim_results


def count_SEIRP(*args, **kwargs):
    """laser_polio.count_SEIRP (model.py:869-899) on the GPU: see
    laser_polio_gb300.ops.count_SEIRP (imported on first use, with torch)."""
    from .ops import count_SEIRP as _count

    return _count(*args, **kwargs)

__all__ = [
    "RI_ABM",
    "SEIR_ABM",
    "SIA_ABM",
    "DiseaseState_ABM",
    "Distribution",
    "LaserFrame",
    "PropertySet",
    "Transmission_ABM",
    "VitalDynamics_ABM",
    "constant",
    "count_SEIRP",
    "create_cumulative_deaths",
    "date",
    "daterange",
    "default_pars",
    "default_run_order",
    "exponential",
    "gamma",
    "get_doy",
    "get_seasonality",
    "lognormal",
    "lognormal_int",
    "normal",
    "poisson",
    "root",
    "save_sim_results",
    "uniform",
]
