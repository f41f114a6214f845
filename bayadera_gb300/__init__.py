"""bayadera_gb300 -- GB300 (sm_103a) engine for Bayadera's ensemble stretch-move MCMC path.

The compute path is libbayadera_gb300.so (C ABI: include/bayadera_gb300.h); this
package is the host-side mirror of uncomplicate.bayadera.core / .mcmc over it.
"""
from . import _native, models  # noqa: F401
from .engine import (Autocorrelation, GB300AcorEngine, GB300BayaderaFactory,  # noqa: F401
                     GB300Stretch, GB300StretchFactory, Histogram, check_model)

__version__ = "0.1.0"
