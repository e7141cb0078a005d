"""GB300-native state-vector engine with qsim's Simulator/StateSpace API.

The compute path is hand-written sm_103a CUDA in libqsim_gb300.so behind a
C ABI (include/qsim_gb300.h); this package is the Python mirror of the
reference's interface over that ABI.  Importing it fails if the library has
not been built: there is no CPU fallback.
"""
from ._native import LIB_PATH, QsgError  # noqa: F401  (raises if missing)
from .api import (Context, MeasurementResult, Rng, Simulator, State,  # noqa: F401
                  StateSpace, default_context)
