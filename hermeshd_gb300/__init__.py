"""hermeshd_gb300: GB300-native DG right-hand side and SSP-RK time step of
HERMESHD (5/10-moment systems), behind the reference's Python call surface.

``from hermeshd_gb300 import hermeshd`` gives the module whose ``hermeshd``
instance has ``main/setup/step/generate_output/cleanup`` with the reference's
signatures (src/hermeshd.py:5-120).  ``Solver``/``Ensemble`` are the
device-tensor API.  All compute runs in libhermes_gb300.so (sm_103a).
"""
from .config import Config, NQ, VARS  # noqa: F401
from . import config, ic  # noqa: F401


def __getattr__(name):
    # lazy: importing the package does not need torch or the CUDA library
    import importlib
    if name in ("Solver", "Ensemble"):
        return getattr(importlib.import_module(__name__ + ".solver"), name)
    if name in ("hermeshd", "solver"):
        return importlib.import_module(__name__ + "." + name)
    raise AttributeError(name)
