"""epetreco_gb300 -- GB300 (sm_103a) implementation of epetreco's MLEM hot path.

The compute lives in ``libepet_gb300.so`` (hand-written CUDA behind the C ABI
of ``include/epet_gb300.h``); this package is the host-side mirror of the
reference's operator surface (``api``) plus geometry descriptors
(``problem``) and synthetic inputs (``phantom``).
"""
from .problem import (CONFIGS, MeasurementSetup, Problem, VoxelGrid, centred_grid, config,
                      two_head_setup)

__all__ = ["CONFIGS", "MeasurementSetup", "Problem", "VoxelGrid", "centred_grid", "config",
           "two_head_setup", "api", "build"]


def __getattr__(name):
    if name in ("api", "build", "phantom"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
