"""GB300-native engine for the G3LHalo aperture-statistics hot path.

The compute path lives in libg3lgpu.so (CUDA, sm_103a); this package is its
Python front-end (``api``), the synthetic table generator (``tables``) and the
standard workloads (``workloads``).
"""
from .api import (FP64, MIXED, NMAPMAP, NNMAP, Context, G3LError, NMapMapModel,  # noqa: F401
                  NNMapModel, Server, hcubature_v, host_densities, lib, library_path,
                  precompute_tables)

__all__ = ["FP64", "MIXED", "NNMAP", "NMAPMAP", "Context", "G3LError", "NNMapModel",
           "NMapMapModel", "Server", "hcubature_v", "host_densities", "lib", "library_path",
           "precompute_tables"]
