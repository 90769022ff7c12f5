"""pbf_gb300 — GB300-native (sm_103a) Position Based Fluids substep path.

A drop-in for the per-substep simulation path of ekpyron/pbf (the ``SPH``
class, its RadixSort and NeighbourCellFinder): hand-written CUDA kernels in
``csrc/`` behind the C ABI of ``include/pbf.h``, with this package as a thin
Python host mirror of the reference's interface.
"""
from ._capi import (PBF_DEV_NONFINITE, PBF_DEV_RUN_OVER_127, PBF_DEV_SORT_TIMEOUT, PBF_DEVICE,
                    PBF_HOST, Params, PbfError, load)
from .sph import SPH, SPHBatch, default_params
from . import scenes

__all__ = ["SPH", "SPHBatch", "Params", "PbfError", "default_params", "load", "scenes", "PBF_HOST",
           "PBF_DEVICE", "PBF_DEV_NONFINITE", "PBF_DEV_SORT_TIMEOUT", "PBF_DEV_RUN_OVER_127"]
