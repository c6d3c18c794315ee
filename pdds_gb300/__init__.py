"""pdds_gb300: GB300-native Feynman-Kac estimation of the PDDSparse interface system.

The compute path is libpdds_gb300.so (hand-written sm_103a CUDA behind the C
ABI of include/pdds.h); this package is its host-side mirror of the
reference's BVP / PDDSparseGM call surface.
"""
from ._capi import (MODE_FP64, MODE_MIXED, MODE_REPLAY_FP64, SOLVE_BICGSTAB_FP64, SOLVE_GMRES_FP32_IR,
                    PDDSError)
from .api import (BVP, Batch, EMFKACSolver, Estimate, Instance, PDDSparseGM, Stencil, read_configuration,
                  release_cached_blocks)
from .checkpoint import estimate_resumable
from .output_files import TimeFile, write_knot_metadata, write_outputs

__all__ = ["BVP", "Batch", "EMFKACSolver", "Estimate", "Stencil", "Instance", "PDDSparseGM", "PDDSError",
           "read_configuration", "release_cached_blocks", "estimate_resumable", "TimeFile", "write_knot_metadata", "write_outputs",
           "MODE_FP64", "MODE_MIXED", "MODE_REPLAY_FP64", "SOLVE_BICGSTAB_FP64", "SOLVE_GMRES_FP32_IR"]
