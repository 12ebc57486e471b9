"""GB300 (sm_103a) subspace normal operator for MRISubspaceRecon.jl workloads.

Python mirror of the reference's public API for the hot path, backed by the
C-ABI library ``libmrsr.so`` (hand-written CUDA kernels, ``csrc/``).  There is
no CPU implementation: every call runs on the current CUDA device.
"""
from . import _lib
from .normalop import NFFTNormalOp, FFTNormalOp, NormalOperator
from .backprojection import calculate_backprojection, forward_model
from .solvers import cg, cg_refined, cg_relaxed, cg_stacked, CgBatch
from .grog import grog_calib, grog_gridding, radial_grog
from .coilmaps import (reconstruct_coilwise, calculate_calibration_kspace, calibration_mask, espirit,
                       calculate_coil_maps)
from . import trajectories, synthetic
from .arrays import jl_empty, jl_zeros, jl_reshape, to_jl, to_host

__all__ = ["NFFTNormalOp", "FFTNormalOp", "NormalOperator", "calculate_backprojection", "forward_model", "cg",
           "cg_refined", "cg_relaxed", "cg_stacked", "CgBatch", "grog_calib", "grog_gridding", "radial_grog", "reconstruct_coilwise",
           "calculate_calibration_kspace", "calibration_mask", "espirit", "calculate_coil_maps", "trajectories", "synthetic",
           "jl_empty", "jl_zeros", "jl_reshape", "to_jl", "to_host"]


def library():
    """The loaded ``libmrsr.so`` (raises if it has not been built)."""
    return _lib.load()
