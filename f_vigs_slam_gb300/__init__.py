"""f_vigs_slam_gb300 -- GB300 (sm_103a) Gaussian-splatting tracking/mapping hot path.

The compute path is the CUDA library libfvgs.so (csrc/), reached through the
C-ABI in include/fvgs.h.  `fvgs` is its Python binding and `synthetic`
generates the seeded workloads.
"""
from . import synthetic  # noqa: F401

__all__ = ["synthetic", "fvgs", "build"]
