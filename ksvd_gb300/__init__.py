"""ksvd_gb300 -- K-SVD dictionary learning (Batch-OMP + approximate K-SVD) on one NVIDIA GB300.

The compute path is ``libksvd_gb300.so``: hand-written sm_103a CUDA kernels behind the C ABI in
``include/ksvd_gb300.h``.  This package holds the build recipe, the ctypes binding, a host-side
mirror of the reference's KSVD interface and the synthetic workload generators.
"""
from .api import KSVD, Handle, KsvdError, random_permutation, PRECISIONS  # noqa: F401
from . import datagen  # noqa: F401

__version__ = "0.1.0"
