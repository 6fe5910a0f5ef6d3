"""letkf_gb300 -- GB300-native (sm_103a) LETKF analysis step.

The compute path is libletkf_gpu.so (hand-written CUDA, C ABI in
include/letkf_gpu.h); this package is its host-side mirror of the reference's
letkf_core / das_letkf interfaces.
"""
from .lib import LETKF_OK, LetkfError  # noqa: F401

__version__ = "0.1.0"
