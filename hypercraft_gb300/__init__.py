"""GB300-native chunk relighter and mesher for HyperCraft.

The product is ``_lib/libhc_gb300.so`` (C ABI in include/hc_gb300.h: hand-written sm_103a CUDA
kernels). This package builds it and offers a thin Python mirror of the reference's mesh task.
"""
from .build import build  # noqa: F401
