"""mpstools_gb300 -- GB300-native (sm_103a) DMRG hot path of MPSTools.

The compute path is libmpsg.so (C++ host + hand-written CUDA kernels) behind the
C ABI declared in include/mpsg.h; this package is its Python binding plus the
model builders used to set up inputs.
"""
from . import models  # noqa: F401

__all__ = ["models"]
