"""sc_gb300 -- GB300-native (sm_103a) Metropolis hot path for patchy spherocylinders.

The energy and move path of SC (robertvacha/SC) behind a C ABI (include/sc_gb300.h),
implemented as hand-written CUDA kernels; this package is the Python host mirror.
"""
from ._lib import ScError, load  # noqa: F401
from .system import ReplicaSet, Surrogate, System  # noqa: F401
