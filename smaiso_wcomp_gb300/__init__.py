"""GB300-native (sm_103a) semi-implicit pseudo-spectral step of smaiso-wcomp.

The compute path is libswc.so (CUDA, built in-tree by build.py) behind the C ABI of
include/swc.h; `engine` is the Python host mirror of that ABI, `ic` the seeded
synthetic initial conditions.
"""
from . import abi  # noqa: F401
from .abi import default_params, derived  # noqa: F401
