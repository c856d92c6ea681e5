"""GB300-native MGBF filtering path (filtering_procedure procs 1, 2, 3, 4, 6,
7 and 8; the analysis<->filter transfers).

The compute path is libmgbf.so (hand-written sm_103a CUDA + C++ host
orchestration) reached through its C-ABI; this package is the Python host
side of that ABI.  There is no CPU fallback.
"""
from ._abi import MGBFError, load as load_library  # noqa: F401
from .mgbf import MGBF, MGBFBatch, MGBFConfig, GroupDesc  # noqa: F401

__all__ = ["MGBF", "MGBFBatch", "MGBFConfig", "GroupDesc", "MGBFError", "load_library"]
