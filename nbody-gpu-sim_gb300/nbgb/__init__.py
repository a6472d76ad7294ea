"""nbgb -- GB300-native (sm_103a) force-and-integrate hot path of nbody-gpu-sim.

The compute path is libnbgb.so (hand-written CUDA kernels behind the C ABI in
include/nbgb.h).  This package is its host-side mirror of the reference's
`include/nbody` interface (api.py), plus initial-condition generators
(ics.py) and the `.nbody` checkpoint format (checkpoint.py).
"""
from .api import *  # noqa: F401,F403
from .api import __all__ as _api_all
from . import ics, checkpoint, serving  # noqa: F401
from ._lib import lib, lib_path, declared_symbols  # noqa: F401

__all__ = list(_api_all) + ["ics", "checkpoint", "lib", "lib_path", "declared_symbols"]
