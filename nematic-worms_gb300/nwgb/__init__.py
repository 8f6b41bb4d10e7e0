"""nwgb — GB300-native step engine for self-propelled nematic worms.

The compute path is libnwgb.so (hand-written sm_103a CUDA behind a C ABI,
include/nwgb.h); this package is the Python host side of that ABI.
"""
from . import abi
from .abi import NwConfig, NwError, default_config, load_library
from .batch import Batch
from .system import ParticleSystem, System

__all__ = ["abi", "NwConfig", "NwError", "default_config", "load_library", "System", "ParticleSystem", "Batch"]
