"""GB300-native device-wide prefix scan (sm_103a), a drop-in for the
ChainedScanDecoupledLookbackDispatcher / ReduceThenScanDispatcher path of
b0nes164/GPUPrefixSums.

The compute path is ``libgps.so`` (hand-written CUDA, C ABI in
``include/gps.h``). Importing this package loads it and raises if it is
missing; there is no other implementation behind these names.
"""
from ._lib import GpsError, lib  # noqa: F401  (loads libgps.so or raises)
from .plan import Plan  # noqa: F401

__all__ = ["Plan", "GpsError", "lib"]
