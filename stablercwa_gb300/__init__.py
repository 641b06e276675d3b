"""GB300-native RCWA solve engine: a drop-in for StableRCWA's rcwa::solve / sweep path.

The compute path is libstablercwa_gb300.so (hand-written sm_103a CUDA behind a C ABI declared in
include/stablercwa_gb300.h); this package is its host-side mirror of the reference's interface.
"""
from .types import TE, TM, Layer, Options, Result, Stack, stack_from_json  # noqa: F401
