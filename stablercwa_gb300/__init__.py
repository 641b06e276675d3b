"""GB300-native RCWA solve engine: a drop-in for StableRCWA's rcwa::solve / sweep path.

The compute path is libstablercwa_gb300.so (hand-written sm_103a CUDA behind a C ABI declared in
include/stablercwa_gb300.h); this package is its host-side mirror of the reference's interface.
"""
from .types import (TE, TM, Layer, Layer2D, Options, Result, Stack, Stack2D, XProfile2D, harmonic_index_2d,  # noqa: F401
                    jones_from_angles_2d, stack2d_from_json, stack_from_json)
