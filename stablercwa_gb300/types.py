"""Value types of the solve path, mirroring StableRCWA's rcwa::Layer / Stack / Options / Result
(include/stablercwa/rcwa1d.hpp:71-164) with the same names and meanings."""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

TE = 0
TM = 1


@dataclass
class Layer:
    """One layer: a uniform film (homogeneous) or a binary/multi-level grating
    (include/stablercwa/rcwa1d.hpp:80-106)."""
    d: float = 0.0
    n: complex = 1.0
    edges: List[float] = field(default_factory=list)
    n_values: List[complex] = field(default_factory=list)
    homogeneous: bool = True

    @staticmethod
    def uniform(thickness, index):
        return Layer(d=float(thickness), n=complex(index), homogeneous=True)

    @staticmethod
    def grating(thickness, boundaries, indices):
        return Layer(d=float(thickness), edges=[float(e) for e in boundaries],
                     n_values=[complex(v) for v in indices], homogeneous=False)


@dataclass
class Stack:
    """Top to bottom: incident medium nI, layers, exit medium nII (include/stablercwa/rcwa1d.hpp:109-114)."""
    nI: complex = 1.0
    layers: List[Layer] = field(default_factory=list)
    nII: complex = 1.0
    period: float = 1.0


@dataclass
class Options:
    """include/stablercwa/rcwa1d.hpp:116-137 and include/stablercwa/eig_types.hpp:25-31 (engine subset)."""
    homogeneous_fast_path: bool = True
    diagnostics: bool = False
    eig_max_iter: int = 30
    eig_eps: float = float(np.finfo(np.float64).eps)


@dataclass
class Result:
    """Per-order amplitudes and efficiencies of one solve (include/stablercwa/rcwa1d.hpp:145-164)."""
    orders: np.ndarray
    R: np.ndarray
    T: np.ndarray
    DEr: np.ndarray
    DEt: np.ndarray
    eig_info: int = 0
    n_eig: int = 0
    n_dense_solve: int = 0
    status: int = 0
    max_eig_residual: float = 0.0

    def reflectance(self):
        return float(np.sum(self.DEr))

    def transmittance(self):
        return float(np.sum(self.DEt))


def stack_from_json(d):
    """Stack from the fixture layout written by tests/golden/export_*.cpp."""
    def c(v):
        return complex(v[0], v[1])
    layers = []
    for L in d["layers"]:
        if "n" in L:
            layers.append(Layer.uniform(L["d"], c(L["n"])))
        else:
            layers.append(Layer.grating(L["d"], L["edges"], [c(v) for v in L["n_values"]]))
    return Stack(nI=c(d["nI"]), layers=layers, nII=c(d["nII"]), period=d["period"])
