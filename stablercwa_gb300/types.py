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
    fourier_method: int = 0      # 0 analytic, 1 FFT-sampled (include/stablercwa/fourier.hpp:15)
    fft_samples: int = 0         # 0: automatic

    @staticmethod
    def uniform(thickness, index):
        return Layer(d=float(thickness), n=complex(index), homogeneous=True)

    @staticmethod
    def grating(thickness, boundaries, indices, fourier_method=0, fft_samples=0):
        return Layer(d=float(thickness), edges=[float(e) for e in boundaries],
                     n_values=[complex(v) for v in indices], homogeneous=False, fourier_method=int(fourier_method),
                     fft_samples=int(fft_samples))


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
    n_dense_solve: int = 0  # the reference's count of dense solves
    status: int = 0
    max_eig_residual: float = 0.0
    n_lu: int = 0  # LU factorisations the engine ran for this point (fewer than n_dense_solve with reduced seams)

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
            layers.append(Layer.grating(L["d"], L["edges"], [c(v) for v in L["n_values"]], L.get("fourier_method", 0),
                                        L.get("fft_samples", 0)))
    return Stack(nI=c(d["nI"]), layers=layers, nII=c(d["nII"]), period=d["period"])


# ---------------------------------------------------------------- 2-D crossed gratings

RAYLEIGH_ANOMALY = 3  # RCWA_SAMPLE_RAYLEIGH


@dataclass
class XProfile2D:
    """Piecewise-constant x profile of one y strip (include/stablercwa/rcwa2d_types.hpp:40-43)."""
    edges: List[float] = field(default_factory=list)
    n_values: List[complex] = field(default_factory=list)


@dataclass
class Layer2D:
    """A uniform layer or K y strips each with an x profile (include/stablercwa/rcwa2d_types.hpp:45-71)."""
    d: float = 0.0
    homogeneous: bool = True
    n: complex = 1.0
    y_edges: List[float] = field(default_factory=list)
    x_profiles: List[XProfile2D] = field(default_factory=list)
    name: str = ""

    @staticmethod
    def uniform(thickness, index, label=""):
        return Layer2D(d=float(thickness), homogeneous=True, n=complex(index), name=label)

    @staticmethod
    def patterned(thickness, y_boundaries, rows, label=""):
        return Layer2D(d=float(thickness), homogeneous=False, y_edges=[float(y) for y in y_boundaries],
                       x_profiles=list(rows), name=label)


@dataclass
class Stack2D:
    """Incident medium nI (real) | layers | exit medium nII, periods Lx, Ly
    (include/stablercwa/rcwa2d_types.hpp:73-78)."""
    nI: float = 1.0
    nII: complex = 1.0
    layers: List[Layer2D] = field(default_factory=list)
    Lx: float = 1.0
    Ly: float = 1.0


def harmonic_index_2d(m, n, M1, M2):
    """include/stablercwa/rcwa2d_types.hpp:110"""
    return (m + M1) * (2 * M2 + 1) + (n + M2)


def jones_from_angles_2d(psi_deg=90.0, delta_deg=0.0):
    """[Es, Ep] = [sin psi exp(i delta), cos psi] (include/stablercwa/rcwa2d_types.hpp:104-108)."""
    psi, delta = np.deg2rad(psi_deg), np.deg2rad(delta_deg)
    return (np.sin(psi) * np.exp(1j * delta), complex(np.cos(psi)))


def stack2d_from_json(d):
    """Stack2D from the fixture layout written by tests/golden/export_rcwa2d.cpp."""
    def c(v):
        return complex(v[0], v[1])
    layers = []
    for L in d["layers"]:
        if "n" in L:
            layers.append(Layer2D.uniform(L["d"], c(L["n"])))
        else:
            rows = [XProfile2D(list(p["edges"]), [c(v) for v in p["n_values"]]) for p in L["x_profiles"]]
            layers.append(Layer2D.patterned(L["d"], L["y_edges"], rows))
    return Stack2D(nI=float(d["nI"]), nII=c(d["nII"]), layers=layers, Lx=float(d["Lx"]), Ly=float(d["Ly"]))
