"""The engine's Hermitian mode formulation for lossless grating layers at high index contrast and high
order, on the CPU (numpy), against the oracle (the reference's own formulation).

For a layer whose permittivities are all real the engine does not run the general eigensolver on the
reference's TM matrix [[1/eps]]^-1 (Kx [[eps]]^-1 Kx - I) (include/stablercwa/rcwa1d.hpp:432-468). It
symmetrises the Fourier coefficients (c_-m = conj(c_m)), factors [[1/eps]] = L L^H, forms L^-1 and L^-H
explicitly, combines four per-layer constants L^-1 X L^-H (X = E, (m_i + m_j) E_ij, m_i m_j E_ij with
E the Hermitian part of [[eps]]^-1, and X = I) with the sample's a^2, a b, b^2, solves that Hermitian
matrix, maps the eigenvectors back with L^-H and normalises each column
(stablercwa_gb300/csrc/smatrix.cuh `toeplitz_cholesky_kernel`, `lower_inverse_kernel`, `pencil_parts`;
csrc/rcwa1d_kernels.cuh `pencil_combine_kernel`). TE solves Kx^2 - [[eps]] as a Hermitian matrix.

The explicit inverse of L and the per-sample combination of large terms (b^2 m_i m_j grows as M^2)
are where a high-contrast, high-order layer could lose accuracy. Here the same arithmetic, in FP64
numpy with LAPACK's Hermitian solver in place of the device's, feeds an exact boundary-value solve of
one grating layer between two half-spaces (the tangential fields W (d + u), V (d - u) matched at both
interfaces, one dense system), and the efficiencies are held to the oracle's at N = 301 harmonics with
silicon- and germanium-like ridges in air: per-order |dDE| <= 1e-10, and the energy balance of the
Hermitian form no worse than the oracle's own.
"""
import numpy as np
import pytest

from stablercwa_gb300 import TE, TM, Layer, Stack

M = 150            # N = 2M + 1 = 301 harmonics
DE_TOL = 1e-10     # per-order efficiencies against the oracle
PERIOD, N_I, N_II = 1.0, 1.0, 1.46

# (ridge and groove index, thickness, ridge fill, wavelength, theta): thin to 5-wavelength-thick layers,
# normal to grazing incidence, one wavelength 1e-9 above a Rayleigh anomaly (order -1 grazing in nI)
CASES = [
    ((3.48, 1.0), 0.5, 0.37, 0.6, 30.0),
    ((3.48, 1.0), 0.5, 0.37, 1.55, 10.0),
    ((3.48, 1.0), 0.5, 0.37, 0.9, 63.0),
    ((4.0, 1.0), 2.0, 0.5, 1.3, 85.0),
    ((3.48, 1.0), 5.0, 0.2, 0.55, 45.0),
    ((3.48, 1.46), 0.05, 0.8, 2.0, 0.0),
    ((4.0, 1.0), 1.0, 0.5, 1.0 / (1.0 + np.sin(np.radians(20.0))) + 1e-9, 20.0),
]


def coefficients(edges, values, period, hmax):
    """c_h = (1/P) integral of the piecewise-constant profile times exp(-2 pi i h x / P), h = -hmax..hmax."""
    edges = np.asarray(edges, float)
    c = np.zeros(2 * hmax + 1, complex)
    for h in range(-hmax, hmax + 1):
        if h == 0:
            c[hmax] = sum(v * (edges[j + 1] - edges[j]) for j, v in enumerate(values)) / period
        else:
            e = np.exp(-2j * np.pi * h * edges / period)
            c[h + hmax] = sum(v * (e[j + 1] - e[j]) for j, v in enumerate(values)) / (-2j * np.pi * h)
    return c


def symmetrised(c):
    """c_-m = conj(c_m) exactly, from the mean of the two (a real profile's coefficients to rounding)."""
    h = len(c) // 2
    out = c.copy()
    for m in range(h + 1):
        s = 0.5 * (c[h + m] + np.conj(c[h - m]))
        out[h + m], out[h - m] = s, np.conj(s)
    return out


def toeplitz(c):
    n = (len(c) + 1) // 2
    i, j = np.indices((n, n))
    return c[i - j + n - 1]


def branch(q):
    """The reference's choice of square root (rcwa1d.hpp:514-518)."""
    q = np.where(q.real < 0.0, -q, q)
    return np.where((q.real < 1e-10) & (q.imag > 0.0), -q, q)


def hermitian_modes(edges, n_values, wl, theta, pol):
    """q, W, V of the grating layer by the engine's Hermitian formulation."""
    n = 2 * M + 1
    a, b = N_I * np.sin(np.radians(theta)), -wl / PERIOD
    m = np.arange(n) - M
    kx = a + b * m
    eps = toeplitz(symmetrised(coefficients(edges, [v * v for v in n_values], PERIOD, 2 * M)))
    if pol == TE:
        A = np.diag(kx * kx) - eps
        lam, X = np.linalg.eigh(0.5 * (A + A.conj().T))
        inv_eps = None
    else:
        inv_eps = toeplitz(symmetrised(coefficients(edges, [1.0 / (v * v) for v in n_values], PERIOD, 2 * M)))
        Ei = np.linalg.inv(eps)
        E = 0.5 * (Ei + Ei.conj().T)
        Li = np.linalg.inv(np.linalg.cholesky(inv_eps))  # explicit L^-1, as lower_inverse_kernel forms it
        LiH = Li.conj().T
        mi, mj = np.meshgrid(m, m, indexing="ij")
        S0, S1, S2, C = (Li @ X @ LiH for X in (E, (mi + mj) * E, (mi * mj) * E, np.eye(n)))
        A = a * a * S0 + a * b * S1 + b * b * S2 - C
        lam, Y = np.linalg.eigh(0.5 * (A + A.conj().T))
        X = LiH @ Y
    W = X / np.linalg.norm(X, axis=0)
    q = branch(np.sqrt(lam.astype(complex)))
    V = W * q if pol == TE else (inv_eps @ W) * q
    return kx, q, W, V


def half_space(nr, kx, pol):
    """q and the diagonal V factor of a homogeneous region (rcwa1d.hpp:522-544)."""
    kz = np.sqrt(nr * nr - kx * kx + 0j)
    kz = np.where(kz.imag < 0.0, -kz, kz)
    kz = np.where((np.abs(kz.imag) < 1e-12) & (kz.real < 0.0), -kz, kz)
    q = kz.imag - 1j * kz.real
    return q, (q if pol == TE else q / (nr * nr))


def efficiencies(edges, n_values, d, wl, theta, pol):
    """DEr, DEt of one grating layer between nI and nII: unknowns R, the layer's downward amplitudes at
    its top, its upward amplitudes at its bottom, T; the field pair W (d + u), V (d - u) continuous at both
    interfaces (evanescent factors only ever multiply amplitudes referred to the near interface)."""
    n = 2 * M + 1
    kx, q, W, V = hermitian_modes(edges, n_values, wl, theta, pol)
    qI, pI = half_space(N_I, kx, pol)
    qII, pII = half_space(N_II, kx, pol)
    X = np.exp(-2.0 * np.pi / wl * q * d)
    I, Z = np.eye(n), np.zeros((n, n))
    system = np.block([[-I, W, W * X, Z],
                       [np.diag(pI), V, -V * X, Z],
                       [Z, W * X, W, -I],
                       [Z, V * X, -V, -np.diag(pII)]])
    inc = np.zeros(n, complex)
    inc[M] = 1.0
    sol = np.linalg.solve(system, np.concatenate([inc, pI * inc, np.zeros(2 * n)]))
    R, T = sol[:n], sol[3 * n:]
    DEr = np.abs(R) ** 2 * (qI / qI[M]).real
    t_factor = qII / qI[M] if pol == TE else (qII / N_II ** 2) / (qI[M] / N_I ** 2)
    return DEr, np.abs(T) ** 2 * t_factor.real


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    return o


@pytest.mark.parametrize("pol", [TM, TE], ids=["TM", "TE"])
@pytest.mark.parametrize("case", CASES, ids=[f"case{k}" for k in range(len(CASES))])
def test_hermitian_form_high_contrast_n301(oracle, case, pol):
    n_values, d, fill, wl, theta = case
    edges = [0.0, fill * PERIOD, PERIOD]
    stack = Stack(nI=N_I, nII=N_II, period=PERIOD, layers=[Layer.grating(d, edges, list(n_values))])
    ref = oracle.solve1d_batch(stack, [(wl, theta)], M, pol)
    assert ref["status"][0] == 0
    DEr, DEt = efficiencies(edges, n_values, d, wl, theta, pol)
    err = max(np.max(np.abs(DEr - ref["DEr"][0])), np.max(np.abs(DEt - ref["DEt"][0])))
    assert err <= DE_TOL, err
    energy = abs(DEr.sum() + DEt.sum() - 1.0)
    energy_ref = abs(ref["DEr"][0].sum() + ref["DEt"][0].sum() - 1.0)
    assert energy <= max(energy_ref, 1e-13), (energy, energy_ref)
