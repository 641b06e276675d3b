"""Lossless gratings of high index contrast at N = 301 harmonics (M = 150) on the GPU, through the C ABI,
against the CPU oracle: the Hermitian eigensolver path with the device Cholesky factor of [[1/eps]], its
explicit triangular inverse and the per-sample pencil combination (stablercwa_gb300/csrc/smatrix.cuh,
csrc/rcwa1d_kernels.cuh), on ridges of index 3.48 and 4.0 in air, layers 0.05 to 5 periods thick,
incidence 0 to 85 degrees and one wavelength 1e-9 above a Rayleigh anomaly. Single points take the
eigensolver's 128-thread CTA form; a sweep of 320 points takes the blocked form with a warp per matrix.
Per-order DEr/DEt within 1e-10 of the oracle; |R + T - 1| no worse than the oracle's own plus 1e-12."""
import numpy as np
import pytest

from oracle import oracle
from stablercwa_gb300 import TE, TM, Layer, Stack
from test_pencil_high_contrast import CASES, M, N_I, N_II, PERIOD

pytestmark = pytest.mark.gpu
DE_TOL = 1e-10
ENERGY_MARGIN = 1e-12


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def stack_of(n_values, d, fill):
    return Stack(nI=N_I, nII=N_II, period=PERIOD,
                 layers=[Layer.grating(d, [0.0, fill * PERIOD, PERIOD], list(n_values))])


def energy(r, k):
    return abs(float(np.sum(r["DEr"][k]) + np.sum(r["DEt"][k])) - 1.0)


@pytest.mark.parametrize("pol", [TM, TE], ids=["TM", "TE"])
def test_single_points_n301(eng, pol):
    worst = 0.0
    for k, (n_values, d, fill, wl, theta) in enumerate(CASES):
        stack = stack_of(n_values, d, fill)
        got = eng.solve1d_arrays(stack, [(wl, theta)], M, pol)
        ref = oracle.solve1d_batch(stack, [(wl, theta)], M, pol)
        assert got["status"][0] == 0 and ref["status"][0] == 0, k
        err = max(float(np.max(np.abs(got["DEr"][0] - ref["DEr"][0]))),
                  float(np.max(np.abs(got["DEt"][0] - ref["DEt"][0]))))
        assert err <= DE_TOL, (k, err)
        assert energy(got, 0) <= energy(ref, 0) + ENERGY_MARGIN, (k, energy(got, 0), energy(ref, 0))
        worst = max(worst, err)
    print(f"worst |dDE| vs oracle at N = 301: {worst:.2e}")


def test_sweep_n301(eng):
    """320 seeded (lambda, theta) points of the silicon-ridge structure in one TM call; eight of them
    against the oracle, the energy balance of all of them."""
    n_values, d, fill = (3.48, 1.0), 0.5, 0.37
    stack = stack_of(n_values, d, fill)
    rng = np.random.default_rng(301)
    pts = np.stack([rng.uniform(0.55, 1.6, 320), rng.uniform(0.0, 70.0, 320)], axis=1)
    got = eng.solve1d_arrays(stack, pts, M, TM)
    assert (got["status"] == 0).all()
    idx = np.linspace(0, len(pts) - 1, 8).astype(int)
    ref = oracle.solve1d_batch(stack, pts[idx], M, TM, threads=8)
    for j, k in enumerate(idx):
        err = max(float(np.max(np.abs(got["DEr"][k] - ref["DEr"][j]))),
                  float(np.max(np.abs(got["DEt"][k] - ref["DEt"][j]))))
        assert err <= DE_TOL, (int(k), err)
        assert energy(got, k) <= energy(ref, j) + ENERGY_MARGIN, (int(k), energy(got, k), energy(ref, j))
    worst_energy = max(energy(got, k) for k in range(len(pts)))
    assert worst_energy <= 1e-11, worst_energy
    print(f"worst |R+T-1| over the 320 points: {worst_energy:.2e}")
