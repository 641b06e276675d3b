"""The engine's own forms of the solve against the reference's sequence on the same inputs, through the C
ABI: the Hermitian eigensolver of lossless grating layers against the general QR (RCWA_GB300_HERMITIAN=0),
and the reduced seam algebra against the reference's interface blocks and stacking solves
(RCWA_GB300_SEAMS=reference), each alone and both together, and the tridiagonal eigenvectors by divide and
conquer (RCWA_GB300_HERM_DC=1) instead of the QL iteration. Seeded random stacks cover several gratings
in a row (grating under grating), films between them, a grating directly on the substrate and directly
under the incident medium, lossless and absorbing gratings; 1-D TE and TM, and conical incidence.
Per-order efficiencies agree within 1e-10 and the amplitudes within 1e-9 (1 + |b|); status, n_eig and
n_dense_solve are identical (the counters report the reference's operations whichever form ran), while
n_lu, the engine's own count of LU factorisations, is never above the reference's sequence's and is
below it wherever a reduced seam replaced an interface block and its stacking solve."""
import contextlib
import os

import numpy as np
import pytest

from stablercwa_gb300 import Layer, Stack

pytestmark = pytest.mark.gpu

PERIOD = 0.7
VARIANTS = {"hermitian": {"RCWA_GB300_SEAMS": "reference"},
            "seams": {"RCWA_GB300_HERMITIAN": "0"},
            "both": {},
            "divide-and-conquer": {"RCWA_GB300_HERM_DC": "1"}}
BASE = {"RCWA_GB300_HERMITIAN": "0", "RCWA_GB300_SEAMS": "reference"}


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


@contextlib.contextmanager
def env(values):
    keys = ("RCWA_GB300_HERMITIAN", "RCWA_GB300_SEAMS", "RCWA_GB300_HERM_DC")
    old = {k: os.environ.get(k) for k in keys}
    try:
        for k in keys:
            os.environ.pop(k, None)
        os.environ.update(values)
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def grating(rng, lossless):
    K = int(rng.integers(2, 5))
    inner = np.sort(rng.uniform(0.0, PERIOD, K - 1)).tolist()
    values = [complex(rng.uniform(1.0, 2.5), 0.0 if lossless else rng.uniform(0.0, 0.1)) for _ in range(K)]
    return Layer.grating(rng.uniform(0.05, 0.4), [0.0, *inner, PERIOD], values)


def film(rng):
    return Layer.uniform(rng.uniform(0.05, 0.3), rng.uniform(1.2, 2.2))


def stacks(seed, lossless):
    """Layer sequences (G grating, F film), top to bottom, each ending on the substrate."""
    rng = np.random.default_rng(seed)
    shapes = ["G", "GG", "GFG", "FGGF", "GGG", "FG", "GFFG"]
    out = []
    for shape in shapes:
        layers = [grating(rng, lossless) if ch == "G" else film(rng) for ch in shape]
        out.append((shape, Stack(nI=1.0, nII=1.46, period=PERIOD, layers=layers)))
    return out


def close(a, b, tol):
    return np.max(np.abs(a - b) / (1.0 + np.abs(b))) <= tol


@pytest.mark.parametrize("lossless", [True, False])
def test_1d_forms_agree(eng, lossless):
    rng = np.random.default_rng(5)
    pts = np.stack([rng.uniform(0.5, 1.5, 24), rng.uniform(0.0, 70.0, 24)], axis=1)
    for shape, stack in stacks(11 if lossless else 12, lossless):
        for pol in (0, 1):
            with env(BASE):
                ref = eng.solve1d_arrays(stack, pts, 12, pol)
            assert (ref["status"] == 0).all(), shape
            for name, values in VARIANTS.items():
                with env(values):
                    got = eng.solve1d_arrays(stack, pts, 12, pol)
                where = (shape, pol, name)
                assert np.array_equal(got["status"], ref["status"]), where
                assert np.array_equal(got["n_eig"], ref["n_eig"]), where
                assert np.array_equal(got["n_dense_solve"], ref["n_dense_solve"]), where
                assert np.all(got["n_lu"] <= ref["n_lu"]) and np.all(ref["n_lu"] <= ref["n_dense_solve"]), where
                if name not in ("hermitian",):  # every shape has a reduced seam (the top or a film over a grating)
                    assert np.all(got["n_lu"] < ref["n_lu"]), where
                for key in ("DEr", "DEt"):
                    assert np.max(np.abs(got[key] - ref[key])) <= 1e-10, (where, key)
                for key in ("R", "T"):
                    assert close(got[key], ref[key], 1e-9), (where, key)


@pytest.mark.parametrize("lossless", [True, False])
def test_conical_forms_agree(eng, lossless):
    rng = np.random.default_rng(6)
    pts = np.stack([rng.uniform(0.5, 1.5, 16), rng.uniform(0.0, 60.0, 16), rng.uniform(0.0, 90.0, 16)], axis=1)
    for shape, stack in stacks(21 if lossless else 22, lossless):
        with env(BASE):
            ref = eng.solve_conical_arrays(stack, pts, 8)
        assert (ref["status"] == 0).all(), shape
        for name, values in VARIANTS.items():
            with env(values):
                got = eng.solve_conical_arrays(stack, pts, 8)
            where = (shape, name)
            for key in ("status", "n_eig", "n_dense_solve", "n_schur"):
                assert np.array_equal(got[key], ref[key]), (where, key)
            assert np.all(got["n_lu"] <= ref["n_lu"]) and np.all(ref["n_lu"] <= ref["n_dense_solve"]), where
            for key in ("DEr", "DEt"):
                assert np.max(np.abs(got[key] - ref[key])) <= 1e-10, (where, key)
            for key in ("Jr", "Jt"):
                assert close(got[key], ref[key], 1e-9), (where, key)
