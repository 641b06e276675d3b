"""GPU eigensolver, LU solve and GEMM through the C ABI, against the oracle and the reference's
golden eigenvalues (tests/test_eig_qr.cpp matrices)."""
import os

import numpy as np
import pytest

from conftest import cvec
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def residual(a, w, v):
    # max_j ||A v_j - l_j v_j|| / (||A||_F ||v_j||)  (include/stablercwa/eig.hpp:38-69)
    fro = np.linalg.norm(a)
    d = a @ v - v * w[None, :]
    return np.max(np.linalg.norm(d, axis=0) / (fro * np.linalg.norm(v, axis=0)))


def match_values(got, ref):
    """max over ref of distance to the nearest unused got value (permutation-invariant)."""
    got = list(got)
    worst = 0.0
    for r in ref:
        k = int(np.argmin([abs(g - r) for g in got]))
        worst = max(worst, abs(got[k] - r))
        got.pop(k)
    return worst


@pytest.mark.parametrize("group", ["4", "8", "16", "32", "64", "128", "256"])
def test_eig_golden(eng, eig_cases, group, monkeypatch):
    monkeypatch.setenv("RCWA_GB300_EIG_GROUP", group)
    for case in eig_cases:
        n = case["n"]
        a = cvec(case["a"]).reshape((n, n), order="F")
        w, v, info, sweeps = eng.eig_batch(a[None], max_iter=case["max_iter"])
        assert info[0] == case["info"], (case["name"], info[0])
        ref = cvec(case["values"])
        scale = max(1.0, np.max(np.abs(ref)))
        if info[0] == 0:
            assert match_values(w[0], ref) <= 1e-11 * scale, case["name"]
            assert residual(a, w[0], v[0]) <= 1e-13, case["name"]
            assert np.allclose(np.linalg.norm(v[0], axis=0), 1.0, atol=1e-13)
        else:
            i = info[0]
            assert match_values(w[0][i:], ref[i:]) <= 1e-11 * scale, case["name"]


def rcwa_matrix(n, index, fill=0.4, lop=0.61, sin_theta=0.2):
    M = n // 2
    e1, e2 = index * index, 1.0
    h = np.subtract.outer(np.arange(n), np.arange(n))
    with np.errstate(invalid="ignore", divide="ignore"):
        eps = np.where(h == 0, fill * e1 + (1 - fill) * e2, (e1 - e2) * np.sin(np.pi * h * fill) / (np.pi * h))
    kx = sin_theta + (np.arange(n) - M) * lop
    return -eps + np.diag(kx * kx)


@pytest.mark.parametrize("n", [41, 81, 121])
def test_eig_batch_vs_oracle(eng, n):
    rng = np.random.default_rng(n)
    mats = [rcwa_matrix(n, complex(rng.uniform(1.3, 2.2), rng.uniform(0, 0.2)), fill=rng.uniform(0.2, 0.6),
                        sin_theta=rng.uniform(-0.5, 0.5)) for _ in range(6)]
    a = np.array(mats)
    w, v, info, sweeps = eng.eig_batch(a)
    for k in range(len(mats)):
        assert info[k] == 0
        wo, vo, io, so = oracle.eig(mats[k])
        assert match_values(w[k], wo) <= 1e-11 * np.max(np.abs(wo))
        assert residual(mats[k], w[k], v[k]) <= 1e-13


def test_lu_solve_and_gemm(eng):
    rng = np.random.default_rng(5)
    for n, nrhs in [(1, 1), (7, 3), (41, 41), (121, 121), (121, 1), (60, 20)]:
        a = rng.standard_normal((4, n, n)) + 1j * rng.standard_normal((4, n, n))
        b = rng.standard_normal((4, n, nrhs)) + 1j * rng.standard_normal((4, n, nrhs))
        x, sing = eng.solve_batch(a, b)
        assert not sing.any()
        for k in range(4):
            xo, so = oracle.solve(a[k], b[k])
            assert np.max(np.abs(x[k] - xo)) <= 1e-10 * max(1.0, np.max(np.abs(xo)))
    z = np.zeros((1, 3, 3), complex)
    z[0, :, 0] = 1.0
    x, sing = eng.solve_batch(z, np.ones((1, 3, 1), complex))
    assert sing[0] and np.isnan(x[0]).all()          # zero pivot: lu.hpp:427-436 throws


@pytest.mark.parametrize("n, nrhs", [(160, 160), (161, 7), (200, 200), (330, 1), (257, 300)])
def test_blocked_lu(eng, n, nrhs):
    """Orders from 100 up run the panel / triangular-solve / GEMM form of the same elimination."""
    rng = np.random.default_rng(n + nrhs)
    a = rng.standard_normal((3, n, n)) + 1j * rng.standard_normal((3, n, n))
    b = rng.standard_normal((3, n, nrhs)) + 1j * rng.standard_normal((3, n, nrhs))
    x, sing = eng.solve_batch(a, b)
    assert not sing.any()
    for k in range(3):
        xo, so = oracle.solve(a[k], b[k])
        assert np.max(np.abs(x[k] - xo)) <= 1e-10 * max(1.0, np.max(np.abs(xo)))
    # a zero pivot in the second panel: singular flag and NaN solution, other systems unaffected
    z = a.copy()
    z[1, :, 40] = 0.0
    z[1, :, 41] = 0.0
    z[1, 41, :] = 0.0
    x, sing = eng.solve_batch(z, b)
    assert sing.tolist() == [False, True, False]
    assert np.isnan(x[1]).all() and np.isfinite(x[0]).all() and np.isfinite(x[2]).all()
    for m, k, n in [(1, 1, 1), (33, 17, 9), (121, 121, 121)]:
        a = rng.standard_normal((3, m, k)) + 1j * rng.standard_normal((3, m, k))
        b = rng.standard_normal((3, k, n)) + 1j * rng.standard_normal((3, k, n))
        c = eng.multiply_batch(a, b)
        for q in range(3):
            assert np.max(np.abs(c[q] - oracle.multiply(a[q], b[q]))) <= 1e-12 * max(1.0, k)


@pytest.mark.parametrize("group", ["4", "16", "32", "128"])
@pytest.mark.parametrize("n", [1, 2, 3, 17, 81, 121])
def test_eig_hermitian_batch(eng, n, group, monkeypatch):
    """rcwa_gpu_eig_hermitian_batch: random Hermitian matrices, the Toeplitz-plus-Kx^2 layer matrices of a
    lossless grating (with exactly repeated eigenvalues at normal incidence) and a diagonal one; eigenvalues
    against numpy's eigh to 1e-13 of the spectral radius, residual <= 1e-13, orthonormal columns to 1e-13.
    A non-Hermitian input is solved through its Hermitian part."""
    monkeypatch.setenv("RCWA_GB300_EIG_GROUP", group)
    rng = np.random.default_rng(n)
    mats = []
    for _ in range(5):
        x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        mats.append(x + x.conj().T)
    M = n // 2
    h = np.subtract.outer(np.arange(n), np.arange(n))
    with np.errstate(invalid="ignore", divide="ignore"):
        eps = np.where(h == 0, 0.4 * 1.46 ** 2 + 0.6, (1.46 ** 2 - 1) * np.sin(np.pi * h * 0.4) / (np.pi * h))
    for kx0 in (0.0, 0.31):
        kx = kx0 + (np.arange(n) - M) * 0.61
        mats.append((np.diag(kx * kx) - eps).astype(np.complex128))
    mats.append(np.diag(rng.standard_normal(n)).astype(np.complex128))
    a = np.array(mats)
    w, v, info = eng.eig_hermitian_batch(a)
    assert (info == 0).all()
    for k in range(len(a)):
        ref = np.linalg.eigvalsh(a[k])
        scale = max(1.0, np.max(np.abs(ref)))
        assert np.max(np.abs(np.sort(w[k]) - ref)) <= 1e-13 * scale * max(1, n) ** 0.5, k
        assert residual(a[k], w[k], v[k]) <= 1e-13, k
        assert np.max(np.abs(v[k].conj().T @ v[k] - np.eye(n))) <= 1e-13 * max(1, n) ** 0.5, k
    # a general matrix: the solver works on (a + a^H) / 2
    g = rng.standard_normal((1, n, n)) + 1j * rng.standard_normal((1, n, n))
    w2, v2, info2 = eng.eig_hermitian_batch(g)
    hpart = (g[0] + g[0].conj().T) / 2
    assert info2[0] == 0 and residual(hpart, w2[0], v2[0]) <= 1e-13
