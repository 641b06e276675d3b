"""The cluster eigensolver (csrc/eig_cluster.cu: one matrix over a thread-block cluster of 8 or 16 SMs,
partial sums and the QR rotation log exchanged through distributed shared memory) against the
one-CTA-per-matrix kernel and against the matrices themselves: the algorithm of
include/stablercwa/eig_qr.hpp:1008-1124 (CORTH, COMQR2, back substitution) at orders 400 and 882, with
RCWA-like layer matrices, a matrix with exactly repeated eigenvalues (the coincident-eigenvalue floor),
and the info contract when the iteration cap is reached."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RESID_TOL = 1e-13   # max_j |A v_j - w_j v_j| / (|A|_F |v_j|), the reference's eigen-pair residual bound


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def layer_matrices(n, batch, seed, loss=0.01):
    """TE matrices Kx^2 - [[eps]] of a binary grating (index 1.46 + loss i, fill 0.3..0.6)."""
    rng = np.random.default_rng(seed)
    M = n // 2
    h = np.subtract.outer(np.arange(n), np.arange(n))
    out = np.empty((batch, n, n), np.complex128)
    for b in range(batch):
        e1 = complex(1.46, loss) ** 2
        fill = rng.uniform(0.3, 0.6)
        with np.errstate(invalid="ignore", divide="ignore"):
            eps = np.where(h == 0, fill * e1 + (1 - fill), (e1 - 1.0) * np.sin(np.pi * h * fill) / (np.pi * h))
        kx = rng.uniform(-0.5, 0.5) + (np.arange(n) - M) * 0.61
        out[b] = np.diag(kx * kx) - eps
    return out


def residual(a, w, v):
    worst = 0.0
    for k in range(a.shape[0]):
        d = a[k] @ v[k] - v[k] * w[k][None, :]
        worst = max(worst, float(np.max(np.linalg.norm(d, axis=0) / (np.linalg.norm(a[k]) * np.linalg.norm(v[k], axis=0)))))
    return worst


def solve(eng, monkeypatch, a, group, max_iter=30):
    monkeypatch.setenv("RCWA_GB300_EIG_GROUP", str(group))
    return eng.eig_batch(a, max_iter=max_iter)


@pytest.mark.parametrize("n,batch", [(400, 3), (882, 1)])
def test_cluster_matches_cta_kernel(eng, monkeypatch, n, batch):
    a = layer_matrices(n, batch, n)
    w, v, info, sweeps = solve(eng, monkeypatch, a, -1)
    w0, v0, info0, sweeps0 = solve(eng, monkeypatch, a, 256)
    assert np.all(info == 0) and np.all(info0 == 0)
    assert residual(a, w, v) <= RESID_TOL
    for k in range(batch):  # the same spectrum: sorted eigenvalues within rounding of the matrix's scale
        scale = np.max(np.abs(w0[k]))
        assert np.max(np.abs(np.sort_complex(w[k]) - np.sort_complex(w0[k]))) <= 1e-12 * scale
    assert np.all(np.abs(sweeps - sweeps0) <= max(3, int(0.02 * n)))  # same iteration, same deflations to rounding


def test_cluster_repeated_eigenvalues(eng, monkeypatch):
    rng = np.random.default_rng(5)
    n = 400
    b = layer_matrices(n // 2, 1, 11)[0]
    q, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    a = (q @ np.kron(np.eye(2), b) @ q.conj().T)[None]  # every eigenvalue twice
    w, v, info, _ = solve(eng, monkeypatch, a, -1)
    assert info[0] == 0
    assert residual(a, w, v) <= 1e-12
    assert np.all(np.isfinite(v))


def test_cluster_iteration_cap(eng, monkeypatch):
    a = layer_matrices(400, 1, 3)
    w, v, info, sweeps = solve(eng, monkeypatch, a, -1, max_iter=1)
    w0, v0, info0, sweeps0 = solve(eng, monkeypatch, a, 256, max_iter=1)
    assert info[0] > 0 and info[0] == info0[0]
    assert sweeps[0] == sweeps0[0]
