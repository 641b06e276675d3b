"""The engine's reduced seam algebra against the reference's interface blocks and stacking, in exact
linear-algebra terms on the CPU (numpy, random complex matrices): the forms the CUDA path evaluates
(stablercwa_gb300/csrc/smatrix.cuh `reduced_seam`, `analytic_over_dense_seam`; the top interfaces of
csrc/rcwa1d.cu and csrc/conical.cu) equal the reference's sequence (include/stablercwa/rcwa1d.hpp:664-712
interface matching and block, :794-808 stack_on, :714-746 and :989-1023 the top) to rounding."""
import numpy as np
import pytest

inv = np.linalg.inv


def crand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def reference_block(tp, tm):
    """Tdd, Rdu, Rud, Tuu of an interface from its matching tp, tm (rcwa1d.hpp:694-712)."""
    tpi = inv(tp)
    rdu = tm @ tpi
    return tp - rdu @ tm, rdu, -tpi @ tm, tpi


def reference_stack(block, r):
    """g and r' of the block stacked on the reflection r below it (rcwa1d.hpp:794-808)."""
    tdd, rdu, rud, tuu = block
    g = inv(np.eye(len(r)) - rdu @ r) @ tdd
    return g, rud + tuu @ r @ g


def matching(Wu, Vu, Wl, Vl):
    """tp, tm with d_b = tp d_a + tm u_a, u_b = tm d_a + tp u_a (rcwa1d.hpp:664-692)."""
    mm, nn = inv(Wl) @ Wu, inv(Vl) @ Vu
    return (mm + nn) / 2, (mm - nn) / 2


@pytest.mark.parametrize("r_kind", ["zero", "diag", "dense"])
def test_reduced_seam(r_kind):
    rng = np.random.default_rng(3)
    n = 11
    Wu, Vu, Wl, Vl = (crand(rng, n, n) for _ in range(4))
    r = {"zero": np.zeros((n, n)), "diag": np.diag(crand(rng, n) * 0.4), "dense": crand(rng, n, n) * 0.1}[r_kind]
    tp, tm = matching(Wu, Vu, Wl, Vl)
    g_ref, r_ref = reference_stack(reference_block(tp, tm), r)
    rp = np.linalg.solve(tp - r @ tm, r @ tp - tm)
    g = tp + tm @ rp
    assert np.max(np.abs(rp - r_ref)) <= 1e-12 * max(1, np.max(np.abs(r_ref)))
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * max(1, np.max(np.abs(g_ref)))
    # singular exactly together: det(tp - r tm) = det(I - r Rdu) det(tp), det(I - r Rdu) = det(I - Rdu r)
    rdu = tm @ inv(tp)
    assert np.isclose(np.linalg.det(tp - r @ tm), np.linalg.det(np.eye(n) - rdu @ r) * np.linalg.det(tp))


def rows_from_relations(w, v, X, Y, d):
    """u_a row by row: from w (d + u) = X where |w| >= |v|, else from v (d - u) = Y."""
    e_row = np.abs(w) >= np.abs(v)
    with np.errstate(divide="ignore", invalid="ignore"):  # the branch not taken may divide by zero
        return np.where(e_row[:, None], X / w[:, None] - d, d - Y / v[:, None])


@pytest.mark.parametrize("planar", [True, False])
def test_analytic_over_dense_seam(planar):
    rng = np.random.default_rng(4)
    n = 10
    W, V = crand(rng, n, n), crand(rng, n, n)
    r = crand(rng, n, n) * 0.1
    if planar:
        w, v = np.ones(n, complex), crand(rng, n)
    else:
        w, v = crand(rng, n), crand(rng, n)
        w[2] = 0.0  # a vanishing factor takes the other relation in its row
        v[5] = 0.0
    # reference: analytic region above (W = diag(w), V = diag(v)), the dense one below
    tp, tm = matching(np.diag(w), np.diag(v), W, V) if (w != 0).all() and (v != 0).all() else (None, None)
    P, Q = v[:, None] * W + w[:, None] * V, v[:, None] * W - w[:, None] * V
    g = np.linalg.solve(P + Q @ r, np.diag(2 * w * v))
    X, Y = W @ (np.eye(n) + r) @ g, V @ (np.eye(n) - r) @ g
    rp = rows_from_relations(w, v, X, Y, np.eye(n))
    # the fields satisfy both tangential relations with u_a = r' d_a, d_b = g d_a
    assert np.max(np.abs(w[:, None] * (np.eye(n) + rp) - X)) <= 1e-11
    assert np.max(np.abs(v[:, None] * (np.eye(n) - rp) - Y)) <= 1e-11
    if tp is not None:
        g_ref, r_ref = reference_stack(reference_block(tp, tm), r)
        assert np.max(np.abs(g - g_ref)) <= 1e-11 * max(1, np.max(np.abs(g_ref)))
        assert np.max(np.abs(rp - r_ref)) <= 1e-11 * max(1, np.max(np.abs(r_ref)))


def test_top_interface():
    """The incident medium (w, v) over a dense region with the dense r below: one column of the
    reference's top solve, R and the downward amplitude d_b."""
    rng = np.random.default_rng(5)
    n, M = 9, 4
    W, V = crand(rng, n, n), crand(rng, n, n)
    r = crand(rng, n, n) * 0.2
    for w, v in ((np.ones(n, complex), crand(rng, n)), (crand(rng, n), crand(rng, n))):
        tp, tm = matching(np.diag(w), np.diag(v), W, V)
        tpi = inv(tp)
        rdu = tm @ tpi
        tdd = tp[:, M] - rdu @ tm[:, M]
        rud = -tpi @ tm[:, M]
        down_ref = np.linalg.solve(np.eye(n) - rdu @ r, tdd)
        R_ref = rud + tpi @ (r @ down_ref)
        P, Q = v[:, None] * W + w[:, None] * V, v[:, None] * W - w[:, None] * V
        e = np.zeros(n, complex)
        e[M] = 2 * w[M] * v[M]
        down = np.linalg.solve(P + Q @ r, e)
        d = np.zeros(n)
        d[M] = 1.0
        R = rows_from_relations(w, v, (W @ (down + r @ down))[:, None], (V @ (down - r @ down))[:, None], d[:, None])[:, 0]
        assert np.max(np.abs(down - down_ref)) <= 1e-12 * max(1, np.max(np.abs(down_ref)))
        assert np.max(np.abs(R - R_ref)) <= 1e-12 * max(1, np.max(np.abs(R_ref)))


def test_hermitian_pencil_mapping():
    """TM: [[1/eps]]^-1 B x = lambda x from L^-1 B L^-H y = lambda y, x = L^-H y; conical: B C x = lambda x
    with C = (L L^H)^-1 from the same Hermitian problem, x = L z and C x = L^-H z."""
    rng = np.random.default_rng(6)
    n = 12
    Bm = crand(rng, n, n)
    Bm = Bm + Bm.conj().T
    Lf = np.tril(crand(rng, n, n)) + 4 * np.eye(n)
    D = Lf @ Lf.conj().T  # Hermitian positive definite, D = [[1/eps]]
    Li = inv(Lf)
    lam, y = np.linalg.eigh(Li @ Bm @ Li.conj().T)
    x = Li.conj().T @ y  # TM
    assert np.max(np.abs(inv(D) @ Bm @ x - x * lam)) <= 1e-10
    z = y
    x2 = Lf @ z  # conical B C
    assert np.max(np.abs(Bm @ inv(D) @ x2 - x2 * lam)) <= 1e-10
    assert np.max(np.abs(inv(D) @ x2 - Li.conj().T @ z)) <= 1e-10
