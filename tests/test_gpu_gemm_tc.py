"""The tensor-core complex product (csrc/gemm_tc.cu: Ozaki bf16 digit slices on tcgen05.mma, exact FP32
group sums, exact int64 accumulation) through rcwa_gpu_multiply_batch, the engine behind the reference's
Options::custom_multiply hook (include/stablercwa/rcwa1d.hpp:125-129), against numpy's FP64 product:
square and ragged shapes, K above one exact-accumulation chunk (2k > 1024), rows and columns scaled
over hundreds of decades, zero rows, and non-finite entries, which must stay non-finite."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# |C - A B| <= TOL * k * 2^-53 * max|A(i,:)| * max|B(:,j)| entrywise: the FP64 product's own error scale
TOL = 4.0


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine, gemm_info
    on, slices, stuck = gemm_info()
    if not on:
        pytest.skip("tensor-core products switched off (RCWA_GB300_GEMM=fp64)")
    assert slices == 7 and stuck == 0
    e = Engine()
    yield e
    e.close()
    assert gemm_info()[2] == 0  # no product kernel gave up on a wait


def rand(rng, *shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def bound(a, b):
    ra = np.max(np.maximum(np.abs(a.real), np.abs(a.imag)), axis=2)  # batch x m
    cb = np.max(np.maximum(np.abs(b.real), np.abs(b.imag)), axis=1)  # batch x n
    k = a.shape[2]
    return TOL * k * 2.0 ** -53 * ra[:, :, None] * cb[:, None, :]


@pytest.mark.parametrize("batch,m,k,n", [(64, 121, 121, 121), (5, 33, 40, 250), (3, 200, 600, 70), (2, 64, 882, 96),
                                         (7, 129, 32, 130)])
def test_matches_fp64_product(eng, batch, m, k, n):
    rng = np.random.default_rng(m * 1000 + k + n)
    a, b = rand(rng, batch, m, k), rand(rng, batch, k, n)
    c = eng.multiply_batch(a, b)
    ref = a @ b
    err = np.abs(c - ref)
    assert np.all(err <= bound(a, b)), float(np.max(err / bound(a, b)))


def test_scaled_rows_columns_and_zeros(eng):
    rng = np.random.default_rng(7)
    batch, m, k, n = 4, 96, 121, 80
    a, b = rand(rng, batch, m, k), rand(rng, batch, k, n)
    a *= 10.0 ** rng.uniform(-150, 150, size=(batch, m, 1))
    b *= 10.0 ** rng.uniform(-150, 150, size=(batch, 1, n))
    a[:, 5, :] = 0.0
    b[:, :, 7] = 0.0
    c = eng.multiply_batch(a, b)
    ref = a @ b
    assert np.all(c[:, 5, :] == 0) and np.all(c[:, :, 7] == 0)
    assert np.all(np.abs(c - ref) <= bound(a, b))


def test_non_finite_propagates(eng):
    rng = np.random.default_rng(9)
    batch, m, k, n = 2, 40, 64, 48
    a, b = rand(rng, batch, m, k), rand(rng, batch, k, n)
    a[0, 3, 10] = np.nan
    b[1, 20, 6] = np.inf
    c = eng.multiply_batch(a, b)
    assert not np.any(np.isfinite(c[0, 3, :]))
    assert not np.any(np.isfinite(c[1, :, 6]))
    ok = np.ones((batch, m, n), bool)
    ok[0, 3, :] = False
    ok[1, :, 6] = False
    assert np.all(np.isfinite(c[ok]))


def test_exact_integer_products_are_bit_exact(eng):
    """Integer entries up to 2^20 with k = 64: every product and sum is an integer below 2^53, exact in FP64, so
    the slice product (exact digit products, exact integer accumulation, one final rounding) must return
    numpy's result bit for bit."""
    rng = np.random.default_rng(11)
    batch, m, k, n = 3, 70, 64, 90
    a = rng.integers(-(1 << 20), 1 << 20, size=(batch, m, k)) + 1j * rng.integers(-(1 << 20), 1 << 20, size=(batch, m, k))
    b = rng.integers(-(1 << 20), 1 << 20, size=(batch, k, n)) + 1j * rng.integers(-(1 << 20), 1 << 20, size=(batch, k, n))
    c = eng.multiply_batch(a, b)
    assert np.array_equal(c, a @ b)
