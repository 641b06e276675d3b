"""FFT-sampled Fourier coefficients on the GPU, through the C ABI, against the reference
(rcwa::fourier_coefficients_fft, include/stablercwa/fourier.hpp:49-83, and the solves that use it:
tests/test_fft.cpp)."""
import numpy as np
import pytest

from conftest import cvec, load_jsonl, rvec
from stablercwa_gb300 import abi
from stablercwa_gb300.types import stack_from_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


@pytest.fixture(scope="module")
def cases():
    return load_jsonl("fft_cases.jsonl")


def test_coefficients(eng, cases):
    seen = 0
    for c in cases:
        if c["kind"] != "coeff":
            continue
        seen += 1
        vals = cvec(c["values"])
        got = eng.fourier_coefficients(c["edges"], vals, c["period"], c["hmax"], method=1, samples=c["samples"])
        tol = 3e-12 * max(1.0, np.max(np.abs(vals)))  # tests/test_fft.cpp:42
        assert np.max(np.abs(got - cvec(c["fft"]))) <= tol, c["name"]
        ana = eng.fourier_coefficients(c["edges"], vals, c["period"], c["hmax"], method=0)
        assert np.max(np.abs(ana - cvec(c["analytic"]))) <= 1e-14 * max(1.0, np.max(np.abs(vals))), c["name"]
    assert seen >= 25


def test_solves_with_fft_layers(eng, cases):
    seen = 0
    for c in cases:
        if c["kind"] != "solve":
            continue
        seen += 1
        stack = stack_from_json(c["stack"])
        pol = 0 if c["pol"] == "TE" else 1
        r = eng.solve1d_arrays(stack, [(c["wavelength"], c["theta"])], c["M"], pol)
        ref = c["ref"]
        der = rvec(ref["DEr"])
        if np.isnan(der).all():  # epsilon or 1/epsilon overflow: numerical failure (tests/test_fft.cpp:119-131)
            assert r["status"][0] == abi.RCWA_SAMPLE_NUMERICAL, c["name"]
            assert np.isnan(r["DEr"][0]).all() and np.isnan(r["DEt"][0]).all(), c["name"]
            continue
        assert r["status"][0] == 0, c["name"]
        for key in ("DEr", "DEt"):
            assert np.max(np.abs(r[key][0] - rvec(ref[key]))) <= 1e-10, (c["name"], key)
        for key in ("R", "T"):
            assert np.max(np.abs(r[key][0] - cvec(ref[key]))) <= 1e-9, (c["name"], key)
        assert int(r["n_dense_solve"][0]) == ref["n_dense_solve"], c["name"]
    assert seen >= 9


def test_conical_with_fft_layers(eng, cases):
    seen = 0
    for c in cases:
        if c["kind"] != "conical":
            continue
        seen += 1
        stack = stack_from_json(c["stack"])
        r = eng.solve_conical(stack, c["wavelength"], c["theta"], c["phi"], c["M"])
        ref = c["ref"]
        for key in ("Jr", "Jt"):
            want = np.array([[complex(*z) for z in row] for row in ref[key]])
            assert np.max(np.abs(r[key] - want)) <= 1e-9, (c["name"], key)
    assert seen >= 2


def test_invalid_settings(eng, cases):
    c = next(c for c in cases if c["name"] == "sampled65536_TE")
    stack = stack_from_json(c["stack"])
    stack.layers[0].fft_samples = 12            # at most 4M: tests/test_fft.cpp:116-118
    with pytest.raises(ValueError):
        eng.solve1d_arrays(stack, [(0.83, 27.0)], 3, 0)
    stack.layers[0].fft_samples = 4194305
    with pytest.raises(ValueError):
        eng.solve1d_arrays(stack, [(0.83, 27.0)], 3, 0)
    stack.layers[0].fft_samples = 0
    stack.layers[0].fourier_method = 7
    with pytest.raises(ValueError):
        eng.solve1d_arrays(stack, [(0.83, 27.0)], 3, 0)
    with pytest.raises(ValueError):
        eng.fourier_coefficients([0.0, 1.0], [1.0], 1.0, 1, method=1, samples=2)   # samples <= 2 hmax
    with pytest.raises(ValueError):
        eng.fourier_coefficients([0.0, 0.7], [1.0], 1.0, 1, method=1, samples=16)  # does not span the period
