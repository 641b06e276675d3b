"""Batched conical-incidence solve on the GPU through the C ABI, against the reference's ten Jones
tables, its own solve_conical outputs (including the Schur-basis degenerate-layer cases) and the
CPU oracle at the benchmark's conical shape. Tolerances: Jones |dJ| <= 1e-9 max(1, |J|) against the
tables (as tests/test_rcwa1d_conical.cpp:231-276); per-channel efficiencies within 1e-10 of the
reference and the oracle."""
import numpy as np
import pytest

from conftest import de_from_ref, jones_from_ref, jones_from_table
from oracle import oracle
from stablercwa_gb300 import Layer, Stack, stack_from_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def test_conical_golden(eng, conical_cases):
    worst = 0.0
    for case in conical_cases:
        s = stack_from_json(case["stack"])
        r = eng.solve_conical(s, case["wavelength"], case["theta"], case["phi"], case["M"])
        ref = case["ref"]
        assert r["status"] == 0, case["name"]
        for key in ("DEr", "DEt"):
            err = np.max(np.abs(r[key] - de_from_ref(ref[key])))
            assert err <= 1e-10, (case["name"], key, err)
            worst = max(worst, err)
        for key in ("Jr", "Jt"):
            want = jones_from_ref(ref[key])
            assert np.max(np.abs(r[key] - want) / np.maximum(1.0, np.abs(want))) <= 1e-9, (case["name"], key)
        if "table" in case:
            for key, tkey in (("Jr", "jr"), ("Jt", "jt")):
                want = jones_from_table(case["table"][tkey])
                assert np.max(np.abs(r[key] - want) / np.maximum(1.0, np.abs(want))) <= 1e-9, (case["name"], key)
        assert r["n_eig"] == ref["n_eig"] and r["n_schur"] == ref["n_schur"], case["name"]
        assert r["n_dense_solve"] == ref["n_dense_solve"], case["name"]
        assert bool(r["degenerate_mode_warning"]) == ref["degenerate_mode_warning"], case["name"]
        assert np.allclose(r["flux_r"], ref["flux_r"], atol=1e-14) and abs(r["ky"] - ref["ky"]) <= 1e-15
    print("worst |dDE| conical GPU vs reference:", worst)


def conical_bench_stack(rng):
    layers = []
    for _ in range(3):
        K = int(rng.integers(2, 5))
        inner = np.sort(rng.uniform(0.0, 0.574, K - 1))
        edges = [0.0, *inner.tolist(), 0.574]
        layers.append(Layer.grating(rng.uniform(0.05, 0.3), edges, rng.uniform(1.0, 2.5, K).tolist()))
    layers.append(Layer.uniform(rng.uniform(0.05, 0.3), complex(1.5 + rng.uniform(0, 0.5), rng.uniform(0, 0.1))))
    return Stack(nI=1.0, nII=1.46, period=0.574, layers=layers)


def test_conical_batch_vs_oracle(eng):
    # the conical benchmark structure at M = 20 on a seeded sample of (lambda, theta, phi)
    rng = np.random.default_rng(7)
    s = conical_bench_stack(rng)
    pts = np.stack([rng.uniform(0.5, 1.6, 12), rng.uniform(0, 60, 12), rng.uniform(0, 90, 12)], axis=1)
    g = eng.solve_conical_arrays(s, pts, 20)
    o = oracle.solve_conical_batch(s, pts, 20, threads=8)
    assert (g["status"] == o["status"]).all()
    ok = g["status"] == 0
    for key in ("DEr", "DEt"):
        assert np.max(np.abs(g[key][ok] - o[key][ok])) <= 1e-10, key
    assert (g["n_schur"] == o["n_schur"]).all()
