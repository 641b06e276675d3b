"""The CPU oracle's 2-D solve (oracle/oracle_rcwa2d.hpp) pinned to the reference: its Eps / Cx / Cy against
the reference's frozen operator tables, its amplitudes and efficiencies against the frozen tables of
tests/rcwa2d_reference.inc and tests/rcwa2d_core_fixture.inc and against the reference's own rcwa::solve2d
outputs (include/stablercwa/rcwa2d.hpp:1359) for every case of tests/golden/rcwa2d_cases.jsonl.gz, its
Rayleigh statuses, energy conservation on the lossless cases, and its near-field harmonics against the
reference's field_at. CPU only: the oracle is the checker the device parity tests can use on inputs the
fixtures do not hold."""
import gzip
import json
import os

import numpy as np
import pytest

from conftest import cvec, rvec
from stablercwa_gb300.types import stack2d_from_json

HERE = os.path.dirname(os.path.abspath(__file__))
OP_TOL = 1e-12   # operators, relative to the matrix's largest entry (test_rcwa2d_reference.cpp:160)
DE_TOL = 1e-10   # per-order efficiencies against the reference's own solve
AMP_TOL = 1e-9   # amplitudes: |a - b| <= 1e-9 + 1e-9 |b|, the reference's frozen-table contract


@pytest.fixture(scope="module")
def cases():
    with gzip.open(os.path.join(HERE, "golden", "rcwa2d_cases.jsonl.gz"), "rt") as f:
        return [json.loads(line) for line in f]


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as o
    return o


def solve(oracle, c):
    jones = complex(*c["jones"][0]), complex(*c["jones"][1])
    r = oracle.solve2d_batch(stack2d_from_json(c["stack"]), [(c["wavelength"], c["theta"], c["phi"], *jones)],
                             c["M1"], c["M2"], laurent=bool(c["laurent"]), threads=1)
    return {k: v[0] for k, v in r.items()}


def close(a, b, atol, rtol):
    return np.all(np.abs(a - b) <= atol + rtol * np.abs(b))


def test_operators_match_reference_tables(oracle, cases):
    count = 0
    for c in cases:
        stack = stack2d_from_json(c["stack"])
        for o in c["operators"]:
            N = o["N"]
            eps, cx, cy, singular = oracle.layer_operators2d(stack.layers[o["layer"]], stack.Lx, stack.Ly, c["M1"],
                                                             c["M2"], laurent=bool(c["laurent"]))
            assert not singular
            for got, key in ((eps, "eps"), (cx, "cx"), (cy, "cy")):
                ref = cvec(o[key]).reshape(N, N)  # row-major in the fixture
                rel = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1.0)
                assert rel <= OP_TOL, (c["name"], key, rel)
                count += 1
    assert count >= 60


def test_frozen_tables(oracle, cases):
    seen = 0
    for c in cases:
        if "table" not in c or c.get("table_status") == 2:
            continue
        seen += 1
        r, t, ref = solve(oracle, c), c["table"], c["ref"]
        assert r["status"] == 0, c["name"]
        atol, rtol = t["atol"], t["rtol"]
        assert close(r["Kx"], rvec(t["Kx"]), atol, rtol) and close(r["Ky"], rvec(t["Ky"]), atol, rtol), c["name"]
        for key in ("kzI", "kzII", "Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"):
            assert close(r[key], cvec(t[key]), atol, rtol), (c["name"], key, np.max(np.abs(r[key] - cvec(t[key]))))
        for key in ("DEr", "DEt"):
            assert close(r[key], rvec(t[key]), atol, rtol), (c["name"], key)
            assert np.max(np.abs(r[key] - rvec(ref[key]))) <= DE_TOL, (c["name"], key)
        if "prop_r" in t:
            assert np.array_equal(r["prop_r"].astype(bool), np.array(t["prop_r"], bool)), c["name"]
            assert np.array_equal(r["prop_t"].astype(bool), np.array(t["prop_t"], bool)), c["name"]
        assert r["n_eig"] == ref["n_eig"], c["name"]
    assert seen >= 30


def test_generated_cases_against_reference_solve(oracle, cases):
    seen = 0
    for c in cases:
        if c["source"] != "generated":
            continue
        seen += 1
        r, ref = solve(oracle, c), c["ref"]
        assert r["status"] == 0 and ref["status"] == 0, c["name"]
        for key in ("Kx", "Ky"):
            assert np.array_equal(r[key], rvec(ref[key])), (c["name"], key)
        for key in ("kzI", "kzII"):
            assert np.array_equal(r[key], cvec(ref[key])), (c["name"], key)
        for key in ("Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"):
            b = cvec(ref[key])
            assert close(r[key], b, AMP_TOL, AMP_TOL), (c["name"], key, np.max(np.abs(r[key] - b)))
        for key in ("DEr", "DEt"):
            assert np.max(np.abs(r[key] - rvec(ref[key]))) <= DE_TOL, (c["name"], key)
        assert r["n_eig"] == ref["n_eig"], c["name"]
    assert seen >= 5


def test_rayleigh_failures(oracle, cases):
    seen = 0
    for c in cases:
        if c.get("table_status") != 2:
            continue
        seen += 1
        stack = stack2d_from_json(c["stack"])
        r = solve(oracle, c)
        assert r["status"] == 3, c["name"]  # RCWA_SAMPLE_RAYLEIGH
        assert np.all(np.isnan(r["DEr"])) and np.all(np.isnan(r["Rs"].real)), c["name"]
        assert np.all(np.isfinite(r["Kx"])) and np.all(np.isfinite(r["kzI"])), c["name"]
        regions = r["rayleigh_regions"]
        for reg in c["rayleigh"]:
            k = 0 if reg["region"] == "incident" else (len(stack.layers) + 1 if reg["region"] == "exit" else reg["layer"] + 1)
            assert regions[k] == 1, (c["name"], reg)
        assert int(regions.sum()) == len(c["rayleigh"]), c["name"]
    assert seen == 5


def test_energy_conservation_lossless(oracle, cases):
    seen = 0
    for c in cases:
        stack = stack2d_from_json(c["stack"])
        indices = [complex(stack.nII)] + [complex(L.n) for L in stack.layers if L.homogeneous]
        indices += [complex(v) for L in stack.layers if not L.homogeneous for p in L.x_profiles for v in p.n_values]
        if any(z.imag != 0.0 for z in indices) or c.get("table_status") == 2:
            continue
        r = solve(oracle, c)
        if r["status"] != 0:
            continue
        seen += 1
        defect = abs(np.sum(r["DEr"]) + np.sum(r["DEt"]) - 1.0)
        assert defect <= 1e-11, (c["name"], defect)
    assert seen >= 20


def test_near_fields_match_reference(oracle):
    """The oracle's near-field harmonics against the reference's rcwa::field_at (every case of
    tests/golden/fields2d_cases.jsonl.gz, zero-thickness and layer-less stacks included) and against the
    frozen Python harmonics within their own tolerances."""
    with gzip.open(os.path.join(HERE, "golden", "fields2d_cases.jsonl.gz"), "rt") as f:
        cases = [json.loads(line) for line in f]
    for c in cases:
        stack = stack2d_from_json(c["stack"])
        jones = complex(*c["jones"][0]), complex(*c["jones"][1])
        arrays, fields = oracle.solve2d_fields(stack, [(c["wavelength"], c["theta"], c["phi"], *jones)], c["M1"], c["M2"],
                                               c["zs"], laurent=bool(c["laurent"]))
        assert arrays["status"][0] == 0, c["name"]
        assert np.max(np.abs(arrays["DEr"][0] - rvec(c["DEr"]))) <= DE_TOL, c["name"]
        want = np.array([[[complex(*z) for z in row] for row in comp] for comp in c["fields"]])  # (6, N, nz)
        err = np.max(np.abs(fields[0] - want) / (1.0 + np.abs(want)))
        assert err <= 1e-11, (c["name"], err)
        if "frozen" in c:
            fz = np.array([[[complex(*z) for z in row] for row in comp] for comp in c["frozen"]])
            assert np.all(np.abs(fields[0] - fz) <= c["near_atol"] + c["near_rtol"] * np.abs(fz)), c["name"]
    assert len(cases) >= 28


def test_n441_point_against_reference(oracle):
    """One point of the benchmark's 2-D workload (Mx = My = 10: N = 441, eigenproblems of order 882) through the oracle
    against the reference's own solve2d output for it: efficiencies within 1e-10 (about a minute on one core)."""
    with gzip.open(os.path.join(HERE, "golden", "rcwa2d_n441_cases.jsonl.gz"), "rt") as f:
        c = json.loads(f.readline())
    assert (c["M1"], c["M2"]) == (10, 10)
    r = solve(oracle, {**c, "laurent": c.get("laurent", 0)})
    ref = c["ref"]
    assert r["status"] == 0 and ref["status"] == 0
    for key in ("DEr", "DEt"):
        assert np.max(np.abs(r[key] - rvec(ref[key]))) <= DE_TOL, key
    assert r["n_eig"] == ref["n_eig"]
