"""GPU 2-D (crossed-grating) solve through the C ABI against the reference: the frozen tables of
tests/rcwa2d_reference.inc and tests/rcwa2d_core_fixture.inc (Kx, Ky, kz, fields, s/p amplitudes,
efficiencies, Rayleigh failures), their Eps / Cx / Cy operators, and the reference's own
rcwa::solve2d outputs for every case (include/stablercwa/rcwa2d.hpp:1359)."""
import numpy as np
import pytest

from conftest import cvec, rvec
from stablercwa_gb300 import abi
from stablercwa_gb300.types import stack2d_from_json

pytestmark = pytest.mark.gpu

DE_TOL = 1e-10        # per-order efficiencies against the reference's own solve
AMP_TOL = 1e-9        # amplitudes: the reference's frozen-table contract |a - b| <= 1e-9 + 1e-9 |b|
OP_TOL = 1e-12        # operators, relative to the matrix's largest entry (test_rcwa2d_reference.cpp:160)


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def jones(c):
    return complex(*c["jones"][0]), complex(*c["jones"][1])


def solve(eng, c):
    return eng.solve2d(stack2d_from_json(c["stack"]), c["wavelength"], c["theta"], c["phi"], c["M1"], c["M2"], jones(c),
                       laurent=bool(c["laurent"]))


def close(a, b, atol, rtol):
    return np.all(np.abs(a - b) <= atol + rtol * np.abs(b))


def test_operators_match_frozen(eng, cases2d):
    worst, count = 0.0, 0
    for c in cases2d:
        stack = stack2d_from_json(c["stack"])
        for o in c["operators"]:
            N = o["N"]
            eps, cx, cy, sing = eng.layer_operators2d(stack.layers[o["layer"]], stack.Lx, stack.Ly, c["M1"], c["M2"],
                                                      laurent=bool(c["laurent"]))
            assert not sing
            for got, key in ((eps, "eps"), (cx, "cx"), (cy, "cy")):
                ref = cvec(o[key]).reshape(N, N)  # row-major in the fixture
                rel = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1.0)
                assert rel <= OP_TOL, (c["name"], key, rel)
                worst = max(worst, rel)
                count += 1
    assert count >= 60


def test_frozen_tables(eng, cases2d):
    worst_de = 0.0
    for c in cases2d:
        if "table" not in c:
            continue
        r = solve(eng, c)
        t = c["table"]
        assert r["status"] == 0, c["name"]
        atol, rtol = t["atol"], t["rtol"]
        assert np.array_equal(r["Kx"], rvec(t["Kx"])) or close(r["Kx"], rvec(t["Kx"]), atol, rtol), c["name"]
        assert close(r["Ky"], rvec(t["Ky"]), atol, rtol), c["name"]
        for key in ("kzI", "kzII", "Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"):
            assert close(r[key], cvec(t[key]), atol, rtol), (c["name"], key, np.max(np.abs(r[key] - cvec(t[key]))))
        for key in ("DEr", "DEt"):
            assert close(r[key], rvec(t[key]), atol, rtol), (c["name"], key)
        if "prop_r" in t:
            assert np.array_equal(r["prop_r"].astype(bool), np.array(t["prop_r"], bool)), c["name"]
            assert np.array_equal(r["prop_t"].astype(bool), np.array(t["prop_t"], bool)), c["name"]
        ref = c["ref"]
        for key in ("DEr", "DEt"):
            d = np.max(np.abs(r[key] - rvec(ref[key])))
            assert d <= DE_TOL, (c["name"], key, d)
            worst_de = max(worst_de, d)
        assert r["n_eig"] == ref["n_eig"], c["name"]
        assert r["n_dense_solve"] == ref["n_dense_solve"], (c["name"], r["n_dense_solve"], ref["n_dense_solve"])


def test_generated_cases_against_reference_solve(eng, cases2d):
    seen = 0
    for c in cases2d:
        if c["source"] != "generated":
            continue
        seen += 1
        r = solve(eng, c)
        ref = c["ref"]
        assert r["status"] == 0 and ref["status"] == 0, c["name"]
        assert np.array_equal(r["Kx"], rvec(ref["Kx"])) and np.array_equal(r["Ky"], rvec(ref["Ky"])), c["name"]
        assert np.array_equal(r["kzI"], cvec(ref["kzI"])) and np.array_equal(r["kzII"], cvec(ref["kzII"])), c["name"]
        for key in ("Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "Rs", "Rp", "Ts", "Tp"):
            b = cvec(ref[key])
            assert close(r[key], b, AMP_TOL, AMP_TOL), (c["name"], key, np.max(np.abs(r[key] - b)))
        for key in ("DEr", "DEt"):
            d = np.max(np.abs(r[key] - rvec(ref[key])))
            assert d <= DE_TOL, (c["name"], key, d)
        assert r["n_eig"] == ref["n_eig"] and r["n_dense_solve"] == ref["n_dense_solve"], c["name"]
    assert seen >= 5


def test_rayleigh_failures(eng, cases2d):
    seen = 0
    for c in cases2d:
        if c.get("table_status") != 2:
            continue
        seen += 1
        stack = stack2d_from_json(c["stack"])
        r = solve(eng, c)
        assert r["status"] == abi.RCWA_SAMPLE_RAYLEIGH, c["name"]
        assert np.all(np.isnan(r["DEr"])) and np.all(np.isnan(r["Rs"].real)), c["name"]
        assert np.all(np.isfinite(r["Kx"])) and np.all(np.isfinite(r["kzI"])), c["name"]
        regions = r["rayleigh_regions"]
        for reg in c["rayleigh"]:
            k = 0 if reg["region"] == "incident" else (len(stack.layers) + 1 if reg["region"] == "exit" else reg["layer"] + 1)
            assert regions[k] == 1, (c["name"], reg)
        assert int(regions.sum()) == len(c["rayleigh"]), c["name"]
        for reg in c["rayleigh"]:
            for m, n in reg["orders"]:
                assert f"({m}, {n})" in r["message"], (c["name"], r["message"])
    assert seen == 5


def test_batch_equals_single_points(eng, cases2d):
    c = next(c for c in cases2d if c["name"] == "pillars_films_oblique")
    stack = stack2d_from_json(c["stack"])
    pts = [(0.83, 23.0, 37.0, 0.6 + 0.2j, 0.7745966692414834), (0.71, 5.0, 80.0, 1.0, 0.0),
           (0.95, 41.0, -20.0, 0.0, 1.0), (0.6, 0.0, 0.0, 1.0, 0.0), (1.1, 60.0, 10.0, 0.5j, 0.5)]
    batch = eng.solve2d_arrays(stack, pts, c["M1"], c["M2"])
    for k, p in enumerate(pts):
        one = eng.solve2d(stack, p[0], p[1], p[2], c["M1"], c["M2"], (p[3], p[4]))
        assert batch["status"][k] == one["status"] == 0
        for key in ("Rs", "Rp", "Ts", "Tp", "DEr", "DEt"):
            assert np.max(np.abs(batch[key][k] - one[key])) <= 1e-12, (k, key)
    # the first point is the fixture case itself
    assert np.max(np.abs(batch["DEr"][0] - rvec(c["ref"]["DEr"]))) <= DE_TOL


def test_energy_conservation_lossless(eng, cases2d):
    for c in cases2d:
        stack = stack2d_from_json(c["stack"])
        lossless = complex(stack.nII).imag == 0 and all(
            (complex(L.n).imag == 0) if L.homogeneous else all(complex(v).imag == 0 for p in L.x_profiles for v in p.n_values)
            for L in stack.layers)
        if not lossless or c["ref"]["status"] != 0:
            continue
        r = solve(eng, c)
        es, ep = jones(c)
        power = abs(es) ** 2 + abs(ep) ** 2
        ref_defect = abs(np.sum(rvec(c["ref"]["DEr"])) + np.sum(rvec(c["ref"]["DEt"])) - power)
        defect = abs(np.sum(r["DEr"]) + np.sum(r["DEt"]) - power)
        # |R + T - |E|^2| <= 1e-12; where the reference itself is that loose (an ill-conditioned case:
        # pillars_films_m6, reference 6.9e-13), the bound is ten times the reference's own defect
        assert defect <= max(1e-12, 10 * ref_defect), (c["name"], defect, ref_defect)


def test_invalid_arguments(eng, cases2d):
    c = next(c for c in cases2d if c["name"] == "ref_9_pillar_sq")
    stack = stack2d_from_json(c["stack"])
    with pytest.raises(ValueError):
        eng.solve2d(stack, 1.0, 90.0, 0.0, 2, 2, (1.0, 0.0))
    with pytest.raises(ValueError):
        eng.solve2d(stack, -1.0, 10.0, 0.0, 2, 2, (1.0, 0.0))
    with pytest.raises(ValueError):
        eng.solve2d(stack, 1.0, 10.0, 0.0, -1, 2, (1.0, 0.0))
    bad = stack2d_from_json(c["stack"])
    bad.layers[0].y_edges = list(reversed(bad.layers[0].y_edges))
    with pytest.raises(ValueError):
        eng.solve2d(bad, 1.0, 10.0, 0.0, 2, 2, (1.0, 0.0))
