"""Planar near fields on the GPU, through the C ABI, against the reference's own rcwa::solve_with_fields +
rcwa::field_at (include/stablercwa/rcwa1d_fields.hpp) on the structures of
tests/test_rcwa_public_fields.cpp and a few more (tests/golden/export_fields.cpp)."""
import numpy as np
import pytest

from conftest import load_jsonl, rvec
from stablercwa_gb300.types import stack_from_json

pytestmark = pytest.mark.gpu

# Field harmonics are compared elementwise as |a - b| <= TOL * (1 + |b|), the form of the reference's own
# close() (tests/test_rcwa_public_fields.cpp:24) and at its tolerance; the largest difference measured
# on these stacks is below 1e-13.
TOL = 5e-12
# 2-D: the same bound (measured worst 2.5e-13, over the reference's frozen cases and problems A-C)
TOL2D = TOL


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


@pytest.fixture(scope="module")
def cases():
    return [c for c in load_jsonl("fields1d_cases.jsonl.gz") if c["kind"] == "planar"]


@pytest.fixture(scope="module")
def conical_cases():
    return [c for c in load_jsonl("fields1d_cases.jsonl.gz") if c["kind"] == "conical"]



def golden_fields(c):
    return np.array([[[complex(*z) for z in row] for row in comp] for comp in c["fields"]])  # (6, n, nz)


def run(eng, c):
    stack = stack_from_json(c["stack"])
    pol = 0 if c["pol"] == "TE" else 1
    return eng.solve1d_fields(stack, [(c["wavelength"], c["theta"])], c["M"], pol, c["zs"])


def test_fields_match_reference(eng, cases):
    worst = 0.0
    for c in cases:
        arrays, fields = run(eng, c)
        assert arrays["status"][0] == 0, c["name"]
        assert np.max(np.abs(arrays["DEr"][0] - rvec(c["DEr"]))) <= 1e-10, c["name"]
        want = golden_fields(c)
        got = fields[0]
        assert got.shape == want.shape, c["name"]
        err = np.max(np.abs(got - want) / (1.0 + np.abs(want)))
        worst = max(worst, err)
        assert err <= TOL, (c["name"], err)
    assert len(cases) >= 12
    print(f"worst relative field difference {worst:.3e}")


def test_batch_equals_single(eng, cases):
    c = next(c for c in cases if c["name"] == "multi_grating_TM")
    stack = stack_from_json(c["stack"])
    pts = [(0.95, -18.0), (0.9, 5.0), (1.1, 33.0)]
    _, many = eng.solve1d_fields(stack, pts, c["M"], 1, c["zs"])
    for p, pt in enumerate(pts):
        _, one = eng.solve1d_fields(stack, [pt], c["M"], 1, c["zs"])
        assert np.max(np.abs(many[p] - one[0]) / (1.0 + np.abs(one[0]))) <= 1e-13
    want = golden_fields(c)
    assert np.max(np.abs(many[0] - want) / (1.0 + np.abs(want))) <= TOL


def test_tangential_continuity(eng, cases):
    # tests/test_rcwa_public_fields.cpp:77-80: Ex, Ey, Hx, Hy continuous across every surface
    c = next(c for c in cases if c["name"] == "mixed_TE")
    stack = stack_from_json(c["stack"])
    for pol in (0, 1):
        zs = []
        for s in (0.0, 0.2, 0.29, 0.42):
            zs += [s - 1e-9, s + 1e-9]
        _, f = eng.solve1d_fields(stack, [(0.83, 27.0)], 3, pol, zs)
        for comp in (0, 1, 3, 4):
            a, b = f[0, comp, :, 0::2], f[0, comp, :, 1::2]
            assert np.all(np.abs(a - b) <= 3e-7 * (1.0 + np.abs(b)))


def test_field_map(eng, cases):
    c = next(c for c in cases if c["name"] == "mixed_far_TM")
    _, f = run(eng, c)
    kxm = rvec(c["kxm"])
    g = eng.field_map(f[0], kxm, c["stack"]["period"], nx=11)
    x = np.arange(11) / 11 * c["stack"]["period"]
    for comp in range(6):
        for iz in range(len(c["zs"])):
            want = np.array([np.sum(f[0, comp, :, iz] * np.exp(-1j * kxm * xx)) for xx in x])
            assert np.allclose(g[comp, iz], want, rtol=5e-12, atol=5e-12)


def test_empty_and_invalid_depths(eng, cases):
    c = cases[0]
    stack = stack_from_json(c["stack"])
    arrays, f = eng.solve1d_fields(stack, [(c["wavelength"], c["theta"])], c["M"], 0, [])
    assert f.shape == (1, 6, 2 * c["M"] + 1, 0)
    assert np.max(np.abs(arrays["DEr"][0] - rvec(c["DEr"]))) <= 1e-10
    for bad in (np.inf, np.nan):
        with pytest.raises(ValueError):
            eng.solve1d_fields(stack, [(c["wavelength"], c["theta"])], c["M"], 0, [0.1, bad])


def run_conical(eng, c):
    stack = stack_from_json(c["stack"])
    jones = [complex(*c["jones"][0]), complex(*c["jones"][1])]
    return eng.solve_conical_fields(stack, [(c["wavelength"], c["theta"], c["phi"])], c["M"], c["zs"], jones)


def test_conical_fields_match_reference(eng, conical_cases):
    worst = {}
    for c in conical_cases:
        arrays, fields = run_conical(eng, c)
        assert arrays["status"][0] == 0, c["name"]
        assert int(arrays["n_schur"][0]) == c["n_schur"], c["name"]
        assert np.max(np.abs(arrays["DEr"][0][:, 0] - rvec(c["DEr_ss"]))) <= 1e-10, c["name"]
        want = golden_fields(c)
        err = np.max(np.abs(fields[0] - want) / (1.0 + np.abs(want)))
        worst[c["name"]] = err
        assert err <= TOL, (c["name"], err)  # the Schur case included: measured below 1e-13
    assert len(conical_cases) >= 8
    print("worst relative conical field difference", {k: f"{v:.2e}" for k, v in worst.items()})


def test_conical_jones_linearity(eng, conical_cases):
    # a common phase on the Jones vector multiplies every field by it (tests/test_rcwa_public_fields.cpp:105-107)
    c = next(c for c in conical_cases if c["name"] == "conical_mixed_jones")
    stack = stack_from_json(c["stack"])
    pt = [(c["wavelength"], c["theta"], c["phi"])]
    j = np.array([complex(*c["jones"][0]), complex(*c["jones"][1])])
    carrier = np.exp(0.73j)
    _, a = eng.solve_conical_fields(stack, pt, c["M"], c["zs"], j)
    _, b = eng.solve_conical_fields(stack, pt, c["M"], c["zs"], j * carrier)
    assert np.all(np.abs(b - carrier * a) <= 2e-12 * (1.0 + np.abs(carrier * a)))
    # the two basis columns combine linearly (after the normalisation of the Jones vector)
    _, s = eng.solve_conical_fields(stack, pt, c["M"], c["zs"], [1.0, 0.0])
    _, p = eng.solve_conical_fields(stack, pt, c["M"], c["zs"], [0.0, 1.0])
    jn = j / np.max(np.abs(np.r_[j.real, j.imag]))
    jn = jn / np.linalg.norm(jn)
    assert np.allclose(jn[0] * s + jn[1] * p, a, rtol=1e-11, atol=1e-12)
    for bad in ([0.0, 0.0], [np.inf, 0.0]):
        with pytest.raises(ValueError):
            eng.solve_conical_fields(stack, pt, c["M"], c["zs"], bad)


def test_conical_batch_equals_single(eng, conical_cases):
    c = next(c for c in conical_cases if c["name"] == "conical_multi_grating")
    stack = stack_from_json(c["stack"])
    pts = [(0.95, -18.0, 63.0), (0.9, 5.0, 10.0), (1.1, 33.0, 80.0)]
    _, many = eng.solve_conical_fields(stack, pts, c["M"], c["zs"], [0.0, 1.0])
    for p, pt in enumerate(pts):
        _, one = eng.solve_conical_fields(stack, [pt], c["M"], c["zs"], [0.0, 1.0])
        assert np.max(np.abs(many[p] - one[0]) / (1.0 + np.abs(one[0]))) <= 1e-13


def test_fields2d_match_reference(eng):
    from stablercwa_gb300.types import stack2d_from_json
    worst = {}
    for c in load_jsonl("fields2d_cases.jsonl.gz"):
        stack = stack2d_from_json(c["stack"])
        jones = [complex(*c["jones"][0]), complex(*c["jones"][1])]
        arrays, fields = eng.solve2d_fields(stack, [(c["wavelength"], c["theta"], c["phi"], jones[0], jones[1])], c["M1"],
                                            c["M2"], c["zs"], laurent=bool(c["laurent"]))
        assert arrays["status"][0] == 0, c["name"]
        assert np.max(np.abs(arrays["DEr"][0] - rvec(c["DEr"]))) <= 1e-10, c["name"]
        want = golden_fields(c)
        err = np.max(np.abs(fields[0] - want) / (1.0 + np.abs(want)))
        worst[c["name"]] = err
        if "frozen" in c:  # and the frozen Python harmonics within their own tolerances
            fz = np.array([[[complex(*z) for z in row] for row in comp] for comp in c["frozen"]])
            assert np.all(np.abs(fields[0] - fz) <= c["near_atol"] + c["near_rtol"] * np.abs(fz)), c["name"]
    print("worst relative 2-D field difference", {k: f"{v:.2e}" for k, v in worst.items()})
    for name, err in worst.items():
        assert err <= TOL2D, (name, err)
    assert len(worst) >= 28


def test_fields2d_failure_and_depth_checks(eng):
    from stablercwa_gb300.types import stack2d_from_json
    c = next(c for c in load_jsonl("fields2d_cases.jsonl.gz") if c["name"] == "problem_a")
    stack = stack2d_from_json(c["stack"])
    jones = [complex(*c["jones"][0]), complex(*c["jones"][1])]
    pt = (c["wavelength"], c["theta"], c["phi"], jones[0], jones[1])
    with pytest.raises(ValueError):
        eng.solve2d_fields(stack, [pt], 1, 1, [0.1, np.nan])
    arrays, f = eng.solve2d_fields(stack, [pt], 1, 1, [])
    assert f.shape == (1, 6, 9, 0) and arrays["status"][0] == 0
    # a point that fails with max_iter = 1 carries NaN fields; the other point of the batch is unaffected
    from stablercwa_gb300.types import Options
    arrays, f = eng.solve2d_fields(stack, [pt], 1, 1, [0.1, 0.5], options=Options(eig_max_iter=1))
    assert arrays["status"][0] != 0 and np.isnan(f).all()
