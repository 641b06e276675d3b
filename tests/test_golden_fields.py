"""The near-field fixtures (tests/golden/export_fields.cpp) hold the physics the reference's own field test
asserts (tests/test_rcwa_public_fields.cpp:69-80): tangential components continuous across every surface,
repeated depths identical, and a depth 5e-13 below an interface clipped onto it."""
import numpy as np

from conftest import load_jsonl


def fields(c):
    return np.array([[[complex(*z) for z in row] for row in comp] for comp in c["fields"]])


def test_fixture_inventory():
    cases = load_jsonl("fields1d_cases.jsonl.gz")
    names = {c["name"] for c in cases}
    for stem in ("mixed", "mixed_far", "schur", "readme_M20", "films", "multi_grating"):
        assert {stem + "_TE", stem + "_TM"} <= names
    assert sum(c["kind"] == "conical" for c in cases) >= 8
    assert next(c for c in cases if c["name"] == "conical_schur_M8")["n_schur"] == 1
    for c in cases:
        assert c["available"] == 1
        assert fields(c).shape == (6, 2 * c["M"] + 1, len(c["zs"]))
        assert np.all(np.isfinite(fields(c)))


def test_conical_zero_thickness_layers_change_nothing():
    # tests/test_rcwa_public_fields.cpp:213-216: zero-thickness layers are skipped, bit for bit
    cases = {c["name"]: c for c in load_jsonl("fields1d_cases.jsonl.gz")}
    assert np.array_equal(fields(cases["conical_mixed_jones"]), fields(cases["conical_zero_layers"]))


def test_tangential_continuity_in_fixtures():
    for c in load_jsonl("fields1d_cases.jsonl.gz"):
        if c["name"].startswith("mixed_far") or c["kind"] != "planar":
            continue
        f = fields(c)
        zs = c["zs"]
        for k in range(len(zs) - 1):
            if abs(zs[k + 1] - zs[k] - 1e-9) < 1e-15:   # an interface and 1e-9 below it
                for comp in (0, 1, 3, 4):
                    a, b = f[comp, :, k], f[comp, :, k + 1]
                    assert np.all(np.abs(a - b) <= 3e-7 * (1.0 + np.abs(b))), (c["name"], k, comp)


def test_repeated_and_clipped_depths():
    for c in load_jsonl("fields1d_cases.jsonl.gz"):
        if not (c["name"].startswith("mixed_far") or c["name"] == "conical_mixed_jones"):
            continue
        f = fields(c)
        # zs = .083, -.12, .42, .2, .2+5e-13, .42+5e-13, .083, .245, 0, 100, -100
        assert np.array_equal(f[:, :, 0], f[:, :, 6])
        assert np.array_equal(f[:, :, 3], f[:, :, 4])


def test_fields2d_fixture_pinned_to_frozen_python():
    # the reference's C++ harmonics agree with the frozen harmonics of its Python authority within the
    # tolerances frozen beside them (tests/test_rcwa2d_fields.cpp:270-290)
    cases = load_jsonl("fields2d_cases.jsonl.gz")
    frozen = [c for c in cases if "frozen" in c]
    assert len(frozen) >= 20
    for c in frozen:
        got, want = fields(c), np.array([[[complex(*z) for z in row] for row in comp] for comp in c["frozen"]])
        assert got.shape == want.shape
        assert np.all(np.abs(got - want) <= c["near_atol"] + c["near_rtol"] * np.abs(want)), c["name"]
    for c in cases:
        assert c["status"] == 0 and c["available"] == 1
        assert fields(c).shape == (6, (2 * c["M1"] + 1) * (2 * c["M2"] + 1), len(c["zs"]))
