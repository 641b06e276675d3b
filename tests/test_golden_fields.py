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


def test_phase_fixture_pinned_to_frozen_python():
    # the reference's slices and phase maps agree with the frozen arrays of its Python authority by the
    # reference test's own criteria (tests/test_rcwa2d_fields.cpp:332-395)
    seen = 0
    for c in load_jsonl("phase_cases.jsonl.gz"):
        if c["kind"] != "slice2d":
            continue
        cv = lambda v: np.array([complex(*z) for z in v])
        got, frozen = cv(c["slice"]), cv(c["frozen_slice"])
        assert np.all(np.abs(got - frozen) <= c["near_atol"] + c["near_rtol"] * np.abs(frozen)), c["name"]
        n = c["nz"] * c["nt"]
        fmask = np.frombuffer(c["frozen_mask"].encode(), np.uint8) == ord("1")
        fcmp = np.frombuffer(c["frozen_comparison"].encode(), np.uint8) == ord("1")
        for comp in range(6):
            sl = slice(comp * n, (comp + 1) * n)
            for key, fkey in (("abs", "frozen_phase_absolute"), ("inc", "frozen_phase_incident")):
                mask = np.frombuffer(c[f"{key}{comp}_mask"].encode(), np.uint8) == ord("1")
                assert np.array_equal(mask, fmask[sl]), (c["name"], comp, key)
                use = ~fcmp[sl]
                ph = np.array([float(x) for x in c[f"{key}{comp}_phase"]])[use]
                want = np.array([float(x) for x in c[fkey]])[sl][use]
                amp = np.abs(frozen[sl][use])
                chord = np.abs(np.exp(1j * ph) - np.exp(1j * want))
                assert np.all(chord <= 2.0 * (c["near_atol"] + c["near_rtol"] * amp) / amp + 5e-14), (c["name"], comp, key)
        seen += 1
    assert seen == 14
