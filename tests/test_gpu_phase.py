"""Field slices and phase maps on the GPU, through the C ABI (rcwa_gpu_field_slice, rcwa_gpu_phase_data), against
the reference's own field_slice / field_map / phase_data (include/stablercwa/rcwa_fields.hpp:326-385,
rcwa_phase.hpp:229-271) on identical inputs, and the whole chain (2-D solve with fields, slice, phase) against
the frozen arrays of the Python authority in tests/rcwa2d_fields_fixture.inc (tests/golden/export_phase.cpp)."""
import numpy as np
import pytest

from conftest import load_jsonl
from stablercwa_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


@pytest.fixture(scope="module")
def cases():
    return load_jsonl("phase_cases.jsonl.gz")


def cv(v):
    a = np.asarray(v, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def rv(v):
    return np.array([float(x) for x in v])


def mask_of(s):
    return np.frombuffer(s.encode(), dtype=np.uint8) == ord("1")


def harmonics_of(cases, c):
    src = c if "harmonics" in c else next(x for x in cases if x["kind"] == "slice2d" and x["id"] == c["id"] and x["plane"] == 0)
    return cv(src["harmonics"]).reshape(6, len(c["kx"]), c["nz"])


def same_phase(got, mask, want, want_mask, tol=1e-12):
    assert np.array_equal(mask, want_mask)
    ok = ~want_mask
    assert np.all(np.isnan(got[~ok]))
    assert np.max(np.abs(got[ok] - want[ok]), initial=0.0) <= tol


def test_slices_match_reference(eng, cases):
    seen = 0
    for c in cases:
        if c["kind"] != "slice2d":
            continue
        seen += 1
        h = harmonics_of(cases, c)
        got = eng.field_slice(h, rv(c["kx"]), rv(c["ky"]), c["plane"], c["nt"], c["period"], c["at"])
        want = cv(c["slice"]).reshape(6, c["nz"], c["nt"])
        assert np.max(np.abs(got - want) / (1.0 + np.abs(want))) <= 5e-12, c["name"]
    assert seen >= 14


def test_phase_matches_reference_on_the_same_grid(eng, cases):
    seen = 0
    for c in cases:
        if c["kind"] == "slice2d":
            grid = cv(c["slice"]).reshape(6, c["nz"], c["nt"])
            for comp in range(6):
                p = eng.phase_data(grid[comp])
                same_phase(p["phase"].ravel(), p["mask"].ravel(), rv(c[f"abs{comp}_phase"]), mask_of(c[f"abs{comp}_mask"]))
                p = eng.phase_data(grid[comp], "incident", incident_k=rv(c["incident_k"]), x=rv(c["x"]), y=rv(c["y"]),
                                   z=rv(c["zs"]))
                same_phase(p["phase"].ravel(), p["mask"].ravel(), rv(c[f"inc{comp}_phase"]), mask_of(c[f"inc{comp}_mask"]))
                seen += 2
        elif c["kind"] == "phase":
            nz, nt = c["nz"], c["nt"]
            grid = cv(c["grid"]).reshape(6, nz, nt)
            row = cv(c["custom_row"])
            opts = {"abs_none": dict(), "abs_both": dict(unwrap="both"),
                    "inc_x": dict(reference="incident", unwrap="x"), "inc_z": dict(reference="incident", unwrap="z"),
                    "custom_both": dict(reference="custom", unwrap="both", custom=row[None, :]),
                    "abs_floor": dict(unwrap="both", phase_floor=0.35)}
            for comp in range(6):
                for key, kw in opts.items():
                    p = eng.phase_data(grid[comp], incident_k=rv(c["incident_k"]), x=rv(c["x"]), y=rv(c["y"]), z=rv(c["z"]),
                                       **kw)
                    same_phase(p["phase"].ravel(), p["mask"].ravel(), rv(c[f"{key}{comp}_phase"]),
                               mask_of(c[f"{key}{comp}_mask"]))
                    assert np.max(np.abs(p["amplitude"].ravel() - rv(c[f"{key}{comp}_amplitude"]))) <= 1e-15 * (
                        1 + np.max(np.abs(grid[comp])))
                    seen += 1
    assert seen >= 276  # 14 slices x 6 components x 2 references + 3 grids x 6 components x 6 option sets


def test_chain_against_frozen_python(eng, cases):
    """2-D solve with fields -> slice -> phase, all on the GPU, against the frozen numpy arrays with the
    reference's own criteria (test_rcwa2d_fields.cpp:332-395): slice values within near_atol + near_rtol |b|,
    phase chords within 2 (atol + rtol |F|) / |F| + 5e-14 where the frozen comparison mask allows, masks equal."""
    from stablercwa_gb300.types import stack2d_from_json
    fields2d = {c["name"]: c for c in load_jsonl("fields2d_cases.jsonl.gz")}  # the stacks of the frozen cases
    seen = 0
    for c in cases:
        if c["kind"] != "slice2d" or c["id"] == 22:
            continue
        ref = fields2d["ref_" + c["name"][:-3]]
        stack = stack2d_from_json(ref["stack"])
        jones = [complex(*c["jones"][0]), complex(*c["jones"][1])]
        _, f = eng.solve2d_fields(stack, [(c["wavelength"], c["theta"], c["phi"], jones[0], jones[1])], c["M1"], c["M2"],
                                  rv(c["zs"]), laurent=bool(c["laurent"]))
        grid = eng.field_slice(f[0], rv(c["kx"]), rv(c["ky"]), c["plane"], c["nt"], c["period"], c["at"])
        frozen = cv(c["frozen_slice"]).reshape(6, c["nz"], c["nt"])
        assert np.all(np.abs(grid - frozen) <= c["near_atol"] + c["near_rtol"] * np.abs(frozen)), c["name"]
        fmask = mask_of(c["frozen_mask"]).reshape(6, -1)
        fcmp = mask_of(c["frozen_comparison"]).reshape(6, -1)
        for comp in range(6):
            for kind, key in (("absolute", "frozen_phase_absolute"), ("incident", "frozen_phase_incident")):
                p = eng.phase_data(grid[comp], kind, incident_k=rv(c["incident_k"]), x=rv(c["x"]), y=rv(c["y"]),
                                   z=rv(c["zs"]))
                assert np.array_equal(p["mask"].ravel(), fmask[comp]), (c["name"], comp, kind)
                want = rv(c[key]).reshape(6, -1)[comp]
                amp = np.abs(frozen[comp].ravel())
                use = ~fcmp[comp]
                chord = np.abs(np.exp(1j * p["phase"].ravel()[use]) - np.exp(1j * want[use]))
                tol = 2.0 * (c["near_atol"] + c["near_rtol"] * amp[use]) / amp[use] + 5e-14
                assert np.all(chord <= tol), (c["name"], comp, kind)
        seen += 1
    assert seen >= 12


def test_slice_and_phase_arguments(eng):
    h = np.ones((6, 3, 2), np.complex128)
    k = np.array([0.1, 0.2, 0.3])
    for bad in (dict(nt=0), dict(at=np.inf), dict(period=0.0), dict(plane=2)):
        args = dict(plane=abi.RCWA_SLICE_XZ, nt=4, period=1.0, at=0.0)
        args.update(bad)
        with pytest.raises(ValueError):
            eng.field_slice(h, k, 0.0, args["plane"], args["nt"], args["period"], args["at"])
    big = np.full((6, 3, 2), 1e308, np.complex128)
    from stablercwa_gb300.engine import EngineError
    with pytest.raises(EngineError):
        eng.field_slice(big, k, 0.0, abi.RCWA_SLICE_XZ, 4, 1.0, 0.0)
    f = np.zeros((2, 3), np.complex128)
    p = eng.phase_data(f)
    assert p["mask"].all() and np.isnan(p["phase"]).all()   # an all-zero field is masked everywhere
    with pytest.raises(ValueError):
        eng.phase_data(f, phase_floor=-1.0)
    with pytest.raises(ValueError):
        eng.phase_data(f, "incident", incident_k=[np.nan, 0, 0], x=[0, 1, 2], y=[0, 0, 0], z=[0, 1])
