"""The JSON front end on the GPU (rcwa_gpu_solve_json on a context, rcwa_gpu_server_solve_json on the serving
loop) against the reference's own replies to the same requests (rcwa::solve_json_reply,
include/stablercwa/rcwa_json.hpp; tests/golden/export_json.cpp): the same text with every number masked
(field order, nulls, indentation), the same integers and strings, and the numbers within the parity bounds."""
import json
import re

import numpy as np
import pytest

from conftest import load_jsonl

pytestmark = pytest.mark.gpu

NUMBER = re.compile(r"-?\d+(\.\d+)?([eE][+-]?\d+)?")


@pytest.fixture(scope="module")
def cases():
    return [c for c in load_jsonl("json_cases.jsonl.gz") if json.loads(c["reply"])["ok"]]


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def masked(text):
    return NUMBER.sub("#", text)


# per-key bounds: efficiencies within the parity bound 1e-10; amplitudes 1e-9; kinematics to rounding
EFF = {"DEr", "DEt", "R_total", "T_total", "DEr_channels", "DEt_channels", "DEr_s", "DEr_p", "DEt_s", "DEt_p"}
AMP = {"R", "T", "Jr", "Jt", "Rs", "Rp", "Ts", "Tp", "Ex_r", "Ey_r", "Ez_r", "Ex_t", "Ey_t", "Ez_t", "flux_unitarity",
       "jones_in"}
KIN = {"kx", "ky", "phi_m_deg", "kzI", "kzII", "flux_r", "flux_t", "Kx", "Ky", "wavelength", "theta_deg", "phi_deg"}
SKIP = {"timing", "max_eig_residual", "max_solve_backward_error", "min_abs_lambda"}


def compare(got, want, key, where):
    if isinstance(want, dict):
        assert list(got.keys()) == list(want.keys()), where
        for k in want:
            if k in SKIP:
                continue
            compare(got[k], want[k], k, f"{where}.{k}")
    elif isinstance(want, list):
        assert isinstance(got, list) and len(got) == len(want), where
        for i, (g, w) in enumerate(zip(got, want)):
            compare(g, w, key, f"{where}[{i}]")
    elif want is None or isinstance(want, (bool, str)) or (isinstance(want, int) and key not in EFF | AMP | KIN):
        assert got == want, (where, got, want)
    else:
        tol = 1e-10 if key in EFF else 1e-9 if key in AMP else 1e-12 * max(1.0, abs(want))
        assert got is not None and abs(got - want) <= tol, (where, got, want)


def check_reply(c, ok, text):
    want = json.loads(c["reply"])
    assert ok, (c["name"], text[:300])
    got = json.loads(text)
    compare(got, want, "", c["name"])
    # the text itself: the same field order, nulls and layout (numbers masked)
    assert masked(text) == masked(c["reply"]), c["name"]


def test_replies_on_a_context(eng, cases):
    for c in cases:
        ok, text = eng.solve_json(c["request"], c["indent"])
        check_reply(c, ok, text)
    assert len(cases) >= 16


def test_replies_on_the_serving_loop(cases):
    from stablercwa_gb300.engine import Server
    srv = Server(slots=8)
    try:
        for c in cases:
            ok, text = srv.solve_json(c["request"], c["indent"])
            check_reply(c, ok, text)
    finally:
        srv.close()


def test_numbers_round_trip(eng, cases):
    """Every number in a reply reads back to the engine's double: the C-ABI result of the same solve."""
    from stablercwa_gb300.types import stack_from_json
    c = next(c for c in cases if c["name"] == "planar_readme_tm_sweep")
    ok, text = eng.solve_json(c["request"])
    reply = json.loads(text)
    rq = json.loads(c["request"])
    stack = stack_from_json({"nI": [1.0, 0.0], "nII": [1.46, 0.0], "period": 0.574,
                             "layers": [{"d": 0.38, "edges": [0.0, 0.1722, 0.574], "n_values": [[1.46, 0.0], [1.0, 0.0]]},
                                        {"d": 0.115, "n": [1.96, 0.0]}]})
    pts = [(p["wavelength"], p["theta_deg"]) for p in rq["points"]]
    direct = eng.solve1d_arrays(stack, pts, rq["M"], 1)
    for p, item in enumerate(reply["results"]):
        assert np.array_equal(np.array(item["DEr"]), direct["DEr"][p])
        assert np.array_equal(np.array([complex(*z) for z in item["R"]]), direct["R"][p])


def chord(a, b):
    return np.abs(np.exp(1j * a) - np.exp(1j * b))


def test_fields_protocol(eng, tmp_path):
    """rcwa_gpu_solve_fields_json against rcwa::solve_fields_json_reply (tests/golden/export_fields_json.cpp):
    the reply text (numbers masked), and the published arrays: fields within 1e-10 (1 + |b|), masks equal,
    phases within 1e-9 on the unit circle, coordinates to rounding. Failures publish nothing."""
    import os
    seen = 0
    for k, c in enumerate(load_jsonl("fields_json_cases.jsonl.gz")):
        out = tmp_path / f"case{k}"
        if c["pre_create"]:
            out.mkdir()
        ok, text = eng.solve_fields_json(c["request"].replace("OUTPUT_DIR", str(out)))
        text = text.replace(str(out), "OUTPUT_DIR")
        assert ok == bool(c["ok"]), (c["name"], text[:300])
        if not ok:
            assert text == c["reply"], (c["name"], text)
            if not c["pre_create"]:
                assert not out.exists()
            continue
        seen += 1
        want, got = json.loads(c["reply"]), json.loads(text)
        assert masked(text) == masked(c["reply"]), c["name"]
        compare(got["results"], want["results"], "", c["name"])
        meta_w, meta_g = want["field_data"], got["field_data"]
        assert meta_g["layers"] == meta_w["layers"] and meta_g["files"] == meta_w["files"], c["name"]
        assert sorted(os.listdir(out)) == sorted(v["name"] for v in meta_w["files"].values())
        f = np.load(out / "fields.npy")
        fw = np.array([complex(*v) for v in c["fields"]]).reshape(f.shape)
        assert np.max(np.abs(f - fw) / (1.0 + np.abs(fw))) <= 1e-10, c["name"]
        m = np.load(out / "phase_mask.npy").astype(bool).ravel()
        mw = np.frombuffer(c["phase_mask"].encode(), np.uint8) == ord("1")
        assert np.array_equal(m, mw), c["name"]
        ph = np.load(out / "phase.npy").ravel()
        pw = np.array([float(v) for v in c["phase"]])
        assert np.all(np.isnan(ph[m])) and np.max(chord(ph[~m], pw[~m])) <= 1e-9, c["name"]
        for key in ("x", "z", "t", "y"):
            if key in c:
                assert np.allclose(np.load(out / f"{key}.npy"), [float(v) for v in c[key]], rtol=0, atol=1e-15)
    assert seen == 6
