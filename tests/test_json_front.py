"""The JSON request front end (rcwa_json_validate, no GPU): every invalid request of the fixture gets the
reference's own reply, byte for byte ({"ok": false, "error", "where"}, rcwa_json.hpp:214-800 and :1254-1270),
and every valid one passes (tests/golden/export_json.cpp)."""
import json

import pytest

from conftest import load_jsonl

pytestmark = pytest.mark.filterwarnings("ignore")


@pytest.fixture(scope="module")
def cases():
    return load_jsonl("json_cases.jsonl.gz")


def test_invalid_requests_get_the_reference_reply(cases):
    from stablercwa_gb300.engine import json_validate
    seen = 0
    for c in cases:
        ref = json.loads(c["reply"])
        ok, reply = json_validate(c["request"], c["indent"])
        if ref["ok"]:
            assert ok and reply == "", c["name"]
            continue
        seen += 1
        assert not ok, c["name"]
        assert reply == c["reply"], (c["name"], reply, c["reply"])
    assert seen >= 70


def test_unimplemented_options_are_request_errors():
    from stablercwa_gb300.engine import json_validate
    base = ('{"mode": "planar", "stack": {"nI": 1.0, "nII": 1.5, "period": 1.0, "layers": []}, "M": 2, '
            '"polarization": "TE", "wavelength": 1.0, "theta_deg": 0.0, "options": %s}')
    for opt, where in (('{"eig": "lr"}', "options.eig"), ('{"linear": "qr"}', "options.linear"),
                       ('{"linear": "lu_nopivot"}', "options.linear"),
                       ('{"homogeneous_fast_path": false}', "options.homogeneous_fast_path")):
        ok, reply = json_validate(base % opt)
        r = json.loads(reply)
        assert not ok and r["where"] == where and "GPU" in r["error"]


def test_parser_edge_cases():
    from stablercwa_gb300.engine import json_validate
    for text, frag in (("", "unexpected end of input"), ('{"a": [1, 2,]}', "unexpected character ']'"),
                       ('{"a": "\\ud800"}', "unpaired surrogate"), ('{"a": tru}', "invalid literal"),
                       ('{"a": 1} x', "after the JSON value"), ('{"a": "\x01"}', "control character"),
                       ("[" * 200 + "]" * 200, "nested too deeply"), ('{"a": 1.}', "decimal point")):
        ok, reply = json_validate(text)
        r = json.loads(reply)
        assert not ok and r["where"] == "" and frag in r["error"], (text[:20], r)
    ok, reply = json_validate('﻿{"mode": 3}')   # a leading BOM is skipped
    assert json.loads(reply)["where"] == "mode"


def test_fields_protocol_request_errors():
    """The near-field protocol's request checks (rcwa_fields_json.hpp:68-151) give the reference's reply."""
    from stablercwa_gb300.engine import fields_json_validate
    seen = 0
    for c in load_jsonl("fields_json_cases.jsonl.gz"):
        ref = json.loads(c["reply"])
        ok, reply = fields_json_validate(c["request"].replace("OUTPUT_DIR", "/tmp/never_created_here/out"))
        if ref["ok"] or ref["where"] == "fields":   # solved, or failing only when run
            assert ok and reply == "", c["name"]
            continue
        seen += 1
        assert not ok and reply == c["reply"], (c["name"], reply)
    assert seen >= 8
