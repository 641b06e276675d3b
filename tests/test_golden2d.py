"""The 2-D golden fixture is consistent before any engine is compared with it (no GPU): the
reference's own rcwa::solve2d outputs written beside each frozen table agree with that table to the
reference's tolerance (tests/test_rcwa2d_reference.cpp:75-110), and the Rayleigh cases list the
regions and orders the frozen tables name."""
import numpy as np

from conftest import cvec, rvec


def test_fixture_covers_the_reference_cases(cases2d):
    names = [c["name"] for c in cases2d]
    assert sum(n.startswith("ref_") for n in names) == 24
    assert sum(n.startswith("core_") for n in names) == 17
    assert sum(c["source"] == "generated" for c in cases2d) >= 5
    assert sum(len(c["operators"]) for c in cases2d) >= 20


def test_reference_outputs_match_frozen_tables(cases2d):
    worst = 0.0
    for c in cases2d:
        if "table" not in c:
            continue
        t, r = c["table"], c["ref"]
        assert r["status"] == 0, c["name"]
        atol, rtol = t["atol"], t["rtol"]
        for key in ("Rs", "Rp", "Ts", "Tp"):
            a, b = cvec(r[key]), cvec(t[key])
            d = np.abs(a - b)
            assert np.all(d <= atol + rtol * np.abs(b)), (c["name"], key)
            worst = max(worst, float(d.max()))
        for key in ("DEr", "DEt"):
            a, b = rvec(r[key]), rvec(t[key])
            assert np.all(np.abs(a - b) <= atol + rtol * np.abs(b)), (c["name"], key)
    assert worst <= 1e-11


def test_rayleigh_cases_name_the_frozen_orders(cases2d):
    seen = 0
    for c in cases2d:
        if c.get("table_status") != 2:
            continue
        seen += 1
        assert c["ref"]["status"] == 2, c["name"]
        assert c["rayleigh"], c["name"]
        if "table_failure" in c:
            orders = sorted(tuple(o) for reg in c["rayleigh"] for o in reg["orders"])
            assert orders == sorted(tuple(o) for o in c["table_failure"]["orders"]), c["name"]
    assert seen == 5
