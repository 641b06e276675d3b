"""The serving loop (rcwa_gpu_server_*): a mix of 1-D, conical and 2-D requests submitted together
gives, for every request, the result the same request gives alone through the direct entry points;
a budget too small for two requests runs them one at a time; wait() honours its timeout."""
import numpy as np
import pytest

from stablercwa_gb300.types import stack2d_from_json, stack_from_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def mix(cases1d, conical_cases, cases2d):
    reqs = []
    for c in cases1d[:8]:
        reqs.append(("1d", stack_from_json(c["stack"]), c))
    for c in conical_cases[:4]:
        reqs.append(("conical", stack_from_json(c["stack"]), c))
    for c in cases2d:
        if c["source"] == "generated" and c["M1"] * c["M2"] <= 9:
            reqs.append(("2d", stack2d_from_json(c["stack"]), c))
    return reqs


def alone(eng, kind, stack, c):
    if kind == "1d":
        pol = 0 if c["pol"] == "TE" else 1
        r = eng.solve1d_arrays(stack, [(c["wavelength"], c["theta"])], c["M"], pol)
        return {k: v[0] for k, v in r.items()}
    if kind == "conical":
        return eng.solve_conical(stack, c["wavelength"], c["theta"], c["phi"], c["M"])
    jones = (complex(*c["jones"][0]), complex(*c["jones"][1]))
    return eng.solve2d(stack, c["wavelength"], c["theta"], c["phi"], c["M1"], c["M2"], jones, laurent=bool(c["laurent"]))


def submit(srv, kind, stack, c):
    if kind == "1d":
        return srv.submit_1d(stack, c["wavelength"], c["theta"], c["M"], 0 if c["pol"] == "TE" else 1)
    if kind == "conical":
        return srv.submit_conical(stack, c["wavelength"], c["theta"], c["phi"], c["M"])
    jones = (complex(*c["jones"][0]), complex(*c["jones"][1]))
    return srv.submit_2d(stack, c["wavelength"], c["theta"], c["phi"], c["M1"], c["M2"], jones, laurent=bool(c["laurent"]))


KEYS = {"1d": ("R", "T", "DEr", "DEt"), "conical": ("Jr", "Jt", "DEr", "DEt"),
        "2d": ("Rs", "Rp", "Ts", "Tp", "DEr", "DEt")}


def test_mix_equals_alone(eng, cases1d, conical_cases, cases2d):
    from stablercwa_gb300.engine import Server
    reqs = mix(cases1d, conical_cases, cases2d)
    assert len({k for k, _, _ in reqs}) == 3
    ref = [alone(eng, k, s, c) for k, s, c in reqs]
    srv = Server(slots=8)
    try:
        tickets = [submit(srv, k, s, c) for k, s, c in reqs]
        out = [srv.wait(t) for t in tickets]
    finally:
        srv.close()
    slots = set()
    for (kind, _, c), r0, (info, r) in zip(reqs, ref, out):
        assert info["code"] == 0, c["name"]
        assert r["status"] == r0["status"], c["name"]
        for key in KEYS[kind]:
            assert np.array_equal(np.asarray(r[key]), np.asarray(r0[key])), (kind, c["name"], key)
        assert info["submit_s"] <= info["start_s"] <= info["finish_s"]
        slots.add(info["slot"])
    assert len(slots) > 1  # the requests really ran on several slots


def test_small_budget_serialises(cases1d):
    from stablercwa_gb300.engine import Server
    srv = Server(slots=4, hbm_budget=1)
    try:
        c = cases1d[0]
        stack = stack_from_json(c["stack"])
        tickets = [srv.submit_1d(stack, c["wavelength"] + 0.01 * k, c["theta"], c["M"]) for k in range(6)]
        infos = [srv.wait(t)[0] for t in tickets]
    finally:
        srv.close()
    spans = sorted((i["start_s"], i["finish_s"]) for i in infos)
    for (s0, f0), (s1, f1) in zip(spans, spans[1:]):
        assert s1 >= f0  # never two at once: each request alone exceeds the budget
    assert all(i["code"] == 0 for i in infos)


def test_wait_timeout(cases2d):
    from stablercwa_gb300.engine import Server
    c = next(c for c in cases2d if c["name"] == "pillars_films_m6")
    srv = Server(slots=2)
    try:
        t = srv.submit_2d(stack2d_from_json(c["stack"]), c["wavelength"], c["theta"], c["phi"], c["M1"], c["M2"],
                          (complex(*c["jones"][0]), complex(*c["jones"][1])))
        assert srv.wait(t, timeout_ms=0) is None
        info, r = srv.wait(t)
        assert info["code"] == 0 and r["status"] == 0
        assert np.max(np.abs(r["DEr"] - np.array([float(x) for x in c["ref"]["DEr"]]))) <= 1e-10
    finally:
        srv.close()
