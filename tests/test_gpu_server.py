"""The serving loop (rcwa_gpu_server_*): a mix of 1-D, conical and 2-D requests submitted together
gives, for every request, the result the same request gives alone through the direct entry points;
requests that differ only in the point share one batched call and match their lone results within the
parity tolerances; a budget too small for two requests runs them one at a time; wait() honours its
timeout."""
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
    srv = Server(slots=8, max_batch=1)  # each request in its own call: results bit for bit
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


def test_same_structure_requests_share_a_call(eng, cases1d, conical_cases, cases2d):
    """Requests of one structure queued together (1-D, conical and 2-D, each at several points) run as one
    batched call per structure (the response reports the batch size), and each result equals the request
    solved alone within 1e-10 on the efficiencies and 1e-9 (1 + |b|) on the amplitudes, with the same
    status; with max_batch = 1 every request runs alone."""
    from stablercwa_gb300.engine import Server
    c1, cc, cp = cases1d[0], conical_cases[0], _pillars(cases2d)
    s1, sc, s2 = stack_from_json(c1["stack"]), stack_from_json(cc["stack"]), stack2d_from_json(cp["stack"])
    jones = (complex(*cp["jones"][0]), complex(*cp["jones"][1]))
    pol = 0 if c1["pol"] == "TE" else 1
    reqs = [("1d", (c1["wavelength"] + 0.011 * k, c1["theta"] + 0.5 * k)) for k in range(10)]
    reqs += [("conical", (cc["wavelength"] + 0.009 * k, cc["theta"] + 0.4 * k, cc["phi"] + 1.0 * k)) for k in range(6)]
    reqs += [("2d", (cp["wavelength"] + 0.007 * k, cp["theta"], cp["phi"])) for k in range(4)]

    def go(srv, kind, p):
        if kind == "1d":
            return srv.submit_1d(s1, p[0], p[1], c1["M"], pol)
        if kind == "conical":
            return srv.submit_conical(sc, p[0], p[1], p[2], cc["M"])
        return srv.submit_2d(s2, p[0], p[1], p[2], cp["M1"], cp["M2"], jones)

    for max_batch in (0, 1):
        srv = Server(slots=1, max_batch=max_batch)
        try:
            # another structure (one order less) keeps the one slot busy while the rest queue
            first = srv.submit_2d(s2, cp["wavelength"], cp["theta"], cp["phi"], cp["M1"] - 1, cp["M2"] - 1, jones)
            tickets = [go(srv, kind, p) for kind, p in reqs]
            srv.wait(first)
            out = [srv.wait(t) for t in tickets]
        finally:
            srv.close()
        batches = {kind: max(info["batch"] for (k2, _), (info, _) in zip(reqs, out) if k2 == kind) for kind in KEYS}
        if max_batch == 1:
            assert all(b == 1 for b in batches.values()), batches
            continue
        assert batches == {"1d": 10, "conical": 6, "2d": 4}, batches
        for (kind, p), (info, r) in zip(reqs, out):
            assert info["code"] == 0
            if kind == "1d":
                r0 = {k: v[0] for k, v in eng.solve1d_arrays(s1, [p], c1["M"], pol).items()}
            elif kind == "conical":
                r0 = eng.solve_conical(sc, p[0], p[1], p[2], cc["M"])
            else:
                r0 = eng.solve2d(s2, p[0], p[1], p[2], cp["M1"], cp["M2"], jones)
            assert r["status"] == r0["status"], (kind, p)
            for key in KEYS[kind]:
                a, b = np.asarray(r[key]), np.asarray(r0[key])
                tol = 1e-10 if key.startswith("DE") else 1e-9
                assert np.max(np.abs(a - b) / (1.0 if key.startswith("DE") else 1.0 + np.abs(b))) <= tol, (kind, key)


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


def _pillars(cases2d):
    return next(c for c in cases2d if c["name"] == "pillars_films_m6")


def _submit_pillars(srv, c, dl=0.0):
    return srv.submit_2d(stack2d_from_json(c["stack"]), c["wavelength"] + dl, c["theta"], c["phi"], c["M1"], c["M2"],
                         (complex(*c["jones"][0]), complex(*c["jones"][1])))


def _footprints(cases1d, cases2d):
    """The admission charge of one large (2-D, N = 169) and one small (1-D) request."""
    from stablercwa_gb300.engine import Server
    srv = Server(slots=1)
    try:
        big = srv.wait(_submit_pillars(srv, _pillars(cases2d)))[0]["footprint_bytes"]
        c = cases1d[0]
        small = srv.wait(srv.submit_1d(stack_from_json(c["stack"]), c["wavelength"], c["theta"], c["M"]))[0]
    finally:
        srv.close()
    return big, small["footprint_bytes"]


def test_admission_budget_and_bypass(cases1d, cases2d):
    """A budget that holds one large request and a few small ones: the second large request waits for
    the first to finish, and small requests submitted behind it start inside the bypass window."""
    from stablercwa_gb300.engine import Server
    big, small = _footprints(cases1d, cases2d)
    assert big > 8 * small
    c1 = cases1d[0]
    stack1 = stack_from_json(c1["stack"])
    srv = Server(slots=4, hbm_budget=int(big + 4 * small), max_bypass_ms=60000)
    try:
        a = _submit_pillars(srv, _pillars(cases2d))
        b = _submit_pillars(srv, _pillars(cases2d), 0.01)
        smalls = [srv.submit_1d(stack1, c1["wavelength"] + 0.01 * k, c1["theta"], c1["M"]) for k in range(3)]
        ia, ib = srv.wait(a)[0], srv.wait(b)[0]
        iss = [srv.wait(t)[0] for t in smalls]
    finally:
        srv.close()
    assert ia["code"] == ib["code"] == 0 and all(i["code"] == 0 for i in iss)
    assert ib["start_s"] >= ia["finish_s"]            # never both large requests at once
    assert all(i["start_s"] < ib["start_s"] for i in iss)  # the small ones bypassed the waiting large one


def test_admission_no_bypass_after_window(cases1d, cases2d):
    """With a bypass window of 1 ms, small requests queued behind a waiting large one keep their order."""
    import time
    from stablercwa_gb300.engine import Server
    big, small = _footprints(cases1d, cases2d)
    c1 = cases1d[0]
    stack1 = stack_from_json(c1["stack"])
    srv = Server(slots=4, hbm_budget=int(big + 4 * small), max_bypass_ms=1)
    try:
        a = _submit_pillars(srv, _pillars(cases2d))
        b = _submit_pillars(srv, _pillars(cases2d), 0.01)
        time.sleep(0.02)  # b has waited longer than the bypass window
        smalls = [srv.submit_1d(stack1, c1["wavelength"] + 0.01 * k, c1["theta"], c1["M"]) for k in range(3)]
        ia, ib = srv.wait(a)[0], srv.wait(b)[0]
        iss = [srv.wait(t)[0] for t in smalls]
    finally:
        srv.close()
    if ib["submit_s"] + 0.001 >= ia["finish_s"]:
        pytest.skip("the first request finished before the window closed")
    assert all(i["start_s"] >= ib["start_s"] for i in iss)


def test_destroy_wakes_waiters(cases2d):
    """Destroying the server while a thread waits (without a timeout) on a queued request wakes that
    thread with RCWA_ECANCELLED (or the result, if the request got to run) instead of leaving it blocked."""
    import threading
    import time
    from stablercwa_gb300 import abi
    from stablercwa_gb300.engine import Server
    c = _pillars(cases2d)
    srv = Server(slots=1)
    tickets = [_submit_pillars(srv, c, 0.01 * k) for k in range(4)]
    got = {}

    def waiter():
        got["r"] = srv.wait(tickets[-1])

    th = threading.Thread(target=waiter)
    th.start()
    time.sleep(0.5)  # the waiter is inside rcwa_gpu_server_wait before destroy begins
    srv.close()
    th.join(timeout=120)
    assert not th.is_alive()
    info, _ = got["r"]
    assert info["code"] in (0, abi.RCWA_ECANCELLED)
