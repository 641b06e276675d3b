"""The CPU oracle against the reference's golden vectors (no GPU).

Pins the restatement in oracle/ to StableRCWA itself: the per-order efficiency tables its tests
hold (tests/test_rcwa1d.cpp:92-325, :1336-1593, tolerance 1e-9 as there) and the reference's own
solve outputs written by tests/golden/export_rcwa1d.cpp (tolerance 1e-12: same algorithm, same
operation order, only libm / contraction differences remain).
"""
import numpy as np
import pytest

from conftest import cvec, rvec
from oracle import oracle
from stablercwa_gb300 import stack_from_json

POL = {"TE": 0, "TM": 1}


def _solve(case):
    s = stack_from_json(case["stack"])
    return oracle.solve1d_batch(s, [(case["wavelength"], case["theta"])], case["M"], POL[case["pol"]])


def test_oracle_matches_reference_solve(cases1d):
    worst = 0.0
    for case in cases1d:
        out = _solve(case)
        ref = case["ref"]
        for key in ("DEr", "DEt"):
            err = np.max(np.abs(out[key][0] - rvec(ref[key])))
            assert err <= 1e-12, (case["name"], key, err)
            worst = max(worst, err)
        for key in ("R", "T"):
            err = np.max(np.abs(out[key][0] - cvec(ref[key])))
            assert err <= 1e-11, (case["name"], key, err)
        assert out["n_eig"][0] == ref["n_eig"], case["name"]
        assert out["n_dense_solve"][0] == ref["n_dense_solve"], case["name"]
        assert out["eig_info"][0] == ref["eig_info"], case["name"]
    print("worst |dDE| oracle vs reference solve:", worst)


def test_oracle_matches_reference_tables(cases1d):
    n_tables = 0
    for case in cases1d:
        if "table" not in case:
            continue
        n_tables += 1
        out = _solve(case)
        err = max(np.max(np.abs(out["DEr"][0] - rvec(case["table"]["der"]))),
                  np.max(np.abs(out["DEt"][0] - rvec(case["table"]["det"]))))
        assert err <= 1e-9, (case["name"], err)
    assert n_tables == 23


def test_cutoff_film_closed_form(cases1d):
    # R = 1/2 (TE), 1/17 (TM): tests/test_rcwa1d.cpp:1868-1883
    for case in cases1d:
        if not case["name"].startswith("cutoff_"):
            continue
        out = _solve(case)
        expected = 0.5 if case["pol"] == "TE" else 1.0 / 17.0
        assert abs(out["DEr"][0].sum() - expected) <= 2e-15
        assert abs(out["DEt"][0].sum() - (1 - expected)) <= 2e-15


def test_oracle_eig_matches_reference(eig_cases):
    for case in eig_cases:
        n = case["n"]
        a = cvec(case["a"]).reshape((n, n), order="F")
        w, v, info, sweeps = oracle.eig(a, max_iter=case["max_iter"])
        assert info == case["info"], case["name"]
        if info == 0:
            ref = cvec(case["values"])
            scale = max(1.0, np.max(np.abs(ref)))
            # same algorithm and order: values match position by position
            assert np.max(np.abs(w - ref)) <= 1e-12 * scale, case["name"]
            assert sweeps == case["sweeps"], case["name"]
            assert oracle.eig_residual(a, w, v) <= 1e-13, case["name"]
        else:
            ref = cvec(case["values"])
            assert np.array_equal(w[info:], ref[info:]) or np.max(np.abs(w[info:] - ref[info:])) <= 1e-12


def test_invalid_arguments_raise():
    from stablercwa_gb300 import Layer, Stack
    s = Stack(nI=1.0, nII=1.46, period=0.574, layers=[Layer.grating(0.38, [0, 0.172, 0.574], [1.46, 1.0])])
    with pytest.raises(oracle.OracleInvalidArgument):
        oracle.solve1d_batch(s, [(1.053, 95.0)], 5, 0)       # |theta| >= 90
    bad = Stack(nI=1.0, nII=1.46, period=0.574, layers=[Layer.grating(0.38, [0, 0.172, 0.5], [1.46, 1.0])])
    with pytest.raises(oracle.OracleInvalidArgument):
        oracle.solve1d_batch(bad, [(1.053, 10.0)], 5, 0)     # edges do not span one period
