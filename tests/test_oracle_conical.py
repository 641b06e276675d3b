"""The CPU conical oracle against the reference's golden vectors (no GPU): the ten Jones tables of
tests/conical_reference.inc (|dJ| <= 1e-9 max(1, |J|), as tests/test_rcwa1d_conical.cpp:231-276
checks) and the reference's own solve_conical outputs, including the Schur-branch cases."""
import numpy as np

from conftest import de_from_ref, jones_from_ref, jones_from_table
from oracle import oracle
from stablercwa_gb300 import stack_from_json


def _solve(case):
    s = stack_from_json(case["stack"])
    return oracle.solve_conical_batch(s, [(case["wavelength"], case["theta"], case["phi"])], case["M"])


def test_conical_oracle_vs_reference(conical_cases):
    for case in conical_cases:
        out = _solve(case)
        ref = case["ref"]
        for key in ("Jr", "Jt"):
            want = jones_from_ref(ref[key])
            err = np.max(np.abs(out[key][0] - want) / np.maximum(1.0, np.abs(want)))
            assert err <= 1e-11, (case["name"], key, err)
        for key in ("DEr", "DEt"):
            assert np.max(np.abs(out[key][0] - de_from_ref(ref[key]))) <= 1e-11, (case["name"], key)
        assert out["n_eig"][0] == ref["n_eig"] and out["n_schur"][0] == ref["n_schur"], case["name"]
        assert out["n_dense_solve"][0] == ref["n_dense_solve"], case["name"]
        assert bool(out["degenerate_mode_warning"][0]) == ref["degenerate_mode_warning"], case["name"]


def test_conical_oracle_vs_tables(conical_cases):
    n = 0
    for case in conical_cases:
        if "table" not in case:
            continue
        n += 1
        out = _solve(case)
        for key, tkey in (("Jr", "jr"), ("Jt", "jt")):
            want = jones_from_table(case["table"][tkey])
            err = np.max(np.abs(out[key][0] - want) / np.maximum(1.0, np.abs(want)))
            assert err <= 1e-9, (case["name"], key, err)
    assert n == 10


def test_schur_cases_present(conical_cases):
    assert sum(1 for c in conical_cases if c["ref"]["n_schur"] > 0) >= 4
