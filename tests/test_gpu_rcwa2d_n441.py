"""2-D solve at the benchmark's full size (Mx = My = 10: N = 441 harmonics, an 882 x 882 eigenproblem
per patterned layer) against the reference's own rcwa::solve2d (include/stablercwa/rcwa2d.hpp:1359) on
six wavelengths of the seeded three-pillar, five-film structure: the first four and the two whose
energy defect is largest (the reference itself gives 1.1e-11 and 3.4e-12 there). Fixture:
tests/golden/rcwa2d_n441_cases.jsonl.gz, written by tests/golden/make_golden.py."""
import numpy as np
import pytest

from conftest import load_jsonl, rvec
from stablercwa_gb300.types import stack2d_from_json

pytestmark = pytest.mark.gpu

DE_TOL = 1e-10          # per-order efficiencies against the reference
ENERGY_MARGIN = 1e-12   # lossless stack: |R + T - 1| no worse than the reference's own plus this
# Where the reference's own defect exceeds the 1e-12 gate, the point is ill-conditioned for both codes:
# at normal incidence the symmetric pillars give exactly repeated mode eigenvalues, and the back
# substitution's coincident-eigenvalue floor (include/stablercwa/eig_qr.hpp:872-877) turns the rounding of
# the Schur form's off-diagonal entry of each pair into eigenvector pairs that are nearly parallel; the
# defect then scales with the condition of W and moves with every rounding difference (the eigensolver's
# partition of its sums, the product kernels). There the engine must stay within this factor of the reference.
ILL_CONDITIONED_FACTOR = 1.5


@pytest.fixture(scope="module")
def crossed():
    cases = load_jsonl("rcwa2d_n441_cases.jsonl.gz")
    assert len(cases) == 6 and all(c["M1"] == c["M2"] == 10 for c in cases)
    return cases


@pytest.fixture(scope="module")
def solved(crossed):
    from stablercwa_gb300.engine import Engine
    eng = Engine()
    try:
        stack = stack2d_from_json(crossed[0]["stack"])
        assert all(c["stack"] == crossed[0]["stack"] for c in crossed)  # one structure, six wavelengths: one batched call
        pts = [(c["wavelength"], c["theta"], c["phi"], complex(*c["jones"][0]), complex(*c["jones"][1])) for c in crossed]
        return eng.solve2d_arrays(stack, pts, 10, 10)
    finally:
        eng.close()


def test_n441_efficiencies_match_reference(crossed, solved):
    worst = 0.0
    for k, c in enumerate(crossed):
        ref = c["ref"]
        assert solved["status"][k] == ref["status"] == 0, c["name"]
        assert solved["eig_info"][k] == ref["eig_info"], c["name"]
        assert solved["n_eig"][k] == ref["n_eig"], c["name"]
        for key in ("DEr", "DEt"):
            d = float(np.max(np.abs(solved[key][k] - rvec(ref[key]))))
            assert d <= DE_TOL, (c["name"], key, d)
            worst = max(worst, d)
    print(f"N = 441 worst |dDE| vs reference {worst:.2e}")


def test_n441_energy_no_worse_than_reference(crossed, solved):
    rows = []
    for k, c in enumerate(crossed):
        ref = c["ref"]
        e_ref = abs(float(np.sum(rvec(ref["DEr"])) + np.sum(rvec(ref["DEt"]))) - 1.0)
        e_gpu = abs(float(np.sum(solved["DEr"][k]) + np.sum(solved["DEt"][k])) - 1.0)
        print(f"{c['name']} lambda={c['wavelength']:.4f}: |R+T-1| engine {e_gpu:.2e}, reference {e_ref:.2e}")
        rows.append((c["name"], e_gpu, e_ref))
    for name, e_gpu, e_ref in rows:
        if e_ref <= ENERGY_MARGIN:
            assert e_gpu <= e_ref + ENERGY_MARGIN, (name, e_gpu, e_ref)
        else:
            assert e_gpu <= ILL_CONDITIONED_FACTOR * e_ref, (name, e_gpu, e_ref)
