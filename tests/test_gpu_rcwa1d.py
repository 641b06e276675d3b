"""Batched 1-D TE/TM solve on the GPU through the C ABI, against the reference's own results
(tests/golden/rcwa1d_cases.jsonl, written by StableRCWA's rcwa::solve), its golden efficiency
tables, and the CPU oracle at the benchmark's shapes. Tolerance: per-order DEr/DEt within 1e-10
absolute; |R + T - 1| <= 1e-12 on lossless stacks."""
import numpy as np
import pytest

from conftest import cvec, rvec
from oracle import oracle
from stablercwa_gb300 import TE, TM, Layer, Options, Stack, stack_from_json

pytestmark = pytest.mark.gpu
POL = {"TE": TE, "TM": TM}


@pytest.fixture(scope="module")
def eng():
    from stablercwa_gb300.engine import Engine
    e = Engine()
    yield e
    e.close()


def test_golden_cases(eng, cases1d):
    worst = 0.0
    for case in cases1d:
        s = stack_from_json(case["stack"])
        r = eng.solve(s, case["wavelength"], case["theta"], case["M"], POL[case["pol"]])
        ref = case["ref"]
        err = max(np.max(np.abs(r.DEr - rvec(ref["DEr"]))), np.max(np.abs(r.DEt - rvec(ref["DEt"]))))
        assert err <= 1e-10, (case["name"], err)
        if "table" in case:
            terr = max(np.max(np.abs(r.DEr - rvec(case["table"]["der"]))),
                       np.max(np.abs(r.DEt - rvec(case["table"]["det"]))))
            assert terr <= 1e-9, (case["name"], terr)
        assert r.status == 0 and r.eig_info == ref["eig_info"], case["name"]
        assert r.n_eig == ref["n_eig"] and r.n_dense_solve == ref["n_dense_solve"], case["name"]
        worst = max(worst, err)
    print("worst |dDE| GPU vs reference:", worst)


def config1_stack():
    return Stack(nI=1.0, nII=1.46, period=0.574,
                 layers=[Layer.grating(0.38, [0.0, 0.172, 0.574], [1.46, 1.0]), Layer.uniform(0.115, 1.96)])


def test_config1_published_values(eng):
    # README.md:106-111: DE(0) R/T 0.026034 / 0.497012, DE(+1) 0.258135 / 0.218818, R+T = 1
    r = eng.solve(config1_stack(), 1.053, 66.36, 20, TE)
    M = 20
    assert abs(r.DEr[M] - 0.026034) < 5e-7 and abs(r.DEt[M] - 0.497012) < 5e-7
    assert abs(r.DEr[M + 1] - 0.258135) < 5e-7 and abs(r.DEt[M + 1] - 0.218818) < 5e-7
    assert abs(r.reflectance() + r.transmittance() - 1.0) <= 1e-12
    o = oracle.solve1d_batch(config1_stack(), [(1.053, 66.36)], 20, TE)
    assert np.max(np.abs(r.DEr - o["DEr"][0])) <= 1e-10 and np.max(np.abs(r.DEt - o["DEt"][0])) <= 1e-10


def mirror_stack(fill=0.4, depth=0.4):
    layers = [Layer.grating(depth, [0.0, fill * 0.574, 0.574], [1.46, 1.0])]
    for _ in range(10):
        layers.append(Layer.uniform(1.053 / (4 * 2.1), 2.1))
        layers.append(Layer.uniform(1.053 / (4 * 1.46), 1.46))
    return Stack(nI=1.0, nII=1.46, period=0.574, layers=layers)


@pytest.mark.parametrize("pol", [TE, TM])
def test_batched_mirror_sweep_vs_oracle(eng, pol):
    # the benchmark's structure at M = 60 (N = 121) on a seeded sample of sweep points
    rng = np.random.default_rng(11 + pol)
    pts = np.stack([rng.uniform(0.9, 1.2, 24), rng.uniform(50, 70, 24)], axis=1)
    s = mirror_stack(rng.uniform(0.3, 0.5), rng.uniform(0.3, 0.5))
    g = eng.solve1d_arrays(s, pts, 60, pol)
    o = oracle.solve1d_batch(s, pts, 60, pol, threads=8)
    assert (g["status"] == 0).all()
    err = max(np.max(np.abs(g["DEr"] - o["DEr"])), np.max(np.abs(g["DEt"] - o["DEt"])))
    assert err <= 1e-10, err
    # lossless stack: |R + T - 1| no worse than the reference's own defect on the same point (which
    # reaches 3.6e-12 here at N = 121), plus 1e-12
    energy = np.abs(g["DEr"].sum(1) + g["DEt"].sum(1) - 1.0)
    ref_energy = np.abs(o["DEr"].sum(1) + o["DEt"].sum(1) - 1.0)
    assert energy.max() <= 2.0 * ref_energy.max() + 1e-12, (energy.max(), ref_energy.max())


def test_failure_contract(eng):
    s = config1_stack()
    r = eng.solve(s, 1.053, 66.36, 20, TE, Options(eig_max_iter=1))
    assert r.status == 2 and r.eig_info > 0
    assert np.isnan(r.R).all() and np.isnan(r.DEr).all() and np.isnan(r.DEt).all()
    with pytest.raises(ValueError):
        eng.solve(s, 1.053, 90.0, 20, TE)
    with pytest.raises(ValueError):
        eng.solve(s, -1.0, 10.0, 20, TE)
    with pytest.raises(ValueError):
        eng.solve(Stack(nI=complex(1, 0.1), nII=1.46, period=0.574, layers=[]), 1.0, 10.0, 5, TE)


def test_pure_films_and_empty_stack(eng):
    s = Stack(nI=1.0, nII=1.45, period=0.8, layers=[Layer.uniform(0.62, 1.72)])
    r = eng.solve(s, 1.053, 41.0, 6, TM)
    o = oracle.solve1d_batch(s, [(1.053, 41.0)], 6, TM)
    assert np.max(np.abs(r.R - o["R"][0])) <= 1e-13
    bare = Stack(nI=1.0, nII=1.45, period=0.8, layers=[])
    r = eng.solve(bare, 1.053, 41.0, 4, TE)
    assert abs(r.reflectance() + r.transmittance() - 1) <= 1e-13
    r0 = eng.solve(s, 1.053, 41.0, 0, TE)
    assert r0.R.shape == (1,)


def test_device_resident_path_matches_host_path(eng):
    import torch
    s = mirror_stack()
    rng = np.random.default_rng(3)
    pts = np.stack([rng.uniform(0.9, 1.2, 64), rng.uniform(50, 70, 64)], axis=1)
    host = eng.solve1d_arrays(s, pts, 30, TE)
    dp = torch.tensor(pts, dtype=torch.float64, device="cuda")
    n = 61
    out = {"R": torch.empty((64, n, 2), dtype=torch.float64, device="cuda"),
           "T": torch.empty((64, n, 2), dtype=torch.float64, device="cuda"),
           "DEr": torch.empty((64, n), dtype=torch.float64, device="cuda"),
           "DEt": torch.empty((64, n), dtype=torch.float64, device="cuda"),
           "status": torch.empty(64, dtype=torch.int32, device="cuda")}
    eng.solve1d_device(s, dp.data_ptr(), 64, 30, TE, {k: v.data_ptr() for k, v in out.items()})
    eng.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    # the device entry point evaluates sin(theta) with the device libm (<= 2 ulp): same parity bar
    o = oracle.solve1d_batch(s, pts, 30, TE, threads=8)
    assert np.max(np.abs(out["DEr"].cpu().numpy() - o["DEr"])) <= 1e-10
    assert np.max(np.abs(out["DEt"].cpu().numpy() - o["DEt"])) <= 1e-10
    assert np.max(np.abs(out["DEr"].cpu().numpy() - host["DEr"])) <= 1e-11


def test_both_polarizations_in_one_call(eng, cases1d):
    """RCWA_TE_TM runs the TE and TM sweeps concurrently; each block equals its own single-polarization sweep."""
    from stablercwa_gb300 import abi
    c = next(c for c in cases1d if c["M"] >= 10)
    stack = stack_from_json(c["stack"])
    pts = [(c["wavelength"], c["theta"]), (c["wavelength"] * 1.07, c["theta"] * 0.5), (c["wavelength"] * 0.93, 3.0)]
    both = eng.solve1d_arrays(stack, pts, c["M"], abi.RCWA_TE_TM)
    for pol in (0, 1):
        one = eng.solve1d_arrays(stack, pts, c["M"], pol)
        for key in ("R", "T", "DEr", "DEt", "status", "n_dense_solve"):
            assert np.array_equal(both[key][pol * len(pts):(pol + 1) * len(pts)], one[key]), (pol, key)
