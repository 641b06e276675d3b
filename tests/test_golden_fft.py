"""FFT-sampled Fourier coefficients, on the CPU (no GPU): the reference's rcwa::fourier_coefficients_fft
outputs in the fixture (tests/test_fft.cpp:36-70 profiles and larger sample counts) equal the sampled
DFT written as a sum of Dirichlet kernels over the runs of equal samples -- the closed form the device
kernel evaluates -- and, on small counts, a direct O(N hmax) quadrature like the reference test's own."""
import numpy as np

from conftest import cvec, load_jsonl


def runs(edges, S, period):
    u = (np.arange(S) + 0.5) / S * period
    seg = np.zeros(S, dtype=np.int64)
    for s in range(1, len(edges) - 1):
        seg[u >= edges[s] - edges[0]] = s
    return seg


def dirichlet(edges, values, period, hmax, S):
    seg = runs(edges, S, period)
    starts = [int(np.searchsorted(seg, s, side="left")) for s in range(len(values))] + [S]
    origin = np.fmod(edges[0], period)
    if origin < 0:
        origin += period
    offset = origin / period + 0.5 / S
    out = np.zeros(2 * hmax + 1, complex)
    for h in range(-hmax, hmax + 1):
        acc = 0j
        for s, v in enumerate(values):
            a, m = starts[s], starts[s + 1] - starts[s]
            if m <= 0:
                continue
            if h == 0:
                d = m
            else:
                r1 = (h * (2 * a + m - 1)) % (2 * S)
                r2 = (h * m) % (2 * S)
                d = np.exp(-1j * np.pi * r1 / S) * np.sin(np.pi * r2 / S) / np.sin(np.pi * h / S)
            acc += v * d
        out[h + hmax] = acc / S * np.exp(-2j * np.pi * h * offset)
    return out


def direct(edges, values, period, hmax, S):
    seg = runs(edges, S, period)
    u = (np.arange(S) + 0.5) / S * period
    h = np.arange(-hmax, hmax + 1)[:, None]
    return (np.asarray(values)[seg][None, :] * np.exp(-2j * np.pi * h * (edges[0] + u[None, :]) / period)).sum(1) / S


def test_closed_form_matches_reference_fft():
    cases = [c for c in load_jsonl("fft_cases.jsonl") if c["kind"] == "coeff"]
    assert len(cases) >= 25
    for c in cases:
        vals = cvec(c["values"])
        ref = cvec(c["fft"])
        got = dirichlet(c["edges"], vals, c["period"], c["hmax"], c["samples"])
        tol = 3e-12 * max(1.0, np.max(np.abs(vals)))
        assert np.max(np.abs(got - ref)) <= tol, c["name"]
        if c["samples"] <= 8192:
            assert np.max(np.abs(direct(c["edges"], vals, c["period"], c["hmax"], c["samples"]) - ref)) <= tol, c["name"]
