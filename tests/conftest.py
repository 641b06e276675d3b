import gzip
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


def load_jsonl(name):
    opener = gzip.open if name.endswith(".gz") else open
    with opener(os.path.join(GOLDEN, name), "rt") as f:
        return [json.loads(line) for line in f if line.strip()]


def cvec(v):
    return np.array([complex(float(a), float(b)) for a, b in v], dtype=np.complex128)


def rvec(v):
    return np.array([float(x) for x in v], dtype=np.float64)


@pytest.fixture(scope="session")
def cases1d():
    return load_jsonl("rcwa1d_cases.jsonl")


@pytest.fixture(scope="session")
def eig_cases():
    return load_jsonl("eig_cases.jsonl")


@pytest.fixture(scope="session")
def conical_cases():
    return load_jsonl("conical_cases.jsonl")


@pytest.fixture(scope="session")
def cases2d():
    return load_jsonl("rcwa2d_cases.jsonl.gz")


def jones_from_table(rows):
    """(n, 4) complex from rows of 8 doubles: ss, sp, ps, pp as (re, im) pairs."""
    a = np.array(rows, dtype=np.float64).reshape(-1, 4, 2)
    return a[..., 0] + 1j * a[..., 1]


def jones_from_ref(rows):
    out = np.empty((len(rows), 4), np.complex128)
    for j, row in enumerate(rows):
        for k in range(4):
            out[j, k] = complex(float(row[k][0]), float(row[k][1]))
    return out


def de_from_ref(rows):
    return np.array([[float(v) for v in row] for row in rows], dtype=np.float64)
