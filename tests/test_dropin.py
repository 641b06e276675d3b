"""The C++ drop-in (include/stablercwa_gb300.hpp) compiled against the StableRCWA headers and linked
with libstablercwa_gb300.so: the reference's own solve, solve_conical and solve2d and the drop-in's
must throw the same std::invalid_argument (same message) for every invalid input, checked on the host
before any device work; a valid solve without a CUDA device must throw std::runtime_error. Runs where
the reference's headers are present ($STABLERCWA_REFERENCE, else /root/reference)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("STABLERCWA_REFERENCE", "/root/reference")


def test_dropin_matches_reference_errors(tmp_path):
    inc = os.path.join(REFERENCE, "include")
    if not os.path.isdir(inc):
        pytest.skip("StableRCWA headers not present")
    from stablercwa_gb300.engine import load_library
    load_library()  # builds the library if needed
    lib_dir = os.path.join(ROOT, "stablercwa_gb300", "_build")
    exe = str(tmp_path / "dropin_check")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-pthread", "-I", inc, "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "dropin", "dropin_check.cpp"), "-L", lib_dir,
                           "-Wl,-rpath," + lib_dir, "-lstablercwa_gb300", "-o", exe])
    import torch
    args = ["device"] if torch.cuda.is_available() else []
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("PASS") >= 30
