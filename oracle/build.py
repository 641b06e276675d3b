"""Build the CPU oracle (TEST INFRASTRUCTURE ONLY).

  python oracle/build.py          -> oracle/_build/liboracle.so  (the restatement; builds anywhere)
  python oracle/build.py --ref    -> also oracle/_ref/ref_solve1d (the StableRCWA sources compiled in
                                     place, for cross-checks; needs the reference checkout)

Compiled with -ffp-contract=off so the oracle's arithmetic is the same on x86-64 and aarch64.
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = ["oracle_dense.hpp", "oracle_rcwa1d.hpp", "oracle_conical.hpp", "oracle_rcwa2d.hpp",
           "../include/stablercwa_gb300.h"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(os.path.join(HERE, d)) > t for d in deps)


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if force or _stale(LIB, SOURCES + HEADERS):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               *[os.path.join(HERE, s) for s in SOURCES], "-o", LIB + ".tmp"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def reference_root():
    """The StableRCWA checkout: $STABLERCWA_REFERENCE, else /root/reference."""
    return os.environ.get("STABLERCWA_REFERENCE", "/root/reference")


def build_reference(reference=None, force=False):
    """Compile the reference's own solve in place (ref_solve1d.cpp includes its headers)."""
    inc = os.path.join(reference or reference_root(), "include")
    if not os.path.isdir(inc):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    exe = os.path.join(REF_OUT, "ref_solve1d")
    if force or _stale(exe, ["ref_solve1d.cpp"]):
        cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", inc, os.path.join(HERE, "ref_solve1d.cpp"), "-o", exe]
        subprocess.check_call(cmd)
    return exe


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build_oracle(a.force))
    if a.ref:
        print(build_reference(force=a.force))
