"""Regenerate the golden fixtures in this directory from the StableRCWA sources.

Usage:  python tests/golden/make_golden.py [--reference /root/reference]

Each exporter (export_*.cpp) compiles one of the reference's own test programs in place (its
main() renamed) together with the reference headers, then writes the test structures, the golden
tables the reference's tests hold, and the reference's own computed results as JSON lines. Needs
g++ and the reference checkout; the fixtures it writes are committed, so the tests themselves never
need the reference.
"""
import argparse
import gzip
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

EXPORTERS = [
    # (source, output, reference test directory it includes from)
    ("export_rcwa1d.cpp", "rcwa1d_cases.jsonl"),
    ("export_eig.cpp", "eig_cases.jsonl"),
    ("export_conical.cpp", "conical_cases.jsonl"),
    ("export_rcwa2d.cpp", "rcwa2d_cases.jsonl.gz"),
    ("export_fft.cpp", "fft_cases.jsonl"),
    ("export_fields.cpp", "fields1d_cases.jsonl.gz"),
    ("export_fields2d.cpp", "fields2d_cases.jsonl.gz"),
    ("export_phase.cpp", "phase_cases.jsonl.gz"),
    ("export_json.cpp", "json_cases.jsonl.gz"),
    ("export_fields_json.cpp", "fields_json_cases.jsonl.gz"),
]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", default=None, help="build only this exporter source")
    args = ap.parse_args()
    inc = os.path.join(args.reference, "include")
    tests = os.path.join(args.reference, "tests")
    if not os.path.isdir(inc):
        sys.exit(f"reference headers not found under {inc}")
    with tempfile.TemporaryDirectory() as tmp:
        for src, out in EXPORTERS:
            if args.only and src != args.only:
                continue
            exe = os.path.join(tmp, src.replace(".cpp", ""))
            cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", inc, "-I", tests,
                   os.path.join(HERE, src), "-o", exe]
            print(" ".join(cmd), flush=True)
            subprocess.check_call(cmd)
            dest = os.path.join(HERE, out)
            plain = os.path.join(tmp, out[:-3]) if out.endswith(".gz") else dest
            subprocess.check_call([exe, plain])
            if plain != dest:  # compressed without a timestamp, so the bytes depend on the content only
                with open(plain, "rb") as src, open(dest, "wb") as raw:
                    with gzip.GzipFile(filename="", mode="wb", fileobj=raw, compresslevel=9, mtime=0) as gz:
                        gz.write(src.read())
            opener = gzip.open if dest.endswith(".gz") else open
            with opener(dest, "rt") as f:
                print(f"  {out}: {sum(1 for _ in f)} cases")


if __name__ == "__main__":
    main()
