"""Time the reference's own 1-D solve against the oracle port on the same host (TEST INFRASTRUCTURE ONLY).

  python oracle/time_ref.py [--points 128] [--threads 8]

Builds oracle/_ref/ref_solve1d from the StableRCWA sources in place (oracle/build.py; needs the
reference checkout, $STABLERCWA_REFERENCE or /root/reference), then solves the same sample of the
benchmark's headline sweep points (TE and TM) with both on the same number of host threads and prints one JSON line:
each one's solves/s and the largest per-order efficiency difference between them. The benchmark host has
no reference sources, so its CPU baseline is the port; this records how the two compare where both exist.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository root, not this folder (whose oracle.py would shadow the package)

import bench  # noqa: E402  (the workload definition)
from oracle import build, oracle  # noqa: E402


def case_text(stack, pts, M, pol, threads):
    rows = [f"{M} {pol} {threads} {len(pts)} {stack.nI.real!r} {complex(stack.nII).real!r} {complex(stack.nII).imag!r} "
            f"{float(stack.period)!r} {len(stack.layers)}"]
    for L in stack.layers:
        if L.homogeneous:
            n = complex(L.n)
            rows.append(f"{float(L.d)!r} 1 {n.real!r} {n.imag!r}")
        else:
            vals = [complex(v) for v in L.n_values]
            rows.append(f"{float(L.d)!r} 0 {len(vals)} " + " ".join(repr(float(e)) for e in L.edges) + " " +
                        " ".join(f"{v.real!r} {v.imag!r}" for v in vals))
    rows += [f"{float(w)!r} {float(t)!r}" for w, t in pts]
    return "\n".join(rows) + "\n"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=128)
    ap.add_argument("--threads", type=int, default=min(8, os.cpu_count() or 1))
    a = ap.parse_args()
    exe = build.build_reference()
    if exe is None:
        print(json.dumps({"unavailable": "no StableRCWA checkout to build the reference from"}))
        return 0
    build.build_oracle()
    stack, pts, _ = bench.workload()
    sample = bench.cpu_sample_points(pts, a.points)
    M = bench.M
    n = 2 * M + 1
    out = {"points": len(sample), "threads": a.threads, "M": M}
    worst = 0.0
    for name, pol in (("TE", 0), ("TM", 1)):
        t0 = time.perf_counter()
        port = oracle.solve1d_batch(stack, sample, M, pol, threads=a.threads)
        t_port = time.perf_counter() - t0
        text = case_text(stack, sample, M, pol, a.threads)
        t0 = time.perf_counter()
        r = subprocess.run([exe], input=text, capture_output=True, text=True, check=True)
        t_ref = time.perf_counter() - t0
        ref = np.array([[float(x) for x in line.split()] for line in r.stdout.strip().splitlines()])
        worst = max(worst, float(np.max(np.abs(ref[:, :n] - port["DEr"]))), float(np.max(np.abs(ref[:, n:] - port["DEt"]))))
        out[name] = {"reference_solves_per_s": len(sample) / t_ref, "port_solves_per_s": len(sample) / t_port}
    out["max_abs_dDE_reference_vs_port"] = worst
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
