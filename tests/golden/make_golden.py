"""Regenerate the golden fixtures in this directory from the StableRCWA sources.

Usage:  python tests/golden/make_golden.py [--reference <StableRCWA checkout>] [--only <exporter or fixture>]

The reference checkout defaults to $STABLERCWA_REFERENCE, else /root/reference.

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


def write_n441_cases(path):
    """The benchmark's seeded 2-D structure (Mx = My = 10, N = 441, 2N = 882) at six of its 256
    wavelengths: the first four and the two whose energy defect is largest, as text for the exporter."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import bench
    stack, pts, _ = bench.workload_crossed2d()
    wls = [p[0] for p in pts]
    picks = list(range(4))
    for target in (0.8462, 0.8656):
        k = min(range(len(wls)), key=lambda i: abs(wls[i] - target))
        if k not in picks:
            picks.append(k)
    def r(x):
        return repr(float(x))
    with open(path, "w") as f:
        for k in picks:
            wl, th, ph, es, ep = pts[k]
            f.write(f"case n441_point{k} {r(wl)} {r(th)} {r(ph)} {bench.CROSSED_M} {bench.CROSSED_M} "
                    f"{r(es.real)} {r(es.imag)} {r(ep.real)} {r(ep.imag)} 0\n")
            nii = complex(stack.nII)
            f.write(f"stack {r(float(stack.nI))} {r(nii.real)} {r(nii.imag)} {r(stack.Lx)} {r(stack.Ly)}\n")
            for L in stack.layers:
                if L.homogeneous:
                    n = complex(L.n)
                    f.write(f"uniform {r(float(L.d))} {r(n.real)} {r(n.imag)}\n")
                    continue
                f.write(f"patterned {r(float(L.d))} {len(L.y_edges) - 1} " + " ".join(r(float(y)) for y in L.y_edges) + "\n")
                for xp in L.x_profiles:
                    vals = " ".join(f"{r(complex(v).real)} {r(complex(v).imag)}" for v in xp.n_values)
                    f.write(f"profile {len(xp.n_values)} " + " ".join(r(float(x)) for x in xp.edges) + " " + vals + "\n")
            f.write("end\n")


# fixtures made by an exporter in a second mode: (source, output, writer of the exporter's input)
LISTED = [("export_rcwa2d.cpp", "rcwa2d_n441_cases.jsonl.gz", write_n441_cases)]


def gzip_into(plain, dest):
    """compressed without a timestamp, so the bytes depend on the content only"""
    with open(plain, "rb") as src, open(dest, "wb") as raw:
        with gzip.GzipFile(filename="", mode="wb", fileobj=raw, compresslevel=9, mtime=0) as gz:
            gz.write(src.read())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("STABLERCWA_REFERENCE", "/root/reference"))
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
            if plain != dest:
                gzip_into(plain, dest)
            opener = gzip.open if dest.endswith(".gz") else open
            with opener(dest, "rt") as f:
                print(f"  {out}: {sum(1 for _ in f)} cases")
        for src, out, writer in LISTED:
            if args.only and src != args.only and out != args.only:
                continue
            exe = os.path.join(tmp, src.replace(".cpp", ""))
            if not os.path.exists(exe):
                cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", inc, "-I", tests, os.path.join(HERE, src), "-o", exe]
                print(" ".join(cmd), flush=True)
                subprocess.check_call(cmd)
            listing = os.path.join(tmp, out + ".txt")
            writer(listing)
            plain = os.path.join(tmp, out[:-3])
            subprocess.check_call([exe, plain, "--cases", listing])
            dest = os.path.join(HERE, out)
            gzip_into(plain, dest)
            with gzip.open(dest, "rt") as f:
                print(f"  {out}: {sum(1 for _ in f)} cases")


if __name__ == "__main__":
    main()
