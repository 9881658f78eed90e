"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/wql_ref.cpp -- the FP64 CPU restatement of the reference's
time step -- and oracle/ref_input.cpp, its own reader of the `.in` files,
into oracle/_build/libwqlref.so (the library's header wql_input.h supplies
only the layout of the parsed record).  FMA contraction is disabled so the restatement
rounds like the reference's x86-64 gfortran build (no FMA at -O5 without
-march).  OpenMP parallelises the stencil loops for the timed CPU baseline;
each grid point is independent, so results do not depend on the thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "libwqlref.so")
SRCS = [os.path.join(HERE, "wql_ref.cpp"), os.path.join(HERE, "ref_input.cpp")]


def build(force=False, verbose=False):
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(s) for s in SRCS + [os.path.join(
            ROOT, "waveqlab3d-gh_gb300", "csrc", "host", "wql_input.h"), os.path.join(HERE, "upwind_tables.inc")])
        if os.path.getmtime(OUT) >= newest:
            return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-I" + os.path.join(ROOT, "waveqlab3d-gh_gb300", "csrc", "host"),
           *SRCS, "-o", OUT + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
