"""Regenerate the golden fixtures from the reference checkout.

The reference's regression suite (src/CMakeLists.txt:104-165,
cmake/run_mpi_test.cmake) runs two 2x21^3 rupture problems and compares six
float32 fault streams against `test_problems/truth/{1,2}` with
python/read_binary.py (max |diff| <= 1e-3).  This script copies the inputs and
those truth streams (plus trup, state, the two station seismograms and, for
the curvilinear case, the fault coordinates and unit vectors shipped beside
the truth) into compressed fixtures so the parity tests run without the
reference present.

Usage:  python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

import numpy as np

CASES = {
    "cart": ("test_rup_cart_fric", "1"),
    "curv": ("test_rup_curv_fric", "2"),
}
STREAMS = {"S": 4, "Svel": 3, "Uface": 9, "Vface": 9, "Uhat": 6, "Vhat": 6,
           "trup": 1, "state": 1}
NGRID, NTIME = 21, 46
GEOMETRY = {"fault_xyz": "fault_topography_AX",
            "fault_normal": "unit_normal_vector_fractal_fault",
            "fault_strike": "unit_strike_vector_fractal_fault",
            "fault_dip": "unit_dip_vector_fractal_fault"}


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    for tag, (prefix, d) in CASES.items():
        src_in = os.path.join(ref, "test_problems", prefix + ".in")
        with open(src_in) as f:
            text = f.read()
        with open(os.path.join(here, prefix + ".in"), "w") as f:
            f.write(text)
        arrays = {}
        for name, ncomp in STREAMS.items():
            path = os.path.join(ref, "test_problems", "truth", d,
                                f"{prefix}_interface.{name}")
            a = np.fromfile(path, dtype="<f4").reshape(NTIME, ncomp, NGRID, NGRID)
            arrays[name] = a
        for st in ("1_11_11", "21_11_11"):
            path = os.path.join(ref, "test_problems", "truth", d, f"{prefix}_{st}.dat")
            arrays["station_" + st] = np.loadtxt(path).astype(np.float64)
        # the fault geometry shipped with the curvilinear truth: x y z and the
        # unit normal, strike and dip vectors per fault point (rows r fastest)
        for key, suffix in GEOMETRY.items():
            path = os.path.join(ref, "test_problems", "truth", d, f"{prefix}_{suffix}.dat")
            if os.path.exists(path):
                arrays[key] = np.loadtxt(path).astype(np.float64)
        np.savez_compressed(os.path.join(here, f"truth_{tag}.npz"), **arrays)
        print(tag, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
