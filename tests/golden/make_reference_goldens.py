"""Imports the reference's own known-answer fixtures into a compact .npz.

The reference tests (tests/tests.cpp:64-422 of fcaballerop/cuPSS) compare
16 / 16^2 / 16^3 results against CSV files in tests/base_truths/ written with
6 decimals: the droplet initial condition (phi_1d, phi_2d, phi_3d) and the
one-step spectral operators lap, iqx, iqy, iqz and 1/q in 1D and 3D, from both
the reference CPU (FFTW) and GPU (cuFFT) paths.  This script reads those CSV
files from a checkout of the reference and stores the value column, in the
reference index order (k*sx*sy + j*sx + i), as float64 arrays.

Usage:  python tests/golden/make_reference_goldens.py /path/to/cuPSS
"""
import os
import sys

import numpy as np


def load(path, dims):
    vals = []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line:
                continue
            parts = [p.strip() for p in line.split(",")]
            vals.append(float(parts[dims]))
    return np.asarray(vals, np.float64)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_reference_goldens.py <path of a cuPSS checkout>")
    root = sys.argv[1]
    bt = os.path.join(root, "tests", "base_truths")
    out = {}
    for name in sorted(os.listdir(bt)):
        dims = 3 if name.endswith("3d") else (2 if name.endswith("2d") else 1)
        out[name] = load(os.path.join(bt, name), dims)
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "reference_base_truths.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
