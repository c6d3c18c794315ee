"""Builds tests/golden/ fixtures from the reference's own recorded run.

The reference repository ships the outputs of one complete run of its CPU
path (4x4 subdomains on [-5,5]^2, 8 knots per interface, N=5000 paths per knot,
h0=0.005, fac = 1.5 1.27 1.2 1.13, Monegros Poisson problem of
BVPs/EDPs/Monegros_Poisson_CPP.hpp, driver main_EXTENDED.cpp):
  Output/Debug/cond.txt   RBF matrix condition numbers per stencil side
  Output/Debug/G.csv, G_var.csv, B.csv, B_var.csv   the estimated system
  Output/solution.csv     interface solution vs analytic
  Output/Debug/times.txt  the phase trace (only its header line is kept)
This script copies those numbers into compact fixtures.  It reads the
reference checkout and is run by hand in a container that has it; the
fixtures it writes are committed so the tests never need the reference.

usage: python tests/golden/make_fixtures.py /path/to/reference
"""
import csv
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    out = os.path.join(HERE, "ref_run_4x4_n8_monegros.npz")
    rows = []
    with open(os.path.join(ref, "Output/Debug/cond.txt")) as f:
        for line in f:
            p = line.strip().split(",")
            if len(p) == 4 and p[0] in ("north", "south", "east", "west"):
                rows.append(("nsew".index(p[0][0]), int(p[1]), float(p[2]), int(p[3])))
    cond = np.array(rows, dtype=np.float64)

    def read(name, cols):
        with open(os.path.join(ref, "Output/Debug", name)) as f:
            r = list(csv.reader(f))[1:]
        return np.array([[float(x) for x in row[:cols]] for row in r])

    G = read("G.csv", 3)
    Gv = read("G_var.csv", 3)
    B = read("B.csv", 3)
    Bv = read("B_var.csv", 3)
    with open(os.path.join(ref, "Output/solution.csv")) as f:
        r = list(csv.reader(f))[1:]
    sol = np.array([[float(x) for x in row[:5]] for row in r])
    np.savez_compressed(out, cond=cond, G=G, G_var=Gv, B=B, B_var=Bv, solution=sol,
                        config=np.array([-5.0, -5.0, 5.0, 5.0, 4, 8, 5000, 0.005,
                                         1.5, 1.27, 1.2, 1.13]))
    print("wrote", out, os.path.getsize(out), "bytes")
    with open(os.path.join(ref, "Output/Debug/times.txt")) as f:
        header = f.readline().strip()
    with open(os.path.join(HERE, "times_header.txt"), "w") as f:
        f.write(header + "\n")
    print("wrote", os.path.join(HERE, "times_header.txt"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py /path/to/reference")
    main(sys.argv[1])
