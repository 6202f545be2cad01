"""Copy the reference's NURBS geometry input files used by the workloads into
tests/golden/geo/ so that tests and benchmarks find them on machines without
the reference checkout.

Run from the repository root in a container that has the reference mounted:
    python tests/golden/make_geometry_fixtures.py /path/to/reference
The files are plain input data (Octave NURBS text, see the .dat loader); they
are copied byte for byte.
"""
import os
import shutil
import sys

FILES = ["sphere.dat", "torus.dat"]


def main(ref_root):
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "geo")
    os.makedirs(out, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(ref_root, "geo", f), os.path.join(out, f))
        print("copied", f)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_geometry_fixtures.py <reference checkout root>")
    main(sys.argv[1])
