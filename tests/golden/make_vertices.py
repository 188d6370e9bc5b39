"""Generates tests/golden/reference_vertices.npz from the Voronoi nuclei the
reference ships with its plotting scripts (plot/run_time_vertices_1.txt and
_2.txt: a count, then one nucleus per line, x y z and two velocities), given
the reference tree's root:

    python tests/golden/make_vertices.py <reference root>   (or MCT_REFERENCE)

The fixture keeps the nuclei (n, 3) and their two values (n, 2) of each file
as float64, so the gridding tests can run on the reference's own models on
machines without the reference tree.
"""
import os
import sys

import numpy as np


def read(path):
    with open(path) as f:
        n = int(f.readline().split()[0])
        rows = [list(map(float, f.readline().split())) for _ in range(n)]
    a = np.array(rows, np.float64)
    return a[:, :3], a[:, 3:5]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCT_REFERENCE")
    if not ref:
        raise SystemExit("usage: make_vertices.py <reference root> (or set MCT_REFERENCE)")
    data = {}
    for k in (1, 2):
        pts, val = read(os.path.join(ref, "plot", "run_time_vertices_%d.txt" % k))
        data["pts%d" % k] = pts
        data["val%d" % k] = val
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vertices.npz"), **data)
    print("wrote", {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
