"""Generates tests/golden/fmm3d_ref.npz from the reference's own
fastMarching3D (fastmarching/fastMarching.cpp), compiled from its sources by
oracle/build_ref.sh. Run in a tree where the reference is present:

    python tests/golden/make_golden.py

The cases are small seeded grids: homogeneous and random velocity, both
orders (0 first order, 1 mixed second order), with a source and receivers in
the interior.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402


def cases():
    rng = np.random.default_rng(20240601)
    out = []
    for trial in range(8):
        nx, ny, nz = (int(v) for v in rng.integers(5, 15, 3))
        dx, dy, dz = 0.5, 0.45, 0.4
        if trial % 3 == 0:
            vel = np.full((nx, ny, nz), 4.0)
        else:
            vel = rng.uniform(3.0, 7.5, (nx, ny, nz))
        xmin, ymin, zmin = -1.0, 2.0, 0.0
        src = np.array([xmin + rng.uniform(0.1, 0.9) * (nx - 1) * dx,
                        ymin + rng.uniform(0.1, 0.9) * (ny - 1) * dy,
                        zmin + rng.uniform(0.1, 0.9) * (nz - 1) * dz])
        nrev = 12
        rev = np.stack([xmin + rng.uniform(0.02, 0.98, nrev) * (nx - 1) * dx,
                        ymin + rng.uniform(0.02, 0.98, nrev) * (ny - 1) * dy,
                        zmin + rng.uniform(0.02, 0.98, nrev) * (nz - 1) * dz], 1)
        for order in (0, 1):
            out.append(dict(nx=nx, ny=ny, nz=nz, h=np.array([dx, dy, dz]),
                            lo=np.array([xmin, ymin, zmin]), vel=vel, src=src, rev=rev,
                            order=order))
    return out


def main():
    oracle.build_reference()
    ref = oracle.load_reference()
    if ref is None:
        raise SystemExit("reference fastMarching3D not available")
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    data = {}
    for i, c in enumerate(cases()):
        vel = np.ascontiguousarray(c["vel"])
        rev = np.ascontiguousarray(c["rev"])
        tt = np.zeros(rev.shape[0])
        tf = np.zeros_like(vel)
        rc = ref.fastMarching3D(c["nx"], c["ny"], c["nz"], *c["h"], *c["lo"], P(vel), P(c["src"]),
                                P(rev), rev.shape[0], c["order"], P(tt), P(tf))
        assert rc == 0
        for k, v in c.items():
            data["c%d_%s" % (i, k)] = v
        data["c%d_ttime" % i] = tt
        data["c%d_tfield" % i] = tf
    data["ncases"] = len(cases())
    np.savez_compressed(os.path.join(os.path.dirname(__file__), "fmm3d_ref.npz"), **data)
    print("wrote", len(cases()), "cases")


if __name__ == "__main__":
    main()
