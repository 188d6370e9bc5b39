"""ORACLE (test infrastructure only): the reference's read-out of stored
travel-time fields for the body-wave location step, restated in plain
Python.

interpolate3d follows Interpolate3d (src/likelihood_body.F90:976-1005) with
point2idx (:1038-1054): the cell of the point (1-based, clamped to
[1, n-1]), its offsets from the cell's first node (z scaled by
grid%scaling), and the sum over the 8 corners of the weights
(1.0 - |(i-1) dx - dsx| / dx) x ... in the loop order i (x), j (y), k (z).
Fields are (nx, ny, nz) arrays, z fastest (Fortran (nz, ny, nx)).
"""
import math


def point2idx(grid, pt):
    s = grid["scaling"]
    ix = math.floor((pt[0] - grid["xmin"]) / grid["dx"]) + 1
    iy = math.floor((pt[1] - grid["ymin"]) / grid["dy"]) + 1
    iz = math.floor((pt[2] - grid["zmin"] / s) / (grid["dz"] / s)) + 1
    ix, iy, iz = max(ix, 1), max(iy, 1), max(iz, 1)
    ix = grid["nx"] - 1 if ix >= grid["nx"] else ix
    iy = grid["ny"] - 1 if iy >= grid["ny"] else iy
    iz = grid["nz"] - 1 if iz >= grid["nz"] else iz
    return ix, iy, iz


def interpolate3d(field, grid, pt):
    dx, dy, dz, s = grid["dx"], grid["dy"], grid["dz"], grid["scaling"]
    ix, iy, iz = point2idx(grid, pt)
    dsx = pt[0] - (grid["xmin"] + (ix - 1) * dx)
    dsy = pt[1] - (grid["ymin"] + (iy - 1) * dy)
    dsz = pt[2] - (grid["zmin"] + (iz - 1) * dz) / s
    qv = 0.0
    for i in (1, 2):
        for j in (1, 2):
            for k in (1, 2):
                w = (1.0 - abs((i - 1) * dx - dsx) / dx) * (1.0 - abs((j - 1) * dy - dsy) / dy) * \
                    (1.0 - abs((k - 1) * dz / s - dsz) / (dz / s))
                qv = qv + w * float(field[ix + i - 2, iy + j - 2, iz + k - 2])
    return qv
