"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: the reference ships only its own noisy
synthetic decks, so every input here is generated from a seed with the stated
shapes and value distributions.
"""
import numpy as np


def voronoi_model_3d(rng, ncells, lo, hi, vs_range, vp_over_vs=None, rho_value=None,
                     monotone_depth=True):
    """Random nuclei in the box [lo, hi] with Vs drawn uniformly in vs_range.

    With monotone_depth, the Vs values are assigned in order of nucleus depth
    so that every grid column's Vs never drops below its top value, which is
    the reference's surface-wave admissibility test (check_model,
    src/likelihood_surf.F90:631-646): the nearest-nucleus map is monotone
    along a vertical line, so depth-sorted values stay depth-sorted.
    Returns points (n, 3) and params (n, 3) = (vp, vs, rho).
    """
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    pts = lo + (hi - lo) * rng.random((ncells, 3))
    vs = rng.uniform(vs_range[0], vs_range[1], ncells)
    if monotone_depth:
        vs = np.sort(vs)[np.argsort(np.argsort(pts[:, 2]))]
    vp = vs * (np.float64(np.float32(1.73)) if vp_over_vs is None else vp_over_vs)
    rho = np.full(ncells, 2.0) if rho_value is not None else 1.74 * vp ** 0.25
    if rho_value is not None:
        rho[:] = rho_value
    return pts, np.stack([vp, vs, rho], 1)


def layered_columns(rng, ncol, nl_range=(12, 40), h_range=(0.05, 0.5), vs_range=(0.2, 3.5),
                    lvl_prob=0.1):
    """Independent 1D columns for the dispersion-precision study: thickness
    uniform in h_range, Vs increasing with depth except that each interior
    layer becomes a low-velocity layer with probability lvl_prob; Vp = 1.73 Vs,
    rho = 1.74 Vp^0.25. Returns (nl, thk, vp, vs, rho) with (ncol, nl_max)
    REAL*4 arrays; the last layer of each column is the half-space (thk 0)."""
    nl = rng.integers(nl_range[0], nl_range[1] + 1, ncol).astype(np.int32)
    nl_max = int(nl_range[1])
    thk = np.zeros((ncol, nl_max), np.float32)
    vs = np.zeros((ncol, nl_max), np.float32)
    for c in range(ncol):
        n = nl[c]
        v = np.sort(rng.uniform(vs_range[0], vs_range[1], n))
        lv = rng.random(n) < lvl_prob
        lv[0] = False
        lv[-1] = False
        v[lv] = v[lv] * 0.7
        thk[c, :n - 1] = rng.uniform(h_range[0], h_range[1], n - 1)
        vs[c, :n] = v
        vs[c, n:] = v[-1]
    vp = (vs * np.float32(1.73)).astype(np.float32)
    rho = (np.float32(1.74) * vp.astype(np.float64) ** 0.25).astype(np.float32)
    return nl, thk, vp, vs, rho
