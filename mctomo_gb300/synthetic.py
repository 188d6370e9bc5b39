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


def surface_workload(rng, nx=41, ny=41, nz=31, extent=(40.0, 40.0, 6.0), nstations=50, nperiods=20,
                     pmin=0.5, pmax=5.0):
    """The batched surface-wave configuration: grid, settings and data dicts
    for SurfaceLikelihood. Stations at seeded uniform positions, every
    station pair once (upper triangle: nsta*(nsta-1)/2 paths per period),
    Rayleigh fundamental-mode phase velocity at log-spaced periods. Observed
    times are straight-ray times at 1.5 km/s with 2% noise; sigma = 2% of the
    time (sigdep with n0 = 0.02, n1 = 0)."""
    grid = dict(nx=nx, ny=ny, nz=nz, xmin=0.0, ymin=0.0, zmin=0.0,
                dx=extent[0] / (nx - 1), dy=extent[1] / (ny - 1), dz=extent[2] / (nz - 1),
                scaling=1.0, water_depth=0.0)
    settings = dict(raylov=1, phase_group=0, dphase=1e-3, gridx=1, gridy=1, sgref=1, sgdic=4, sgext=8,
                    order=1, sigdep=1, material_law=2, rho_value=2.0, precision=1, tt_precision=0)
    margin = 0.05 * np.array(extent[:2])
    st = margin + (np.array(extent[:2]) - 2 * margin) * rng.random((nstations, 2))
    periods = np.geomspace(pmin, pmax, nperiods)
    freqs = 1.0 / periods
    srs = np.triu(np.ones((nstations, nstations), np.int32), 1).reshape(-1)
    raystat = np.tile(srs, (nperiods, 1))
    dist = np.hypot(st[:, None, 0] - st[None, :, 0], st[:, None, 1] - st[None, :, 1]).reshape(-1)
    tt = dist / 1.5
    ttime = np.tile(tt, (nperiods, 1)) * (1 + 0.02 * rng.standard_normal((nperiods, tt.size)))
    data = dict(src=st, rev=st, freqs=freqs, raystat=raystat, ttime=ttime, sigma=None,
                nrays=int(raystat.sum()))
    return grid, settings, data


def surface_chain_models(rng, nchains, ncell_max, grid, ncell_range=(10, 400), vs_range=(0.3, 2.5)):
    """One Voronoi model per chain with an uneven cell count, Vs sorted by
    nucleus depth (so every model passes check_model). Returns ncells,
    points (nchains, ncell_max, 3), params (nchains, ncell_max, 3)."""
    lo = np.array([grid["xmin"], grid["ymin"], grid["zmin"]])
    hi = lo + np.array([grid["dx"] * (grid["nx"] - 1), grid["dy"] * (grid["ny"] - 1), grid["dz"] * (grid["nz"] - 1)])
    ncells = rng.integers(ncell_range[0], ncell_range[1] + 1, nchains).astype(np.int32)
    points = np.zeros((nchains, ncell_max, 3))
    params = np.zeros((nchains, ncell_max, 3))
    for c in range(nchains):
        p, q = voronoi_model_3d(rng, int(ncells[c]), lo, hi, vs_range, rho_value=2.0)
        points[c, :ncells[c]] = p
        params[c, :ncells[c]] = q
    return ncells, points, params


def perturb_chain_models(rng, ncells, points, params, grid, vs_range=(0.3, 2.5)):
    """A move proposal per chain: one nucleus is displaced in depth order
    (keeping Vs sorted by depth), so each proposal changes one Voronoi cell."""
    lo = np.array([grid["xmin"], grid["ymin"], grid["zmin"]])
    ext = np.array([grid["dx"] * (grid["nx"] - 1), grid["dy"] * (grid["ny"] - 1), grid["dz"] * (grid["nz"] - 1)])
    points = points.copy(); params = params.copy()
    for c in range(len(ncells)):
        n = int(ncells[c])
        i = rng.integers(n)
        newp = np.clip(points[c, i] + rng.normal(0, 0.05, 3) * ext, lo, lo + ext)
        points[c, i] = newp
        order = np.argsort(points[c, :n, 2])
        vs = np.sort(params[c, :n, 1])
        params[c, order, 1] = vs
        params[c, :n, 0] = params[c, :n, 1] * np.float64(np.float32(1.73))
    return points, params


def body_workload(rng, nx=101, ny=101, nz=51, extent=(50.0, 50.0, 25.0), nevents=200, nstations=60, np_=2):
    """The 3D body-wave configuration: events at seeded uniform positions
    inside the grid, at 4-80 % of its depth (1-20 km for the default 25 km),
    with origin times uniform on [0, 1] s, stations at the
    surface kept off the grid's maximum x/y faces (where the reference's
    trilinear read-out multiplies times), P and S picks for every pair, noise
    sigma 0.03 s (P) / 0.06 s (S). Observed times are straight-ray times at
    6 / 3.5 km/s plus noise and origin time. Returns grid, settings, data,
    event locations (nevents, 4)."""
    grid = dict(nx=nx, ny=ny, nz=nz, xmin=0.0, ymin=0.0, zmin=0.0,
                dx=extent[0] / (nx - 1), dy=extent[1] / (ny - 1), dz=extent[2] / (nz - 1),
                scaling=1.0, water_depth=0.0)
    ev = np.column_stack([rng.uniform(0.02, 0.98, nevents) * extent[0], rng.uniform(0.02, 0.98, nevents) * extent[1],
                          rng.uniform(0.04, 0.8, nevents) * extent[2], rng.uniform(0.0, 1.0, nevents)])
    sta = np.column_stack([rng.uniform(0.02, 0.95, nstations) * extent[0],
                           rng.uniform(0.02, 0.95, nstations) * extent[1], np.zeros(nstations)])
    dist = np.sqrt(((ev[:, None, :3] - sta[None, :, :]) ** 2).sum(-1)).reshape(-1)   # (src j, rev k)
    sig = np.array([0.03, 0.06])[:np_]
    vel = np.array([6.0, 3.5])[:np_]
    t0 = np.repeat(ev[:, 3], nstations)
    ttime = np.stack([dist / vel[p] + t0 + sig[p] * rng.standard_normal(dist.size) for p in range(np_)])
    raystat = np.ones((np_, dist.size), np.int32)
    settings = dict(order=1, np=np_, sigdep=0)
    sigma = np.stack([np.full(dist.size, sig[p]) for p in range(np_)])
    data = dict(nsrc=nevents, rev=sta, raystat=raystat, ttime=ttime, sigma=sigma, nrays=int(raystat.sum()))
    return grid, settings, data, ev


def voronoi_phase_maps(rng, nmaps, nvx, nvz, dx, dz, ncell=50, vrange=(0.4, 2.2)):
    """Piecewise-constant 2D phase-velocity maps (Voronoi cells of uniform
    random velocity), padded by one vertex on each side by edge copy, the
    layout modrays takes: (nmaps, nvx+2, nvz+2)."""
    out = np.zeros((nmaps, nvx + 2, nvz + 2))
    X, Z = np.meshgrid(np.arange(nvx) * dx, np.arange(nvz) * dz, indexing="ij")
    for m in range(nmaps):
        pts = rng.uniform(0, 1, (ncell, 2)) * [(nvx - 1) * dx, (nvz - 1) * dz]
        vals = rng.uniform(vrange[0], vrange[1], ncell)
        d = (X[..., None] - pts[:, 0]) ** 2 + (Z[..., None] - pts[:, 1]) ** 2
        out[m, 1:-1, 1:-1] = vals[np.argmin(d, -1)]
        out[m, 0] = out[m, 1]; out[m, -1] = out[m, -2]
        out[m, :, 0] = out[m, :, 1]; out[m, :, -1] = out[m, :, -2]
    return out


def tt2d_workload(rng, nx=51, ny=51, extent=10.0, nstations=16, inset=0.5, noise=0.05, datatype=0):
    """The plain 2D travel-time configuration: a square grid over extent km,
    nstations equally spaced on a square perimeter inset from the edges (the
    reference's refined-source pass reads undefined memory for sources on
    the maximum edges), every station a source to every other one, observed
    times = straight-ray times at 3 km/s plus Gaussian noise. datatype 1
    adds differential times of every source pair at every receiver (zero,
    i.e. absent, where the receiver is one of the two sources) with
    cross-correlation coefficients in [0.5, 1]. Returns grid, settings,
    data for TravelTime2DLikelihood."""
    grid = dict(nx=nx, ny=ny, nz=1, xmin=0.0, ymin=0.0, zmin=0.0, dx=extent / (nx - 1), dy=extent / (ny - 1),
                dz=1.0, scaling=1.0, water_depth=0.0)
    side = extent - 2 * inset
    s = np.arange(nstations) * (4 * side / nstations)
    st = np.zeros((nstations, 2))
    for n, a in enumerate(s):
        e, f = int(a // side), a % side
        st[n] = [(inset + f, inset), (extent - inset, inset + f), (extent - inset - f, extent - inset),
                 (inset, extent - inset - f)][e]
    raystat = (1 - np.eye(nstations, dtype=np.int32)).reshape(-1)
    dist = np.hypot(st[:, None, 0] - st[None, :, 0], st[:, None, 1] - st[None, :, 1])
    tt = (dist / 3.0 + noise * rng.standard_normal(dist.shape)) * (1 - np.eye(nstations))
    settings = dict(gridx=1, gridy=1, sgref=1, sgdic=5, sgext=10, order=1, sigdep=0, datatype=datatype, straight=0,
                    precision=0)
    data = dict(src=st, rev=st, raystat=raystat, ttime=tt.reshape(-1), sigma=np.full(raystat.size, noise),
                nrays=int(raystat.sum()))
    if datatype == 1:
        pairs = [(i, j) for i in range(nstations) for j in range(i + 1, nstations)]
        dt = np.zeros((len(pairs), nstations))
        dcc = rng.uniform(0.5, 1.0, dt.shape)
        for d, (i, j) in enumerate(pairs):
            for k in range(nstations):
                if k not in (i, j):
                    dt[d, k] = tt[j, k] - tt[i, k] + 0.01 * rng.standard_normal()
        data.update(dtime=dt, dcc=dcc, ndtime=int((dt != 0).sum()))
    return grid, settings, data


def tt2d_chain_models(rng, nchains, ncell_max, grid, ncell_range=(4, 100), vrange=(2.0, 4.0)):
    """2D Voronoi models (nuclei uniform in the domain, velocity uniform on
    vrange): ncells, points (nchains, ncell_max, 2), params (nchains,
    ncell_max, 3) with the velocity first."""
    lo = np.array([grid["xmin"], grid["ymin"]])
    hi = lo + np.array([grid["dx"] * (grid["nx"] - 1), grid["dy"] * (grid["ny"] - 1)])
    ncells = rng.integers(ncell_range[0], ncell_range[1] + 1, nchains).astype(np.int32)
    points = np.zeros((nchains, ncell_max, 2))
    params = np.zeros((nchains, ncell_max, 3))
    for c in range(nchains):
        n = int(ncells[c])
        points[c, :n] = lo + (hi - lo) * rng.random((n, 2))
        params[c, :n, 0] = rng.uniform(vrange[0], vrange[1], n)
        params[c, :n, 1] = params[c, :n, 0] / 1.73
        params[c, :n, 2] = 2.0
    return ncells, points, params


def serving_models(kind, grid, ncell_max, ncell_range):
    """(new_model, propose) for one chain of a serving stream: new_model(rng)
    draws a Voronoi model (ncells, points, params) padded to ncell_max;
    propose(rng, model) returns the proposal. kind "tt2d": 2D cells with
    velocity on [2, 4] km/s and value-change proposals; "surface": 3D cells
    with Vs on [0.3, 2.5] km/s; "body" / "joint": 3D cells with Vp on
    [3, 7.5] km/s, Vs = Vp / 1.73; 3D proposals move one nucleus and keep Vs
    sorted by depth (perturb_chain_models)."""
    if kind == "tt2d":
        def new_model(rng):
            nc, p, q = tt2d_chain_models(rng, 1, ncell_max, grid, ncell_range=ncell_range)
            return int(nc[0]), p[0], q[0]

        def propose(rng, model):
            nc, p, q = model
            q = q.copy()
            i = int(rng.integers(nc))
            q[i, 0] = float(np.clip(q[i, 0] + rng.normal(0.0, 0.1), 2.0, 4.0))
            q[i, 1] = q[i, 0] / 1.73
            return nc, p, q
        return new_model, propose
    vs_range = (0.3, 2.5) if kind == "surface" else (3.0 / 1.73, 7.5 / 1.73)
    lo = np.array([grid["xmin"], grid["ymin"], grid["zmin"]])
    hi = lo + np.array([grid["dx"] * (grid["nx"] - 1), grid["dy"] * (grid["ny"] - 1), grid["dz"] * (grid["nz"] - 1)])

    def new_model(rng):
        n = int(rng.integers(ncell_range[0], ncell_range[1] + 1))
        p, q = voronoi_model_3d(rng, n, lo, hi, vs_range, rho_value=2.0)
        pts = np.zeros((ncell_max, 3)); par = np.zeros((ncell_max, 3))
        pts[:n] = p; par[:n] = q
        return n, pts, par

    def propose(rng, model):
        nc, p, q = model
        p2, q2 = perturb_chain_models(rng, np.array([nc]), p[None], q[None], grid, vs_range)
        return nc, p2[0], q2[0]
    return new_model, propose
