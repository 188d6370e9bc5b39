"""Small fixed cases of the hot kernels, for profilers.

    python -m mctomo_gb300.profcase fm2d [--precision P] [--maps M] [--repeat R]
    python -m mctomo_gb300.profcase eik3 [--order O]
    python -m mctomo_gb300.profcase eik3heap [--order O] [--solves N]
    python -m mctomo_gb300.profcase disp [--precision P] [--columns N] [--study]
    python -m mctomo_gb300.profcase grid
    python -m mctomo_gb300.profcase tiles [--chains N]

fm2d: M Voronoi phase maps of 41 x 41 vertices (1 km spacing), 50 stations
between 2 and 38 km, every station pair once, source refinement 4 x over
8 cells (the surface-wave likelihood's fm2d settings); R calls of
mct_modrays_batch. eik3: 8 velocity grids of 101 x 101 x 51 nodes (0.5 km),
120 solves. eik3heap: the exact heap march, N solves (default 8) on 4
Voronoi grids of 51 x 51 x 26 nodes (0.5 km, velocities 3-7.5 km/s). disp: N layered columns (12-40 layers, no low-velocity layers),
20 Rayleigh fundamental-mode phase periods log-spaced 0.5-5 s, the surface
likelihood's search increment 1e-3 km/s; with --study, N columns of the
dispersion-precision study instead (12-40 layers with a 10 % low-velocity
layer chance, 60 periods 0.2-20 s, fundamental and first overtone, phase and
group, multimode). grid: nearest-nucleus gridding of a
101 x 101 x 51 grid over 50 x 50 x 25 km from 800 nuclei. Each case prints
one line and exits 0. tiles: the body-wave forward (101 x 101 x 51 grid, 200
events, 60 stations, P and S, first order) of N chains with each
configuration of the 3D tile solver forced in turn, then the tuned one; one
line per configuration.
"""
import argparse
import time

import numpy as np

from . import forward, synthetic


def fm2d(precision=1, maps=16, repeat=2):
    rng = np.random.default_rng(0)
    nvx = nvz = 41
    st = rng.uniform(2.0, 38.0, (50, 2))
    srs = np.triu(np.ones((50, 50), np.int32), 1)
    velv = synthetic.voronoi_phase_maps(rng, maps, nvx, nvz, 1.0, 1.0)
    for _ in range(repeat):
        t0 = time.perf_counter()
        tt = forward.modrays_batch(st, st, srs, nvx, nvz, 0.0, 0.0, 1.0, 1.0, velv, sgdl=4, sgs=8,
                                   precision=precision)
        dt = time.perf_counter() - t0
    print(f"fm2d precision={precision} maps={maps} solves={maps * 49} last_call_s={dt:.4f} t01={tt[0, 0, 1]:.6f}")


def eik3(order=0):
    rng = np.random.default_rng(1)
    nx, ny, nz = 101, 101, 51
    h = (0.5, 0.5, 0.5)
    lo = (0.0, 0.0, 0.0)
    z = np.arange(nz) * h[2]
    vels = np.stack([np.broadcast_to(3.0 + 0.08 * z * (1 + 0.1 * g), (nx, ny, nz)).copy() *
                     (1 + 0.05 * rng.standard_normal((nx, ny, nz))) for g in range(8)])
    nsolve = 120
    grid = (np.arange(nsolve) % 8).astype(np.int32)
    srcs = rng.uniform([2, 2, 1], [48, 48, 20], (nsolve, 3))
    rev = rng.uniform([2, 2, 0], [48, 48, 0.5], (60, 3))
    t0 = time.perf_counter()
    tt, _, passes = forward.eikonal3d_batch(vels, h, lo, grid, srcs, rev, order=order)
    dt = time.perf_counter() - t0
    print(f"eik3 order={order} solves={nsolve} passes={passes} call_s={dt:.4f} t00={tt[0, 0]:.6f}")


def eik3heap(order=1, solves=8):
    rng = np.random.default_rng(4)
    shape = (51, 51, 26)
    h = (0.5, 0.5, 0.5)
    lo = np.zeros(3); hi = (np.array(shape) - 1) * 0.5
    X, Y, Z = np.meshgrid(*[np.arange(k) * 0.5 for k in shape], indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    vels = []
    for g in range(4):
        pts, par = synthetic.voronoi_model_3d(rng, 120, lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        d = ((nodes[:, None, :] - pts[None]) ** 2).sum(-1)
        vels.append((par[:, 1] * 1.73)[d.argmin(1)].reshape(shape))
    vels = np.stack(vels)
    grid = (np.arange(solves) % 4).astype(np.int32)
    srcs = rng.uniform([1, 1, 0], [24, 24, 0.2], (solves, 3))
    rev = rng.uniform([1, 1, 1], [24, 24, 12], (40, 3))
    t0 = time.perf_counter()
    tt, _, _ = forward.eikonal3d_batch(vels, h, lo, grid, srcs, rev, order=order, solver="heap")
    dt = time.perf_counter() - t0
    print(f"eik3heap order={order} solves={solves} call_s={dt:.4f} t00={tt[0, 0]:.6f}")


def disp(precision=1, columns=4096, study=False):
    rng = np.random.default_rng(2)
    if study:
        nl, thk, vp, vs, rho = synthetic.layered_columns(rng, columns, nl_range=(12, 40), lvl_prob=0.1)
        periods = np.geomspace(0.2, 20.0, 60)
        kw = dict(mode=2, multimode=True)
    else:
        nl, thk, vp, vs, rho = synthetic.layered_columns(rng, columns, lvl_prob=0.0)
        periods = np.geomspace(0.5, 5.0, 20)
        kw = {}
    t0 = time.perf_counter()
    cp, _, ierr, cnt = forward.surfdisp_batch(nl, thk, vp, vs, rho, periods, 2, int(study), 1e-3,
                                              precision=precision, **kw)
    dt = time.perf_counter() - t0
    print(f"disp precision={precision} columns={columns} study={int(study)} call_s={dt:.4f} ierr={int((ierr != 0).sum())} "
          f"evals_fp64={cnt[0]} evals_fp32={cnt[1]} cp00={cp[0, 0, 0]:.6f}")


def grid():
    rng = np.random.default_rng(3)
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0])
    shape = (101, 101, 51)
    st = (hi - lo) / (np.array(shape) - 1)
    pts, par = synthetic.voronoi_model_3d(rng, 800, lo, hi, (1.7, 4.3))
    t0 = time.perf_counter()
    sid, _, _, _ = forward.kdtree_to_grid(pts, par, *shape, lo, st)
    dt = time.perf_counter() - t0
    print(f"grid nodes={sid.size} nuclei=800 call_s={dt:.4f} sid0={int(sid.ravel()[0])}")


def tiles(chains=32):
    from . import BodyLikelihood, lib
    L = lib()
    rng = np.random.default_rng(5)
    grid, settings, data, ev = synthetic.body_workload(rng)
    settings["order"] = 0
    settings["solver"] = 0x10
    lo = np.zeros(3); hi = np.array([50.0, 50.0, 25.0]); ncell_max = 800
    ncells = rng.integers(20, ncell_max + 1, chains).astype(np.int32)
    pts = np.zeros((chains, ncell_max, 3)); par = np.zeros((chains, ncell_max, 3))
    for c in range(chains):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (3.0 / 1.73, 7.5 / 1.73))
        q[:, 0] = q[:, 1] * 1.73
        pts[c, :ncells[c]] = p; par[c, :ncells[c]] = q
    locs = np.repeat(ev[None], chains, 0)
    n0 = np.zeros((chains, 2)); n1 = np.full((chains, 2), 0.05)
    lk = BodyLikelihood(grid, settings, data, nslots=chains, ncell_max=ncell_max)
    old = L.mct_debug_eik3_tile_config(-1, 0, 0, 0, 0)
    ref = None
    for cfg in list(range(20)) + [-1]:
        L.mct_debug_eik3_tile_config(cfg, 0, 0, 0, 0)
        lk.forward(ncells, pts, par, locs, n0, n1)
        t0 = time.perf_counter()
        out = lk.forward(ncells, pts, par, locs, n0, n1)
        dt = time.perf_counter() - t0
        ref = out if ref is None else ref
        print(f"tiles cfg={cfg} chains={chains} forward_s={dt:.3f} passes={lk.phase_time(0)[1]} "
              f"max_like_diff={float(np.max(np.abs(out[:, 0] - ref[:, 0]))):.3g}", flush=True)
    print(f"tiles tuned_cfg={L.mct_debug_eik3_tile_config(-2, 101, 101, 51, 0)}")
    L.mct_debug_eik3_tile_config(old, 0, 0, 0, 0)
    lk.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case", choices=["fm2d", "eik3", "eik3heap", "disp", "grid", "tiles"])
    ap.add_argument("--chains", type=int, default=32)
    ap.add_argument("--solves", type=int, default=8)
    ap.add_argument("--columns", type=int, default=4096)
    ap.add_argument("--precision", type=int, default=1)
    ap.add_argument("--maps", type=int, default=16)
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--order", type=int, default=None)
    ap.add_argument("--study", action="store_true")
    a = ap.parse_args(argv)
    if a.case == "fm2d":
        fm2d(a.precision, a.maps, a.repeat)
    elif a.case == "eik3":
        eik3(a.order or 0)
    elif a.case == "eik3heap":
        eik3heap(1 if a.order is None else a.order, a.solves)
    elif a.case == "disp":
        disp(a.precision, a.columns, a.study)
    elif a.case == "tiles":
        tiles(a.chains)
    else:
        grid()


if __name__ == "__main__":
    main()
