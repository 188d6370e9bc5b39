"""GPU parity of the batched surface-wave likelihood (gridding -> dispersion
-> fm2d -> misfit) against the oracle's composition of the reference path,
including the commit / reject semantics of the device-resident chain state
and results that do not depend on which other chains share the batch."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import SurfaceLikelihood, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TT_TOL = 1e-4      # s, travel times (the stated accuracy bound)
LIKE_RTOL = 1e-6


def small_case(seed, nchains=4, ncell_max=60):
    rng = np.random.default_rng(seed)
    grid, settings, data = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0),
                                                      nstations=9, nperiods=6, pmin=0.5, pmax=3.0)
    ncells, pts, par = synthetic.surface_chain_models(rng, nchains, ncell_max, grid, ncell_range=(6, ncell_max))
    return rng, grid, settings, data, ncells, pts, par


def oracle_like(orc, grid, settings, data, n, pts, par, n0, n1):
    gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
    gd = np.array([grid[k] for k in ("xmin", "ymin", "zmin", "dx", "dy", "dz", "scaling", "water_depth")])
    iset = np.array([settings[k] for k in ("raylov", "gridx", "gridy", "sgref", "sgdic", "sgext", "order",
                                           "sigdep", "material_law")], np.int32)
    npd = len(data["freqs"])
    pv = np.zeros((npd, grid["nx"], grid["ny"]))
    pt = np.zeros((npd, len(data["src"]), len(data["rev"])))
    out = np.zeros(4)
    rc = orc.orc_surf_likelihood(P(gi), P(gd), P(iset), settings["dphase"], settings["rho_value"], int(n),
                                 P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), npd,
                                 P(np.ascontiguousarray(data["freqs"])), len(data["src"]),
                                 P(np.ascontiguousarray(data["src"])), len(data["rev"]),
                                 P(np.ascontiguousarray(data["rev"])), P(np.ascontiguousarray(data["raystat"], np.int32)),
                                 P(np.ascontiguousarray(data["ttime"])), None, data["nrays"],
                                 P(np.ascontiguousarray(n0)), P(np.ascontiguousarray(n1)), None, P(pv), P(pt), P(out))
    assert rc == 0
    return out, pt, pv


def check_chain(orc, lk, idx, grid, settings, data, n, pts, par, n0, n1, out):
    eo, ept, epv = oracle_like(orc, grid, settings, data, n, pts, par, n0, n1)
    pt, pv = lk.phase_time(idx)
    assert int(out[3]) == int(eo[3])
    assert np.max(np.abs(pv - epv)) <= 1e-5
    m = np.asarray(data["raystat"]).reshape(pt.shape) == 1
    assert np.max(np.abs(pt[m] - ept[m])) <= TT_TOL
    if eo[3] == 0:
        np.testing.assert_allclose(out[:3], eo[:3], rtol=LIKE_RTOL)


@pytest.mark.parametrize("precision", [0, 1])
def test_surface_batch_matches_oracle(orc, gpulib, precision):
    rng, grid, settings, data, ncells, pts, par = small_case(1)
    settings["precision"] = precision
    settings["tt_precision"] = 0
    lk = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=pts.shape[1])
    npd = len(data["freqs"])
    n0 = np.full((4, npd), 0.02); n1 = np.full((4, npd), 0.01)
    out = lk.forward(np.arange(4), ncells, pts, par, n0, n1)
    for c in range(4):
        check_chain(orc, lk, c, grid, settings, data, ncells[c], pts[c], par[c], n0[c], n1[c], out[c])
    lk.close()


def test_surface_commit_and_reject_semantics(orc, gpulib):
    rng, grid, settings, data, ncells, pts, par = small_case(2)
    lk = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=pts.shape[1])
    npd = len(data["freqs"])
    n0 = np.full((4, npd), 0.02); n1 = np.full((4, npd), 0.0)
    lk.forward(np.arange(4), ncells, pts, par, n0, n1)
    lk.commit(np.ones(4, np.int32))
    pts2, par2 = synthetic.perturb_chain_models(rng, ncells, pts, par, grid)
    out2 = lk.forward(np.arange(4), ncells, pts2, par2, n0, n1)   # only changed columns recomputed
    for c in range(4):
        check_chain(orc, lk, c, grid, settings, data, ncells[c], pts2[c], par2[c], n0[c], n1[c], out2[c])
    lk.commit(np.array([1, 0, 1, 0], np.int32))
    pts3, par3 = synthetic.perturb_chain_models(rng, ncells, pts2, par2, grid)
    out3 = lk.forward(np.arange(4), ncells, pts3, par3, n0, n1)   # chains 1, 3 start from the first model
    for c in range(4):
        check_chain(orc, lk, c, grid, settings, data, ncells[c], pts3[c], par3[c], n0[c], n1[c], out3[c])
    lk.close()


def test_surface_result_is_the_same_alone_and_in_the_mix(gpulib):
    rng, grid, settings, data, ncells, pts, par = small_case(3, nchains=6)
    lk = SurfaceLikelihood(grid, settings, data, nslots=6, ncell_max=pts.shape[1])
    npd = len(data["freqs"])
    n0 = np.full((6, npd), 0.02); n1 = np.full((6, npd), 0.0)
    mix = lk.forward(np.arange(6), ncells, pts, par, n0, n1)
    mix_pt = [lk.phase_time(i)[0] for i in range(6)]
    for c in (0, 3, 5):
        alone = lk.forward(np.array([c]), ncells[c:c + 1], pts[c:c + 1], par[c:c + 1], n0[c:c + 1], n1[c:c + 1])
        np.testing.assert_array_equal(alone[0], mix[c])
        np.testing.assert_array_equal(lk.phase_time(0)[0], mix_pt[c])
    lk.close()


def test_surface_rejects_models_failing_check_model(gpulib):
    rng, grid, settings, data, ncells, pts, par = small_case(4, nchains=2)
    par = par.copy()
    # a slow deep cell under a fast top one violates vs(k>1) >= vs(1)
    n = ncells[0]
    top = np.argmin(pts[0, :n, 2]); deep = np.argmax(pts[0, :n, 2])
    par[0, deep, 1] = par[0, top, 1] * 0.5
    lk = SurfaceLikelihood(grid, settings, data, nslots=2, ncell_max=pts.shape[1])
    npd = len(data["freqs"])
    out = lk.forward(np.arange(2), ncells, pts, par, np.full((2, npd), 0.02), np.zeros((2, npd)))
    assert int(out[0, 3]) & 1 and out[0, 0] > 1e300
    assert int(out[1, 3]) == 0
    lk.close()


@pytest.mark.parametrize("tt_precision", [1, 2])
def test_surface_reduced_precision_travel_times(orc, gpulib, tt_precision):
    rng, grid, settings, data, ncells, pts, par = small_case(5)
    settings["precision"] = 1
    settings["tt_precision"] = tt_precision
    lk = SurfaceLikelihood(grid, settings, data, nslots=4, ncell_max=pts.shape[1])
    npd = len(data["freqs"])
    n0 = np.full((4, npd), 0.02); n1 = np.full((4, npd), 0.01)
    out = lk.forward(np.arange(4), ncells, pts, par, n0, n1)
    for c in range(4):
        eo, ept, epv = oracle_like(orc, grid, settings, data, ncells[c], pts[c], par[c], n0[c], n1[c])
        pt, pv = lk.phase_time(c)
        m = np.asarray(data["raystat"]).reshape(pt.shape) == 1
        err = np.abs(pt[m] - ept[m])
        if tt_precision == 1:      # double-float: within the bound on every path
            assert err.max() <= TT_TOL
        else:                      # fixed point: approximate mode
            assert np.quantile(err, 0.99) <= TT_TOL and err.max() <= 5e-2
        if eo[3] == 0:
            np.testing.assert_allclose(out[c, :3], eo[:3], rtol=1e-2)
    lk.close()
