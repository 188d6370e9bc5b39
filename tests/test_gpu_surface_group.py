"""GPU parity of the surface-wave likelihood with group velocities (travel
times along the rays of the phase field, phaseGroup = 1) and with straight
rays (isStraight = 1), against the oracle's composition of the reference
path, including commit/reject and the noise-only likelihood on the
committed group times and ray lengths."""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import SurfaceLikelihood, synthetic

pytestmark = pytest.mark.gpu
P = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
TT_TOL = 1e-4
LIKE_RTOL = 1e-6


def case(seed, nchains=3, ncell_max=40):
    rng = np.random.default_rng(seed)
    grid, settings, data = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0),
                                                      nstations=8, nperiods=4, pmin=0.5, pmax=3.0)
    ncells, pts, par = synthetic.surface_chain_models(rng, nchains, ncell_max, grid, ncell_range=(6, ncell_max))
    return rng, grid, settings, data, ncells, pts, par


def oracle_like(orc, grid, settings, data, n, pts, par, n0, n1):
    gi = np.array([grid["nx"], grid["ny"], grid["nz"]], np.int32)
    gd = np.array([grid[k] for k in ("xmin", "ymin", "zmin", "dx", "dy", "dz", "scaling", "water_depth")])
    iset = np.array([settings[k] for k in ("raylov", "gridx", "gridy", "sgref", "sgdic", "sgext", "order",
                                           "sigdep", "material_law")], np.int32)
    npd = len(data["freqs"])
    pv = np.zeros((npd, grid["nx"], grid["ny"])); gv = np.zeros_like(pv)
    pt = np.zeros((npd, len(data["src"]), len(data["rev"]))); sd = np.zeros_like(pt)
    out = np.zeros(4)
    rc = orc.orc_surf_likelihood_ex(P(gi), P(gd), P(iset), settings["dphase"], settings["rho_value"], int(n),
                                    P(np.ascontiguousarray(pts[:n])), P(np.ascontiguousarray(par[:n])), npd,
                                    P(np.ascontiguousarray(data["freqs"])), len(data["src"]),
                                    P(np.ascontiguousarray(data["src"])), len(data["rev"]),
                                    P(np.ascontiguousarray(data["rev"])),
                                    P(np.ascontiguousarray(data["raystat"], np.int32)),
                                    P(np.ascontiguousarray(data["ttime"])), None, data["nrays"],
                                    P(np.ascontiguousarray(n0)), P(np.ascontiguousarray(n1)), None,
                                    settings["phase_group"], settings.get("straight", 0), P(pv), P(gv), P(pt), P(sd),
                                    P(out))
    assert rc == 0
    return out, pt, sd


@pytest.mark.parametrize("mode", ["group", "straight_group", "straight_phase"])
@pytest.mark.parametrize("tt_precision", [0, 1])
def test_surface_group_modes_match_oracle(orc, gpulib, mode, tt_precision):
    rng, grid, settings, data, ncells, pts, par = case(7)
    settings = dict(settings, phase_group=0 if mode == "straight_phase" else 1,
                    straight=1 if mode.startswith("straight") else 0, tt_precision=tt_precision)
    nch = len(ncells)
    npd = len(data["freqs"])
    n0 = np.full((nch, npd), 0.02); n1 = np.full((nch, npd), 0.01)
    lk = SurfaceLikelihood(grid, settings, data, nslots=nch, ncell_max=pts.shape[1])
    out = lk.forward(np.arange(nch), ncells, pts, par, n0, n1)
    m = np.asarray(data["raystat"]).reshape(npd, len(data["src"]), len(data["rev"])) == 1
    for c in range(nch):
        eo, ept, esd = oracle_like(orc, grid, settings, data, ncells[c], pts[c], par[c], n0[c], n1[c])
        pt, _ = lk.phase_time(c)
        assert int(out[c, 3]) == int(eo[3])
        tol = 1e-9 if (tt_precision == 0 or mode.startswith("straight")) else TT_TOL
        assert np.max(np.abs(pt[m] - ept[m])) <= tol
        if eo[3] == 0:
            np.testing.assert_allclose(out[c, :3], eo[:3], rtol=LIKE_RTOL)
    # commit everything, then the noise-only likelihood on the committed
    # times with srdist by mode
    lk.commit(np.ones(nch, np.int32))
    m0 = np.full((nch, npd), 0.03); m1 = np.full((nch, npd), 0.02)
    nz = lk.noise_likelihood(np.arange(nch), m0, m1)
    for c in range(nch):
        if out[c, 3] != 0:
            continue
        eo, _, _ = oracle_like(orc, grid, settings, data, ncells[c], pts[c], par[c], m0[c], m1[c])
        if eo[3] == 0:
            np.testing.assert_allclose(nz[c, :3], eo[:3], rtol=LIKE_RTOL if tt_precision == 0 else 1e-4)
    lk.close()


def test_surface_group_commit_and_reject(orc, gpulib):
    rng, grid, settings, data, ncells, pts, par = case(8, nchains=3)
    settings = dict(settings, phase_group=1, tt_precision=0)
    npd = len(data["freqs"])
    n0 = np.full((3, npd), 0.02); n1 = np.full((3, npd), 0.01)
    lk = SurfaceLikelihood(grid, settings, data, nslots=3, ncell_max=pts.shape[1])
    lk.forward(np.arange(3), ncells, pts, par, n0, n1)
    lk.commit(np.array([1, 0, 1], np.int32))
    pts2, par2 = synthetic.perturb_chain_models(rng, ncells, pts, par, grid)
    out2 = lk.forward(np.arange(3), ncells, pts2, par2, n0, n1)   # chain 1 starts from nothing committed
    m = np.asarray(data["raystat"]).reshape(npd, len(data["src"]), len(data["rev"])) == 1
    for c in range(3):
        eo, ept, _ = oracle_like(orc, grid, settings, data, ncells[c], pts2[c], par2[c], n0[c], n1[c])
        pt, _ = lk.phase_time(c)
        assert int(out2[c, 3]) == int(eo[3])
        assert np.max(np.abs(pt[m] - ept[m])) <= 1e-9
    lk.close()
