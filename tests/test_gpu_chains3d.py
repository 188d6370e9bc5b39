"""GPU: seeded 3D surface-wave chains driven by the restated sampler
(mct_rng_* and mct_mcmc_*, src/mt19937.f90 and src/mcmc_loc2.f90) give the
same chains on the device-resident likelihood (mct_surf_*) as on the
oracle's restatement of the reference path.

Each chain runs the reference's Metropolis-Hastings loop: a proposal of the
type proposeType2 picks (birth, death, move, value change, and for sigdep
the surface noise change), the acceptance test, and the reference's redo of
a proposal whose model the likelihood rejects (like = huge), with the same
type and acceptance draw. The same seeds on both sides must give the same
accept / reject sequence, -log L within LIKE_RTOL at every step, and the
same final models.
"""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import SurfaceLikelihood, sampler, synthetic
from test_gpu_surface import oracle_like, small_case

pytestmark = pytest.mark.gpu
LIKE_RTOL = 1e-6
MAX_TRY = 1000   # the reference's maxTryNum (src/mcmc_loc2.f90:52)


def mcmc_settings(grid, ncell_max, sigdep):
    ext = [grid["d" + a] * (grid["n" + a] - 1) for a in "xyz"]
    return dict(ncell_min=4, ncell_max=ncell_max, kernel=1, datatype=2, sigdep=sigdep, locate=0,
                xmin=grid["xmin"], xmax=grid["xmin"] + ext[0], ymin=grid["ymin"], ymax=grid["ymin"] + ext[1],
                zmin=grid["zmin"], zmax=grid["zmin"] + ext[2], vpmin=0.5, vpmax=4.5, vsmin=0.3, vsmax=2.5,
                sigma_vp=0.1, sigma_vs=0.08, sigma_vp2=0.1, sigma_vs2=0.08, pd=5.0, pd2=8.0,
                sigma_bn0=0.0, sigma_bn1=0.0, bn0_min=0.0, bn0_max=1.0, bn1_min=0.0, bn1_max=1.0,
                sigma_sn0=0.002, sigma_sn1=0.01, sn0_min=0.001, sn0_max=0.1, sn1_min=0.0, sn1_max=0.5)


def run_chain(chain, like_fn, noise_fn, commit_fn, niter):
    """The reference's loop for one chain; like_fn(chain) -> (like, status)
    of the chain's current model, noise_fn(chain) -> like of its committed
    model with its current noise levels, commit_fn(accept) after a model
    forward. Returns the trace [(iteration, type, accepted, like)]."""
    like_cur, st = like_fn(chain)
    assert st == 0
    commit_fn(1)
    trace = []
    step = sampler.McmcStep()
    for it in range(1, niter + 1):
        redo, tries = False, 0
        while True:
            snap = chain.snapshot()
            chain.propose(it, redo, step)
            if not step.valid:
                chain.restore(snap)
                trace.append((it, step.ptype, False, None))
                break
            if step.ptype <= 4:
                like, st = like_fn(chain)
                if st != 0:                       # like = huge: redo the proposal
                    chain.restore(snap)
                    commit_fn(0)
                    tries += 1
                    redo = tries < MAX_TRY
                    continue
            else:
                like = noise_fn(chain)
            acc = chain.accept(step, like, like_cur)
            if step.ptype <= 4:
                commit_fn(1 if acc else 0)
            if acc:
                like_cur = like
            else:
                chain.restore(snap)
            trace.append((it, step.ptype, bool(acc), like))
            break
    return trace


@pytest.mark.parametrize("sigdep", [0, 1])
def test_seeded_surface_chains_match_oracle(orc, gpulib, sigdep):
    ncell_max = 40
    rng, grid, settings, data, ncells, pts, par = small_case(3, nchains=2, ncell_max=ncell_max)
    settings["sigdep"] = 1
    npd = len(data["freqs"])
    mset = mcmc_settings(grid, ncell_max, sigdep)
    lk = SurfaceLikelihood(grid, settings, data, nslots=2, ncell_max=ncell_max)
    niter = 120
    try:
        for c in range(2):
            sn0, sn1 = np.full(npd, 0.02), np.zeros(npd)
            gpu = sampler.Chain(mset, 1000 + c, ncells[c], pts[c], par[c], snoise0=sn0, snoise1=sn1)
            cpu = sampler.Chain(mset, 1000 + c, ncells[c], pts[c], par[c], snoise0=sn0, snoise1=sn1)
            sl = np.array([c], np.int32)

            def gpu_like(ch):
                o = lk.forward(sl, [ch.ncells], ch.points[None], ch.params[None], ch.sn0[None], ch.sn1[None])
                return o[0, 0], int(o[0, 3])

            def gpu_noise(ch):
                return lk.noise_likelihood(sl, ch.sn0[None], ch.sn1[None])[0, 0]

            def cpu_like(ch):
                o, _, _ = oracle_like(orc, grid, settings, data, ch.ncells, ch.points, ch.params, ch.sn0, ch.sn1)
                return o[0], int(o[3])

            tg = run_chain(gpu, gpu_like, gpu_noise, lambda a: lk.commit(np.array([a], np.int32)), niter)
            tc = run_chain(cpu, cpu_like, lambda ch: cpu_like(ch)[0], lambda a: None, niter)
            assert len(tg) == len(tc) == niter
            for (i1, p1, a1, l1), (i2, p2, a2, l2) in zip(tg, tc):
                assert (i1, p1, a1) == (i2, p2, a2), (i1, p1, a1, i2, p2, a2)
                if l1 is not None:
                    np.testing.assert_allclose(l1, l2, rtol=LIKE_RTOL)
            assert gpu.ncells == cpu.ncells
            np.testing.assert_array_equal(gpu.points, cpu.points)
            np.testing.assert_array_equal(gpu.params, cpu.params)
            np.testing.assert_array_equal(gpu.sn0, cpu.sn0)
            # the chains moved: some proposals of several types were accepted
            assert sum(a for _, _, a, _ in tg) >= 3
            assert len({p for _, p, _, _ in tg}) >= 3
            gpu.close(); cpu.close()
    finally:
        lk.close()
