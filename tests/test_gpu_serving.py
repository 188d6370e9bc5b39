"""GPU end to end of the serving loop: a Poisson stream of chains of four
kinds (2D travel times, surface waves, body waves, joint surface + body) is
served by batched workers on their own contexts and streams, with chains
admitted into free slots between steps and leaving after their proposals;
then every chain is run again alone through a one-slot context, one call
per proposal (the plain drop-in). Each chain's trace (its -log L after each
step, which also fixes every Metropolis decision) is the same in the mix as
alone, bit for bit (the body kinds use the exact heap march here; the tile
solver's times agree alone and in the mix within a few fixed-point units,
tests/test_gpu_body.py)."""
import time

import numpy as np
import pytest

from mctomo_gb300 import BodyLikelihood, SurfaceLikelihood, TravelTime2DLikelihood, serving, synthetic

pytestmark = pytest.mark.gpu
PROPOSALS = 3


def kinds(single):
    """Backends of the four kinds on small shapes; single: one-slot contexts
    with one chain per call."""
    rng = np.random.default_rng(90)
    n = 1 if single else 3
    g2, s2, d2 = synthetic.tt2d_workload(rng)
    nm, pr = synthetic.serving_models("tt2d", g2, 30, (4, 30))
    tt2d = serving.TT2DBackend(TravelTime2DLikelihood(g2, s2, d2, nslots=n, ncell_max=30), n, nm, pr,
                               single=single)
    gs, ss, ds = synthetic.surface_workload(rng, nx=21, ny=19, nz=11, extent=(20.0, 18.0, 3.0), nstations=8,
                                            nperiods=4, pmin=0.5, pmax=3.0)
    nm, pr = synthetic.serving_models("surface", gs, 30, (6, 30))
    surf = serving.SurfaceBackend(SurfaceLikelihood(gs, ss, ds, nslots=n, ncell_max=30), n, nm, pr, 4,
                                  single=single)
    gb, sb, db, ev = synthetic.body_workload(rng, nx=31, ny=29, nz=17, extent=(15.0, 14.0, 8.0), nevents=24,
                                             nstations=9)
    sb["order"] = 1
    sb["solver"] = 0x20        # the exact heap march: times independent of the call's other chains
    nm, pr = synthetic.serving_models("body", gb, 30, (6, 30))
    body = serving.BodyBackend(BodyLikelihood(gb, sb, db, nslots=n, ncell_max=30), n, nm, pr, ev, single=single)
    # joint: the body grid's models on a surface context over the same area
    gj, sj, dj = synthetic.surface_workload(rng, nx=16, ny=15, nz=9, extent=(15.0, 14.0, 8.0), nstations=6,
                                            nperiods=3, pmin=0.5, pmax=3.0)
    nmj, prj = synthetic.serving_models("joint", gb, 30, (6, 30))
    js = serving.SurfaceBackend(SurfaceLikelihood(gj, sj, dj, nslots=n, ncell_max=30), n, nmj, prj, 3,
                                single=single)
    jb = serving.BodyBackend(BodyLikelihood(gb, sb, db, nslots=n, ncell_max=30), n, nmj, prj, ev, single=single)
    return {"tt2d": tt2d, "surface": surf, "body": body, "joint": serving.JointBackend(js, jb)}


def test_served_chains_are_the_same_alone_and_in_the_mix(gpulib):
    rng = np.random.default_rng(91)
    names = ["tt2d", "surface", "body", "joint"]
    arrivals = serving.poisson_arrivals(rng, 20.0, 1.0, names)
    assert len(arrivals) >= 8
    backends = kinds(False)
    workers = [serving.Worker(k, backends[k], PROPOSALS) for k in names]
    stats, mix = serving.run_stream(workers, arrivals, duration=90.0, window=(0.0, 90.0), seed=3, until_done=True)
    assert all(ch.t_done is not None for ch in mix), [(ch.kind, ch.nprop) for ch in mix]
    for w in workers:
        assert len(w.done) == stats["kinds"][w.kind]["arrived"]
    # slots were reused when more chains of a kind arrived than it has slots
    assert any(stats["kinds"][k]["arrived"] > 3 for k in names)
    alone = kinds(True)
    for ch in mix:
        w = serving.Worker(ch.kind, alone[ch.kind], PROPOSALS, plain=True)
        w.start()
        c1 = serving.Chain(ch.cid, ch.kind, time.perf_counter(), 3 * 1000003 + ch.cid)
        w.submit(c1)
        t0 = time.time()
        while c1.t_done is None and w.error is None and time.time() - t0 < 120:
            time.sleep(0.002)
        w.stop.set(); w.join()
        assert w.error is None, w.error
        assert c1.trace == ch.trace, (ch.kind, ch.cid)
        assert all(np.isfinite(ch.trace)) and len(ch.trace) == PROPOSALS + 1
