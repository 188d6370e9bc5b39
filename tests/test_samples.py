"""CPU: the sample stream (mct_mcmc_record, mct_samples_write / _read).

The byte layout is the reference's write_samples (src/run_time_info.f90:
306-340, stream access, unpadded): the reference's own reader
plot/plot_point_values.m:46-56 takes int32 step, 1-byte accepted, int32
vindex, int64 ncells, misfit, unweighted misfit, like, the coordinates (2
in the 2D code), 3 values, noise0, noise1. The records follow the MCMC
loop's filling (src/mcmc_loc2.f90:253-263, 305-315, 345-355, 425-436,
487-497, 578-582)."""
import struct

import numpy as np
import pytest

from mctomo_gb300 import sampler

SETTINGS = dict(ncell_min=2, ncell_max=20, kernel=1, datatype=2, sigdep=1, locate=0, xmin=0.0, xmax=10.0,
                ymin=0.0, ymax=8.0, zmin=0.0, zmax=3.0, vpmin=0.5, vpmax=4.5, vsmin=0.3, vsmax=2.5,
                sigma_vp=0.1, sigma_vs=0.08, sigma_vp2=0.1, sigma_vs2=0.08, pd=5.0, pd2=8.0,
                sigma_bn0=0.0, sigma_bn1=0.0, bn0_min=0.0, bn0_max=1.0, bn1_min=0.0, bn1_max=1.0,
                sigma_sn0=0.002, sigma_sn1=0.01, sn0_min=0.001, sn0_max=0.1, sn1_min=0.0, sn1_max=0.5)


def make_chain(seed=3, n=6):
    rng = np.random.default_rng(seed)
    pts = rng.uniform([0, 0, 0], [10, 8, 3], (n, 3))
    vs = np.sort(rng.uniform(0.3, 2.5, n))
    par = np.stack([vs * 1.73, vs, np.full(n, 2.0)], 1)
    return sampler.Chain(SETTINGS, seed, n, pts, par, snoise0=[0.02, 0.03], snoise1=[0.1, 0.2])


def test_records_follow_the_loop():
    ch = make_chain()
    step = sampler.McmcStep()
    seen = set()
    try:
        for it in range(1, 400):
            snap = ch.snapshot()
            ch.propose(it, False, step)
            accepted = bool(step.valid) and (it % 3 != 0)
            if not accepted:
                ch.restore(snap)
            sm = ch.record(step, accepted, 100.0 + it, 50.0 + it, 25.0 + it)
            assert sm.step == step.ptype and sm.accepted == int(accepted)
            assert (sm.ncells, sm.like, sm.misfit, sm.unweighted_misfit) == (ch.ncells, 100.0 + it, 50.0 + it,
                                                                               25.0 + it)
            i = step.index - 1
            if not accepted:
                assert sm.vindex == 0 and not any(sm.coord) and not any(sm.values) and sm.noise0 == sm.noise1 == 0
            elif step.ptype == 1:       # birth: the new nucleus and its values
                assert sm.vindex == 0 and list(sm.coord) == list(ch.points[i]) and list(sm.values) == list(ch.params[i])
            elif step.ptype == 2:       # death: the removed cell
                assert sm.vindex == step.index and not any(sm.coord) and not any(sm.values)
            elif step.ptype == 3:       # move: the moved nucleus
                assert sm.vindex == step.index and list(sm.coord) == list(ch.points[i]) and not any(sm.values)
            elif step.ptype == 4:       # value change: the new values
                assert sm.vindex == step.index and not any(sm.coord) and list(sm.values) == list(ch.params[i])
            elif step.ptype == 6:       # surface-wave noise
                assert sm.vindex == step.index and (sm.noise0, sm.noise1) == (ch.sn0[i], ch.sn1[i])
            if accepted:
                seen.add(step.ptype)
    finally:
        ch.close()
    assert {1, 2, 3, 4, 6} <= seen


@pytest.mark.parametrize("dim", [2, 3])
def test_stream_layout_and_round_trip(tmp_path, dim):
    recs = []
    for k in range(5):
        s = sampler.Sample()
        s.step, s.accepted, s.vindex, s.ncells = k + 1, k % 2, 3 * k, 10 ** 10 + k
        s.misfit, s.unweighted_misfit, s.like = 1.5 * k, 2.5 * k, -3.25 * k
        s.coord[:] = [k + 0.1, k + 0.2, k + 0.3]
        s.values[:] = [4.0 + k, 2.0 + k, 2.5]
        s.noise0, s.noise1 = 0.01 * k, 0.02 * k
        recs.append(s)
    f = tmp_path / "samples_1.out"
    sampler.write_samples(f, recs[:2], dim)
    sampler.write_samples(f, recs[2:], dim)           # appends, as write_samples does
    raw = f.read_bytes()
    fmt = "<iBiq3d" + "d" * dim + "3d2d"
    assert len(raw) == 5 * struct.calcsize(fmt) == 5 * (81 + 8 * dim)
    for k, s in enumerate(recs):
        v = struct.unpack_from(fmt, raw, k * struct.calcsize(fmt))
        assert v[:4] == (s.step, s.accepted, s.vindex, s.ncells)
        assert v[4:7] == (s.misfit, s.unweighted_misfit, s.like)
        assert list(v[7:7 + dim]) == list(s.coord[:dim])
        assert list(v[7 + dim:10 + dim]) == list(s.values) and v[10 + dim:] == (s.noise0, s.noise1)
    back = sampler.read_samples(f, 10, dim)
    assert len(back) == 5
    for a, b in zip(back, recs):
        assert (a.step, a.accepted, a.vindex, a.ncells, a.like) == (b.step, b.accepted, b.vindex, b.ncells, b.like)
        assert list(a.coord[:dim]) == list(b.coord[:dim]) and list(a.values) == list(b.values)
