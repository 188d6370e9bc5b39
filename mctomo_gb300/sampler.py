"""The sampler's random stream and proposal steps (C ABI mct_rng_*,
mct_mcmc_*), mirroring the reference's mt19937 module and the
Metropolis-Hastings steps of src/mcmc_loc2.f90.

Chain holds one chain's state (RTI%points, RTI%parameters, noise levels)
and its generator; propose() applies one proposal in place (the caller keeps
a snapshot to restore on rejection, as the reference does) and accept()
runs the acceptance test.
"""
import ctypes

import numpy as np

from ._lib import check, lib

_D = ctypes.c_double
_I = ctypes.c_int
_P = ctypes.c_void_p


class McmcSet(ctypes.Structure):
    """The T_MCMC_SET fields the proposal steps read (include/mctomo.h)."""
    _fields_ = [(n, _I) for n in ("ncell_min", "ncell_max", "kernel", "datatype", "sigdep", "locate")] + \
               [(n, _D) for n in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "vpmin", "vpmax", "vsmin", "vsmax",
                                  "sigma_vp", "sigma_vs", "sigma_vp2", "sigma_vs2", "pd", "pd2",
                                  "sigma_bn0", "sigma_bn1", "bn0_min", "bn0_max", "bn1_min", "bn1_max",
                                  "sigma_sn0", "sigma_sn1", "sn0_min", "sn0_max", "sn1_min", "sn1_max")]


class McmcState(ctypes.Structure):
    _fields_ = [("ncells", _I), ("points", _P), ("parameters", _P), ("nbnoise", _I), ("nsnoise", _I),
                ("bnoise0", _P), ("bnoise1", _P), ("snoise0", _P), ("snoise1", _P)]


class McmcStep(ctypes.Structure):
    _fields_ = [("ptype", _I), ("index", _I), ("valid", _I), ("prob", _D), ("random", _D)]


class Chain:
    """One chain: seed for init_genrand, the initial nuclei (ncells, points
    (ncell_max, 3), params (ncell_max, 3)) and noise levels."""

    def __init__(self, settings, seed, ncells, points, params, snoise0=(), snoise1=(), bnoise0=(), bnoise1=()):
        self.set = McmcSet(**settings)
        self.rng = ctypes.c_void_p()
        check("mct_rng_create", lib().mct_rng_create(seed, ctypes.byref(self.rng)))
        nmax = self.set.ncell_max
        self.ncells = int(ncells)
        self.points = np.zeros((nmax, 3)); self.points[:ncells] = points[:ncells]
        self.params = np.zeros((nmax, 3)); self.params[:ncells] = params[:ncells]
        self.sn0 = np.array(snoise0, np.float64); self.sn1 = np.array(snoise1, np.float64)
        self.bn0 = np.array(bnoise0, np.float64); self.bn1 = np.array(bnoise1, np.float64)

    def close(self):
        if self.rng:
            lib().mct_rng_destroy(self.rng)
            self.rng = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def snapshot(self):
        return (self.ncells, self.points.copy(), self.params.copy(), self.sn0.copy(), self.sn1.copy(),
                self.bn0.copy(), self.bn1.copy())

    def restore(self, snap):
        self.ncells = snap[0]
        for dst, src in zip((self.points, self.params, self.sn0, self.sn1, self.bn0, self.bn1), snap[1:]):
            dst[...] = src

    def propose(self, it, redo=False, step=None):
        """One proposal of iteration it applied in place; with redo, the type
        and acceptance draw of step are kept. Returns the step."""
        step = step if step is not None else McmcStep()
        ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
        st = McmcState(self.ncells, self.points.ctypes.data, self.params.ctypes.data, self.bn0.size, self.sn0.size,
                       ptr(self.bn0), ptr(self.bn1), ptr(self.sn0), ptr(self.sn1))
        check("mct_mcmc_propose", lib().mct_mcmc_propose(ctypes.byref(self.set), self.rng, int(it), 1 if redo else 0,
                                                        ctypes.byref(st), ctypes.byref(step)))
        self.ncells = st.ncells
        return step

    def accept(self, step, like_new, like_old):
        return lib().mct_mcmc_accept(ctypes.byref(self.set), ctypes.byref(step), float(like_new),
                                     float(like_old)) == 1

    def record(self, step, accepted, like, misfit, unweighted_misfit):
        """The iteration's T_SAMPLE after the acceptance test (the state as
        restored on rejection)."""
        ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
        st = McmcState(self.ncells, self.points.ctypes.data, self.params.ctypes.data, self.bn0.size, self.sn0.size,
                       ptr(self.bn0), ptr(self.bn1), ptr(self.sn0), ptr(self.sn1))
        sm = Sample()
        check("mct_mcmc_record", lib().mct_mcmc_record(ctypes.byref(st), ctypes.byref(step), 1 if accepted else 0,
                                                       float(like), float(misfit), float(unweighted_misfit),
                                                       ctypes.byref(sm)))
        return sm

    def accept_tempered(self, step, like_new, like_old, temperature):
        """The acceptance test of mcmc_pt: the likelihood ratio over the
        chain's temperature."""
        rc = lib().mct_mcmc_accept_tempered(ctypes.byref(self.set), ctypes.byref(step), float(like_new),
                                            float(like_old), float(temperature))
        return check("mct_mcmc_accept_tempered", rc) == 1


class Sample(ctypes.Structure):
    """T_SAMPLE (src/run_time_info.f90:62-76): one iteration's record."""
    _fields_ = [("step", _I), ("accepted", _I), ("vindex", _I), ("ncells", ctypes.c_longlong),
                ("misfit", _D), ("unweighted_misfit", _D), ("like", _D), ("coord", _D * 3), ("values", _D * 3),
                ("noise0", _D), ("noise1", _D)]


def write_samples(filename, samples, dim=3):
    """Appends records to a sample stream file (write_samples' layout)."""
    arr = (Sample * len(samples))(*samples)
    check("mct_samples_write", lib().mct_samples_write(str(filename).encode(), int(dim), arr, len(samples)))


def read_samples(filename, n, dim=3):
    """Up to n records of a sample stream file."""
    arr = (Sample * n)()
    got = check("mct_samples_read", lib().mct_samples_read(str(filename).encode(), int(dim), arr, n))
    return list(arr[:got])


class Pt(ctypes.Structure):
    _fields_ = [("nchains", _I), ("number_of_1s", _I), ("jump_type", _I), ("values0", _P), ("values", _P),
                ("indices", _P), ("accepted", ctypes.c_longlong), ("total", ctypes.c_longlong)]


class Tempering:
    """Parallel tempering over chains 1..n (mct_pt_*): ladder = number_of_1s
    ones followed by the temperature file's values; jump_type as in the
    reference's settings. choose() and swap() draw from the given chain's
    generator (the reference uses its first process's stream)."""

    def __init__(self, ladder, number_of_1s, jump_type=0):
        self.values0 = np.ascontiguousarray(ladder, np.float64)
        n = self.values0.size
        self.values = np.zeros(n)
        self.indices = np.zeros(n, np.int32)
        self.pt = Pt(n, int(number_of_1s), int(jump_type), self.values0.ctypes.data, self.values.ctypes.data,
                     self.indices.ctypes.data, 0, 0)
        check("mct_pt_init", lib().mct_pt_init(ctypes.byref(self.pt)))

    def choose(self, chain):
        t1, t2 = _I(), _I()
        check("mct_pt_choose", lib().mct_pt_choose(ctypes.byref(self.pt), chain.rng, ctypes.byref(t1),
                                                   ctypes.byref(t2)))
        return t1.value, t2.value

    def swap(self, chain, t1, t2, like1, like2):
        rc = lib().mct_pt_swap(ctypes.byref(self.pt), chain.rng, int(t1), int(t2), float(like1), float(like2))
        return check("mct_pt_swap", rc) == 1

    @property
    def accepted(self):
        return self.pt.accepted

    @property
    def total(self):
        return self.pt.total
