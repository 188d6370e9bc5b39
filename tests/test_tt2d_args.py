"""CPU: argument checks of the 2D travel-time context that return before
any device work (the library loads without a GPU)."""
import ctypes

import numpy as np

from mctomo_gb300 import _lib
from mctomo_gb300.surface import Grid
from mctomo_gb300.tt2d import TT2DData, TT2DSettings


def _create(nsrc, nrev, datatype):
    lib = _lib.lib()
    g = Grid(nx=11, ny=11, nz=1, xmin=0.0, ymin=0.0, zmin=0.0, dx=1.0, dy=1.0, dz=1.0, scaling=1.0,
             water_depth=0.0)
    s = TT2DSettings(gridx=1, gridy=1, sgref=0, sgdic=1, sgext=1, order=1, sigdep=1, datatype=datatype, straight=0,
                     precision=0)
    src = np.zeros((nsrc, 2)) + 1.0; rev = np.zeros((nrev, 2)) + 2.0
    rays = np.ones(nsrc * nrev, np.int32); tt = np.ones(nsrc * nrev)
    ndd = nsrc * (nsrc - 1) // 2
    dt = np.ones((max(ndd, 1), nrev)); dcc = np.zeros_like(dt)
    d = TT2DData(nsrc, nrev, src.ctypes.data, rev.ctypes.data, rays.ctypes.data, tt.ctypes.data, None, nsrc * nrev,
                 dt.ctypes.data, dcc.ctypes.data, 0)
    h = ctypes.c_void_p()
    return lib.mct_tt2d_create(ctypes.byref(g), ctypes.byref(s), ctypes.byref(d), 2, 10, ctypes.byref(h))


def test_swapped_index_read_outside_dtime_is_refused():
    # 2 sources, 10 receivers: the reference's test abs(dat%dtime(ddindex,k,1))
    # reads element ddindex + (k-1)*nrev of a (10, 1) array
    assert _create(2, 10, 1) == -1
    assert b"outside dtime" in _lib.lib().mct_last_error()


def test_bad_settings_are_refused():
    assert _create(3, 3, 2) == -1     # datatype 2 is not a travel-time likelihood
