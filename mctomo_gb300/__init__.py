"""GB300 (sm_103a) forward-modelling hot path of MCTomo's rjMCMC.

The compute runs in ``libmctomo_gpu.so`` (hand-written CUDA, C ABI in
include/mctomo.h). This package is the Python mirror of the reference's
forward-modelling call surface (kdtree_to_grid, surfdisp96 / surfmodes,
modrays, fastMarching3D and the likelihood calls of the surface-wave,
body-wave and 2D travel-time paths).
"""
from ._lib import MctError, lib, LIB_PATH  # noqa: F401
from .surface import SurfaceLikelihood  # noqa: F401
from .body import BodyLikelihood  # noqa: F401
from .tt2d import TravelTime2DLikelihood  # noqa: F401
from .forward import (  # noqa: F401
    kdtree_to_grid, surfdisp96, surfdisp_mmodes, surfmodes, surfmodes_para, modes_para, grt_batch, surfmodes_route,
    surfdisp_batch,
    modrays, modrays_batch,
    modrays_group_batch, fast_marching3d, eikonal3d_batch,
)

__version__ = "0.1.0"
