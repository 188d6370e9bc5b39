"""GPU: the allocation-free gridding entry point gives the same grids as the
allocating one (bit-exact, two calls in a row), through the C ABI.

Named to be collected last, so that it also runs after every other test has
used the library in the same process.
"""
import ctypes

import numpy as np
import pytest

from mctomo_gb300 import synthetic

pytestmark = pytest.mark.gpu

NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024


def _inputs(torch, d, nchains, ncell_max, shape, seed, with_box):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    lo = np.array([-2.0, 0.5, 0.0]); st = np.array([0.5, 0.45, 0.3])
    hi = lo + st * (np.array(shape) - 1)
    ncells = rng.integers(max(4, ncell_max // 3), ncell_max + 1, nchains).astype(np.int32)
    pts = np.zeros((nchains, ncell_max, d)); par = np.zeros((nchains, ncell_max, 3))
    for c in range(nchains):
        p, q = synthetic.voronoi_model_3d(rng, int(ncells[c]), lo, hi, (0.3, 2.5))
        pts[c, :ncells[c]] = p[:, :d]
        par[c, :ncells[c]] = q
    boxes = None
    if with_box:
        b = []
        for _ in range(nchains):
            ix = np.sort(rng.integers(1, nx + 1, 2)); iy = np.sort(rng.integers(1, ny + 1, 2))
            iz = np.sort(rng.integers(1, nz + 1, 2)) if d == 3 else np.array([1, 1])
            b.append([ix[0], ix[1], iy[0], iy[1], iz[0], iz[1]])
        boxes = torch.tensor(np.array(b, np.int32), device="cuda")
    dev = dict(ncells=torch.tensor(ncells, device="cuda"),
               pts=torch.tensor(pts, device="cuda"), par=torch.tensor(par, device="cuda"),
               lo=torch.tensor(lo[:d].copy(), device="cuda"), st=torch.tensor(st[:d].copy(), device="cuda"),
               box=boxes)
    return dev, lo, st


def _run(torch, lib, fn, d, nchains, ncell_max, shape, dev, lo, st):
    nx, ny, nz = shape
    nodes = nx * ny * (nz if d == 3 else 1)
    # outputs start from a sentinel so nodes outside the boxes are compared too
    sid = torch.full((nchains, nodes), -7, dtype=torch.int32, device="cuda")
    vel = torch.full((3, nchains, nodes), -1.5, dtype=torch.float64, device="cuda")
    lo_h = np.ascontiguousarray(lo[:3]); st_h = np.ascontiguousarray(st[:3])
    s = torch.cuda.current_stream().cuda_stream
    box = dev["box"].data_ptr() if dev["box"] is not None else None
    rc = getattr(lib, fn)(d, nchains, ncell_max, dev["ncells"].data_ptr(), dev["pts"].data_ptr(),
                          dev["par"].data_ptr(), nx, ny, nz if d == 3 else 1,
                          lo_h.ctypes.data_as(ctypes.c_void_p), st_h.ctypes.data_as(ctypes.c_void_p),
                          box, sid.data_ptr(), vel[0].data_ptr(), vel[1].data_ptr(), vel[2].data_ptr(), s)
    assert rc == 0, lib.mct_last_error()
    torch.cuda.synchronize()
    return sid.cpu().numpy(), vel.cpu().numpy()


@pytest.mark.parametrize("d,nchains,ncell_max,shape,with_box", [
    (3, 4, 300, (41, 37, 23), False),
    (3, 6, 120, (30, 28, 17), True),
    (2, 5, 60, (51, 47, 1), False),
])
def test_noalloc_matches_allocating_entry(gpulib, d, nchains, ncell_max, shape, with_box):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    dev, lo, st = _inputs(torch, d, nchains, ncell_max, shape, 100 + nchains, with_box)
    ref = _run(torch, gpulib, "mct_grid_nearest_batch_device", d, nchains, ncell_max, shape, dev, lo, st)
    assert (ref[0][:, :] > 0).any()
    for _ in range(2):  # two calls in a row reuse the fixed scratch
        got = _run(torch, gpulib, "mct_grid_nearest_batch_device_noalloc", d, nchains, ncell_max, shape,
                   dev, lo, st)
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])


def test_noalloc_resolves_ties_like_allocating_entry(gpulib):
    # Nuclei mirrored across grid planes put many nodes at exactly equal
    # distances from two nuclei. Those nodes are resolved by the kd-tree
    # search, whose per-chain tree storage sits in the fixed scratch array.
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(9)
    nchains, shape = 3, (21, 21, 11)
    lo = np.zeros(3); st = np.ones(3)
    models, bases = [], []
    for c in range(nchains):
        base = rng.integers(1, 19, (40 + 10 * c, 3)).astype(float)
        base[:, 2] = rng.integers(1, 10, len(base))
        p = np.unique(np.concatenate([base + [0.5, 0, 0], base - [0.5, 0, 0], base + [0, 0.5, 0.5]]), axis=0)
        models.append(p)
        bases.append(base)
    ncell_max = max(len(p) for p in models)
    pts = np.zeros((nchains, ncell_max, 3)); par = np.zeros((nchains, ncell_max, 3))
    for c, p in enumerate(models):
        pts[c, :len(p)] = p
        par[c, :len(p)] = np.stack([np.arange(len(p)) + 1.0, np.arange(len(p)) * 0.5 + 1, np.ones(len(p))], 1)
    # the inputs really hold exact ties: grid node `base` lies halfway
    # between its nucleus pair at x +- 0.5, with nothing closer
    d2 = ((models[0][None] - bases[0][:, None]) ** 2).sum(-1)
    d2.sort(axis=1)
    assert (d2[:, 0] == d2[:, 1]).all()
    ncells = np.array([len(p) for p in models], np.int32)
    dev = dict(ncells=torch.tensor(ncells, device="cuda"), pts=torch.tensor(pts, device="cuda"),
               par=torch.tensor(par, device="cuda"), box=None)
    ref = _run(torch, gpulib, "mct_grid_nearest_batch_device", 3, nchains, ncell_max, shape, dev, lo, st)
    for _ in range(2):
        got = _run(torch, gpulib, "mct_grid_nearest_batch_device_noalloc", 3, nchains, ncell_max, shape,
                   dev, lo, st)
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])


def test_noalloc_rejects_oversized_call(gpulib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    # 64 chains of a 101x101x51 grid need ~133 MB of tie lists: rejected
    # before anything is launched, with the size in the message
    nx, ny, nz, nchains, ncell_max = 101, 101, 51, 64, 100
    assert 4 * nchains * nx * ny * nz > NOALLOC_SCRATCH_BYTES
    lo = np.zeros(3); st = np.ones(3)
    rc = gpulib.mct_grid_nearest_batch_device_noalloc(
        3, nchains, ncell_max, None, None, None, nx, ny, nz,
        lo.ctypes.data_as(ctypes.c_void_p), st.ctypes.data_as(ctypes.c_void_p),
        None, None, None, None, None, None)
    assert rc == -1
    assert b"scratch" in gpulib.mct_last_error()
