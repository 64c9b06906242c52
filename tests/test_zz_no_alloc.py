"""The flood entry point that allocates no device memory, vf_flood_noalloc.

It exists for callers that cannot allocate while this step runs (their
device memory belongs to a pool of their own, or must not grow after
start-up): they pass their own device buffers and the library uses a fixed
scratch array of its own.  This test calls it through the C ABI on device
buffers owned by the test and checks its labels against the regular flood
entry point (vf_fracture through a grid), bit for bit, on two calls in a
row.  The file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as Vs

pytestmark = pytest.mark.gpu


def _device_call(vf, occ, seeds, dfunc, expect=0):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = torch.from_numpy(occ.astype(np.uint16).view(np.int16)).cuda()
    out = torch.full(occ.shape, -1, dtype=torch.int16, device="cuda")
    s = torch.from_numpy(seeds.astype(np.uint32).view(np.int32).reshape(-1, 4)).cuda() \
        if len(seeds) else None
    torch.cuda.synchronize()
    X, Y, Z = occ.shape
    st = vf.lib().vf_flood_noalloc(C.c_void_p(g.data_ptr()), C.c_void_p(out.data_ptr()),
                                   X, Y, Z, C.c_void_p(s.data_ptr()) if s is not None else None,
                                   len(seeds), dfunc, None)
    assert st == expect, vf.lib().vf_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint16)


def _regular(vf, ctx, occ, seeds, dfunc):
    grid = vf.RegularGrid(occ.shape, None, None, ctx)
    grid.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(dfunc)
    fr.build(grid, seeds)
    return grid.data()


def test_flood_noalloc_matches_regular_entry_point_twice(vf, ctx, oracle_lib):
    v, f = Vs.vessel_mesh(64, 48, 5)
    mn, mx = Vs.mesh_aabb(v)
    dims = Vs.grid_dims(mn, mx, 60)   # Z % 8 == 4: padded rows inside the scratch
    occ = O.voxelize(v, f, dims, mn, mx)
    cases = [(O.seeder_uniform(occ, 9, 3, 2), 1), (O.seeder_uniform(occ, 21, 4, 2), 2)]
    for seeds, dfunc in cases:  # two calls in a row share the scratch array
        got = _device_call(vf, occ, seeds, dfunc)
        exp = _regular(vf, ctx, occ, seeds, dfunc)
        assert np.array_equal(got, exp)
        assert np.array_equal(got, O.flood(occ, seeds, dfunc)[0])


def test_flood_noalloc_edge_cases(vf, ctx, oracle_lib):
    rng = np.random.default_rng(11)
    # no seeds: occupied voxels come out FREE (1), empty ones EMPTY (0)
    occ = (rng.random((20, 17, 9)) < 0.6).astype(np.uint16)
    got = _device_call(vf, occ, np.zeros((0, 4), np.uint32), 1)
    assert np.array_equal(got, O.flood(occ, np.zeros((0, 4), np.uint32), 1)[0])
    assert np.array_equal(got, (occ != 0).astype(np.uint16))
    # grids one voxel wide along each axis (seeds picked directly: the
    # seeder needs two layers per axis)
    for shape in ((1, 23, 40), (31, 1, 18), (12, 26, 1)):
        occ = (rng.random(shape) < 0.7).astype(np.uint16)
        occv = np.argwhere(occ != 0)
        pick = occv[rng.choice(len(occv), 3, replace=False)]
        seeds = np.concatenate([pick, np.arange(2, 5)[:, None]], axis=1).astype(np.uint32)
        for dfunc in (1, 2):
            got = _device_call(vf, occ, seeds, dfunc)
            assert np.array_equal(got, O.flood(occ, seeds, dfunc)[0]), shape


def test_flood_noalloc_rejects_bad_seeds(vf, ctx):
    occ = np.ones((16, 16, 16), np.uint16)
    # a seed outside the grid, and a label with a sub-seed prefix (> 255)
    outside = np.array([[3, 3, 3, 2], [3, 16, 3, 3]], np.uint32)
    _device_call(vf, occ, outside, 1, expect=vf.ERR_INVALID)
    prefixed = np.array([[3, 3, 3, 2], [9, 9, 9, 2 | (1 << 8)]], np.uint32)
    _device_call(vf, occ, prefixed, 2, expect=vf.ERR_INVALID)
    # the next valid call is unaffected by the failed ones
    seeds = np.array([[1, 2, 3, 2], [12, 12, 12, 3]], np.uint32)
    got = _device_call(vf, occ, seeds, 1)
    assert np.array_equal(got, O.flood(occ, seeds, 1)[0])


def test_flood_noalloc_rejects_oversize(vf, ctx):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = torch.zeros(8, dtype=torch.int16, device="cuda")
    st = vf.lib().vf_flood_noalloc(C.c_void_p(g.data_ptr()), C.c_void_p(g.data_ptr()),
                                   512, 512, 512, None, 0, 1, None)
    assert st == vf.ERR_RANGE
    assert b"scratch" in vf.lib().vf_last_error()
