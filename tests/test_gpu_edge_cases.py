"""GPU parity edge cases of the mesh, point-cloud, impact and grid-pass paths: grids
touching every border, odd sizes, degenerate meshes, rays on the box faces
and signed-zero directions, extreme nearSeeds settings.  Bit-exact against
the oracle, as the main parity tests."""
import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as Vs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _mesh_parity(vf, ctx, g0, mn, mx, params):
    g = vf.RegularGrid(g0.shape, mn, mx, ctx)
    g.upload(g0)
    g.triangulate(params)
    got = g.meshes_arrays()
    e = O.triangulate(g0, mn, mx, params.nonboundary_iterations, params.nonboundary_weight,
                      params.boundary_iterations, params.boundary_weight)
    for a, b in zip(got, e):
        if a.dtype == np.float32:
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        else:
            assert np.array_equal(a, b)
    return g, got


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 2, 9), (2, 7, 2), (5, 5, 8), (4, 3, 17)])
def test_mesh_labels_on_every_border(vf, ctx, shape):
    rng = np.random.default_rng(sum(shape))
    g0 = rng.integers(2, 9, size=shape).astype(np.uint16)  # every voxel labelled
    g0 |= (rng.random(shape) < 0.3).astype(np.uint16) << 15
    g, _ = _mesh_parity(vf, ctx, g0, [0, 0, 0], list(shape), vf.MCParams(2, 0.5, 2, 0.5))
    g.close()


def test_mesh_single_voxel_corners(vf, ctx):
    for at in [(0, 0, 0), (6, 0, 0), (0, 5, 0), (0, 0, 10), (6, 5, 10)]:
        g0 = np.ones((7, 6, 11), np.uint16)
        g0[at] = 2
        g, got = _mesh_parity(vf, ctx, g0, [-1, -1, -1], [1, 1, 1], vf.MCParams(1, 0.9, 1, 0.2))
        assert len(got[3]) == 6 and len(got[4]) == 8
        g.close()


def test_point_clouds_small_counts_and_degenerate_meshes(vf, ctx):
    verts, faces = Vs.vessel_mesh(16, 12, 5)
    v4 = np.concatenate([verts, np.zeros((len(verts), 1), np.float32)], axis=1)
    f4 = np.concatenate([faces, np.zeros((len(faces), 1), np.uint32)], axis=1)
    for S in (1, 2, len(faces) - 1, len(faces), len(faces) + 1):
        got = vf.sample_mesh(verts, faces, S, 7, ctx)
        e = O.sample_mesh(v4, f4, S, 7, 0)
        assert np.array_equal(got.view(np.uint32), e.view(np.uint32)), S
    # every triangle degenerate (zero area): the area ratio is NaN, each face 1 sample
    dv = np.zeros((3, 3), np.float32)
    df = np.array([[0, 1, 2], [0, 0, 1], [2, 1, 0]], np.uint32)
    dv4 = np.concatenate([dv, np.zeros((3, 1), np.float32)], axis=1)
    df4 = np.concatenate([df, np.zeros((3, 1), np.uint32)], axis=1)
    for S in (2, 3, 10):
        got = vf.sample_mesh(dv, df, S, 3, ctx)
        e = O.sample_mesh(dv4, df4, S, 3, 0)
        assert np.array_equal(got.view(np.uint32), e.view(np.uint32)), S


def test_rays_on_box_faces_and_signed_zeros(vf, ctx):
    g0 = np.zeros((12, 10, 14), np.uint16)
    g0[3:9, 2:8, 4:11] = 1
    mn, mx = np.array([0, 0, 0], np.float32), np.array([12, 10, 14], np.float32)
    g = vf.RegularGrid(g0.shape, mn, mx, ctx)
    g.upload(g0)
    rays = []
    for o in ([0, 5.5, 7.5], [12, 5.5, 7.5], [6.5, 0, 7.5], [6.5, 10, 7.5], [6.5, 5.5, 0],
              [6.5, 5.5, 14], [3, 2, 4], [9, 8, 11]):
        for d in ([1, 0, 0], [-1, -0.0, 0], [0, 1, -0.0], [0, -1, 0], [-0.0, 0, 1], [0, 0, -1],
                  [1, 1, 1], [-1, 0.5, -0.25], [0.0, -0.0, -0.5]):
            rays.append(o + d)
    r = np.array(rays, np.float32)
    got = g.rayEntryVoxels(r)
    for i, rr in enumerate(r):
        e = O.ray_entry(g0, mn, mx, rr[:3], rr[3:])
        exp = np.array(e if e is not None else (0xFFFFFFFF,) * 3, np.uint32)
        assert np.array_equal(got[i], exp), (rr, got[i], exp)
    g.close()


@pytest.mark.parametrize("spread,nseeds", [(1, 1), (12, 8), (15, 4)])
def test_near_seeds_extreme_settings(vf, ctx, spread, nseeds):
    g0 = np.zeros((30, 32, 34), np.uint16)
    g0[5:25, 6:26, 7:27] = 1
    g = vf.RegularGrid(g0.shape, None, None, ctx)
    g.upload(g0)
    frags = O.seeder_uniform(g0, 3, 5, 1)
    got = vf.Seeder.nearSeeds(g, frags, 2, nseeds, spread, 13)
    assert np.array_equal(got, O.near_seeds(g0, frags, 2, nseeds, spread, 13))
    g.close()


# ---- grid passes on ragged grids: partial bricks in x, y and z ------------
# (Z = 13, 45, 66: the last z brick holds fewer than 32 voxels, so the row
# kernels' lanes past Zk / Zp must stay idle; X, Y are not multiples of 16)
@pytest.mark.parametrize("shape,gseed", [((21, 17, 13), 3), ((37, 29, 45), 4), ((18, 40, 66), 5)])
def test_grid_passes_on_ragged_grids(vf, ctx, shape, gseed):
    rng = np.random.default_rng(gseed)
    occ = (rng.random(shape) < 0.6).astype(np.uint16)
    seeds = O.seeder_uniform(occ, 9, gseed, 2)
    g = vf.RegularGrid(shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(2)
    fr.build(g, seeds)
    lab, _ = O.flood(occ, seeds, 2)
    assert np.array_equal(g.data(), lab)
    for amp, period, seed in ((2.0, 5, 7), (1.3, 16, 8)):
        g.upload(lab)
        g.perturb(amp, period, seed)
        assert np.array_equal(g.data(), O.perturb(lab, amp, period, seed))
    for bs in (0, 1, 2):
        g.upload(lab)
        g.detectBoundaries(bs)
        assert np.array_equal(g.data(), O.detect_boundaries(lab, bs))
    g.close()
