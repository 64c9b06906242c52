"""GPU parity: every stage of the CUDA path, called through the C ABI,
bit-exact against the CPU oracle on the same seeded inputs, and every
golden case end to end (batched and plain paths).

Tolerance: none.  Labels, occupancy and counts are integer results and must
be identical; the float parts (tri-box SAT, tetra cross-sections, noise,
erosion activation) round exactly as the oracle does.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as Vs

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _mg():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


CASES = sorted(json.load(open(os.path.join(GOLD, "cases.json"))))


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


# (angular, profile, mesh seed, max_dim): includes Z % 8 == 4 and dims that
# are not multiples of the 16x16x32 brick
VOX_CASES = [(32, 24, 1, 32), (48, 36, 2, 60), (64, 48, 3, 76), (96, 72, 4, 100), (40, 30, 5, 44),
             (12, 9, 6, 128), (24, 18, 7, 200), (200, 150, 8, 64)]  # coarse/fine meshes


def _mesh(A, P, ms, md):
    v, f = Vs.vessel_mesh(A, P, ms)
    mn, mx = Vs.mesh_aabb(v)
    return v, f, mn, mx, Vs.grid_dims(mn, mx, md)


@pytest.mark.parametrize("case", VOX_CASES)
def test_voxelize(vf, ctx, case):
    v, f, mn, mx, dims = _mesh(*case)
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    got = g.data()
    exp = O.voxelize(v, f, dims, mn, mx)
    assert np.array_equal(got, exp), f"{int((got != exp).sum())} voxels differ"


def _soup(seed):
    """Open, non-manifold and degenerate meshes: random triangle soups (some on
    a coarse lattice, so vertices share slice planes and pixel centres),
    faces with a repeated vertex, duplicated faces."""
    rng = np.random.default_rng(seed)
    nv = int(rng.integers(3, 60))
    nf = int(rng.integers(1, 90))
    v = rng.random((nv, 3)).astype(np.float32)
    if seed % 3 == 0:
        v = (np.round(v * 8) / 8).astype(np.float32)
    f = rng.integers(0, nv, (nf, 3)).astype(np.uint32)
    if seed % 4 == 1:
        f = np.concatenate([f, f[: nf // 2]])
    dims = tuple(int(x) for x in rng.integers(4, 48, 3))
    return v, f, v.min(0), v.max(0), dims


@pytest.mark.parametrize("seed", range(12))
def test_voxelize_open_and_degenerate_meshes(vf, ctx, seed):
    v, f, mn, mx, dims = _soup(seed)
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    got = g.data()
    exp = O.voxelize(v, f, dims, mn, mx)
    assert np.array_equal(got, exp), f"{int((got != exp).sum())} voxels differ"


@pytest.mark.parametrize("scale,offset", [(1.0, (1000.0, -500.0, 2000.0)), (1e-3, (0.0, 0.0, 0.0)),
                                          (250.0, (-3.0e4, 1.0e4, 7.0)), (1.0, (0.3, 0.1, -0.2))])
def test_voxelize_offset_and_scaled_meshes(vf, ctx, scale, offset):
    # large coordinates against small cells: float rounding in the SAT is a
    # sizeable fraction of a cell, so candidate pruning must not drop a cell
    v, f = Vs.vessel_mesh(48, 36, 11)
    v = (v.astype(np.float64) * scale + np.array(offset)).astype(np.float32)
    mn, mx = Vs.mesh_aabb(v)
    dims = Vs.grid_dims(mn, mx, 64)
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    got = g.data()
    exp = O.voxelize(v, f, dims, mn, mx)
    assert np.array_equal(got, exp), f"{int((got != exp).sum())} voxels differ"


def test_voxelize_closed_mesh_with_extra_faces(vf, ctx):
    # a closed vessel plus duplicated faces (even and odd edge multiplicities)
    v, f = Vs.vessel_mesh(24, 18, 3)
    mn, mx = Vs.mesh_aabb(v)
    f2 = np.concatenate([f, f[:50], f[10:13]])
    dims = Vs.grid_dims(mn, mx, 48)
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f2)
    assert np.array_equal(g.data(), O.voxelize(v, f2, dims, mn, mx))


def test_voxelize_anisotropic_cells(vf, ctx):
    v, f = Vs.vessel_mesh(40, 30, 9)
    mn, mx = Vs.mesh_aabb(v)
    dims = (36, 52, 28)  # cells are not cubes
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    assert np.array_equal(g.data(), O.voxelize(v, f, dims, mn, mx))


@pytest.fixture(scope="module")
def occ64(vf, ctx):
    v, f, mn, mx, dims = _mesh(64, 48, 3, 64)
    return O.voxelize(v, f, dims, mn, mx), mn, mx


@pytest.mark.parametrize("loc", [0, 1, 2])
def test_seeds(vf, ctx, occ64, loc):
    occ, mn, mx = occ64
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    n = 3 if loc == 0 else 24
    got = vf.Seeder.uniform(g, n, 1234 + loc, loc)
    exp = O.seeder_uniform(occ, n, 1234 + loc, loc)
    assert np.array_equal(got, exp)


def test_fracture_seeds_with_extra(vf, ctx, occ64):
    occ, mn, mx = occ64
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    p = vf.Params.default(num_seeds=7, num_extra_seeds=14, seed=5, seed_location=vf.BOTH,
                          merge_distance=vf.MANHATTAN)
    got = vf.Seeder.fracture_seeds(g, p)
    exp = O.fracture_seeds(occ, 7, 14, vf.BOTH, vf.MANHATTAN, 5)
    assert np.array_equal(got, exp)


def test_seed_search_error(vf, ctx):
    occ = np.zeros((16, 16, 16), np.uint16)
    occ[4, 4, 4] = 1
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    with pytest.raises(vf.VFError) as e:
        vf.Seeder.uniform(g, 2, 1, vf.BOTH)
    assert e.value.status == vf.ERR_SEED_SEARCH


@pytest.mark.parametrize("dfunc", [0, 1, 2])
@pytest.mark.parametrize("nseeds", [1, 8, 40])
def test_flood_vessel(vf, ctx, occ64, dfunc, nseeds):
    occ, mn, mx = occ64
    seeds = O.seeder_uniform(occ, nseeds, 77 + nseeds, 2)
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(dfunc)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, dfunc)
    got = g.data()
    assert np.array_equal(got, exp), f"{int((got != exp).sum())} voxels differ"


@pytest.mark.parametrize("dfunc", [1, 2])
def test_flood_plain_matches_oracle(vf, ctx, occ64, dfunc):
    occ, mn, mx = occ64
    seeds = O.seeder_uniform(occ, 9, 5, 2)
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(dfunc)
    waves = fr.build_plain(g, seeds)
    exp, ewaves = O.flood(occ, seeds, dfunc)
    assert np.array_equal(g.data(), exp)
    assert waves == ewaves  # same number of BFS waves as the oracle


@pytest.mark.parametrize("shape,frac,gseed", [((37, 29, 45), 0.55, 0), ((70, 18, 66), 0.7, 1),
                                              ((20, 90, 36), 0.62, 2)])
@pytest.mark.parametrize("dfunc", [1, 2])
def test_flood_random_grids(vf, ctx, shape, frac, gseed, dfunc):
    rng = np.random.default_rng(gseed)
    occ = (rng.random(shape) < frac).astype(np.uint16)
    seeds = O.seeder_uniform(occ, 12, gseed, 2)
    g = vf.RegularGrid(shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(dfunc)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, dfunc)
    assert np.array_equal(g.data(), exp)


def test_flood_maze_long_paths(vf, ctx):
    """A serpentine corridor: geodesic distances far above the brick size,
    many passes, and a tie in the middle."""
    X, Y, Z = 40, 34, 70
    occ = np.zeros((X, Y, Z), np.uint16)
    for y in range(0, Y, 2):
        occ[:, y, :] = 1
        if y + 1 < Y:
            occ[:, y + 1, (Z - 1) if (y // 2) % 2 == 0 else 0] = 1
    seeds = np.array([[3, 0, 0, 2], [5, Y - 1, Z - 1, 3]], np.uint32)
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(vf.MANHATTAN)
    fr.build(g, seeds)
    exp, waves = O.flood(occ, seeds, 1)
    assert waves > 500
    assert np.array_equal(g.data(), exp)


def test_flood_extra_seed_prefixes(vf, ctx, occ64):
    occ, mn, mx = occ64
    seeds = O.fracture_seeds(occ, 6, 14, 2, 0, 99)
    assert (seeds[:, 3] > 255).any()
    for dfunc in (1, 2):
        g = vf.RegularGrid(occ.shape, mn, mx, ctx)
        g.upload(occ)
        fr = vf.FloodFracturer()
        fr.setDistanceFunction(dfunc)
        fr.build(g, seeds)
        exp, _ = O.flood(occ, seeds, dfunc)
        assert np.array_equal(g.data(), exp)
        g2 = vf.RegularGrid(occ.shape, mn, mx, ctx)
        g2.upload(occ)
        fr.build_plain(g2, seeds)
        assert np.array_equal(g2.data(), exp)


def test_flood_seed_on_empty_voxel(vf, ctx):
    occ = np.zeros((20, 20, 40), np.uint16)
    occ[2:18, 2:18, 2:38] = 1
    seeds = np.array([[0, 0, 0, 2], [10, 10, 20, 3]], np.uint32)  # first seed outside
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    vf.FloodFracturer().build(g, seeds, vf.Params.default(distance=vf.CHEBYSHEV))
    exp, _ = O.flood(occ, seeds, 2)
    assert np.array_equal(g.data(), exp)


@pytest.mark.parametrize("dfunc", [0, 1, 2])
def test_naive(vf, ctx, occ64, dfunc):
    occ, mn, mx = occ64
    seeds = O.seeder_uniform(occ, 33, 4, 2)
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    vf.NaiveFracturer().build(g, seeds, vf.Params.default(distance=dfunc))
    assert np.array_equal(g.data(), O.naive(occ, seeds, dfunc))


@pytest.fixture(scope="module")
def labelled64(occ64):
    occ, mn, mx = occ64
    seeds = O.seeder_uniform(occ, 10, 3, 2)
    lab, _ = O.flood(occ, seeds, 2)
    return lab, mn, mx


@pytest.mark.parametrize("amp,period,seed", [(2.0, 16, 1), (1.0, 4, 2), (3.0, 7, 3), (0.6, 1, 4)])
def test_perturb(vf, ctx, labelled64, amp, period, seed):
    lab, mn, mx = labelled64
    g = vf.RegularGrid(lab.shape, mn, mx, ctx)
    g.upload(lab)
    g.perturb(amp, period, seed)
    assert np.array_equal(g.data(), O.perturb(lab, amp, period, seed))


@pytest.mark.parametrize("bs", [0, 1, 2, 3])
def test_detect_boundaries(vf, ctx, labelled64, bs):
    lab, mn, mx = labelled64
    g = vf.RegularGrid(lab.shape, mn, mx, ctx)
    g.upload(lab)
    g.detectBoundaries(bs)
    assert np.array_equal(g.data(), O.detect_boundaries(lab, bs))


@pytest.mark.parametrize("etype,size,iters,p,thr", [(0, 3, 1, 0.5, 0.5), (1, 3, 3, 0.5, 0.5),
                                                    (2, 5, 2, 0.8, 0.4), (0, 7, 1, 1.0, 0.6),
                                                    (1, 4, 1, 0.3, 0.5)])
def test_erode(vf, ctx, labelled64, etype, size, iters, p, thr):
    lab, mn, mx = labelled64
    g = vf.RegularGrid(lab.shape, mn, mx, ctx)
    g.upload(lab)
    g.erode(etype, size, iters, p, thr, 17)
    exp = O.erode(lab, etype, size, iters, p, thr, 17)
    got = g.data()
    assert np.array_equal(got, exp), f"{int((got != exp).sum())} voxels differ"


def test_remove_isolated_and_undo_mask(vf, ctx, labelled64):
    lab, mn, mx = labelled64
    b = O.detect_boundaries(lab)
    g = vf.RegularGrid(lab.shape, mn, mx, ctx)
    g.upload(b)
    g.removeIsolatedRegions()
    assert np.array_equal(g.data(), O.remove_isolated(b))
    g.undoMask()
    assert np.array_equal(g.data(), O.undo_mask(O.remove_isolated(b)))


def test_counts(vf, ctx, labelled64):
    lab, mn, mx = labelled64
    b = O.detect_boundaries(lab)
    b[0, 0, 0] = 700  # a value above 255 goes through the global bins
    g = vf.RegularGrid(lab.shape, mn, mx, ctx)
    g.upload(b)
    c, occ = g.countValues(1024)
    ec, eocc = O.count_values(b, 1024)
    assert occ == eocc and np.array_equal(c, ec)
    with pytest.raises(vf.VFError) as e:
        g.countValues(256)
    assert e.value.status == vf.ERR_RANGE


def test_fracture_model(vf, ctx):
    mg = _mg()
    v, f, mn, mx, dims, p, kw = mg.case_inputs("flood_euclid_noise_erode_64")
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    params = vf.Params.default(**kw)
    seeds = vf.fracture_model(g, params)
    gold = np.load(os.path.join(GOLD, "flood_euclid_noise_erode_64.npz"))
    assert np.array_equal(seeds, gold["seeds"])
    assert np.array_equal(g.data(), gold["labels"])


# ---- golden cases end to end ------------------------------------------------
def _spec(vf, name):
    mg = _mg()
    v, f, mn, mx, dims, p, kw = mg.case_inputs(name)
    meta = json.load(open(os.path.join(GOLD, "cases.json")))[name]
    assert mg.mesh_sha(v, f) == meta["mesh_sha256"]
    return vf.JobSpec(v, f, vf.Params.default(**kw), dims=dims, aabb=(mn, mx), ncounts=1024)


def _check_gold(name, spec, res):
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    assert res.status == 0
    assert np.array_equal(spec.labels, gold["labels"]), name
    nz = np.nonzero(spec.counts)[0]
    assert np.array_equal(nz, gold["count_values"]) and np.array_equal(spec.counts[nz],
                                                                          gold["count_numbers"])
    assert res.nseeds == gold["seeds"].shape[0]


@pytest.mark.parametrize("name", CASES)
def test_golden_batched(vf, ctx, name):
    spec = _spec(vf, name)
    (res,) = vf.batch_run([spec], ctx)
    _check_gold(name, spec, res)


@pytest.mark.parametrize("name", CASES)
def test_golden_plain(vf, ctx, name):
    spec = _spec(vf, name)
    (res,) = vf.plain_run([spec], ctx)
    _check_gold(name, spec, res)


def test_golden_all_in_one_batch(vf, ctx):
    specs = [_spec(vf, n) for n in CASES]
    res = vf.batch_run(specs, ctx)
    for n, s, r in zip(CASES, specs, res):
        _check_gold(n, s, r)


# ---- RLE export (RegularGrid::exportRLE) on the GPU --------------------------
def _rle_decode(buf):
    X, Y, Z = np.frombuffer(buf[:12], "<u4")
    runs = np.frombuffer(buf[12:], dtype=np.dtype([("v", "<u2"), ("n", "<u4")]))
    return np.repeat(runs["v"], runs["n"]).reshape(X, Y, Z)


def test_rle_export_reference_fixture(vf, ctx):
    # the reference's own exported grid: decoded, uploaded, exported again on
    # the GPU, byte for byte
    buf = open(os.path.join(GOLD, "AL_12B_grid_128r.rle"), "rb").read()
    g = _rle_decode(buf)
    grid = vf.RegularGrid(g.shape, None, None, ctx)
    grid.upload(g)
    assert grid.exportRLE() == buf


@pytest.mark.parametrize("kind", ["random_runs", "uniform", "alternating", "sparse", "odd_z"])
def test_rle_export_matches_oracle(vf, ctx, kind):
    rng = np.random.default_rng(sum(map(ord, kind)))
    shape = {"odd_z": (9, 7, 13), "alternating": (17, 5, 40)}.get(kind, (33, 20, 52))
    if kind == "random_runs":
        g = np.repeat(rng.integers(0, 6, size=shape[0] * shape[1] * shape[2] // 7 + 1), 7)
        g = g[:np.prod(shape)].reshape(shape).astype(np.uint16)
    elif kind == "uniform":
        g = np.full(shape, 3, np.uint16)
    elif kind == "alternating":
        g = (np.arange(np.prod(shape)) % 2 + 2).reshape(shape).astype(np.uint16)
    elif kind == "sparse":
        g = np.zeros(shape, np.uint16)
        g[rng.random(shape) < 0.02] = 0x8005  # bit 15 set: the full 16-bit value is exported
    else:
        g = rng.integers(0, 3, size=shape).astype(np.uint16)
    grid = vf.RegularGrid(shape, None, None, ctx)
    grid.upload(g)
    got = grid.exportRLE()
    assert got == O.rle_encode(g)
    assert np.array_equal(_rle_decode(got), g)


def test_rle_export_after_fracture(vf, ctx, occ64):
    occ, mn, mx = occ64
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(vf.MANHATTAN)
    fr.build(g, O.seeder_uniform(occ, 8, 5, 2))
    g.detectBoundaries(1)
    assert g.exportRLE() == O.rle_encode(g.data())


# ---- limits and edge cases --------------------------------------------------
def test_flood_max_seed_count_and_limit(vf, ctx):
    rng = np.random.default_rng(11)
    shape = (40, 36, 44)
    occ = (rng.random(shape) < 0.9).astype(np.uint16)
    seeds = O.seeder_uniform(occ, 4095, 3, 2).copy()  # the most a flood takes (12-bit slots)
    assert seeds.shape[0] == 4095
    # fragment labels 2..255 with sub-seed prefixes, as mergeSeeds makes them
    i = np.arange(4095)
    seeds[:, 3] = (i % 254 + 2) | ((i // 254) << 8)
    g = vf.RegularGrid(shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(vf.CHEBYSHEV)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, vf.CHEBYSHEV)
    assert np.array_equal(g.data(), exp)
    more = np.concatenate([seeds, seeds[:1]])
    with pytest.raises(vf.VFError) as e:
        fr.build(g, more)
    assert e.value.status == vf.ERR_RANGE


@pytest.mark.parametrize("dfunc", [1, 2])
def test_flood_long_thin_grid(vf, ctx, dfunc):
    # a 2048-voxel corridor: geodesic distances far beyond one brick, more than
    # a hundred brick passes, two fronts meeting in the middle
    shape = (2048, 2, 4)
    occ = np.ones(shape, np.uint16)
    seeds = np.array([[0, 0, 0, 2], [2047, 1, 3, 3]], np.uint32)
    g = vf.RegularGrid(shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(dfunc)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, dfunc)
    assert np.array_equal(g.data(), exp)


def test_flood_rejects_labels_without_fragment_id(vf, ctx, occ64):
    occ, mn, mx = occ64
    seeds = O.seeder_uniform(occ, 4, 9, 2).copy()
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    for bad in (0x100, 0x201, 0x8002):
        seeds[1, 3] = bad
        with pytest.raises(vf.VFError) as e:
            fr.build(g, seeds)
        assert e.value.status == vf.ERR_INVALID
        with pytest.raises(O.OracleError):
            O.flood(occ, seeds, vf.MANHATTAN)


def test_smallest_grid_and_extreme_labels(vf, ctx):
    occ = np.ones((2, 2, 2), np.uint16)
    seeds = np.array([[0, 0, 0, 0x7FFF >> 8 << 8 | 0xFF], [1, 1, 1, 2]], np.uint32)  # labels 0x7FFF, 2
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(vf.MANHATTAN)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, vf.MANHATTAN)
    assert np.array_equal(g.data(), exp)
    with pytest.raises(vf.VFError):
        vf.RegularGrid((1, 8, 8), None, None, ctx)  # dims below 2


def _serpentine(n_path, length=1450):
    """A one-voxel corridor in the x = 0 layer of a (2, rows, length) grid
    that runs along z and turns at alternate ends: n_path voxels, the geodesic
    distance from its first voxel to its last is n_path - 1.  (Along z a brick
    visit carries the front across the whole brick in one sweep.)"""
    rows = 2 * (n_path // (length + 1) + 2)
    occ = np.zeros((2, rows, length), np.uint16)
    k, y = 0, 0
    while k < n_path:
        take = min(length, n_path - k)
        if (y // 2) % 2 == 0:
            occ[0, y, :take] = 1
        else:
            occ[0, y, length - take:] = 1
        k += take
        if k < n_path:  # the connector to the next corridor row
            occ[0, y + 1, length - 1 if (y // 2) % 2 == 0 else 0] = 1
            k += 1
        y += 2
    return occ


def test_flood_distance_limit(vf, ctx):
    """Keys hold geodesic distances up to 2^20 - 2: a corridor whose far end
    sits exactly at that distance floods like the oracle (the distance-limit
    check runs and finds nothing); one voxel further is VF_ERR_RANGE."""
    limit = (1 << 20) - 2
    seeds = np.array([[0, 0, 0, 2]], np.uint32)
    occ = _serpentine(limit + 1)
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    fr = vf.FloodFracturer()
    fr.setDistanceFunction(vf.MANHATTAN)
    fr.build(g, seeds)
    exp, _ = O.flood(occ, seeds, vf.MANHATTAN)
    assert np.array_equal(g.data(), exp)
    occ = _serpentine(limit + 2)
    g = vf.RegularGrid(occ.shape, None, None, ctx)
    g.upload(occ)
    with pytest.raises(vf.VFError) as e:
        fr.build(g, seeds)
    assert e.value.status == vf.ERR_RANGE
