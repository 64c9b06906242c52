"""CPU tests of the oracle: known-answer cases, independent brute-force
restatements, the reference's RLE fixture and the golden fixtures.

The reference ships no tests for this path, so the oracle is pinned here by
(1) hand-worked cases, (2) independent Python restatements on small grids,
(3) an analytic inside test of the synthetic vessel for the voxelizer, and
(4) byte equality with the reference's own RLE output fixture.
"""
import collections
import hashlib
import itertools
import json
import os

import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as V

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _build(oracle_lib):
    return oracle_lib


# ---- tri-box SAT (Intersections3D.h:204-258) -------------------------------
@pytest.mark.parametrize("tri,box,expect", [
    (((0.2, 0.2, 0.5), (0.8, 0.2, 0.5), (0.5, 0.8, 0.5)), ((0, 0, 0), (1, 1, 1)), True),
    (((2, 2, 2), (3, 2, 2), (2, 3, 2)), ((0, 0, 0), (1, 1, 1)), False),
    # triangle in the plane of a box face
    (((0, 0, 1), (1, 0, 1), (0, 1, 1)), ((0, 0, 0), (1, 1, 1)), True),
    # triangle touching only a box corner
    (((1, 1, 1), (2, 1, 1), (1, 2, 1)), ((0, 0, 0), (1, 1, 1)), True),
    # large triangle cutting through the box
    (((-5, -5, 0.5), (5, -5, 0.5), (0, 5, 0.5)), ((0, 0, 0), (1, 1, 1)), True),
    # triangle parallel to a face, just outside
    (((0, 0, 1.001), (1, 0, 1.001), (0, 1, 1.001)), ((0, 0, 0), (1, 1, 1)), False),
    # edge crossing the box diagonally, plane misses the corner region
    (((1.5, -0.5, 0.5), (1.5, 0.4, 0.5), (2.5, 0.0, 0.5)), ((0, 0, 0), (1, 1, 1)), False),
])
def test_tri_box_known(tri, box, expect):
    assert O.tri_box(*tri, *box) == expect


def test_tri_box_matches_sampling():
    """SAT never says 'no' for a triangle with a sample point inside the box."""
    rng = np.random.default_rng(1)
    for _ in range(300):
        t = rng.uniform(-0.5, 1.5, size=(3, 3)).astype(np.float32)
        w = rng.dirichlet([1, 1, 1], size=200)
        pts = w @ t
        inside = np.all((pts > 0.01) & (pts < 0.99), axis=1).any()
        if inside:
            assert O.tri_box(t[0], t[1], t[2], (0, 0, 0), (1, 1, 1))


# ---- voxelizer -------------------------------------------------------------
@pytest.mark.parametrize("A,P,maxd", [(48, 36, 48), (64, 48, 64)])
def test_voxelizer_matches_analytic_vessel(A, P, maxd):
    v, f = V.vessel_mesh(A, P, 42)
    mn, mx = V.mesh_aabb(v)
    dims = V.grid_dims(mn, mx, maxd)
    shell = O.voxelize(v, f, dims, mn, mx, 1).astype(bool)
    par = O.voxelize(v, f, dims, mn, mx, 2).astype(bool)
    both = O.voxelize(v, f, dims, mn, mx, 3).astype(bool)
    assert np.array_equal(both, shell | par)
    X, Y, Z = dims
    cs = (mx - mn) / np.array(dims, np.float32)
    xi, yi, zi = np.meshgrid(np.arange(X), np.arange(Y), np.arange(Z), indexing="ij")
    # tetra parity samples at pixel centres in x,z and on the lower y face
    px, py, pz = mn[0] + (xi + 0.5) * cs[0], mn[1] + yi * cs[1], mn[2] + (zi + 0.5) * cs[2]
    a = V._cubic_coeffs(42)
    r = lambda z: 0.3 + 0.15 * np.sin(3 * z) + (((a[3] * z + a[2]) * z + a[1]) * z + a[0])
    rho = np.hypot(px, py)
    inside = (pz >= 0) & (pz <= 1) & (rho <= r(pz)) & ~((pz > 0.03) & (rho < r(pz) - 0.03))
    mism = par != inside
    assert mism.sum() < 0.05 * inside.sum()
    assert not (mism & ~shell).any(), "parity differs from the analytic solid away from the surface"


def test_voxelizer_empty_and_invalid():
    g = O.voxelize(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), (8, 8, 8),
                   (0, 0, 0), (1, 1, 1))
    assert not g.any()
    with pytest.raises(O.OracleError):
        O.voxelize(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.uint32), (8, 8, 8),
                   (0, 0, 0), (1, 1, 1))


def test_grid_dims_rule():
    # CADScene::allocateMeshGrid: longest axis -> max_voxels, others multiple of 4
    assert O.grid_dims((0, 0, 0), (1, 1, 1), 128) == (128, 128, 128)
    assert O.grid_dims((0, 0, 0), (0.5, 1, 0.3), 128) == (64, 128, 40)  # 38.4 -> 38 -> up to 40
    assert O.grid_dims((0, 0, 0), (1, 0.25, 1), 130) == (128, 32, 128)
    for mn, mx, m in [((0, 0, 0), (0.93, 0.93, 1.0), 128), ((0, 0, 0), (0.7, 1, 0.2), 200)]:
        assert O.grid_dims(mn, mx, m) == V.grid_dims(mn, mx, m)


# ---- seeding (Seeder.cpp:154-208) -----------------------------------------
def _occ_grid(n=24, seed=0, frac=0.3):
    rng = np.random.default_rng(seed)
    return (rng.random((n, n, n)) < frac).astype(np.uint16)


@pytest.mark.parametrize("loc", [0, 1, 2])
def test_seeder_uniform_properties(loc):
    g = _occ_grid(frac=0.97 if loc == 0 else 0.3)  # INNER needs fully occupied 3^3 windows
    s = O.seeder_uniform(g, 20, 7, loc)
    assert s.shape == (20, 4)
    pos = [tuple(int(c) for c in r[:3]) for r in s]
    assert pos == sorted(pos) and len(set(pos)) == 20
    assert list(s[:, 3]) == list(range(2, 22))
    X = g.shape[0]
    for x, y, z in pos:
        assert g[x, y, z] != 0
        assert max(x, y, z) <= X - 2  # int(U*(dim-1)) never reaches the last layer
        w = g[max(x - 1, 0):x + 2, max(y - 1, 0):y + 2, max(z - 1, 0):z + 2]
        bnd = bool((w == 0).any())
        if loc == 1:
            assert bnd
        if loc == 0:
            assert not bnd


def test_seeder_deterministic_and_seed_dependent():
    g = _occ_grid()
    a = O.seeder_uniform(g, 10, 42, 2)
    assert np.array_equal(a, O.seeder_uniform(g, 10, 42, 2))
    assert not np.array_equal(a, O.seeder_uniform(g, 10, 43, 2))


def test_seeder_search_error():
    g = np.zeros((16, 16, 16), np.uint16)
    g[3, 3, 3] = 1
    with pytest.raises(O.OracleError) as e:
        O.seeder_uniform(g, 2, 1, 2)
    assert e.value.status == O.ERR_SEED_SEARCH


def test_merge_seeds_known():
    frags = np.array([[0, 0, 0, 2], [10, 10, 10, 3]], np.uint32)
    seeds = np.array([[1, 1, 1, 0], [9, 9, 9, 0], [2, 0, 0, 0], [5, 5, 5, 0]], np.uint32)
    m = O.merge_seeds(frags, seeds, 0)
    # nearest fragment; per-fragment counter in list order; tie (5,5,5) -> first
    assert list(m[:, 3]) == [2 | 1 << 8, 3 | 1 << 8, 2 | 2 << 8, 2 | 3 << 8]


# ---- flood (FloodFracturer.cpp:98-191) ------------------------------------
def _brute_geodesic(grid, seeds, conn):
    """Independent restatement: multi-source BFS distance, ties to the lowest
    seed index (later seeds win a shared voxel)."""
    X, Y, Z = grid.shape
    occ = grid != 0
    offs = [o for o in itertools.product((-1, 0, 1), repeat=3) if any(o)]
    if conn == 6:
        offs = [o for o in offs if sum(map(abs, o)) == 1]
    best = {}
    for i, (x, y, z, w) in enumerate(seeds):
        best[(int(x), int(y), int(z))] = (0, i)
    q = collections.deque(sorted(best, key=lambda p: best[p]))
    dist = {p: best[p] for p in best}
    # Dijkstra with unit weights and lexicographic (dist, idx) keys
    import heapq
    heap = [(d, i, p) for p, (d, i) in dist.items()]
    heapq.heapify(heap)
    done = {}
    while heap:
        d, i, p = heapq.heappop(heap)
        if p in done:
            continue
        done[p] = (d, i)
        for o in offs:
            n = (p[0] + o[0], p[1] + o[1], p[2] + o[2])
            if not (0 <= n[0] < X and 0 <= n[1] < Y and 0 <= n[2] < Z) or not occ[n]:
                continue
            if n not in done and (n not in dist or (d + 1, i) < dist[n]):
                dist[n] = (d + 1, i)
                heapq.heappush(heap, (d + 1, i, n))
    out = np.where(occ, 1, 0).astype(np.uint16)
    for p, (d, i) in done.items():
        out[p] = seeds[i][3] & 0xFF
    return out


@pytest.mark.parametrize("conn,dfunc", [(6, 1), (26, 2), (26, 0)])
@pytest.mark.parametrize("gseed", [0, 1, 2])
def test_flood_equals_geodesic_nearest_seed(conn, dfunc, gseed):
    g = _occ_grid(12, gseed, 0.6)
    s = O.seeder_uniform(g, 5, gseed + 10, 2)
    fl, waves = O.flood(g, s, dfunc)
    assert np.array_equal(fl, _brute_geodesic(g, s, conn))
    assert waves > 0


def test_flood_single_seed_fills_component_and_leaves_others_free():
    g = np.zeros((10, 10, 10), np.uint16)
    g[1:4, 1:4, 1:4] = 1   # seeded component
    g[6:9, 6:9, 6:9] = 1   # unseeded component
    fl, _ = O.flood(g, np.array([[2, 2, 2, 2]], np.uint32), 1)
    assert (fl[1:4, 1:4, 1:4] == 2).all()
    assert (fl[6:9, 6:9, 6:9] == 1).all()  # stays FREE
    assert (fl[g == 0] == 0).all()


def test_flood_tie_goes_to_lowest_seed_index():
    g = np.ones((1, 1, 9), np.uint16)
    s = np.array([[0, 0, 0, 2], [0, 0, 8, 3]], np.uint32)
    fl, _ = O.flood(g, s, 1)
    assert list(fl[0, 0]) == [2, 2, 2, 2, 2, 3, 3, 3, 3]  # voxel 4 is equidistant -> index 0


def test_flood_ball_shapes():
    g = np.ones((9, 9, 9), np.uint16)
    s = np.array([[4, 4, 4, 2], [0, 0, 0, 3], [8, 8, 8, 4]], np.uint32)
    man, _ = O.flood(g, s, 1)
    che, _ = O.flood(g, s, 2)
    c = np.array([4, 4, 4])
    idx = np.indices(g.shape).reshape(3, -1).T
    # voxels within graph distance 2 of the centre seed are always its own
    for p in idx:
        if np.abs(p - c).sum() <= 2:
            assert man[tuple(p)] == 2
        if np.abs(p - c).max() <= 2:
            assert che[tuple(p)] == 2


def test_flood_later_duplicate_seed_wins_voxel():
    g = np.ones((4, 4, 4), np.uint16)
    s = np.array([[1, 1, 1, 2], [1, 1, 1, 5]], np.uint32)
    fl, _ = O.flood(g, s, 2)
    assert (fl == 5).all()


def test_flood_extra_seed_prefix_cleanup():
    """Sub-seeds of one fragment that end disconnected from the fragment's
    minimum prefix are reset and re-flooded (disjoint cleanup)."""
    g = np.ones((1, 1, 11), np.uint16)
    # fragment 2 has sub-seeds at both ends, fragment 3 sits in the middle
    s = np.array([[0, 0, 0, 2 | 1 << 8], [0, 0, 5, 3 | 1 << 8], [0, 0, 10, 2 | 2 << 8]],
                 np.uint32)
    fl, _ = O.flood(g, s, 1)
    # the prefix-2 region of fragment 2 (right end) is not connected to its
    # prefix-1 region -> FREE -> re-flooded from the survivors (fragment 3)
    assert list(fl[0, 0]) == [2, 2, 2, 3, 3, 3, 3, 3, 3, 3, 3]


def test_flood_invalid_seed():
    g = np.ones((4, 4, 4), np.uint16)
    with pytest.raises(O.OracleError):
        O.flood(g, np.array([[9, 0, 0, 2]], np.uint32), 1)
    with pytest.raises(O.OracleError):
        O.flood(g, np.array([[0, 0, 0, 1]], np.uint32), 1)


# ---- naive (NaiveFracturer.cpp:26-68) ------------------------------------
@pytest.mark.parametrize("dfunc", [0, 1, 2])
def test_naive_matches_bruteforce(dfunc):
    g = _occ_grid(10, 4, 0.5)
    s = O.seeder_uniform(g, 6, 1, 2)
    out = O.naive(g, s, dfunc)
    idx = np.indices(g.shape).reshape(3, -1).T.astype(np.int64)
    d = idx[:, None, :] - s[None, :, :3].astype(np.int64)
    if dfunc == 0:
        dist = np.sqrt((d.astype(np.float32) ** 2).sum(-1, dtype=np.float32), dtype=np.float32)
    elif dfunc == 1:
        dist = np.abs(d).sum(-1).astype(np.float32)
    else:
        dist = np.abs(d).max(-1).astype(np.float32)
    lab = s[np.argmin(dist, axis=1), 3].reshape(g.shape)  # argmin keeps the first = lowest index
    exp = np.where(g != 0, lab, 0)
    assert np.array_equal(out, exp)


# ---- grid passes -----------------------------------------------------------
def test_detect_boundaries_known():
    g = np.zeros((5, 5, 5), np.uint16)
    g[1:4, 1:4, 1:4] = 2
    g[3, 1:4, 1:4] = 3
    out = O.detect_boundaries(g, 1)
    assert (out[2, 1:4, 1:4] == (2 | 0x8000)).all()   # touches label 3
    assert (out[3, 1:4, 1:4] == (3 | 0x8000)).all()
    assert (out[1, 1:4, 1:4] == 2).all()              # EMPTY neighbours do not count
    again = O.detect_boundaries(out, 1)
    assert np.array_equal(again, out)


def test_remove_isolated_known():
    g = np.zeros((6, 6, 6), np.uint16)
    g[1:5, 1:5, 1:5] = 2
    g[0, 0, 0] = 7  # isolated voxel
    out = O.remove_isolated(g)
    assert out[0, 0, 0] == 0
    assert (out[2:4, 2:4, 2:4] == 2).all()
    assert out[1, 1, 1] == 2  # corner of the cube: 7 equal neighbours >= 6


def test_erode_square_removes_thin_features():
    g = np.zeros((8, 8, 8), np.uint16)
    g[2:6, 2:6, 2:6] = 2
    g[2:6, 2:6, 6] = 3
    out = O.erode(g, 0, 3, 1, 1.0, 0.5, 1)
    # every voxel of the one-voxel-thick label-3 plate is a boundary voxel with
    # few equal neighbours -> removed; the cube core keeps its label
    assert not (out[:, :, 6] == (3 | 0x8000)).any()
    assert ((out[3:5, 3:5, 3:5] & 0x7FFF) == 2).all()


def test_erode_probability_zero_only_removes_isolated():
    g = _occ_grid(10, 2, 0.7) * 2
    out = O.erode(g, 1, 3, 2, 0.0, 0.5, 5)
    assert np.array_equal(out, O.remove_isolated(O.detect_boundaries(O.detect_boundaries(g))))


def test_counts_and_undo_mask():
    g = np.array([0, 1, 2, 2 | 0x8000, 3, 300, 3], np.uint16).reshape(1, 1, 7)
    c, occ = O.count_values(g, 512)
    assert occ == 5 and c[2] == 2 and c[3] == 2 and c[300] == 1 and c[1] == 0
    assert list(O.undo_mask(g)[0, 0]) == [0, 1, 2, 2, 3, 300, 3]
    with pytest.raises(O.OracleError):
        O.count_values(g, 256)


def test_perturb_zero_amplitude_and_locality():
    g = _occ_grid(16, 3, 0.8) * 2
    g[8:, :, :] = np.where(g[8:] != 0, 3, 0)
    assert np.array_equal(O.perturb(g, 0.0, 8, 1), g)
    out = O.perturb(g, 1.0, 4, 1)
    assert np.array_equal(out == 0, g == 0)          # occupancy never changes
    assert set(np.unique(out)) <= {0, 2, 3}
    # a voxel only takes a label found within +-1 voxel
    diff = np.argwhere(out != g)
    for x, y, z in diff.tolist():
        w = g[max(x - 1, 0):x + 2, max(y - 1, 0):y + 2, max(z - 1, 0):z + 2]
        assert out[x, y, z] in w


# ---- RLE format: the reference's own fixture ------------------------------
def _rle_decode(buf):
    X, Y, Z = np.frombuffer(buf[:12], "<u4")
    runs = np.frombuffer(buf[12:], dtype=np.dtype([("v", "<u2"), ("n", "<u4")]))
    return np.repeat(runs["v"], runs["n"]).reshape(X, Y, Z)


def test_rle_roundtrip_reference_fixture():
    path = os.path.join(GOLD, "AL_12B_grid_128r.rle")
    buf = open(path, "rb").read()
    g = _rle_decode(buf)
    assert g.shape == (128, 110, 128)
    assert int((g != 0).sum()) == 111152
    assert O.rle_encode(g) == buf


# ---- golden fixtures --------------------------------------------------------
def _cases():
    with open(os.path.join(GOLD, "cases.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_matches_golden(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    meta = _cases()[name]
    v, f, mn, mx, dims, p, _ = mg.case_inputs(name)
    assert mg.mesh_sha(v, f) == meta["mesh_sha256"], "vessel generator changed"
    assert list(dims) == meta["dims"]
    labels, counts, seeds = O.run_job(v, f, dims, mn, mx, p)
    gold = np.load(os.path.join(GOLD, name + ".npz"))
    assert np.array_equal(labels, gold["labels"])
    assert np.array_equal(seeds, gold["seeds"])
    nz = np.nonzero(counts)[0]
    assert np.array_equal(nz, gold["count_values"]) and np.array_equal(counts[nz], gold["count_numbers"])
    assert hashlib.sha256(labels.tobytes()).hexdigest() == meta["labels_sha256"]
