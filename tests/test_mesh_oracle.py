"""CPU tests of the fragment-mesh oracle (RegularGrid::toTriangleMesh) and of
the marching-cubes case table shared by the kernels and the oracle."""
from __future__ import annotations

import hashlib
import json
import os
import re

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE_H = os.path.join(ROOT, "voxelfragmentml_gb300", "csrc", "vf_mc_table.h")
GOLDEN = os.path.join(ROOT, "tests", "golden", "mc_tables.json")
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6),
         (3, 7)]


def _table():
    src = open(TABLE_H).read()
    body = src[src.index("VF_MC_TRIANGLES[256]"):]
    body = body[body.index("{") + 1:body.index("};")]
    rows = re.findall(r'"([0-9a-f]*)"', body)
    assert len(rows) == 256
    return [[int(ch, 16) for ch in r] for r in rows]


def _crossing(c):
    m = 0
    for i, (a, b) in enumerate(EDGES):
        if ((c >> a) & 1) != ((c >> b) & 1):
            m |= 1 << i
    return m


def test_case_table_matches_reference_digest():
    ref = json.load(open(GOLDEN))
    rows = _table()
    canon = ";".join(",".join(str(e) for e in r) for r in rows)
    assert hashlib.sha256(canon.encode()).hexdigest() == ref["triangles_sha256"]
    assert sum(len(r) // 3 for r in rows) == ref["triangle_count_total"]
    # the reference's edge-flag table is the set of edges whose corners differ
    edges = ",".join(str(_crossing(c)) for c in range(256))
    assert hashlib.sha256(edges.encode()).hexdigest() == ref["edges_sha256"]


def test_case_table_uses_exactly_the_crossing_edges():
    for c, r in enumerate(_table()):
        assert len(r) % 3 == 0 and len(r) <= 15
        used = 0
        for e in r:
            used |= 1 << e
        assert used == _crossing(c), c


def _single(value=2, bit15=False, dims=(3, 3, 3), at=(1, 1, 1)):
    g = np.ones(dims, np.uint16)
    g[at] = value | (0x8000 if bit15 else 0)
    return g


def test_single_voxel_is_an_octahedron():
    vals, vo, fo, v, f = O.triangulate(_single(), [0, 0, 0], [3, 3, 3])
    assert list(vals) == [2] and list(vo) == [0, 6] and list(fo) == [0, 8]
    # lattice point p maps to s*p + min - s (s = 1): the voxel's lower corner
    # sits at (1, 1, 1), its face midpoints half a voxel below it
    exp = [(0.5, 1, 1), (1.5, 1, 1), (1, 0.5, 1), (1, 1.5, 1), (1, 1, 0.5), (1, 1, 1.5)]
    assert np.array_equal(v[:, :3], np.array(exp, np.float32))
    assert not v[:, 3].any() and not f[:, 3].any()
    # closed: every edge in two faces, opposite orientation; normals outward
    edges = {}
    for a, b, c, _ in f:
        for e in ((a, b), (b, c), (c, a)):
            edges[e] = edges.get(e, 0) + 1
    assert len(edges) == 24 and all(edges.get((b, a)) == 1 for (a, b) in edges)
    centre = np.array([1, 1, 1], np.float32)
    for a, b, c, _ in f:
        n = np.cross(v[b, :3] - v[a, :3], v[c, :3] - v[a, :3])
        assert np.dot(n, (v[a, :3] + v[b, :3] + v[c, :3]) / 3 - centre) > 0


def test_single_voxel_boundary_flags():
    # bit 15 on the voxel flags the triangles of the cells whose lattice point
    # (largest x, smallest y and z corner) is that voxel, and their vertices
    vals, vo, fo, v, f = O.triangulate(_single(bit15=True), [0, 0, 0], [3, 3, 3])
    assert list(vals) == [2]
    assert 0 < f[:, 3].sum() < len(f)
    for a, b, c, w in f:
        assert w == max(v[a, 3], v[b, 3], v[c, 3])


def test_smoothing_known_answer():
    # one non-boundary iteration, weight 0.5: each octahedron vertex moves
    # halfway to the mean of its four neighbours, the voxel's lower corner
    _, _, _, v, _ = O.triangulate(_single(), [0, 0, 0], [3, 3, 3], nb_iters=1, nb_weight=0.5)
    exp = [(0.75, 1, 1), (1.25, 1, 1), (1, 0.75, 1), (1, 1.25, 1), (1, 1, 0.75), (1, 1, 1.25)]
    assert np.array_equal(v[:, :3], np.array(exp, np.float32))
    # boundary iterations move only boundary vertices; weight 0 moves nothing
    _, _, _, v0, _ = O.triangulate(_single(), [0, 0, 0], [3, 3, 3])
    _, _, _, v1, _ = O.triangulate(_single(), [0, 0, 0], [3, 3, 3], b_iters=3, b_weight=0.5)
    assert np.array_equal(v0, v1)
    _, _, _, v2, _ = O.triangulate(_single(), [0, 0, 0], [3, 3, 3], nb_iters=4, nb_weight=0.0)
    assert np.array_equal(v0, v2)


def test_solid_box_is_closed_genus_zero():
    g = np.ones((9, 8, 7), np.uint16)
    g[2:7, 1:6, 2:5] = 5
    vals, vo, fo, v, f = O.triangulate(g, [-1, -2, 0], [1, 2, 3.5])
    assert list(vals) == [5]
    V, F = len(v), len(f)
    edges = {}
    for a, b, c, _ in f:
        for e in ((a, b), (b, c), (c, a)):
            edges[e] = edges.get(e, 0) + 1
    assert all(n == 1 for n in edges.values()) and all((b, a) in edges for (a, b) in edges)
    assert V - len(edges) // 2 + F == 2
    # fused vertices = exposed voxel faces of the box
    assert V == 2 * (5 * 5 + 5 * 3 + 5 * 3)


def test_two_fragments_share_positions_not_vertices():
    g = np.ones((4, 3, 3), np.uint16)
    g[1, 1, 1] = 2
    g[2, 1, 1] = 3
    vals, vo, fo, v, f = O.triangulate(g, [0, 0, 0], [4, 3, 3])
    assert list(vals) == [2, 3] and list(vo) == [0, 6, 12] and list(fo) == [0, 8, 16]
    # each mesh indexes its own vertices; the two voxels' facing midpoints coincide
    assert f[:8, :3].max() < 6 and f[8:, :3].max() < 6
    a = {tuple(p) for p in v[:6, :3]}
    b = {tuple(p) for p in v[6:, :3]}
    assert len(a & b) == 1


def test_empty_and_unlabelled_grids():
    for fill in (0, 1):
        g = np.full((5, 4, 3), fill, np.uint16)
        vals, vo, fo, v, f = O.triangulate(g, [0, 0, 0], [1, 1, 1])
        assert len(vals) == 0 and len(v) == 0 and len(f) == 0 and list(vo) == [0]


def test_vertex_order_follows_owner_voxel_then_direction():
    rng = np.random.default_rng(3)
    g = rng.integers(0, 5, size=(6, 5, 7)).astype(np.uint16)
    vals, vo, fo, v, f = O.triangulate(g, [0, 0, 0], [6, 5, 7])
    X, Y, Z = g.shape
    for i, val in enumerate(vals):
        keys = []
        for p in v[vo[i]:vo[i + 1], :3]:
            q = p + 1.0  # lattice coordinates (s = 1, min = 0)
            ax = int(np.argmax(np.abs(q - np.round(q)) > 0.25))
            lo = q.copy(); lo[ax] -= 0.5
            hi = q.copy(); hi[ax] += 0.5
            cand = []
            for end, other, up in ((lo, hi, 1), (hi, lo, 0)):
                x, y, z = (int(round(t)) - 1 for t in end)
                if 0 <= x < X and 0 <= y < Y and 0 <= z < Z and (g[x, y, z] & 0x7FFF) == val:
                    cand.append(((x * Y + y) * Z + z) * 6 + 2 * ax + up)
            assert len(cand) == 1
            keys.append(cand[0])
        assert keys == sorted(keys) and len(set(keys)) == len(keys)
