"""CPU tests of the point-sampling oracle (CADModel::sampleCPU)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O


def _mesh(dims=(9, 8, 7), seed=2):
    rng = np.random.default_rng(seed)
    g = np.ones(dims, np.uint16)
    g[2:7, 1:6, 2:5] = 5
    g[rng.random(dims) < 0.1] = 1
    vals, vo, fo, v, f = O.triangulate(g, [-1, -2, 0], [1, 2, 3.5])
    return v[vo[0]:vo[1]], f[fo[0]:fo[1]]


def _face_of(v, f, p, tol=1e-5):
    """faces whose triangle contains p (barycentric, double)"""
    hits = []
    for t, (a, b, c, _) in enumerate(f):
        A, B, Cc = (v[i, :3].astype(np.float64) for i in (a, b, c))
        u, w = B - A, Cc - A
        n = np.cross(u, w)
        nn = np.dot(n, n)
        if nn == 0:
            continue
        d = p - A
        if abs(np.dot(d, n)) / np.sqrt(nn) > tol:
            continue
        s = np.dot(np.cross(d, w), n) / nn
        r = np.dot(np.cross(u, d), n) / nn
        if s >= -tol and r >= -tol and s + r <= 1 + tol:
            hits.append(t)
    return hits


@pytest.mark.parametrize("S", [7, 40, 500])
def test_points_lie_on_the_mesh(S):
    v, f = _mesh()
    pts = O.sample_mesh(v, f, S, 11, 5)
    assert len(pts) == S
    assert np.all(pts[:, 3] == 1.0)
    for p in pts[:: max(1, len(pts) // 40)]:
        assert _face_of(v, f, p[:3].astype(np.float64)), p


def test_few_samples_use_distinct_faces():
    v, f = _mesh()
    S = len(f) // 3
    pts = O.sample_mesh(v, f, S, 3, 5)
    assert len(pts) == S
    faces = [tuple(_face_of(v, f, p[:3].astype(np.float64))) for p in pts]
    assert all(faces)
    # one point per chosen face, in face order: the smallest containing face
    # index strictly increases (points on shared edges may touch two faces)
    firsts = [fs[0] for fs in faces]
    assert firsts == sorted(firsts)


def test_exact_count_rules_and_determinism():
    v, f = _mesh()
    T = len(f)
    assert len(O.sample_mesh(v, f, T, 1, 5)) == T          # S == T: one per face
    assert len(O.sample_mesh(v, f, T + 1, 1, 5)) == T + 1  # S > T: oversampled, cut to S
    a = O.sample_mesh(v, f, 300, 9, 5)
    assert np.array_equal(a, O.sample_mesh(v, f, 300, 9, 5))
    assert not np.array_equal(a, O.sample_mesh(v, f, 300, 10, 5))
    assert not np.array_equal(a, O.sample_mesh(v, f, 300, 9, 6))  # the mesh key
    assert len(O.sample_mesh(v, f, 0, 9, 5)) == 0
    assert len(O.sample_mesh(v, f[:0], 100, 9, 5)) == 0


def test_large_triangles_get_more_samples():
    # two triangles, one 100x the area of the other: S = 202 samples split about
    # 100:1 (ceil of each share), then cut to S
    v = np.array([[0, 0, 0, 0], [10, 0, 0, 0], [0, 10, 0, 0],
                  [0, 0, 1, 0], [1, 0, 1, 0], [0, 1, 1, 0]], np.float32)
    f = np.array([[0, 1, 2, 0], [3, 4, 5, 0]], np.uint32)
    pts = O.sample_mesh(v, f, 202, 4, 0)
    assert len(pts) == 202
    on_small = int((pts[:, 2] == 1.0).sum())
    assert 1 <= on_small <= 4
