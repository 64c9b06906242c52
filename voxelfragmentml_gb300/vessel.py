"""Synthetic vessel meshes: closed, watertight surfaces of revolution.

The reference generates its dataset from scanned archaeological vessels
loaded with assimp and normalised to a unit box (CADModel.cpp:112-180,
scale at :148-151).  Those meshes are not available, so a seeded generator
stands in for them with the same shape class (a thin-walled pot):

* outer radius profile ``r(z) = 0.3 + 0.15 sin(3z) + c(z)`` over
  ``z in [0, 1]``, ``c`` a seeded cubic with coefficients in [-0.02, 0.02];
* an inner wall ``r(z) - thickness`` from ``z = thickness`` to 1, a bottom
  disc on each side and a rim annulus at ``z = 1`` close the surface;
* ``A`` angular x ``P`` profile samples give ``4*A*P`` triangles
  (128x96 -> 49,152; 256x192 -> 196,608; 512x384 -> 786,432).

Vertices are float32 and faces uint32 (3 per triangle).  All trigonometry
is evaluated with a fixed float64 polynomial using only IEEE add and
multiply, so the same mesh comes out bit-for-bit on x86 and on Arm.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["vessel_mesh", "mesh_aabb", "grid_dims", "samples_for_triangles"]

_TWO_PI = 2.0 * math.pi


def _sin64(x: np.ndarray) -> np.ndarray:
    """sin for float64 arrays: reduction to [-pi, pi], Taylor series to x^27."""
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / _TWO_PI + 0.5)
    r = x - k * _TWO_PI
    r2 = r * r
    term = r.copy()
    acc = r.copy()
    for n in range(1, 14):
        term = term * r2
        term = term / float((2 * n) * (2 * n + 1))
        acc = acc - term if n % 2 == 1 else acc + term
    return acc


def _cos64(x: np.ndarray) -> np.ndarray:
    return _sin64(np.asarray(x, dtype=np.float64) + 0.5 * math.pi)


def _cubic_coeffs(seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    return rng.uniform(-0.02, 0.02, size=4)


def vessel_mesh(angular: int = 128, profile: int = 96, seed: int = 42,
                thickness: float = 0.03):
    """Return ``(vertices float32 [n,3], faces uint32 [m,3])``."""
    A, P = int(angular), int(profile)
    if A < 3 or P < 2:
        raise ValueError("need angular >= 3 and profile >= 2")
    a = _cubic_coeffs(seed)
    th = np.arange(A, dtype=np.float64) * (_TWO_PI / A)
    ct, st = _cos64(th), _sin64(th)

    def radius(z):
        return 0.3 + 0.15 * _sin64(3.0 * z) + (((a[3] * z + a[2]) * z + a[1]) * z + a[0])

    zo = np.arange(P, dtype=np.float64) / (P - 1)
    zi = thickness + zo * (1.0 - thickness)
    ro = radius(zo)
    ri = radius(zi) - thickness

    def rings(r, z):
        x = r[:, None] * ct[None, :]
        y = r[:, None] * st[None, :]
        zz = np.broadcast_to(z[:, None], x.shape)
        return np.stack([x, y, zz], axis=-1).reshape(-1, 3)

    outer = rings(ro, zo)                      # index j*A + i
    inner = rings(ri, zi)                      # offset P*A
    verts = np.concatenate([outer, inner,
                            [[0.0, 0.0, 0.0], [0.0, 0.0, thickness]]]).astype(np.float32)
    oc, ic = 2 * P * A, 2 * P * A + 1
    i = np.arange(A, dtype=np.int64)
    i1 = (i + 1) % A
    faces = []
    for j in range(P - 1):                     # outer wall, outward
        a0, a1 = j * A + i, j * A + i1
        b0, b1 = (j + 1) * A + i, (j + 1) * A + i1
        faces.append(np.stack([a0, a1, b1], 1))
        faces.append(np.stack([a0, b1, b0], 1))
    off = P * A
    for j in range(P - 1):                     # inner wall, facing the axis
        a0, a1 = off + j * A + i, off + j * A + i1
        b0, b1 = off + (j + 1) * A + i, off + (j + 1) * A + i1
        faces.append(np.stack([a0, b1, a1], 1))
        faces.append(np.stack([a0, b0, b1], 1))
    faces.append(np.stack([np.full(A, oc), i1, i], 1))                 # outer bottom
    faces.append(np.stack([np.full(A, ic), off + i, off + i1], 1))     # inner bottom
    t0, t1 = (P - 1) * A + i, (P - 1) * A + i1                        # rim annulus
    u0, u1 = off + (P - 1) * A + i, off + (P - 1) * A + i1
    faces.append(np.stack([t0, t1, u1], 1))
    faces.append(np.stack([t0, u1, u0], 1))
    faces = np.concatenate(faces).astype(np.uint32)
    return np.ascontiguousarray(verts), np.ascontiguousarray(faces)


def mesh_aabb(verts: np.ndarray):
    """Mesh AABB (float32 min, max), the grid AABB of RegularGrid::setAABB."""
    return verts.min(axis=0).astype(np.float32), verts.max(axis=0).astype(np.float32)


def grid_dims(aabb_min, aabb_max, max_voxels: int):
    """CADScene::allocateMeshGrid (CADScene.cpp:545-561): scale the longest
    axis to ``max_voxels`` and round every axis to a multiple of 4 that does
    not exceed it.  Float32 arithmetic as in the reference."""
    mn = np.asarray(aabb_min, np.float32)
    mx = np.asarray(aabb_max, np.float32)
    size = (mx - mn).astype(np.float32)
    longest = np.float32(size.max())
    dims = []
    for a in range(3):
        v = np.float32(np.float32(max_voxels) * size[a]) / longest
        d = int(np.floor(np.float32(v)))
        while d % 4:
            d += 1
        while d % 4 or d > max_voxels:
            d -= 1
        dims.append(d)
    return tuple(dims)


def samples_for_triangles(n_triangles: int):
    """(angular, profile) with 4*A*P ~= n_triangles and P = 3A/4."""
    A = max(8, int(round(math.sqrt(n_triangles / 3.0))))
    P = max(4, int(round(0.75 * A)))
    return A, P
