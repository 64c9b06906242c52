"""GPU parity of the fragment meshes (RegularGrid::toTriangleMesh): the CUDA
path through the C ABI against the CPU oracle, bit for bit.

Tolerance: none.  Vertex positions are exact lattice midpoints mapped by the
grid's affine map, and the smoothing sums fixed-point integers, then rounds
each float step as written; both sides round identically, so positions
compare as raw float32 bits.
"""
import json
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(json.load(open(os.path.join(GOLD, "cases.json"))))


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _mg():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _compare(vf, ctx, labels, mn, mx, params=None):
    dims = labels.shape
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.upload(labels)
    if params is None:
        params = vf.MCParams.default(max(dims))
    sizes = g.triangulate(params)
    vals, vo, fo, v, f = g.meshes_arrays()
    e = O.triangulate(labels, mn, mx, params.nonboundary_iterations, params.nonboundary_weight,
                      params.boundary_iterations, params.boundary_weight)
    assert sizes == (len(e[0]), len(e[3]), len(e[4]))
    assert np.array_equal(vals, e[0])
    assert np.array_equal(vo, e[1]) and np.array_equal(fo, e[2])
    assert np.array_equal(f, e[4]), f"{int((f != e[4]).any(axis=1).sum())} faces differ"
    bad = (v.view(np.uint32) != e[3].view(np.uint32)).any(axis=1)
    assert not bad.any(), f"{int(bad.sum())} of {len(v)} vertices differ"
    g.close()
    return sizes


@pytest.mark.parametrize("name", CASES)
def test_mesh_golden_label_grids(vf, ctx, name):
    mg = _mg()
    _, _, mn, mx, dims, _, _ = mg.case_inputs(name)
    labels = np.load(os.path.join(GOLD, name + ".npz"))["labels"]
    F, V, T = _compare(vf, ctx, labels, mn, mx)
    assert F >= 2 and V > 0 and T > 0


@pytest.mark.parametrize("shape,nlab,seed", [((5, 7, 33), 4, 1), ((17, 3, 65), 3, 2),
                                             ((2, 2, 2), 3, 3), ((33, 31, 30), 6, 4),
                                             ((3, 40, 1 + 96), 2, 5)])
def test_mesh_random_label_grids(vf, ctx, shape, nlab, seed):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, nlab + 2, size=shape).astype(np.uint16)
    g |= (rng.random(shape) < 0.2).astype(np.uint16) << 15
    p = vf.MCParams(3, 0.7, 2, 0.3)
    _compare(vf, ctx, g, [-1.5, 0.25, -3.0], [2.0, 1.75, 5.5], p)


def test_mesh_many_fragments_two_split_passes(vf, ctx):
    # more than 256 fragment values: the stable split takes two 8-bit passes
    rng = np.random.default_rng(11)
    g = rng.integers(2, 700, size=(30, 24, 36)).astype(np.uint16)
    g[rng.random(g.shape) < 0.3] = 1
    F, _, _ = _compare(vf, ctx, g, [0, 0, 0], [1, 1, 1], vf.MCParams(1, 0.9, 1, 0.2))
    assert F > 256


def test_mesh_blocks_and_large_labels(vf, ctx):
    g = np.ones((20, 18, 22), np.uint16)
    g[2:9, 3:15, 1:20] = 0x7FFF
    g[9:18, 3:15, 1:20] = 0x0102 | 0x8000
    g[5, 5, 5] = 0
    _compare(vf, ctx, g, [0, 0, 0], [2, 2, 2])


def test_mesh_empty_grid(vf, ctx):
    for fill in (0, 1):
        g = vf.RegularGrid((6, 5, 4), None, None, ctx)
        g.upload(np.full((6, 5, 4), fill, np.uint16))
        assert g.triangulate() == (0, 0, 0)
        assert g.toTriangleMesh() == []
        g.close()


def test_mesh_after_fracture_model(vf, ctx):
    mg = _mg()
    v, f, mn, mx, dims, _, kw = mg.case_inputs("flood_chebyshev_noise_60")
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    vf.fracture_model(g, vf.Params.default(**kw))
    labels = g.data()
    meshes = g.toTriangleMesh()
    counts, _ = g.countValues()
    assert [m.value for m in meshes] == list(np.nonzero(counts)[0])
    e = O.triangulate(labels, mn, mx, *_default_args(vf, dims))
    for i, m in enumerate(meshes):
        assert np.array_equal(m.faces, e[4][e[2][i]:e[2][i + 1]])
        assert np.array_equal(m.vertices.view(np.uint32), e[3][e[1][i]:e[1][i + 1]].view(np.uint32))
    g.close()


def _default_args(vf, dims):
    p = vf.MCParams.default(max(dims))
    return p.nonboundary_iterations, p.nonboundary_weight, p.boundary_iterations, p.boundary_weight


def test_mesh_repeat_is_identical(vf, ctx):
    labels = np.load(os.path.join(GOLD, CASES[0] + ".npz"))["labels"]
    g = vf.RegularGrid(labels.shape, [0, 0, 0], [1, 1, 1], ctx)
    g.upload(labels)
    g.triangulate()
    a = g.meshes_arrays()
    g.triangulate()
    b = g.meshes_arrays()
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint8) if x.dtype == np.float32 else x,
                              y.view(np.uint8) if y.dtype == np.float32 else y)
    g.close()
