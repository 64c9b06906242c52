"""GPU parity of point sampling (CADModel::sampleCPU) against the CPU oracle,
bit for bit: every fragment mesh of a triangulated grid, and a caller mesh.

Tolerance: none.  Areas, the chunked double sum, the sample counts and every
point coordinate round exactly as the oracle does.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as Vs

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(json.load(open(os.path.join(GOLD, "cases.json"))))


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _grid(vf, ctx, name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    _, _, mn, mx, dims, _, _ = m.case_inputs(name)
    labels = np.load(os.path.join(GOLD, name + ".npz"))["labels"]
    g = vf.RegularGrid(labels.shape, mn, mx, ctx)
    g.upload(labels)
    return g


@pytest.mark.parametrize("name", CASES[:4])
@pytest.mark.parametrize("S,seed", [(64, 1), (1024, 80), (20000, 5)])
def test_fragment_point_clouds_match_oracle(vf, ctx, name, S, seed):
    g = _grid(vf, ctx, name)
    g.triangulate()
    vals, vo, fo, v, f = g.meshes_arrays()
    clouds = g.samplePointClouds(S, seed)
    assert len(clouds) == len(vals)
    for i, val in enumerate(vals):
        e = O.sample_mesh(v[vo[i]:vo[i + 1]], f[fo[i]:fo[i + 1]], S, seed, int(val))
        got = clouds[i]
        assert got.shape == e.shape, (val, got.shape, e.shape)
        bad = (got.view(np.uint32) != e.view(np.uint32)).any(axis=1)
        assert not bad.any(), f"value {val}: {int(bad.sum())} of {len(e)} points differ"
    g.close()


def test_host_mesh_matches_oracle(vf, ctx):
    verts, faces = Vs.vessel_mesh(48, 36, 9)
    v4 = np.concatenate([verts, np.zeros((len(verts), 1), np.float32)], axis=1)
    f4 = np.concatenate([faces, np.zeros((len(faces), 1), np.uint32)], axis=1)
    for S in (100, len(faces), 3 * len(faces)):
        got = vf.sample_mesh(verts, faces, S, 42, ctx)
        e = O.sample_mesh(v4, f4, S, 42, 0)
        assert got.shape == e.shape and np.array_equal(got.view(np.uint32), e.view(np.uint32))


def test_sampling_edge_cases(vf, ctx):
    g = vf.RegularGrid((6, 5, 4), None, None, ctx)
    g.upload(np.ones((6, 5, 4), np.uint16))
    g.triangulate()
    assert g.samplePointClouds(128) == []
    g.close()
    verts, faces = Vs.vessel_mesh(12, 9, 3)
    assert len(vf.sample_mesh(verts, faces, 0, 1, ctx)) == 0
