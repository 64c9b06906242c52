"""Parity pinned to the reference's own code.

The reference's tri-box test (Intersections3D.h:204-258 on its Triangle3D and
AABB), NaiveFracturer::buildCPU (NaiveFracturer.cpp:26-68) and
Seeder::mergeSeeds (Seeder.cpp:115-152) compile unchanged from the reference
checkout against the stand-ins in oracle/ref_shim/ (oracle/Makefile, target
`ref`).  These tests compare the oracle's restatements with them:
  - always, against tests/golden/ref_pins.npz (their outputs on seeded
    inputs, made by tests/golden/make_ref_pins.py);
  - where the reference checkout is present, live on fresh random inputs.
The GPU tests compare the CUDA path with the oracle, and the naive fracturer
on the GPU with the same fixture (tests/test_gpu_ref_pin.py)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_pins.npz")


@pytest.fixture(scope="module")
def pins(oracle_lib):
    return np.load(GOLD)


def test_oracle_tri_box_matches_reference_fixture(pins):
    tris, boxes, hit = pins["tribox_tris"], pins["tribox_boxes"], pins["tribox_hit"]
    assert 0 < int(hit.sum()) < len(hit)
    got = np.array([O.tri_box(t[0:3], t[3:6], t[6:9], b[0:3], b[3:6]) for t, b in zip(tris, boxes)],
                   np.uint8)
    assert np.array_equal(got, hit)


@pytest.mark.parametrize("gi", [0, 1, 2])
@pytest.mark.parametrize("dfunc", [0, 1, 2])
def test_oracle_naive_matches_reference_fixture(pins, gi, dfunc):
    grid, seeds = pins[f"naive{gi}_grid"], pins[f"naive{gi}_seeds"]
    assert np.array_equal(O.naive(grid, seeds, dfunc), pins[f"naive{gi}_labels{dfunc}"])


@pytest.mark.parametrize("mi", range(6))
def test_oracle_merge_seeds_matches_reference_fixture(pins, mi):
    frags, seeds = pins[f"merge{mi}_frags"], pins[f"merge{mi}_seeds"]
    for d in (0, 1, 2):
        got = np.asarray(O.merge_seeds(frags, seeds.copy(), d)).reshape(-1, 4)
        assert np.array_equal(got[:, 3], pins[f"merge{mi}_labels{d}"])


@pytest.fixture(scope="module")
def ref(oracle_lib):
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference checkout not present: the fixture tests cover the pin")
    return R


def test_oracle_tri_box_matches_reference_live(ref):
    rng = np.random.default_rng(77)
    n = 100000
    tris = (rng.random((n, 9)) * 4 - 2).astype(np.float32)
    tris[: n // 4] = np.round(tris[: n // 4] * 2) / 2  # on faces, edges, corners
    cell = rng.choice([1.0, 0.5, 0.125, 1e-3], size=(n, 1)).astype(np.float32)
    lo = (rng.integers(-3, 3, (n, 3)) * cell).astype(np.float32)
    boxes = np.concatenate([lo, lo + cell], 1).astype(np.float32)
    hit = np.zeros(n, np.uint8)
    P = C.c_void_p
    ref.vfr_tri_box_batch(tris.ctypes.data_as(P), boxes.ctypes.data_as(P), n, hit.ctypes.data_as(P))
    got = np.array([O.tri_box(t[0:3], t[3:6], t[6:9], b[0:3], b[3:6]) for t, b in zip(tris, boxes)],
                   np.uint8)
    assert 0 < int(hit.sum()) < n
    assert np.array_equal(got, hit)


def test_oracle_naive_and_merge_match_reference_live(ref):
    rng = np.random.default_rng(78)
    P = C.c_void_p
    for _ in range(12):
        shape = tuple(int(v) for v in rng.integers(3, 30, 3))
        occ = (rng.random(shape) < 0.5).astype(np.uint16)
        cells = np.argwhere(occ != 0)
        ns = int(rng.integers(1, min(40, len(cells)) + 1))
        pick = cells[rng.choice(len(cells), ns, replace=False)]
        seeds = np.concatenate([pick, rng.integers(2, 256, (ns, 1))], 1).astype(np.uint32)
        for d in (0, 1, 2):
            g = occ.copy()
            assert ref.vfr_naive(g.ctypes.data_as(P), *shape, seeds.ctypes.data_as(P), ns, d) == 0
            assert np.array_equal(O.naive(occ, seeds, d), g)
        frags = seeds.copy()
        extra = np.concatenate([rng.integers(0, 30, (50, 3)), np.zeros((50, 1))], 1).astype(np.uint32)
        for d in (0, 1, 2):
            s = extra.copy()
            assert ref.vfr_merge_seeds(frags.ctypes.data_as(P), ns, s.ctypes.data_as(P), 50, d) == 0
            got = np.asarray(O.merge_seeds(frags, extra.copy(), d)).reshape(-1, 4)
            assert np.array_equal(got[:, 3], s[:, 3])


@pytest.mark.parametrize("mi", range(6))
def test_library_merge_seeds_matches_reference_fixture(pins, mi):
    # vf_merge_seeds is host code of the library (no GPU needed)
    from voxelfragmentml_gb300 import build as B
    B.build()
    import voxelfragmentml_gb300 as V
    frags, seeds = pins[f"merge{mi}_frags"], pins[f"merge{mi}_seeds"]
    for d in (0, 1, 2):
        got = np.asarray(V.Seeder.mergeSeeds(frags, seeds.copy(), d)).reshape(-1, 4)
        assert np.array_equal(got[:, 3], pins[f"merge{mi}_labels{d}"])
