"""CPU tests of the impact-path oracle: RegularGrid::rayTraversalAmanatidesWoo
(the voxel a ray enters first) and Seeder::nearSeeds."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O


def _box_grid():
    g = np.zeros((20, 22, 24), np.uint16)
    g[4:16, 5:18, 6:20] = 1
    return g


def test_ray_axis_aligned_known_answers():
    g = _box_grid()
    lo, hi = [0, 0, 0], [20, 22, 24]  # one unit per voxel
    # +x through voxel row (y=11, z=12): first occupied x is 4 -> 1-based (5, 12, 13)
    assert O.ray_entry(g, lo, hi, [-5, 11.5, 12.5], [1, 0, 0]) == (5, 12, 13)
    # -x from the far side: first occupied x is 15 -> 16
    assert O.ray_entry(g, lo, hi, [30, 11.5, 12.5], [-1, 0, 0]) == (16, 12, 13)
    # +z and -y
    assert O.ray_entry(g, lo, hi, [10.5, 11.5, -3], [0, 0, 2]) == (11, 12, 7)
    assert O.ray_entry(g, lo, hi, [10.5, 40, 12.5], [0, -0.5, 0]) == (11, 18, 13)


def test_ray_misses_and_empty_paths():
    g = _box_grid()
    lo, hi = [0, 0, 0], [20, 22, 24]
    assert O.ray_entry(g, lo, hi, [-5, 11.5, 12.5], [-1, 0, 0]) is None  # points away
    assert O.ray_entry(g, lo, hi, [-5, 30, 12.5], [1, 0, 0]) is None     # passes beside the box
    assert O.ray_entry(g, lo, hi, [-5, 1.5, 1.5], [1, 0, 0]) is None     # only EMPTY voxels


def test_ray_starting_inside_the_box():
    g = _box_grid()
    lo, hi = [0, 0, 0], [20, 22, 24]
    # inside an occupied voxel: the walk starts there
    assert O.ray_entry(g, lo, hi, [10.5, 11.5, 12.5], [1, 0.3, 0.2]) == (11, 12, 13)
    # inside, in EMPTY space, heading into the block
    assert O.ray_entry(g, lo, hi, [1.5, 11.5, 12.5], [1, 0, 0]) == (5, 12, 13)


def test_ray_zero_direction_rejected():
    g = _box_grid()
    with pytest.raises(O.OracleError):
        O.ray_entry(g, [0, 0, 0], [20, 22, 24], [-5, 11, 12], [0, 0, 0])


def test_ray_oblique_steps_one_voxel_at_a_time():
    # a lone voxel is found by diagonal rays from every octant
    g = np.zeros((9, 9, 9), np.uint16)
    g[4, 4, 4] = 7
    for sx in (-1, 1):
        for sy in (-1, 1):
            for sz in (-1, 1):
                o = [4.5 - 10 * sx, 4.5 - 10 * sy, 4.5 - 10 * sz]
                assert O.ray_entry(g, [0, 0, 0], [9, 9, 9], o, [sx, sy, sz]) == (5, 5, 5)


def _near_case(seed=7):
    g = _box_grid()
    frags = O.seeder_uniform(g, 4, seed, 1)
    return g, frags


def _is_boundary(g, v):
    X, Y, Z = g.shape
    x, y, z = v
    box = g[max(x - 1, 0):min(x + 1, X - 1) + 1, max(y - 1, 0):min(y + 1, Y - 1) + 1,
            max(z - 1, 0):min(z + 1, Z - 1) + 1]
    return bool((box == 0).any())


@pytest.mark.parametrize("impacts,nseeds,spread,seed", [(1, 8, 5, 1), (3, 20, 2, 2), (5, 5, 1, 3),
                                                        (2, 32, 5, 4)])
def test_near_seeds_properties(impacts, nseeds, spread, seed):
    g, frags = _near_case()
    out = O.near_seeds(g, frags, impacts, nseeds, spread, seed)
    assert np.array_equal(out[:len(frags)], frags)
    new = out[len(frags):]
    assert 1 <= len(new) <= nseeds
    assert list(new[:, 3]) == list(range(frags[-1, 3] + 1, frags[-1, 3] + 1 + len(new)))
    keys = [tuple(int(c) for c in v[:3]) for v in new]
    assert keys == sorted(keys) and len(set(keys)) == len(keys)
    half = min(g.shape) // 2
    for v in keys:
        assert g[v] != 0 and _is_boundary(g, v)
        d = np.sqrt(((frags[:, :3].astype(np.float64) - np.array(v)) ** 2).sum(axis=1))
        assert d.min() <= half + 1e-6
    # deterministic in the seed
    assert np.array_equal(out, O.near_seeds(g, frags, impacts, nseeds, spread, seed))


def test_near_seeds_places_every_seed_with_enough_impacts():
    g, frags = _near_case()
    # the first impact may take all pending seeds; with many impacts they all go
    out = O.near_seeds(g, frags, 40, 12, 3, 11)
    assert len(out) - len(frags) == 12


def test_near_seeds_search_error_and_invalid_arguments():
    g = np.ones((12, 12, 12), np.uint16)  # no EMPTY voxel: no surface
    frags = np.array([[5, 5, 5, 2]], np.uint32)
    with pytest.raises(O.OracleError) as e:
        O.near_seeds(g, frags, 1, 3, 2, 5)
    assert e.value.status == O.ERR_SEED_SEARCH
    with pytest.raises(O.OracleError):
        O.near_seeds(g, frags, 1, 3, 0, 5)  # spreading 0
    with pytest.raises(O.OracleError):
        O.near_seeds(g, np.zeros((0, 4), np.uint32), 1, 3, 2, 5)  # no seed to impact
    # no impacts: the seeds come back unchanged
    assert np.array_equal(O.near_seeds(g, frags, 0, 3, 2, 5), frags)
