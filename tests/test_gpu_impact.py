"""GPU parity of the impact path (CADScene::hit + Seeder::nearSeeds): ray entry
voxels and near seeds through the C ABI against the CPU oracle.

Tolerance: none.  The ray walk rounds every float step as the oracle does,
and the seed draws come from the same counter-based hash, so indices and
seeds must be identical.
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


def _case(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    _, _, mn, mx, dims, _, _ = m.case_inputs(name)
    return np.load(os.path.join(GOLD, name + ".npz"))["labels"], np.asarray(mn), np.asarray(mx)


def _rays(mn, mx, n, seed):
    rng = np.random.default_rng(seed)
    c = (mn + mx) / 2
    ext = (mx - mn)
    o = c + (rng.random((n, 3)) - 0.5) * ext * 3.0      # inside and outside the box
    tgt = c + (rng.random((n, 3)) - 0.5) * ext * 0.8
    d = tgt - o
    # some axis-aligned and some with zero components
    d[: n // 8, 1:] = 0
    d[n // 8: n // 4, 2] = 0
    d[n // 4: n // 4 + 4] = -d[n // 4: n // 4 + 4]      # pointing away
    d[np.all(d == 0, axis=1)] = [1, 0, 0]
    return np.concatenate([o, d], axis=1).astype(np.float32)


@pytest.mark.parametrize("name", CASES[:4])
def test_ray_entry_matches_oracle(vf, ctx, name):
    labels, mn, mx = _case(name)
    g = vf.RegularGrid(labels.shape, mn, mx, ctx)
    g.upload(labels)
    rays = _rays(mn, mx, 512, 3)
    got = g.rayEntryVoxels(rays)
    for i, r in enumerate(rays):
        e = O.ray_entry(labels, mn, mx, r[:3], r[3:])
        exp = np.array(e if e is not None else (0xFFFFFFFF,) * 3, np.uint32)
        assert np.array_equal(got[i], exp), (i, r, got[i], exp)
    assert (got[:, 0] != 0xFFFFFFFF).sum() > 64  # many rays hit
    g.close()


def test_ray_entry_single_and_errors(vf, ctx):
    g0 = np.zeros((20, 22, 24), np.uint16)
    g0[4:16, 5:18, 6:20] = 3
    g = vf.RegularGrid(g0.shape, [0, 0, 0], [20, 22, 24], ctx)
    g.upload(g0)
    assert g.getClosestEntryVoxel([-5, 11.5, 12.5], [1, 0, 0]) == (5, 12, 13)
    assert g.getClosestEntryVoxel([-5, 30, 12.5], [1, 0, 0]) is None
    with pytest.raises(vf.VFError):
        g.getClosestEntryVoxel([-5, 11.5, 12.5], [0, 0, 0])
    g.close()


@pytest.mark.parametrize("name", CASES[:3])
@pytest.mark.parametrize("impacts,nseeds,spread,seed", [(1, 32, 5, 80), (3, 16, 2, 7),
                                                        (6, 40, 1, 9)])
def test_near_seeds_match_oracle(vf, ctx, name, impacts, nseeds, spread, seed):
    labels, mn, mx = _case(name)
    occ = (labels != 0).astype(np.uint16)  # the voxelized grid nearSeeds runs on
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    frags = O.seeder_uniform(occ, 6, seed, 1)
    got = vf.Seeder.nearSeeds(g, frags, impacts, nseeds, spread, seed)
    exp = O.near_seeds(occ, frags, impacts, nseeds, spread, seed)
    assert np.array_equal(got, exp)
    assert len(got) > len(frags)
    g.close()


def test_near_seeds_from_a_ray_impact(vf, ctx):
    # CADScene::hit: the entry voxel becomes the one given seed (label 2)
    labels, mn, mx = _case(CASES[0])
    occ = (labels != 0).astype(np.uint16)
    g = vf.RegularGrid(occ.shape, mn, mx, ctx)
    g.upload(occ)
    c = (mn + mx) / 2
    hit = g.getClosestEntryVoxel(c - np.array([0, 0, 2 * (mx[2] - mn[2])]), [0, 0.05, 1])
    assert hit is not None
    frags = np.array([[*hit, 2]], np.uint32)
    got = vf.Seeder.nearSeeds(g, frags, 1, 32, 5, 80)
    assert np.array_equal(got, O.near_seeds(occ, frags, 1, 32, 5, 80))
    g.close()


def test_near_seeds_errors_match(vf, ctx):
    full = np.ones((16, 16, 16), np.uint16)  # no EMPTY voxel: no surface to seed
    g = vf.RegularGrid(full.shape, None, None, ctx)
    g.upload(full)
    frags = np.array([[5, 5, 5, 2]], np.uint32)
    with pytest.raises(vf.VFError) as e:
        vf.Seeder.nearSeeds(g, frags, 1, 3, 2, 5)
    assert e.value.status == vf.ERR_SEED_SEARCH
    with pytest.raises(vf.VFError):
        vf.Seeder.nearSeeds(g, frags, 1, 3, 0, 5)
    assert np.array_equal(vf.Seeder.nearSeeds(g, frags, 0, 3, 2, 5), frags)
    g.close()


# ---- impacts inside CADScene::fractureModel (num_impacts > 0) ---------------
def _job(name):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.case_inputs(name)


def _oracle_params(vf, p):
    q = O.Params()
    for name, _ in O.Params._fields_:
        setattr(q, name, getattr(p, name))
    return q


@pytest.mark.parametrize("name,impacts,bias,focus,extra", [
    ("flood_manhattan_48", 2, 32, 5, 0), ("flood_chebyshev_noise_60", 1, 12, 3, 0),
    ("flood_extra_seeds_44", 3, 20, 5, 16)])
def test_fracture_model_with_impacts(vf, ctx, name, impacts, bias, focus, extra):
    v, f, mn, mx, dims, _, kw = _job(name)
    kw = dict(kw, num_impacts=impacts, bias_seeds=bias, bias_focus=focus)
    if extra:
        kw["num_extra_seeds"] = extra
    p = vf.Params.default(**kw)
    g = vf.RegularGrid(dims, mn, mx, ctx)
    g.fill(v, f)
    seeds = vf.fracture_model(g, p)
    lab, cnt, es = O.run_job(v, f, dims, mn, mx, _oracle_params(vf, p), ncounts=1024)
    assert np.array_equal(seeds, es)
    assert len(seeds) > p.num_seeds  # the impacts placed seeds
    assert np.array_equal(g.data(), lab)
    g.close()


def test_batch_and_plain_paths_with_impacts(vf, ctx):
    specs, exp = [], []
    for name in ("flood_manhattan_48", "naive_euclid_40"):
        v, f, mn, mx, dims, _, kw = _job(name)
        p = vf.Params.default(**dict(kw, num_impacts=2, bias_seeds=16, bias_focus=4))
        specs.append(vf.JobSpec(v, f, p, dims=dims, aabb=(mn, mx), ncounts=1024))
        exp.append(O.run_job(v, f, dims, mn, mx, _oracle_params(vf, p), ncounts=1024))
    res = vf.batch_run(specs, ctx)
    for s, r, (lab, cnt, es) in zip(specs, res, exp):
        assert r.status == 0 and r.nseeds == len(es)
        assert np.array_equal(s.labels, lab)
        assert np.array_equal(s.counts, cnt[:1024])
    plain = [vf.JobSpec(s.verts, s.faces, s.params, dims=s.dims, aabb=s.aabb, ncounts=1024)
             for s in specs]
    vf.plain_run(plain, ctx)
    for a, b in zip(plain, specs):
        assert np.array_equal(a.labels, b.labels)


def test_ray_batches_walk_the_occupancy_bits(vf, ctx):
    # 4096 rays or more read a packed occupancy bitmap; the answers stay the oracle's
    labels, mn, mx = _case(CASES[1])
    g = vf.RegularGrid(labels.shape, mn, mx, ctx)
    g.upload(labels)
    rays = _rays(mn, mx, 6000, 17)
    got = g.rayEntryVoxels(rays)
    assert np.array_equal(got, O.ray_entry_batch(labels, mn, mx, rays))
    assert np.array_equal(got[:100], g.rayEntryVoxels(rays[:100]))  # the direct path agrees
    g.close()
