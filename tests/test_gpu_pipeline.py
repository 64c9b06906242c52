"""GPU tests of the job runners: mixed batches of uneven jobs, the server
(continuous batching), determinism alone vs in a mix, admission control and
error statuses."""
import os
import time

import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import vessel as Vs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _job(vf, i, ncounts=512, pinned=False):
    """A small job of the mixed workload: uneven dims, metric and noise drawn
    per job."""
    rng = np.random.default_rng(1000 + i)
    tris = int(rng.integers(1500, 12000))
    A, P = Vs.samples_for_triangles(tris)
    v, f = Vs.vessel_mesh(A, P, 500 + i)
    mn, mx = Vs.mesh_aabb(v)
    dims = tuple(int(4 * round(d / 4)) for d in np.exp(rng.uniform(np.log(24), np.log(72), 3)))
    p = vf.Params.default(
        algorithm=vf.FLOOD if i % 5 else vf.NAIVE, distance=int(rng.integers(0, 3)),
        num_seeds=int(rng.integers(2, 12)), seed=7 + i, seed_location=vf.BOTH,
        noise_amplitude=float(rng.uniform(0, 3)) if i % 3 else 0.0, noise_period=16,
        erode=int(i % 4 == 1), erosion_type=int(rng.integers(0, 3)), erosion_iterations=1)
    return vf.JobSpec(v, f, p, dims=dims, aabb=(mn, mx), ncounts=ncounts, tag=i, pinned=pinned)


def _oracle_job(spec):
    P = spec.params
    q = O.Params()
    for name, _ in O.Params._fields_:
        setattr(q, name, getattr(P, name))
    return O.run_job(spec.verts, spec.faces, spec.dims, spec.aabb[0], spec.aabb[1], q,
                     ncounts=spec.counts.shape[0])


def test_mixed_batch_matches_oracle_and_alone(vf, ctx):
    specs = [_job(vf, i) for i in range(14)]
    res = vf.batch_run(specs, ctx)
    for s, r in zip(specs, res):
        assert r.status == 0
        lab, cnt, seeds = _oracle_job(s)
        assert np.array_equal(s.labels, lab), f"job {s.tag}"
        assert np.array_equal(s.counts, cnt)
        assert r.voxels == int(np.prod(s.dims)) and r.occupied == int(cnt.sum())
    # the same job alone gives the same bits
    for i in (0, 5, 9):
        alone = _job(vf, i)
        (r,) = vf.batch_run([alone], ctx)
        assert np.array_equal(alone.labels, specs[i].labels)


def test_resident_batch_graph_replays_match(vf, ctx):
    # prepare once, execute three times: the first execute captures the stage
    # chain as a CUDA graph, the next ones replay it; every run gives the
    # batch_run bits
    specs = [_job(vf, i, pinned=True) for i in range(10)]
    ref = [_job(vf, i) for i in range(10)]
    vf.batch_run(ref, ctx)
    rb = vf.ResidentBatch(specs, ctx)
    for k in range(3):
        for s in specs:
            s.labels[...] = 0xFFFF
            s.counts[...] = 0
        res = rb.execute(download=True)
        assert rb.graph, "resident chain without host steps runs as a CUDA graph"
        for a, b, r in zip(specs, ref, res):
            assert r.status == 0
            assert np.array_equal(a.labels, b.labels), f"execute {k} job {a.tag}"
            assert np.array_equal(a.counts, b.counts)


def test_resident_batch_with_host_steps_runs_direct(vf, ctx):
    # sub-seed prefixes need the host-driven competition loop: no graph, same bits
    specs, ref = [], []
    for lst in (specs, ref):
        for i in range(3):
            s = _job(vf, 40 + i)
            s.params.algorithm = vf.FLOOD
            s.params.num_extra_seeds = 3
            lst.append(s)
    vf.batch_run(ref, ctx)
    rb = vf.ResidentBatch(specs, ctx)
    for k in range(2):
        res = rb.execute(download=True)
        assert not rb.graph
        for a, b, r in zip(specs, ref, res):
            assert r.status == 0
            assert np.array_equal(a.labels, b.labels)


def test_autotune_and_settings_do_not_change_results(vf, ctx):
    ref = [_job(vf, i) for i in range(8)]
    vf.batch_run(ref, ctx)
    saved = ctx.tuning()
    try:
        chosen = ctx.autotune([_job(vf, i) for i in range(8)])
        assert chosen["parity_grid"] in (4, 8, 16, 32) and chosen["shell_grid"] in (6, 12, 24)
        assert chosen["flood_sweeps"] in (8, 16, 32, 96) and chosen["flood_ctas"] in (0, 2, 3)
        assert ctx.tuning() == chosen
        # extreme settings: one sweep per brick visit (every brick re-queues
        # itself until its keys settle), one CTA per SM, minimal grids
        for kw in (chosen, dict(flood_sweeps=1, flood_ctas=1, parity_grid=1, shell_grid=1),
                   dict(flood_sweeps=3, flood_ctas=0, parity_grid=64, shell_grid=64)):
            ctx.set_tuning(**kw)
            got = [_job(vf, i) for i in range(8)]
            for r in vf.batch_run(got, ctx):
                assert r.status == 0
            for a, b in zip(got, ref):
                assert np.array_equal(a.labels, b.labels), kw
                assert np.array_equal(a.counts, b.counts)
        with pytest.raises(vf.VFError):
            ctx.set_tuning(flood_sweeps=0)
    finally:
        ctx.set_tuning(**saved)


def test_pinned_outputs_any_dims_match_pageable(vf, ctx):
    # pinned outputs are written by the download kernels (16-byte units when
    # Z % 4 == 0, rows otherwise); pageable ones by copies: same bits
    dims_list = [(30, 27, 25), (31, 22, 36), (24, 40, 44), (17, 19, 23)]
    mk = lambda pinned: [_job(vf, 60 + i, pinned=pinned) for i in range(len(dims_list))]
    a, b = mk(True), mk(False)
    for lst in (a, b):
        for s, d in zip(lst, dims_list):
            s.dims = d
            if s.labels is not None:
                s.labels = (vf.pinned_array(d, np.uint16) if lst is a else np.zeros(d, np.uint16))
                s.labels[...] = 0
    ra, rb_ = vf.batch_run(a, ctx), vf.batch_run(b, ctx)
    for x, y, r1, r2 in zip(a, b, ra, rb_):
        assert r1.status == 0 and r2.status == 0
        assert np.array_equal(x.labels, y.labels) and np.array_equal(x.counts, y.counts)
        assert (x.labels != 0).any()


def test_plain_matches_batched(vf, ctx):
    specs = [_job(vf, i) for i in range(6)]
    plain = [_job(vf, i) for i in range(6)]
    vf.batch_run(specs, ctx)
    res = vf.plain_run(plain, ctx)
    for a, b, r in zip(specs, plain, res):
        assert r.status == 0
        assert np.array_equal(a.labels, b.labels) and np.array_equal(a.counts, b.counts)


def test_server_continuous_batching_same_results(vf, ctx):
    specs = [_job(vf, i) for i in range(20)]
    ref = [_job(vf, i) for i in range(20)]
    vf.batch_run(ref, ctx)
    srv = vf.Server(ctx, max_inflight=3, max_batch=4)
    try:
        got = []
        for s in specs[:8]:
            srv.submit(s)
        time.sleep(0.01)
        for s in specs[8:]:  # arrive while the first micro-batches run
            srv.submit(s)
        deadline = time.time() + 120
        while len(got) < len(specs) and time.time() < deadline:
            got += srv.poll(64, wait_ms=100)
        assert len(got) == len(specs)
        for r in got:
            assert r.status == 0
            assert r.done_ms >= r.submit_ms
            s = specs[r.user_tag]
            assert np.array_equal(s.labels, ref[r.user_tag].labels)
            assert np.array_equal(s.counts, ref[r.user_tag].counts)
    finally:
        srv.close()


def test_server_admission_respects_budget(vf, ctx):
    specs = [_job(vf, i) for i in range(6)]
    srv = vf.Server(ctx, hbm_budget=1, max_inflight=2, max_batch=8)  # admits one job at a time
    try:
        for s in specs:
            srv.submit(s)
        got = []
        deadline = time.time() + 120
        while len(got) < len(specs) and time.time() < deadline:
            got += srv.poll(64, wait_ms=100)
        assert len(got) == len(specs) and all(r.status == 0 for r in got)
    finally:
        srv.close()


def test_job_errors_are_statuses(vf, ctx):
    ok = _job(vf, 2)
    bad = _job(vf, 3)
    bad.params.num_seeds = 300  # above 254 fragment ids
    with pytest.raises(vf.VFError) as e:
        vf.batch_run([ok, bad], ctx)
    assert e.value.status == vf.ERR_RANGE
    # a job whose seeds cannot be found fails alone; the rest of the batch is fine
    tiny = _job(vf, 4)
    tiny.verts = (tiny.verts * 0.01).astype(np.float32)  # mesh far smaller than its grid
    tiny.params.num_seeds = 200
    res = vf.batch_run([_job(vf, 6), tiny], ctx)
    assert res[0].status == 0 and res[1].status == vf.ERR_SEED_SEARCH


def test_context_budget_oom(vf):
    c = vf.Context(0, hbm_budget=1 << 20)
    try:
        with pytest.raises(vf.VFError) as e:
            vf.batch_run([_job(vf, 1)], c)
        assert e.value.status == vf.ERR_OOM
    finally:
        c.close()


def test_arenas_fall_back_below_doubled_size(vf):
    # arenas grow to twice the size asked for; under a budget that cannot
    # hold the doubled sizes they take 1/8 more or the exact size instead,
    # and the batch runs with the same results
    v, f = Vs.vessel_mesh(128, 96, 42)
    mn, mx = Vs.mesh_aabb(v)
    p = vf.Params.default(distance=vf.CHEBYSHEV, num_seeds=8, seed=42, seed_location=vf.BOTH)
    spec = vf.JobSpec(v, f, p, dims=Vs.grid_dims(mn, mx, 128), aabb=(mn, mx), ncounts=256)
    big = vf.Context(0)
    try:
        (r0,) = vf.batch_run([spec], big)
        assert r0.status == 0
        lab0 = spec.labels.copy()
        doubled = big.bytes_in_use
    finally:
        big.close()
    tight = vf.Context(0, hbm_budget=doubled - (1 << 20))
    try:
        spec.labels[...] = 0
        (r1,) = vf.batch_run([spec], tight)
        assert r1.status == 0
        assert tight.bytes_in_use <= doubled - (1 << 20)
        assert np.array_equal(spec.labels, lab0)
    finally:
        tight.close()


def test_config1_vessel_128(vf, ctx):
    """128-max-dim vessel, 8 fragments, Manhattan flood, seed 42 (the
    CPU-runnable configuration) against the oracle."""
    v, f = Vs.vessel_mesh(128, 96, 42)
    mn, mx = Vs.mesh_aabb(v)
    dims = Vs.grid_dims(mn, mx, 128)
    p = vf.Params.default(distance=vf.MANHATTAN, num_seeds=8, seed=42, seed_location=vf.BOTH)
    spec = vf.JobSpec(v, f, p, dims=dims, aabb=(mn, mx), ncounts=256)
    (r,) = vf.batch_run([spec], ctx)
    lab, cnt, _ = _oracle_job(spec)
    assert r.status == 0 and np.array_equal(spec.labels, lab) and np.array_equal(spec.counts, cnt)


def test_batch_with_empty_mesh_job(vf, ctx):
    # a job without triangles (grid and AABB given) stays empty and fails its
    # seed search alone; its neighbours in the batch are unaffected
    ok1, ok2 = _job(vf, 7), _job(vf, 8)
    ref = [_job(vf, 7), _job(vf, 8)]
    vf.batch_run(ref, ctx)
    p = vf.Params.default(num_seeds=4, seed_location=vf.BOTH)
    empty = vf.JobSpec(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), p,
                       dims=(20, 24, 28), aabb=((0, 0, 0), (1, 1, 1)), ncounts=256, tag=99)
    res = vf.batch_run([ok1, empty, ok2], ctx)
    assert res[0].status == 0 and res[2].status == 0
    assert res[1].status == vf.ERR_SEED_SEARCH
    assert not empty.labels.any()
    assert np.array_equal(ok1.labels, ref[0].labels) and np.array_equal(ok2.labels, ref[1].labels)


def test_large_batch_matches_small_batches(vf, ctx):
    # 40 jobs in one batch (pinned and pageable outputs mixed) and the same
    # jobs in batches of 8 give the same bits
    n = 40
    big = [_job(vf, 100 + i, pinned=(i % 2 == 0)) for i in range(n)]
    small = [_job(vf, 100 + i) for i in range(n)]
    res = vf.batch_run(big, ctx)
    for k in range(0, n, 8):
        for r in vf.batch_run(small[k:k + 8], ctx):
            assert r.status == 0
    for a, b, r in zip(big, small, res):
        assert r.status == 0 and r.user_tag == a.tag
        assert np.array_equal(a.labels, b.labels), f"job {a.tag}"
        assert np.array_equal(a.counts, b.counts)


def test_pipeline_overlapped_batches_match_batch_run(vf, ctx):
    """vf_pipeline_*: batches in flight (pinned and pageable outputs, odd
    dims) give the bits of vf_batch_run, collected in submission order; a
    full pipeline refuses another batch; collect with nothing in flight is an
    error."""
    ref = {}
    for i in range(12):
        s = _job(vf, i)
        vf.batch_run([s], ctx)
        ref[i] = (s.labels.copy(), s.counts.copy())
    pipe = vf.Pipeline(ctx, depth=2)
    batches = [[_job(vf, i, pinned=bool(i % 2)) for i in range(k, k + 4)] for k in (0, 4, 8)]
    pipe.submit(batches[0])
    pipe.submit(batches[1])
    with pytest.raises(vf.VFError) as e:
        pipe.submit(batches[2])
    assert e.value.status == vf.ERR_BUSY
    done = [pipe.collect()]
    pipe.submit(batches[2])
    done += [pipe.collect(), pipe.collect()]
    for b, res in zip(batches, done):
        assert len(res) == len(b)
        for s, r in zip(b, res):
            assert r.status == 0
            assert np.array_equal(s.labels, ref[s.tag][0]), f"job {s.tag}"
            assert np.array_equal(s.counts, ref[s.tag][1])
    with pytest.raises(vf.VFError):
        pipe.collect()
    pipe.close()
