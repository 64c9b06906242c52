"""Full-size parity of the benchmark configurations: the 256^3 vessel
(Euclidean, noise A=2 P=16, one 3x3x3 erosion), the 512^3 vessel (64
fragments, Chebyshev, noise) and jobs of the mixed-256 batch at their own
sizes, each through the batched path and compared bit for bit (labels and
per-fragment counts) with the oracle's whole job."""
import numpy as np
import pytest

import oracle as O
from voxelfragmentml_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _oracle_run(spec):
    q = O.Params()
    for name, _ in O.Params._fields_:
        setattr(q, name, getattr(spec.params, name))
    return O.run_job(spec.verts, spec.faces, spec.dims, spec.aabb[0], spec.aabb[1], q,
                     ncounts=spec.counts.shape[0])


def _check(vf, ctx, job, plain=False):
    spec = W.to_spec(job, vf, want_labels=True, ncounts=256)
    (r,) = vf.batch_run([spec], ctx)
    assert r.status == 0, vf.lib().vf_last_error()
    lab, cnt, _ = _oracle_run(spec)
    assert int(np.count_nonzero(spec.labels != lab)) == 0
    assert np.array_equal(spec.counts, cnt)
    assert r.occupied == int(cnt.sum())
    if plain:
        ps = W.to_spec(job, vf, want_labels=True, ncounts=256)
        (pr,) = vf.plain_run([ps], ctx)
        assert pr.status == 0
        assert np.array_equal(ps.labels, lab)
        assert np.array_equal(ps.counts, cnt)
    return r


def test_config2_256_euclidean_noise_erosion(vf, ctx):
    # 256x192 vessel (196,608 triangles), 256^3, 16 fragments, Euclidean,
    # value-noise perturbation A=2 P=16, one 3x3x3 erosion pass
    r = _check(vf, ctx, W.single(256, 256, 192, 16, 0, 2.0, 16, True, 42, 42), plain=True)
    assert r.fragments >= 2


def test_config3_512_chebyshev_noise(vf, ctx):
    # 512x384 vessel (786,432 triangles), 512^3, 64 fragments, Chebyshev, noise
    r = _check(vf, ctx, W.single(512, 512, 384, 64, 2, 2.0, 16, False, 42, 42))
    assert r.fragments >= 32


def test_mixed256_headline_jobs_full_size(vf, ctx):
    # the largest job of the headline batch, and jobs of every metric, at
    # their own (uneven) sizes, in one batch
    jobs = W.mixed(256)
    big = max(jobs, key=lambda j: int(np.prod(j["dims"])))
    pick = [big] + [next(j for j in jobs if j["distance"] == d and j is not big) for d in (0, 1, 2)]
    specs = [W.to_spec(j, vf, want_labels=True, ncounts=256) for j in pick]
    res = vf.batch_run(specs, ctx)
    for s, r in zip(specs, res):
        assert r.status == 0
        lab, cnt, _ = _oracle_run(s)
        assert int(np.count_nonzero(s.labels != lab)) == 0, f"job {s.tag} dims {s.dims}"
        assert np.array_equal(s.counts, cnt)
