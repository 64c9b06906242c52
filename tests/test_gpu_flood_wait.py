"""The flood relaxation's bounded device wait: its pass barrier gives up
after a spin limit, sets an error word and returns, so the call fails with
VF_ERR_TIMEOUT instead of hanging, and the context stays usable.  The test
sets a limit of a few spins on a grid that needs many passes (the wait runs
out), then floods the same grid on the same context at the default limit and
compares with the oracle bit for bit."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _corridor():
    # a serpentine corridor: hundreds of BFS waves, many relaxation passes
    X, Y, Z = 40, 34, 70
    occ = np.zeros((X, Y, Z), np.uint16)
    for y in range(0, Y, 2):
        occ[:, y, :] = 1
        if y + 1 < Y:
            occ[:, y + 1, (Z - 1) if (y // 2) % 2 == 0 else 0] = 1
    seeds = np.array([[3, 0, 0, 2], [5, Y - 1, Z - 1, 3]], np.uint32)
    return occ, seeds


def test_flood_barrier_wait_runs_out_then_context_recovers(vf):
    occ, seeds = _corridor()
    exp, _ = O.flood(occ, seeds, 1)
    ctx = vf.Context(0)
    try:
        L = vf.lib()
        assert L.vf_ctx_set_flood_wait_limit(ctx.h, 2) == vf.OK
        g = vf.RegularGrid(occ.shape, None, None, ctx)
        g.upload(occ)
        fr = vf.FloodFracturer()
        fr.setDistanceFunction(vf.MANHATTAN)
        with pytest.raises(vf.VFError) as e:
            fr.build(g, seeds)
        assert e.value.status == vf.ERR_TIMEOUT
        g.close()
        # default limit: the same context floods the grid correctly
        assert L.vf_ctx_set_flood_wait_limit(ctx.h, 0) == vf.OK
        g = vf.RegularGrid(occ.shape, None, None, ctx)
        g.upload(occ)
        fr.build(g, seeds)
        assert np.array_equal(g.data(), exp)
        # and a batched job after it
        from voxelfragmentml_gb300 import vessel as Vs
        v, f = Vs.vessel_mesh(48, 36, 3)
        mn, mx = Vs.mesh_aabb(v)
        p = vf.Params.default(distance=vf.CHEBYSHEV, num_seeds=6, seed=5, seed_location=vf.BOTH)
        spec = vf.JobSpec(v, f, p, dims=Vs.grid_dims(mn, mx, 60), aabb=(mn, mx), ncounts=256)
        (r,) = vf.batch_run([spec], ctx)
        assert r.status == 0
        q = O.Params()
        for name, _ in O.Params._fields_:
            setattr(q, name, getattr(p, name))
        lab, cnt, _ = O.run_job(v, f, spec.dims, mn, mx, q, ncounts=256)
        assert np.array_equal(spec.labels, lab) and np.array_equal(spec.counts, cnt)
        g.close()
    finally:
        ctx.close()
