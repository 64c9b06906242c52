"""Synthetic workloads of the benchmarks (seeded; identical on every host).

* ``mixed(n)``  -- the batching workload: n vessels with uneven grids, each
  axis log-uniform in [64, 384] (x and z rounded to multiples of 4 as
  CADScene.cpp:254-265 does), 5k-200k triangles (log-uniform), 2-32
  fragments, metric and noise amplitude (0-3 voxels, period 16) drawn per
  job, flood fracture, detectBoundaries(1).
* ``single(max_dim, angular, profile, ...)`` -- one vessel job.

Jobs are plain dicts; ``to_spec`` turns one into a JobSpec with its mesh.
"""
from __future__ import annotations

import math

import numpy as np

from . import vessel as _vs


def mixed(n: int = 256, master_seed: int = 2024):
    rng = np.random.default_rng(master_seed)
    jobs = []
    lo, hi = math.log(64), math.log(384)
    for i in range(n):
        d = [int(round(math.exp(rng.uniform(lo, hi)))) for _ in range(3)]
        d[0] = max(64, 4 * round(d[0] / 4))
        d[2] = max(64, 4 * round(d[2] / 4))
        tris = int(round(math.exp(rng.uniform(math.log(5000), math.log(200000)))))
        jobs.append(dict(index=i, dims=tuple(d), triangles=tris,
                         fragments=int(rng.integers(2, 33)), distance=int(rng.integers(0, 3)),
                         amplitude=float(rng.uniform(0.0, 3.0)), period=16,
                         mesh_seed=master_seed * 1000 + i, seed=int(rng.integers(1, 2**31))))
    return jobs


def single(max_dim=128, angular=128, profile=96, fragments=8, distance=1, amplitude=0.0,
           period=16, erode=False, mesh_seed=42, seed=42):
    return dict(index=0, dims=None, max_dim=max_dim, angular=angular, profile=profile,
                fragments=fragments, distance=distance, amplitude=amplitude, period=period,
                erode=erode, mesh_seed=mesh_seed, seed=seed)


def mesh_for(job):
    if "angular" in job:
        A, P = job["angular"], job["profile"]
    else:
        A, P = _vs.samples_for_triangles(job["triangles"])
    return _vs.vessel_mesh(A, P, job["mesh_seed"])


def params_for(job, V):
    kw = dict(algorithm=V.FLOOD, distance=job["distance"], num_seeds=job["fragments"],
              seed=job["seed"], seed_location=V.BOTH, noise_amplitude=job["amplitude"],
              noise_period=job["period"], boundary_size=1)
    if job.get("erode"):
        kw.update(erode=1, erosion_type=V.SQUARE, erosion_size=3, erosion_iterations=1)
    return kw


def to_spec(job, V, want_labels=True, ncounts=256, pinned=False):
    v, f = mesh_for(job)
    mn, mx = _vs.mesh_aabb(v)
    dims = job["dims"] or _vs.grid_dims(mn, mx, job["max_dim"])
    p = V.Params.default(**params_for(job, V))
    if pinned:
        pv = V.pinned_array(v.shape, np.float32)
        pv[...] = v
        pf = V.pinned_array(f.shape, np.uint32)
        pf[...] = f
        v, f = pv, pf
    spec = V.JobSpec(v, f, p, dims=dims, aabb=(mn, mx), want_labels=False, ncounts=ncounts,
                     tag=job["index"], pinned=pinned)
    if want_labels:
        spec.labels = V.pinned_array(spec.dims, np.uint16) if pinned else np.zeros(spec.dims, np.uint16)
    return spec
