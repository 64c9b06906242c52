"""Generate the golden fixtures of the parity tests.

Each case is a synthetic vessel (voxelfragmentml_gb300.vessel, bit-identical
on x86 and Arm) run through the CPU oracle's whole job
(oracle.run_job: voxelize -> seeds -> fracture -> perturb -> erode |
detectBoundaries -> counts).  Stored per case: the parameters, the mesh's
SHA-256, the grid dims/AABB, the seeds, the uint16 label grid and the
per-fragment counts (compressed .npz).

The reference RLE fixture (docs/decompress/samples/AL_12B_grid_128r.rle of
the reference project, an occupancy grid written by RegularGrid::exportRLE)
is copied next to the cases when the reference tree is available; it pins
the RLE format and the x-major voxel order.

Run:  python tests/golden/make_golden.py [reference_root]
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from voxelfragmentml_gb300 import vessel  # noqa: E402

# name: (angular, profile, mesh_seed, max_dim, params)
CASES = {
    "flood_manhattan_48": (48, 36, 42, 48, dict(algorithm=1, distance=1, num_seeds=8, seed=42,
                                                seed_location=2)),
    "flood_euclid_noise_erode_64": (64, 48, 7, 64, dict(
        algorithm=1, distance=0, num_seeds=16, seed=11, seed_location=2,
        noise_amplitude=2.0, noise_period=16, erode=1, erosion_type=0, erosion_size=3,
        erosion_iterations=1)),
    "flood_chebyshev_noise_60": (64, 48, 3, 60, dict(
        algorithm=1, distance=2, num_seeds=12, seed=5, seed_location=2,
        noise_amplitude=1.5, noise_period=8)),
    "naive_euclid_40": (40, 30, 9, 40, dict(algorithm=0, distance=0, num_seeds=10, seed=3,
                                            seed_location=1)),
    "flood_extra_seeds_44": (44, 33, 13, 44, dict(
        algorithm=1, distance=2, num_seeds=6, num_extra_seeds=12, seed=21, seed_location=1)),
    "flood_ellipse_erode2_52": (52, 39, 17, 52, dict(
        algorithm=1, distance=1, num_seeds=5, seed=8, seed_location=0, erode=1,
        erosion_type=1, erosion_size=3, erosion_iterations=2, erosion_probability=0.6)),
    "flood_cross_erode_boundary2_36": (36, 27, 19, 36, dict(
        algorithm=1, distance=0, num_seeds=4, seed=99, seed_location=2, erode=1,
        erosion_type=2, erosion_size=5, erosion_iterations=1)),
    "flood_boundary3_40": (40, 30, 23, 40, dict(algorithm=1, distance=2, num_seeds=7, seed=31,
                                                seed_location=2, boundary_size=3)),
}


def default_params(**kw) -> oracle.Params:
    p = oracle.Params()
    p.algorithm, p.distance, p.num_seeds, p.num_extra_seeds = 1, 2, 8, 0
    p.merge_distance, p.seed_location, p.seed = 0, 1, 80
    p.noise_amplitude, p.noise_period = 0.0, 16
    p.erode, p.erosion_type, p.erosion_size, p.erosion_iterations = 0, 1, 3, 3
    p.erosion_probability, p.erosion_threshold, p.boundary_size = 0.5, 0.5, 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def mesh_sha(v, f) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(v, np.float32).tobytes())
    h.update(np.ascontiguousarray(f, np.uint32).tobytes())
    return h.hexdigest()


def case_inputs(name):
    A, P, mseed, max_dim, kw = CASES[name]
    v, f = vessel.vessel_mesh(A, P, mseed)
    mn, mx = vessel.mesh_aabb(v)
    dims = vessel.grid_dims(mn, mx, max_dim)
    return v, f, mn, mx, dims, default_params(**kw), kw


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_golden.py <root of the reference checkout>")
    ref_root = sys.argv[1]
    index = {}
    for name in CASES:
        v, f, mn, mx, dims, p, kw = case_inputs(name)
        labels, counts, seeds = oracle.run_job(v, f, dims, mn, mx, p)
        nz = np.nonzero(counts)[0]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), labels=labels, seeds=seeds,
                            count_values=nz.astype(np.uint32), count_numbers=counts[nz])
        index[name] = {"mesh_sha256": mesh_sha(v, f), "dims": list(dims),
                       "aabb_min": [float(x) for x in mn], "aabb_max": [float(x) for x in mx],
                       "params": kw, "occupied": int(counts.sum()),
                       "labels_sha256": hashlib.sha256(labels.tobytes()).hexdigest()}
        print(name, dims, "occupied", int(counts.sum()), "fragments", len(nz))
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(index, fh, indent=1, sort_keys=True)
    src = os.path.join(ref_root, "docs", "decompress", "samples", "AL_12B_grid_128r.rle")
    if os.path.exists(src):
        shutil.copyfile(src, os.path.join(HERE, "AL_12B_grid_128r.rle"))
        print("copied reference RLE fixture")


if __name__ == "__main__":
    main()
