"""Generate tests/golden/ref_pins.npz from the reference's own code.

The reference pin (oracle/_ref/libvfref.so, built by `make -C oracle ref`
from the reference checkout) runs, unchanged:
  - Intersections3D::intersect(Triangle3D&, AABB&) (Intersections3D.h:204-258)
  - NaiveFracturer::buildCPU (NaiveFracturer.cpp:26-68)
  - Seeder::mergeSeeds (Seeder.cpp:115-152)
This script feeds them seeded inputs and stores inputs and outputs, so that
machines without the reference checkout (the GPU tests) still compare against
the reference's results.

usage: make_ref_pins.py <reference MeshFragments/Source directory>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def tri_box_cases(rng, n):
    """Triangles against voxel-sized boxes, many of them touching or grazing."""
    tris = (rng.random((n, 9)) * 4 - 2).astype(np.float32)
    cell = rng.choice([1.0, 0.5, 0.25, 1e-3, 3e4], size=(n, 1)).astype(np.float32)
    corner = rng.integers(-2, 2, (n, 3)).astype(np.float32) * cell
    # a third of the triangles have vertices on the box's faces or edges
    k = n // 3
    tris[:k] = (np.round(tris[:k] * 4) / 4).astype(np.float32)
    boxes = np.concatenate([corner, corner + cell], 1).astype(np.float32)
    scale = np.where(cell > 1e3, cell, 1.0).astype(np.float32)
    tris = (tris * scale).astype(np.float32)
    return tris, boxes


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_ref_pins.py <reference MeshFragments/Source directory>")
    import ctypes as C
    import oracle as O
    path = O.build_ref(sys.argv[1])
    R = O.ref_lib()
    if R is None:
        raise SystemExit(f"reference pin not built ({path})")
    P = C.c_void_p
    rng = np.random.default_rng(20261204)
    out = {}
    tris, boxes = tri_box_cases(rng, 3000)
    res = np.zeros(len(tris), np.uint8)
    R.vfr_tri_box_batch(tris.ctypes.data_as(P), boxes.ctypes.data_as(P), len(tris),
                        res.ctypes.data_as(P))
    out.update(tribox_tris=tris, tribox_boxes=boxes, tribox_hit=res)
    for gi, shape in enumerate([(20, 17, 23), (31, 9, 14), (12, 28, 19)]):
        occ = (rng.random(shape) < 0.55).astype(np.uint16)
        cells = np.argwhere(occ != 0)
        ns = [5, 17, 40][gi]
        pick = cells[rng.choice(len(cells), ns, replace=False)]
        labels = np.arange(2, 2 + ns) if gi != 1 else rng.integers(2, 250, ns)
        seeds = np.concatenate([pick, labels[:, None]], 1).astype(np.uint32)
        out[f"naive{gi}_grid"] = occ
        out[f"naive{gi}_seeds"] = seeds
        for d in (0, 1, 2):
            g = occ.copy()
            assert R.vfr_naive(g.ctypes.data_as(P), *shape, seeds.ctypes.data_as(P), ns, d) == 0
            out[f"naive{gi}_labels{d}"] = g
    for mi in range(6):
        nf, ns = [3, 8, 20, 1, 12, 30][mi], [10, 25, 60, 5, 40, 90][mi]
        frags = np.concatenate([rng.integers(0, 48 if mi % 2 else 4, (nf, 3)),
                                (2 + np.arange(nf))[:, None]], 1).astype(np.uint32)
        seeds = np.concatenate([rng.integers(0, 48, (ns, 3)), np.zeros((ns, 1))], 1).astype(np.uint32)
        out[f"merge{mi}_frags"] = frags
        out[f"merge{mi}_seeds"] = seeds
        for d in (0, 1, 2):
            s = seeds.copy()
            assert R.vfr_merge_seeds(frags.ctypes.data_as(P), nf, s.ctypes.data_as(P), ns, d) == 0
            out[f"merge{mi}_labels{d}"] = s[:, 3].copy()
    np.savez_compressed(os.path.join(HERE, "ref_pins.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
