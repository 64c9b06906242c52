"""Pin the marching-cubes case table against the reference.

Reads MarchingCubes.cpp of the reference project (its _triangleTable and
_edgeTable arrays) and writes tests/golden/mc_tables.json: SHA-256 digests of
both tables in a canonical text form.  tests/test_mesh_oracle.py recomputes
the digests from voxelfragmentml_gb300/csrc/vf_mc_table.h, so the table the
kernels and the oracle use is pinned to the reference's own.

Canonical forms: triangles -- for each of the 256 configurations, the edge
indices before the first -1 joined by ',', configurations joined by ';';
edge flags -- the 256 values in decimal joined by ','.

Run:  python tests/golden/make_mc_table_fixture.py [reference_root]
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def canonical_triangles(rows):
    return ";".join(",".join(str(e) for e in r) for r in rows)


def canonical_edges(vals):
    return ",".join(str(v) for v in vals)


def digest(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def main(ref_root: str) -> None:
    path = os.path.join(ref_root, "MeshFragments", "Source", "Graphics", "Core", "MarchingCubes.cpp")
    src = open(path, encoding="utf-8", errors="replace").read()
    body = re.search(r"_triangleTable\[256 \* 16\] = \{(.*?)\};", src, re.S).group(1)
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(vals) == 4096
    rows = []
    for c in range(256):
        r = []
        for v in vals[16 * c:16 * c + 16]:
            if v < 0:
                break
            r.append(v)
        rows.append(r)
    body = re.search(r"_edgeTable\[256\] = \{(.*?)\};", src, re.S).group(1)
    edges = [int(v, 0) for v in re.findall(r"0x[0-9a-fA-F]+|\d+", body)]
    assert len(edges) == 256
    out = {
        "source": "MeshFragments/Source/Graphics/Core/MarchingCubes.cpp (_triangleTable, _edgeTable)",
        "triangles_sha256": digest(canonical_triangles(rows)),
        "edges_sha256": digest(canonical_edges(edges)),
        "triangle_count_total": sum(len(r) // 3 for r in rows),
    }
    with open(os.path.join(HERE, "mc_tables.json"), "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")
    print(out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_mc_table_fixture.py <root of the reference checkout>")
    main(sys.argv[1])
