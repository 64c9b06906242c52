"""ctypes binding of the CPU oracle (oracle/vf_oracle.c).

TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
Imported by tests/, __graft_entry__.smoke() and bench.py's CPU arms; the
product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libvforacle.so")
_lib = None

OK, ERR_INVALID, ERR_SEED_SEARCH, ERR_RANGE = 0, 1, 4, 5


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (seconds)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < max(
                os.path.getmtime(os.path.join(_HERE, f))
                for f in ("vf_oracle.c", "vf_oracle_mesh.c", "vf_oracle_impact.c",
                          "vf_oracle_sample.c", "vf_oracle.h",
                          "Makefile",
                          os.path.join("..", "voxelfragmentml_gb300", "csrc",
                                       "vf_mc_table.h")))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_REF_LIB = os.path.join(_HERE, "_ref", "libvfref.so")
_ref = None


def build_ref(ref_root: str | None = None) -> str | None:
    """Compile the reference pin (`make ref`: the reference's own tri-box,
    NaiveFracturer::buildCPU and Seeder::mergeSeeds, unchanged, against the
    stand-ins in oracle/ref_shim/) when the reference checkout is present;
    None when it is not."""
    src = ref_root or os.environ.get("VF_REFERENCE_SOURCE", "")
    if not src:
        for cand in (os.path.join(_HERE, "..", "..", "reference", "MeshFragments", "Source"),):
            if os.path.isdir(cand):
                src = cand
    if not src or not os.path.isdir(src):
        return _REF_LIB if os.path.exists(_REF_LIB) else None
    r = subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={os.path.abspath(src)}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference pin build failed:\n" + r.stderr[-4000:])
    return _REF_LIB


def ref_lib():
    """The compiled reference pin (vfr_tri_box, vfr_tri_box_batch, vfr_naive,
    vfr_merge_seeds), or None when it cannot be built here."""
    global _ref
    if _ref is None:
        path = build_ref()
        if not path or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        P, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.vfr_tri_box.restype = i32
        L.vfr_tri_box.argtypes = [P, P, P, P, P]
        L.vfr_tri_box_batch.restype = None
        L.vfr_tri_box_batch.argtypes = [P, P, u32, P]
        L.vfr_naive.restype = i32
        L.vfr_naive.argtypes = [P, u32, u32, u32, P, u32, i32]
        L.vfr_merge_seeds.restype = i32
        L.vfr_merge_seeds.argtypes = [P, u32, P, u32, i32]
        _ref = L
    return _ref


class Params(C.Structure):
    _fields_ = [("algorithm", C.c_int32), ("distance", C.c_int32),
                ("num_seeds", C.c_int32), ("num_extra_seeds", C.c_int32),
                ("merge_distance", C.c_int32), ("seed_location", C.c_int32),
                ("seed", C.c_uint64), ("noise_amplitude", C.c_float),
                ("noise_period", C.c_uint32), ("erode", C.c_int32),
                ("erosion_type", C.c_int32), ("erosion_size", C.c_int32),
                ("erosion_iterations", C.c_int32),
                ("erosion_probability", C.c_float),
                ("erosion_threshold", C.c_float), ("boundary_size", C.c_int32),
                ("num_impacts", C.c_int32), ("bias_seeds", C.c_int32), ("bias_focus", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.c_void_p
        u32, u64, i32, f32 = C.c_uint32, C.c_uint64, C.c_int, C.c_float
        sig = {
            "vfo_hash": (u64, [u64, u32, u64]),
            "vfo_u01": (f32, [u64]),
            "vfo_voxelize": (i32, [P, u32, P, u32, u32, u32, u32, P, P, P, i32]),
            "vfo_tri_box": (i32, [P, P, P, P, P]),
            "vfo_grid_dims": (None, [P, P, u32, P]),
            "vfo_seeder_uniform": (i32, [P, u32, u32, u32, u32, u64, i32, P]),
            "vfo_merge_seeds": (i32, [P, u32, P, u32, i32]),
            "vfo_fracture_seeds": (i32, [P, u32, u32, u32, u32, u32, i32, i32, u64, u32, u32,
                                         u32, P, P]),
            "vfo_flood": (i32, [P, u32, u32, u32, P, u32, i32, P]),
            "vfo_naive": (i32, [P, u32, u32, u32, P, u32, i32]),
            "vfo_perturb": (i32, [P, u32, u32, u32, f32, u32, u64]),
            "vfo_detect_boundaries": (None, [P, u32, u32, u32, i32]),
            "vfo_remove_isolated": (None, [P, u32, u32, u32]),
            "vfo_erode": (i32, [P, u32, u32, u32, i32, u32, u32, f32, f32, u64]),
            "vfo_undo_mask": (None, [P, u32, u32, u32]),
            "vfo_count_values": (i32, [P, u32, u32, u32, P, u32, P]),
            "vfo_run_job": (i32, [P, u32, P, u32, u32, u32, u32, P, P, P, P, P, u32, P, P]),
            "vfo_rle_encode": (C.c_size_t, [P, u32, u32, u32, P, C.c_size_t]),
            "vfo_triangulate": (i32, [P, u32, u32, u32, P, P, u32, f32, u32, f32,
                                      P, P, P, P, P, P, P, P]),
            "vfo_ray_entry": (i32, [P, u32, u32, u32, P, P, P, P, P]),
            "vfo_sample_mesh": (i32, [P, P, u32, u32, u64, u32, P, P]),
            "vfo_ray_entry_batch": (i32, [P, u32, u32, u32, P, P, P, u32, P]),
            "vfo_near_seeds": (i32, [P, u32, u32, u32, P, u32, u32, u32, u32, u64, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


class OracleError(RuntimeError):
    def __init__(self, status, what):
        super().__init__(f"{what}: oracle status {status}")
        self.status = status


def _check(st, what):
    if st != OK:
        raise OracleError(st, what)


def voxelize(verts, faces, dims, aabb_min, aabb_max, mode=3):
    X, Y, Z = (int(d) for d in dims)
    v = np.ascontiguousarray(verts, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.uint32)
    g = np.empty((X, Y, Z), dtype=np.uint16)
    mn, mx = _f3(aabb_min), _f3(aabb_max)
    _check(lib().vfo_voxelize(_p(v), v.shape[0], _p(f), f.shape[0], X, Y, Z,
                              _p(mn), _p(mx), _p(g), mode), "voxelize")
    return g


def tri_box(p0, p1, p2, bmin, bmax):
    a = [_f3(x) for x in (p0, p1, p2, bmin, bmax)]
    return bool(lib().vfo_tri_box(*[_p(x) for x in a]))


def grid_dims(aabb_min, aabb_max, max_voxels):
    out = np.zeros(3, np.uint32)
    mn, mx = _f3(aabb_min), _f3(aabb_max)
    lib().vfo_grid_dims(_p(mn), _p(mx), int(max_voxels), _p(out))
    return tuple(int(x) for x in out)


def seeder_uniform(grid, n, seed, location):
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    out = np.zeros((max(n, 1), 4), np.uint32)
    _check(lib().vfo_seeder_uniform(_p(g), *g.shape, int(n), int(seed),
                                    int(location), _p(out)), "seeder_uniform")
    return out[:n]


def fracture_seeds(grid, n_main, n_extra, location, merge_dfunc, seed, num_impacts=0,
                   bias_seeds=32, bias_focus=5):
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    cap = 2 * (n_main + (bias_seeds if num_impacts else 0)) + n_extra
    out = np.zeros((max(cap, 1), 4), np.uint32)
    n = C.c_uint32(0)
    _check(lib().vfo_fracture_seeds(_p(g), *g.shape, int(n_main), int(n_extra),
                                    int(location), int(merge_dfunc), int(seed), int(num_impacts),
                                    int(bias_seeds), int(bias_focus), _p(out), C.byref(n)),
           "fracture_seeds")
    return out[:n.value]


def merge_seeds(frags, seeds, dfunc):
    f = np.ascontiguousarray(frags, dtype=np.uint32)
    s = np.array(seeds, dtype=np.uint32, copy=True, order="C")
    _check(lib().vfo_merge_seeds(_p(f), f.shape[0], _p(s), s.shape[0], int(dfunc)),
           "merge_seeds")
    return s


def flood(grid, seeds, dfunc):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    s = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4)
    waves = C.c_uint32(0)
    _check(lib().vfo_flood(_p(g), *g.shape, _p(s), s.shape[0], int(dfunc),
                           C.byref(waves)), "flood")
    return g, waves.value


def naive(grid, seeds, dfunc):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    s = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4)
    _check(lib().vfo_naive(_p(g), *g.shape, _p(s), s.shape[0], int(dfunc)), "naive")
    return g


def perturb(grid, amplitude, period, seed):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    _check(lib().vfo_perturb(_p(g), *g.shape, float(amplitude), int(period),
                             int(seed)), "perturb")
    return g


def detect_boundaries(grid, size=1):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    lib().vfo_detect_boundaries(_p(g), *g.shape, int(size))
    return g


def remove_isolated(grid):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    lib().vfo_remove_isolated(_p(g), *g.shape)
    return g


def erode(grid, etype, size, iterations, probability, threshold, seed):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    _check(lib().vfo_erode(_p(g), *g.shape, int(etype), int(size), int(iterations),
                           float(probability), float(threshold), int(seed)), "erode")
    return g


def undo_mask(grid):
    g = np.array(grid, dtype=np.uint16, copy=True, order="C")
    lib().vfo_undo_mask(_p(g), *g.shape)
    return g


def count_values(grid, ncounts=32768):
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    c = np.zeros(ncounts, np.uint32)
    occ = C.c_uint64(0)
    _check(lib().vfo_count_values(_p(g), *g.shape, _p(c), ncounts, C.byref(occ)),
           "count_values")
    return c, occ.value


def run_job(verts, faces, dims, aabb_min, aabb_max, params: Params, ncounts=32768):
    X, Y, Z = (int(d) for d in dims)
    v = np.ascontiguousarray(verts, dtype=np.float32)
    f = np.ascontiguousarray(faces, dtype=np.uint32)
    g = np.empty((X, Y, Z), dtype=np.uint16)
    c = np.zeros(ncounts, np.uint32)
    cap = 2 * (params.num_seeds + (params.bias_seeds if params.num_impacts > 0 else 0)) + \
        params.num_extra_seeds
    s = np.zeros((max(cap, 1), 4), np.uint32)
    ns = C.c_uint32(0)
    mn, mx = _f3(aabb_min), _f3(aabb_max)
    _check(lib().vfo_run_job(_p(v), v.shape[0], _p(f), f.shape[0], X, Y, Z,
                             _p(mn), _p(mx), C.byref(params), _p(g), _p(c), ncounts,
                             _p(s), C.byref(ns)), "run_job")
    return g, c, s[:ns.value]


def rle_encode(grid):
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    n = lib().vfo_rle_encode(_p(g), *g.shape, None, 0)
    out = np.zeros(n, np.uint8)
    lib().vfo_rle_encode(_p(g), *g.shape, _p(out), n)
    return out.tobytes()


def triangulate(grid, aabb_min, aabb_max, nb_iters=0, nb_weight=0.9, b_iters=0, b_weight=0.2):
    """RegularGrid::toTriangleMesh: (values, vert_off, face_off, verts (V, 4)
    float32, faces (T, 4) uint32), meshes concatenated in value order."""
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    X, Y, Z = g.shape
    lo, hi = _f3(aabb_min), _f3(aabb_max)
    F, V, T = C.c_uint32(), C.c_uint64(), C.c_uint64()
    args = (_p(g), X, Y, Z, _p(lo), _p(hi), nb_iters, nb_weight, b_iters, b_weight,
            C.byref(F), C.byref(V), C.byref(T))
    _check(lib().vfo_triangulate(*args, None, None, None, None, None), "triangulate")
    vals = np.zeros(F.value, np.uint16)
    vo = np.zeros(F.value + 1, np.uint64)
    fo = np.zeros(F.value + 1, np.uint64)
    verts = np.zeros((V.value, 4), np.float32)
    faces = np.zeros((T.value, 4), np.uint32)
    _check(lib().vfo_triangulate(*args, _p(vals), _p(vo), _p(fo), _p(verts), _p(faces)),
           "triangulate")
    return vals, vo, fo, verts, faces


def ray_entry(grid, aabb_min, aabb_max, origin, direction):
    """RegularGrid::getClosestEntryVoxel: the 1-based index of the first
    occupied voxel on the ray, or None."""
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    lo, hi, o, d = _f3(aabb_min), _f3(aabb_max), _f3(origin), _f3(direction)
    out = np.zeros(3, np.uint32)
    _check(lib().vfo_ray_entry(_p(g), *g.shape, _p(lo), _p(hi), _p(o), _p(d), _p(out)), "ray_entry")
    return None if out[0] == 0xFFFFFFFF else tuple(int(v) for v in out)


def near_seeds(grid, frags, num_impacts, num_seeds, spreading, seed):
    """Seeder::nearSeeds: frags followed by the seeds placed around impacts."""
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    f = np.ascontiguousarray(frags, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros((f.shape[0] + num_seeds + 1, 4), np.uint32)
    n = C.c_uint32()
    _check(lib().vfo_near_seeds(_p(g), *g.shape, _p(f), f.shape[0], num_impacts, num_seeds,
                                spreading, seed, _p(out), C.byref(n)), "near_seeds")
    return out[:n.value]


def ray_entry_batch(grid, aabb_min, aabb_max, rays):
    """ray_entry for (n, 6) rays at once (OpenMP): (n, 3) uint32, 0xFFFFFFFF on a miss."""
    g = np.ascontiguousarray(grid, dtype=np.uint16)
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    lo, hi = _f3(aabb_min), _f3(aabb_max)
    out = np.zeros((r.shape[0], 3), np.uint32)
    _check(lib().vfo_ray_entry_batch(_p(g), *g.shape, _p(lo), _p(hi), _p(r), r.shape[0], _p(out)),
           "ray_entry_batch")
    return out


def sample_mesh(verts4, faces4, max_samples, seed, key=0):
    """CADModel::sampleCPU: (n, 4) float32 points (x, y, z, 1) on the mesh
    (verts4: (V, 4) float32, faces4: (T, 4) uint32 mesh-local indices)."""
    v = np.ascontiguousarray(verts4, dtype=np.float32).reshape(-1, 4)
    f = np.ascontiguousarray(faces4, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros((max(max_samples, 1), 4), np.float32)
    n = C.c_uint64()
    _check(lib().vfo_sample_mesh(_p(v), _p(f), f.shape[0], max_samples, seed, key, _p(out),
                                 C.byref(n)), "sample_mesh")
    return out[:n.value]
