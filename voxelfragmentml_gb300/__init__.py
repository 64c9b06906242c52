"""GB300 voxelize -> seed -> fracture -> perturb/erode -> count pipeline.

Python binding of the C ABI in include/vf.h (library
voxelfragmentml_gb300/_build/libvfgb300.so, built by build.py for
sm_103a).  The classes mirror the reference's interface:

* :class:`RegularGrid`  -- RegularGrid (DataStructures/RegularGrid.h): fill,
  detectBoundaries, erode, undoMask, countValues, data;
* :class:`Seeder`       -- Seeder::uniform / mergeSeeds (Fracturer/Seeder.h);
* :class:`FloodFracturer`, :class:`NaiveFracturer` -- Fracturer::build
  (Fracturer/Fracturer.h:28-57);
* :func:`fracture_model` -- CADScene::fractureModel;
* :func:`batch_run`, :func:`plain_run`, :class:`Server` -- whole jobs.

There is no CPU fallback: every call runs on the GPU through the library,
and loading fails with an error when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import vessel  # noqa: F401  (synthetic inputs)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvfgb300.so")

OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_SEED_SEARCH, ERR_RANGE, ERR_TIMEOUT, \
    ERR_NOT_BUILT, ERR_BUSY = range(9)
NAIVE, FLOOD = 0, 1
EUCLIDEAN, MANHATTAN, CHEBYSHEV = 0, 1, 2
SQUARE, ELLIPSE, CROSS = 0, 1, 2
INNER, OUTER, BOTH = 0, 1, 2
MAX_SEEDS = 4095
STAGES = ("upload", "tetrahedra", "parity", "shell", "combine", "seeds", "fracture", "perturb",
          "erode_boundaries", "counts", "download")


class VFError(RuntimeError):
    """A non-zero vf_status from the library."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class Params(C.Structure):
    """vf_params: the hot-path fields of FractureParameters."""
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

    @classmethod
    def default(cls, **kw) -> "Params":
        p = cls()
        lib().vf_params_default(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def seed_capacity(self) -> int:
        """Seeds fractureModel may use: 2 * (main + nearSeeds' bias) + extra."""
        bias = self.bias_seeds if self.num_impacts > 0 else 0
        return 2 * (self.num_seeds + bias) + self.num_extra_seeds


class Job(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("nverts", C.c_uint32),
                ("faces", C.c_void_p), ("nfaces", C.c_uint32),
                ("dims", C.c_uint32 * 3), ("max_dim", C.c_uint32),
                ("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3),
                ("params", Params), ("out_labels", C.c_void_p),
                ("out_counts", C.c_void_p), ("ncounts", C.c_uint32),
                ("user_tag", C.c_uint64)]


class JobResult(C.Structure):
    _fields_ = [("status", C.c_int), ("dims", C.c_uint32 * 3), ("nseeds", C.c_uint32),
                ("voxels", C.c_uint64), ("occupied", C.c_uint64),
                ("fragments", C.c_uint32), ("flood_passes", C.c_uint32),
                ("submit_ms", C.c_double), ("done_ms", C.c_double),
                ("user_tag", C.c_uint64)]


EXPORTS = {
    "vf_params_default": (None, [C.c_void_p]),
    "vf_last_error": (C.c_char_p, []),
    "vf_status_string": (C.c_char_p, [C.c_int]),
    "vf_version": (C.c_char_p, []),
    "vf_ctx_create": (C.c_int, [C.c_int, C.c_size_t, C.c_void_p]),
    "vf_ctx_destroy": (C.c_int, [C.c_void_p]),
    "vf_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "vf_ctx_bytes_in_use": (C.c_size_t, [C.c_void_p]),
    "vf_host_alloc": (C.c_void_p, [C.c_size_t]),
    "vf_host_free": (None, [C.c_void_p]),
    "vf_host_numa_node": (C.c_int, [C.c_void_p]),
    "vf_ctx_host_numa": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_ctx_copy_bandwidth": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "vf_grid_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_void_p, C.c_void_p, C.c_void_p]),
    "vf_grid_destroy": (C.c_int, [C.c_void_p]),
    "vf_grid_dims": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_dims_for_aabb": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_grid_upload": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_grid_download": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_voxelize": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "vf_sample_seeds": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_void_p]),
    "vf_merge_seeds": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int]),
    "vf_fracture_seeds": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vf_fracture": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_uint32]),
    "vf_fracture_plain": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_perturb": (C.c_int, [C.c_void_p, C.c_float, C.c_uint32, C.c_uint64]),
    "vf_detect_boundaries": (C.c_int, [C.c_void_p, C.c_int]),
    "vf_erode": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_float,
                           C.c_float, C.c_uint64]),
    "vf_remove_isolated": (C.c_int, [C.c_void_p]),
    "vf_undo_mask": (C.c_int, [C.c_void_p]),
    "vf_count_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_fracture_model": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vf_job_footprint": (C.c_size_t, [C.c_void_p]),
    "vf_batch_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_plain_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_batch_prepare": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_batch_execute": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "vf_ctx_stage_ms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_ctx_flood_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vf_ctx_flood_counters": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_ctx_last_graph": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_ctx_flood_pass_sizes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_grid_export_rle": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "vf_grid_sample_meshes": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p,
                                        C.c_void_p]),
    "vf_grid_points": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vf_sample_mesh": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                 C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]),
    "vf_ray_entry_voxels": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_near_seeds": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]),
    "vf_mc_params_default": (None, [C.c_uint32, C.c_void_p]),
    "vf_grid_triangulate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "vf_grid_meshes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p]),
    "vf_grid_mesh_phase_ms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_grid_mesh_counters": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_ctx_set_tuning": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_ctx_get_tuning": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_ctx_set_flood_wait_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
    "vf_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "vf_server_create": (C.c_int, [C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_void_p]),
    "vf_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "vf_server_poll": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int]),
    "vf_server_destroy": (C.c_int, [C.c_void_p]),
    "vf_pipeline_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_pipeline_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vf_pipeline_collect": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vf_pipeline_destroy": (C.c_int, [C.c_void_p]),
    "vf_flood_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]),
    "vf_ctx_event_record": (C.c_int, [C.c_void_p, C.c_int]),
    "vf_ctx_event_elapsed": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "vf_ctx_last_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libvfgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise VFError(ERR_NOT_BUILT,
                          f"{LIB_PATH} is missing: run voxelfragmentml_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != OK:
        msg = lib().vf_last_error()
        raise VFError(status, msg.decode() if msg else "error")


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


class Context:
    """vf_ctx: one device, one stream, an HBM budget."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        h = C.c_void_p()
        _check(lib().vf_ctx_create(device, hbm_budget, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().vf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        _check(lib().vf_ctx_synchronize(self.h))

    @property
    def bytes_in_use(self) -> int:
        return lib().vf_ctx_bytes_in_use(self.h)

    def stage_ms(self):
        """Device ms per stage of the last batched run (see STAGES)."""
        a = (C.c_float * 11)()
        _check(lib().vf_ctx_stage_ms(self.h, a, 11))
        return dict(zip(STAGES, list(a)))

    TUNING = ("parity_grid", "shell_grid", "flood_sweeps", "flood_ctas")

    def tuning(self) -> dict:
        v = (C.c_int32 * 4)()
        _check(lib().vf_ctx_get_tuning(self.h, v, 4))
        return dict(zip(self.TUNING, list(v)))

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        v = (C.c_int32 * 4)(*[int(cur[k]) for k in self.TUNING])
        _check(lib().vf_ctx_set_tuning(self.h, v, 4))

    def autotune(self, specs) -> dict:
        """vf_autotune over the jobs of `specs` (JobSpec list); returns the
        chosen settings, which stay on this context."""
        jobs = (Job * len(specs))(*[s.job() for s in specs])
        v = (C.c_int32 * 4)()
        _check(lib().vf_autotune(self.h, jobs, len(specs), v, 4))
        return dict(zip(self.TUNING, list(v)))

    def flood_pass_sizes(self):
        """Bricks queued per pass of the last batched flood."""
        a = (C.c_uint32 * 256)()
        _check(lib().vf_ctx_flood_pass_sizes(self.h, a, 256))
        return [v for v in a if v]

    def host_numa(self) -> int:
        """Host NUMA node closest to the device (-1: none reported)."""
        n = C.c_int(-1)
        _check(lib().vf_ctx_host_numa(self.h, C.byref(n)))
        return n.value

    def copy_bandwidth(self, nbytes: int = 256 << 20):
        """(H2D, D2H) GB/s between pinned host memory and the device."""
        a, b = C.c_float(), C.c_float()
        _check(lib().vf_ctx_copy_bandwidth(self.h, nbytes, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_stats(self):
        la, vis, by = C.c_uint64(), C.c_uint64(), C.c_uint64()
        ms = C.c_float()
        _check(lib().vf_ctx_last_stats(self.h, C.byref(la), C.byref(ms), C.byref(by), C.byref(vis)))
        pa, sw, mh = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().vf_ctx_flood_stats(self.h, C.byref(pa), C.byref(sw), C.byref(mh)))
        cn = (C.c_uint64 * 20)()
        _check(lib().vf_ctx_flood_counters(self.h, cn, 20))
        return {"launches": la.value, "flood_ms": ms.value, "flood_bytes": by.value,
                "flood_visits": vis.value, "flood_passes": pa.value, "flood_sweeps": sw.value,
                "flood_maxit_hits": mh.value, "flood_active_row_sweeps": cn[6],
                "flood_busy_warp_sweeps": cn[2],
                "flood_key_changes": cn[7],
                "flood_barrier_timeouts": cn[3],
                # first out-of-range access the relaxation skipped (0: none)
                "flood_anomaly": (cn[8], cn[9], cn[10]),
                "flood_empty_visits": cn[16],
                "flood_visits_no_change": cn[17],
                # SM cycles summed over the relaxation CTAs, per phase of their work
                "flood_phase_cycles": {k: 256 * cn[11 + i] for i, k in enumerate(
                    ("claim", "staging", "sweeps", "writeback_enqueue", "pass_barrier"))}}


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class MCParams(C.Structure):
    """vf_mc_params: the smoothing fields of FractureParameters used by
    MarchingCubes::triangulateFieldGPU (MarchingCubes.cpp:400-401)."""
    _fields_ = [("nonboundary_iterations", C.c_uint32), ("nonboundary_weight", C.c_float),
                ("boundary_iterations", C.c_uint32), ("boundary_weight", C.c_float)]

    @classmethod
    def default(cls, max_voxels: int) -> "MCParams":
        p = cls()
        lib().vf_mc_params_default(int(max_voxels), C.byref(p))
        return p


class FragmentMesh:
    """One fragment's mesh as CADModel::insert receives it: vertices (V, 4)
    float32 (x, y, z, boundary) and faces (F, 4) uint32 (three vertex
    indices, boundary)."""

    def __init__(self, value, vertices, faces):
        self.value, self.vertices, self.faces = int(value), vertices, faces

    def __repr__(self):
        return (f"FragmentMesh(value={self.value}, vertices={len(self.vertices)}, "
                f"faces={len(self.faces)})")


class RegularGrid:
    """Device-resident uint16 label grid, x-major (RegularGrid.h:142-367)."""

    def __init__(self, dims, aabb_min=None, aabb_max=None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        X, Y, Z = (int(d) for d in dims)
        mn = _f3(aabb_min if aabb_min is not None else (0, 0, 0))
        mx = _f3(aabb_max if aabb_max is not None else (X, Y, Z))
        h = C.c_void_p()
        _check(lib().vf_grid_create(self.ctx.h, X, Y, Z, _p(mn), _p(mx), C.byref(h)))
        self.h, self.dims = h, (X, Y, Z)
        self.aabb_min, self.aabb_max = mn, mx

    def close(self):
        if getattr(self, "h", None):
            lib().vf_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def getNumSubdivisions(self):
        return self.dims

    def fill(self, verts, faces):
        """RegularGrid::fill(Model3D*): voxelize a triangle mesh."""
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        _check(lib().vf_voxelize(self.h, _p(v), v.shape[0], _p(f), f.shape[0]))

    def upload(self, grid: np.ndarray):
        g = np.ascontiguousarray(grid, dtype=np.uint16)
        if g.shape != self.dims:
            raise ValueError(f"grid shape {g.shape} != {self.dims}")
        _check(lib().vf_grid_upload(self.h, _p(g)))

    def data(self) -> np.ndarray:
        """RegularGrid::updateGrid + data(): copy the labels to the host."""
        g = np.empty(self.dims, dtype=np.uint16)
        _check(lib().vf_grid_download(self.h, _p(g)))
        return g

    def detectBoundaries(self, boundary_size: int = 1):
        _check(lib().vf_detect_boundaries(self.h, boundary_size))

    def exportRLE(self, path=None) -> bytes:
        """RegularGrid::exportRLE: the grid as run-length records (computed on
        the GPU); also written to `path` when given."""
        n = C.c_size_t(0)
        _check(lib().vf_grid_export_rle(self.h, None, 0, C.byref(n)))
        buf = (C.c_ubyte * max(n.value, 1))()
        _check(lib().vf_grid_export_rle(self.h, buf, n.value, C.byref(n)))
        data = bytes(buf)[:n.value]
        if path is not None:
            with open(path, "wb") as fh:
                fh.write(data)
        return data

    def erode(self, erosion_type=ELLIPSE, size=3, iterations=3, probability=0.5,
              threshold=0.5, seed=80):
        _check(lib().vf_erode(self.h, erosion_type, size, iterations, probability,
                              threshold, seed))

    def removeIsolatedRegions(self):
        _check(lib().vf_remove_isolated(self.h))

    def undoMask(self):
        _check(lib().vf_undo_mask(self.h))

    def perturb(self, amplitude: float, period: int, seed: int):
        _check(lib().vf_perturb(self.h, amplitude, period, seed))

    def countValues(self, ncounts: int = 32768):
        c = np.zeros(ncounts, np.uint32)
        occ = C.c_uint64()
        _check(lib().vf_count_values(self.h, _p(c), ncounts, C.byref(occ)))
        return c, occ.value

    def getClosestEntryVoxel(self, origin, direction):
        """RegularGrid::getClosestEntryVoxel: the 1-based index of the first
        occupied voxel on the ray (as CADScene::hit uses it), or None."""
        r = self.rayEntryVoxels(np.concatenate([_f3(origin), _f3(direction)]).reshape(1, 6))
        return None if r[0, 0] == 0xFFFFFFFF else tuple(int(v) for v in r[0])

    def rayEntryVoxels(self, rays):
        """Entry voxels of many rays (n, 6: origin, direction) on the GPU:
        (n, 3) uint32, 0xFFFFFFFF rows for misses."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros((r.shape[0], 3), np.uint32)
        _check(lib().vf_ray_entry_voxels(self.h, _p(r), r.shape[0], _p(out)))
        return out

    def triangulate(self, params: MCParams | None = None):
        """vf_grid_triangulate: build every fragment's mesh on the device and
        return (meshes, vertices, faces) counts."""
        F, V, T = C.c_uint32(), C.c_uint64(), C.c_uint64()
        _check(lib().vf_grid_triangulate(self.h, C.byref(params) if params is not None else None,
                                         C.byref(F), C.byref(V), C.byref(T)))
        self._mesh_sizes = (F.value, V.value, T.value)
        return self._mesh_sizes

    def meshes_arrays(self):
        """The last triangulation as concatenated arrays: (values, vert_off,
        face_off, verts (V, 4) float32, faces (T, 4) uint32)."""
        F, V, T = self._mesh_sizes
        vals = np.zeros(max(F, 1), np.uint16)
        vo = np.zeros(F + 1, np.uint64)
        fo = np.zeros(F + 1, np.uint64)
        verts = np.zeros((V, 4), np.float32)
        faces = np.zeros((T, 4), np.uint32)
        _check(lib().vf_grid_meshes(self.h, _p(vals), _p(vo), _p(fo), _p(verts), _p(faces)))
        return vals[:F], vo, fo, verts, faces

    def mesh_phase_ms(self):
        """Device ms of the last triangulation's phases: counts, size read-back,
        records + split + outputs, smoothing lists, smoothing iterations,
        local indices."""
        ms = np.zeros(6, np.float32)
        _check(lib().vf_grid_mesh_phase_ms(self.h, _p(ms), 6))
        return [float(x) for x in ms]

    def mesh_counters(self):
        """Sizes of the last triangulation: vertices, faces, boundary vertices,
        smoothing face incidences, neighbour entries, boundary-vertex entries."""
        c = np.zeros(6, np.uint64)
        _check(lib().vf_grid_mesh_counters(self.h, _p(c), 6))
        return [int(x) for x in c]

    def samplePointClouds(self, max_samples: int, seed: int = 80):
        """CADModel::sampleCPU of every mesh of the last triangulation: a list of
        (n, 4) float32 point arrays (x, y, z, 1), one per fragment value."""
        F = self._mesh_sizes[0]
        offs = np.zeros(F + 1, np.uint64)
        n = C.c_uint64()
        _check(lib().vf_grid_sample_meshes(self.h, max_samples, seed, _p(offs), C.byref(n)))
        pts = np.zeros((max(n.value, 1), 4), np.float32)
        if n.value:
            _check(lib().vf_grid_points(self.h, _p(pts)))
        return [pts[offs[i]:offs[i + 1]] for i in range(F)]

    def toTriangleMesh(self, params: MCParams | None = None):
        """RegularGrid::toTriangleMesh (RegularGrid.cpp:443-486): one smoothed
        marching-cubes mesh per fragment value, in ascending value order."""
        self.triangulate(params)
        vals, vo, fo, verts, faces = self.meshes_arrays()
        return [FragmentMesh(v, verts[vo[i]:vo[i + 1]], faces[fo[i]:fo[i + 1]])
                for i, v in enumerate(vals)]


class Seeder:
    """Seeder::uniform / mergeSeeds (Fracturer/Seeder.h:59-76)."""

    @staticmethod
    def uniform(grid: RegularGrid, nseeds: int, seed: int, location: int = OUTER):
        out = np.zeros((max(nseeds, 1), 4), np.uint32)
        _check(lib().vf_sample_seeds(grid.h, nseeds, seed, location, _p(out)))
        return out[:nseeds]

    @staticmethod
    def mergeSeeds(frags, seeds, dfunc: int):
        f = np.ascontiguousarray(frags, dtype=np.uint32).reshape(-1, 4)
        s = np.array(seeds, dtype=np.uint32, copy=True, order="C").reshape(-1, 4)
        _check(lib().vf_merge_seeds(_p(f), f.shape[0], _p(s), s.shape[0], dfunc))
        return s

    @staticmethod
    def nearSeeds(grid: RegularGrid, frags, numImpacts: int, numSeeds: int, spreading: int,
                  seed: int = 80):
        """Seeder::nearSeeds (Seeder.cpp:49-113): frags followed by seeds placed
        on surface voxels around numImpacts randomly chosen frags."""
        f = np.ascontiguousarray(frags, dtype=np.uint32).reshape(-1, 4)
        out = np.zeros((f.shape[0] + numSeeds + 1, 4), np.uint32)
        n = C.c_uint32()
        _check(lib().vf_near_seeds(grid.h, _p(f), f.shape[0], numImpacts, numSeeds, spreading,
                                   seed, _p(out), C.byref(n)))
        return out[:n.value]

    @staticmethod
    def fracture_seeds(grid: RegularGrid, params: Params):
        cap = params.seed_capacity()
        out = np.zeros((max(cap, 1), 4), np.uint32)
        n = C.c_uint32()
        _check(lib().vf_fracture_seeds(grid.h, C.byref(params), _p(out), C.byref(n)))
        return out[:n.value]


class _Fracturer:
    algorithm = FLOOD

    def __init__(self):
        self._dfunc = MANHATTAN

    def setDistanceFunction(self, dfunc: int) -> bool:
        if dfunc not in (EUCLIDEAN, MANHATTAN, CHEBYSHEV):
            return False
        self._dfunc = dfunc
        return True

    def build(self, grid: RegularGrid, seeds, params: Params | None = None):
        s = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4)
        d = params.distance if params is not None else self._dfunc
        _check(lib().vf_fracture(grid.h, self.algorithm, d, _p(s), s.shape[0]))


class FloodFracturer(_Fracturer):
    """FloodFracturer::build (Fracturer/FloodFracturer.cpp:98-191)."""
    algorithm = FLOOD

    def build_plain(self, grid: RegularGrid, seeds) -> int:
        """Reference-shaped flood: one launch + host read per BFS wave."""
        s = np.ascontiguousarray(seeds, dtype=np.uint32).reshape(-1, 4)
        waves = C.c_uint32()
        _check(lib().vf_fracture_plain(grid.h, self._dfunc, _p(s), s.shape[0], C.byref(waves)))
        return waves.value


class NaiveFracturer(_Fracturer):
    """NaiveFracturer::build (Fracturer/NaiveFracturer.cpp:26-68)."""
    algorithm = NAIVE


def fracture_model(grid: RegularGrid, params: Params):
    """CADScene::fractureModel on a voxelized grid; returns the seeds used."""
    cap = params.seed_capacity()
    out = np.zeros((max(cap, 1), 4), np.uint32)
    n = C.c_uint32()
    _check(lib().vf_fracture_model(grid.h, C.byref(params), _p(out), C.byref(n)))
    return out[:n.value]


def sample_mesh(verts, faces, max_samples: int, seed: int = 80, ctx: "Context | None" = None):
    """CADModel::sampleCPU of one mesh on the GPU: (n, 4) float32 points."""
    ctx = ctx or default_context()
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
    out = np.zeros((max(max_samples, 1), 4), np.float32)
    n = C.c_uint64()
    _check(lib().vf_sample_mesh(ctx.h, _p(v), v.shape[0], _p(f), f.shape[0], max_samples, seed,
                                _p(out), C.byref(n)))
    return out[:n.value]


def dims_for_aabb(aabb_min, aabb_max, max_voxels: int):
    out = np.zeros(3, np.uint32)
    _check(lib().vf_dims_for_aabb(_p(_f3(aabb_min)), _p(_f3(aabb_max)), max_voxels, _p(out)))
    return tuple(int(x) for x in out)


# ---- whole jobs ----------------------------------------------------------------
class JobSpec:
    """A job with its host buffers kept alive (mesh, labels, counts)."""

    def __init__(self, verts, faces, params: Params, dims=None, aabb=None, max_dim=0,
                 want_labels=True, ncounts=256, tag=0, pinned=None):
        self.verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        if aabb is None:
            aabb = (self.verts.min(0), self.verts.max(0))
        self.aabb = (_f3(aabb[0]), _f3(aabb[1]))
        if dims is None:
            dims = dims_for_aabb(self.aabb[0], self.aabb[1], max_dim)
        self.dims = tuple(int(d) for d in dims)
        self.params = params
        if pinned:
            # page-locked outputs: the library writes labels straight into them
            self.labels = pinned_array(self.dims, np.uint16) if want_labels else None
            self.counts = pinned_array((ncounts,), np.uint32) if ncounts else None
            if self.labels is not None:
                self.labels[...] = 0
            if self.counts is not None:
                self.counts[...] = 0
        else:
            self.labels = np.zeros(self.dims, np.uint16) if want_labels else None
            self.counts = np.zeros(ncounts, np.uint32) if ncounts else None
        self.tag = tag

    def job(self) -> Job:
        j = Job()
        j.verts = self.verts.ctypes.data
        j.nverts = self.verts.shape[0]
        j.faces = self.faces.ctypes.data
        j.nfaces = self.faces.shape[0]
        for a in range(3):
            j.dims[a] = self.dims[a]
            j.aabb_min[a] = float(self.aabb[0][a])
            j.aabb_max[a] = float(self.aabb[1][a])
        j.params = self.params
        j.out_labels = self.labels.ctypes.data if self.labels is not None else None
        j.out_counts = self.counts.ctypes.data if self.counts is not None else None
        j.ncounts = self.counts.shape[0] if self.counts is not None else 0
        j.user_tag = self.tag
        return j


def _run(fn, specs, ctx):
    ctx = ctx or default_context()
    arr = (Job * len(specs))(*[s.job() for s in specs])
    res = (JobResult * len(specs))()
    st = fn(ctx.h, arr, len(specs), res)
    if st != OK and all(r.status == OK for r in res):
        _check(st)
    return list(res)


def batch_run(specs, ctx: Context | None = None):
    """Batched path: every stage once over all jobs (vf_batch_run)."""
    return _run(lib().vf_batch_run, specs, ctx)


class Pipeline:
    """vf_pipeline_*: up to `depth` batches in flight; the download of one
    batch runs while the next one computes.  submit() returns once the batch
    is issued; collect() waits for the oldest batch and returns its results.
    The specs' host buffers stay referenced until their batch is collected."""

    def __init__(self, ctx: Context | None = None, depth: int = 2):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _check(lib().vf_pipeline_create(self.ctx.h, depth, C.byref(h)))
        self.h = h
        self._inflight = []  # (specs, job array) of the batches in flight, oldest first

    def submit(self, specs):
        specs = list(specs)
        arr = (Job * len(specs))(*[s.job() for s in specs])
        _check(lib().vf_pipeline_submit(self.h, arr, len(specs)))
        self._inflight.append((specs, arr))

    def collect(self):
        if not self._inflight:
            raise VFError(ERR_INVALID, "no batch in flight")
        specs, _ = self._inflight[0]
        res = (JobResult * len(specs))()
        n = C.c_uint32()
        st = lib().vf_pipeline_collect(self.h, res, len(specs), C.byref(n))
        if st == OK or n.value:
            self._inflight.pop(0)
        if st != OK and all(r.status == OK for r in res[:n.value]):
            _check(st)
        return list(res[:n.value])

    def close(self):
        if getattr(self, "h", None):
            lib().vf_pipeline_destroy(self.h)
            self.h = None
            self._inflight = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ResidentBatch:
    """vf_batch_prepare / vf_batch_execute: inputs uploaded once, then
    every execute() runs all stages on the HBM-resident inputs."""

    def __init__(self, specs, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.specs = list(specs)
        self._jobs = (Job * len(self.specs))(*[s.job() for s in self.specs])
        _check(lib().vf_batch_prepare(self.ctx.h, self._jobs, len(self.specs)))

    def execute(self, download: bool = False):
        res = (JobResult * len(self.specs))()
        st = lib().vf_batch_execute(self.ctx.h, 1 if download else 0, res)
        if st != OK and all(r.status == OK for r in res):
            _check(st)
        g = C.c_int(0)
        _check(lib().vf_ctx_last_graph(self.ctx.h, C.byref(g)))
        self.graph = bool(g.value)  # the stage chain ran as a CUDA graph
        return list(res)


def pinned_array(shape, dtype):
    """A numpy array in page-locked host memory (vf_host_alloc); freed when
    the array is garbage collected."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    n = max(count * dt.itemsize, 1)
    p = lib().vf_host_alloc(n)
    if not p:
        raise VFError(ERR_OOM, "pinned host allocation failed")
    buf = (C.c_ubyte * n).from_address(p)
    buf._owner = _PinnedOwner(p)  # lives as long as the buffer
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


class _PinnedOwner:
    def __init__(self, p):
        self.p = p

    def __del__(self):
        try:
            lib().vf_host_free(self.p)
        except Exception:
            pass


def plain_run(specs, ctx: Context | None = None):
    """Plain path: one job at a time, per-wave flood (vf_plain_run)."""
    return _run(lib().vf_plain_run, specs, ctx)


class Server:
    """vf_server: continuous batching with HBM admission control."""

    def __init__(self, ctx: Context | None = None, hbm_budget: int = 0, max_inflight: int = 3,
                 max_batch: int = 128):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _check(lib().vf_server_create(self.ctx.h, hbm_budget, max_inflight, max_batch, C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, spec: JobSpec) -> int:
        t = C.c_uint64()
        j = spec.job()
        _check(lib().vf_server_submit(self.h, C.byref(j), C.byref(t)))
        self._keep[spec.tag] = spec
        return t.value

    def poll(self, max_results: int = 256, wait_ms: int = 0):
        out = (JobResult * max_results)()
        n = C.c_uint32()
        _check(lib().vf_server_poll(self.h, out, max_results, C.byref(n), wait_ms))
        res = list(out[:n.value])
        return res

    def close(self):
        if getattr(self, "h", None):
            lib().vf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
