/*
 * vf.h -- C ABI of the GB300 voxelize -> seed -> fracture -> perturb/erode
 * -> count pipeline (library libvfgb300.so).
 *
 * The entry points replace the reference's fracture path, which is C++ over
 * OpenGL compute shaders:
 *   RegularGrid    (MeshFragments/Source/DataStructures/RegularGrid.h:142-367)
 *   Seeder         (MeshFragments/Source/Fracturer/Seeder.h:59-76)
 *   Fracturer      (MeshFragments/Source/Fracturer/Fracturer.h:28-57) with
 *                  FloodFracturer / NaiveFracturer
 *   CADScene::fractureModel (MeshFragments/Source/Graphics/Application/
 *                  CADScene.cpp:624-691), the orchestration order.
 *
 * Conventions
 *   - Plain C types only; every call returns a vf_status (0 = VF_OK).  No
 *     exception crosses the ABI.  vf_last_error() gives a message for the
 *     last failing call on the calling thread.
 *   - Label grids are uint16, x-major, index x*Y*Z + y*Z + z
 *     (RegularGrid.cpp:1031-1034).  0 EMPTY, 1 FREE, >1 labels; bits 0-7
 *     fragment id, 8-14 sub-seed prefix, 15 boundary flag.
 *   - Host pointers are the caller's; the library copies what it needs.
 *     Grids live on the device, owned by the context, until destroyed.
 *   - One context per device and per host thread at a time: calls on one
 *     context are serialised by the caller.  Work runs on the context's
 *     CUDA stream; calls that return host data synchronise it.
 *   - Results are deterministic: identical inputs give identical bits, in
 *     isolation, in a batch and under the server.
 */
#ifndef VF_H
#define VF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int vf_status;
#define VF_OK 0
#define VF_ERR_INVALID 1     /* bad argument (dims, pointers, enum values) */
#define VF_ERR_CUDA 2        /* CUDA runtime error; context may be unusable */
#define VF_ERR_OOM 3         /* allocation failed or over the HBM budget */
#define VF_ERR_SEED_SEARCH 4 /* Seeder::SeederSearchError (Seeder.h:19-22) */
#define VF_ERR_RANGE 5       /* value out of the representable range */
#define VF_ERR_TIMEOUT 6     /* a bounded device wait gave up */
#define VF_ERR_NOT_BUILT 7   /* CUDA path unavailable (no device / no kernel image) */
#define VF_ERR_BUSY 8        /* server queue full */

/* FractureParameters::FractureAlgorithm (FractureParameters.h:20) */
#define VF_NAIVE 0
#define VF_FLOOD 1
/* fracturer::DistanceFunction (Fracturer.h:10-14) */
#define VF_EUCLIDEAN 0
#define VF_MANHATTAN 1
#define VF_CHEBYSHEV 2
/* FractureParameters::ErosionType (FractureParameters.h:26) */
#define VF_SQUARE 0
#define VF_ELLIPSE 1
#define VF_CROSS 2
/* Seeder::Location (Seeder.h:24) */
#define VF_INNER 0
#define VF_OUTER 1
#define VF_BOTH 2

#define VF_MAX_SEEDS 4095u  /* seeds per fracture (12-bit seed slot) */
#define VF_MAX_DIM 4096u    /* per axis */

typedef struct vf_ctx vf_ctx;
typedef struct vf_grid vf_grid;
typedef struct vf_server vf_server;
typedef struct vf_pipeline vf_pipeline;

/* Fracture parameters: the hot-path fields of FractureParameters
 * (FractureParameters.h:43-85, defaults :91-145). */
typedef struct vf_params {
  int32_t algorithm;          /* _fractureAlgorithm: VF_FLOOD | VF_NAIVE */
  int32_t distance;           /* _distanceFunction */
  int32_t num_seeds;          /* _numSeeds (fragments, <= 254) */
  int32_t num_extra_seeds;    /* _numExtraSeeds (sub-seeds merged into fragments) */
  int32_t merge_distance;     /* _mergeSeedsDistanceFunction */
  int32_t seed_location;      /* Seeder::Location of the main seeds */
  uint64_t seed;              /* _seed: all random draws derive from it */
  float noise_amplitude;      /* boundary perturbation, voxels (0 = off) */
  uint32_t noise_period;      /* perturbation noise lattice period, voxels */
  int32_t erode;              /* _erode */
  int32_t erosion_type;       /* _erosionConvolution */
  int32_t erosion_size;       /* _erosionSize */
  int32_t erosion_iterations; /* _erosionIterations */
  float erosion_probability;  /* _erosionProbability */
  float erosion_threshold;    /* _erosionThreshold */
  int32_t boundary_size;      /* detectBoundaries(1) when not eroding */
  int32_t num_impacts;        /* _numImpacts: > 0 places bias_seeds more main
                                 seeds around impacts (Seeder::nearSeeds) */
  int32_t bias_seeds;         /* _biasSeeds: seeds nearSeeds may place */
  int32_t bias_focus;         /* _biasFocus: nearSeeds spreading */
} vf_params;

/* FractureParameters() defaults (FractureParameters.h:91-145), with
 * num_extra_seeds 0 and seed_location VF_OUTER as in CADScene.cpp:633;
 * num_impacts 0, bias_seeds 32, bias_focus 5. */
void vf_params_default(vf_params* p);

const char* vf_last_error(void);
const char* vf_status_string(vf_status s);
/* library version string and the GPU architecture it was built for */
const char* vf_version(void);

/* ---- context ------------------------------------------------------------
 * hbm_budget: bytes of device memory the context may hold (0 = 90% of free).
 * Replaces the GL context + ComputeShader runtime (ComputeShader.h:74-190). */
vf_status vf_ctx_create(int device, size_t hbm_budget, vf_ctx** out);
vf_status vf_ctx_destroy(vf_ctx* ctx);
vf_status vf_ctx_synchronize(vf_ctx* ctx);
/* bytes currently held by grids and scratch */
size_t vf_ctx_bytes_in_use(const vf_ctx* ctx);
/* pinned host memory for fast uploads/downloads.  Buffers of 1 MiB or more
 * are placed on the host NUMA node closest to the current device (preferred
 * policy, then cudaHostRegister, mapped); smaller ones, or hosts without a
 * NUMA node for the device, come from cudaMallocHost.  Free with
 * vf_host_free. */
void* vf_host_alloc(size_t bytes);
void vf_host_free(void* p);
/* NUMA node of the host page holding p (-1 unknown); no reference
 * counterpart, for placement checks */
int vf_host_numa_node(const void* p);
/* host NUMA node closest to the context's device (cudaDevAttrHostNumaId;
 * -1 when the system reports none) */
vf_status vf_ctx_host_numa(vf_ctx* ctx, int* node);
/* host link probe: best of 3 copies of `bytes` between a vf_host_alloc
 * buffer and device memory on the context's stream, GB/s each way */
vf_status vf_ctx_copy_bandwidth(vf_ctx* ctx, size_t bytes, float* h2d_gbs, float* d2h_gbs);

/* ---- grid (RegularGrid) --------------------------------------------------
 * RegularGrid(aabb, subdivisions) + setAABB (RegularGrid.cpp:21-27, 426-441):
 * cellSize = (aabb_max - aabb_min) / dims. */
vf_status vf_grid_create(vf_ctx* ctx, uint32_t X, uint32_t Y, uint32_t Z,
                         const float aabb_min[3], const float aabb_max[3],
                         vf_grid** out);
vf_status vf_grid_destroy(vf_grid* g);
vf_status vf_grid_dims(const vf_grid* g, uint32_t dims[3]);
/* CADScene::allocateMeshGrid dims rule (CADScene.cpp:545-561) */
vf_status vf_dims_for_aabb(const float aabb_min[3], const float aabb_max[3],
                           uint32_t max_voxels, uint32_t dims_out[3]);
/* RegularGrid::updateSSBO / updateGrid (RegularGrid.cpp:505-515) */
vf_status vf_grid_upload(vf_grid* g, const uint16_t* host_grid);
vf_status vf_grid_download(vf_grid* g, uint16_t* host_grid);

/* RegularGrid::exportRLE (RegularGrid.cpp:672-714) into memory: u32 X, Y, Z,
 * then one {u16 value, u32 repetitions} record per run of equal labels in
 * x-major order, packed little endian.  *written = the size in bytes; out =
 * NULL with cap = 0 only queries it; VF_ERR_RANGE if cap is smaller or the
 * grid has 2^32 voxels or more. */
vf_status vf_grid_export_rle(vf_grid* g, uint8_t* out, size_t cap, size_t* written);

/* ---- fragment meshes (RegularGrid::toTriangleMesh) -----------------------
 * Smoothing of MarchingCubes::triangulateFieldGPU (MarchingCubes.cpp:
 * 396-401): iterations over the non-boundary, then the boundary vertices. */
typedef struct vf_mc_params {
  uint32_t nonboundary_iterations; /* maxVoxels * _nonBoundaryMCIterations */
  float nonboundary_weight;        /* _nonBoundaryMCWeight */
  uint32_t boundary_iterations;    /* maxVoxels * _boundaryMCIterations */
  float boundary_weight;           /* _boundaryMCWeight */
} vf_mc_params;
/* FractureParameters defaults (FractureParameters.h:93-94, 109-110):
 * iterations = (unsigned)(max_voxels * 0.048f), weights 0.9 and 0.2;
 * max_voxels is the largest voxelization size. */
void vf_mc_params_default(uint32_t max_voxels, vf_mc_params* p);

/* RegularGrid::toTriangleMesh (RegularGrid.cpp:443-486): one marching-cubes
 * mesh per fragment value (label & 0x7FFF > 1, ascending), the field
 * "label == value" on the grid padded by one FREE voxel (MarchingCubes::
 * setGrid), vertices fused, moved by the grid's box (s = size / dims,
 * p * s + min - s), face flags = max of vertex flags, then Laplacian
 * smoothing.  p = NULL: vf_mc_params_default(max(dims)).  The meshes stay on
 * the device; *nmeshes, *nverts and *nfaces give their sizes.  The reference
 * leaves vertex and face order to GPU atomics; here vertices follow the
 * fragment voxel the vertex's edge leaves (x-major) then the direction
 * -x,+x,-y,+y,-z,+z, faces follow the marched cell (x-major) then the case
 * table, and a vertex is a boundary vertex when any triangle using it is. */
vf_status vf_grid_triangulate(vf_grid* g, const vf_mc_params* p, uint32_t* nmeshes,
                              uint64_t* nverts, uint64_t* nfaces);
/* The meshes of the last vf_grid_triangulate, to host memory (any pointer may
 * be NULL): values[nmeshes]; vert_offsets / face_offsets [nmeshes + 1], mesh
 * i = vertices [vert_offsets[i], vert_offsets[i+1]); verts 4 floats per vertex
 * (x, y, z, boundary 0/1); faces 4 uint32 per face (three vertex indices
 * within the mesh, boundary 0/1) -- the vec4 / uvec4 layouts CADModel::insert
 * receives (MarchingCubes.cpp:403-406). */
vf_status vf_grid_meshes(vf_grid* g, uint16_t* values, uint64_t* vert_offsets,
                         uint64_t* face_offsets, float* verts, uint32_t* faces);
/* Device time of the last vf_grid_triangulate's phases, CUDA events on the
 * grid's stream: [0] face masks + counts, [1] the wait for the sizes (host
 * round trip), [2] vertex and triangle records + split by fragment +
 * positions and faces, [3] smoothing neighbour lists, [4] smoothing
 * iterations, [5] mesh-local face indices. */
vf_status vf_grid_mesh_phase_ms(const vf_grid* g, float* ms, uint32_t n);
/* Sizes of the last vf_grid_triangulate: [0] vertices, [1] faces, [2]
 * boundary vertices, [3] face incidences the smoothing sums, [4] distinct
 * neighbour entries, [5] those of boundary vertices (0 without smoothing). */
vf_status vf_grid_mesh_counters(const vf_grid* g, uint64_t* out, uint32_t n);

/* RegularGrid::fill(Model3D*) (RegularGrid.cpp:173-212): occupancy = FP32
 * tri-box SAT shell (Intersections3D.h:204-258) OR tetra-parity interior
 * (Tetravoxelizer.cpp:42-92, 198-315).  verts: 3 floats per vertex, faces:
 * 3 uint32 per triangle, host memory.  Writes 0/1 into the grid. */
vf_status vf_voxelize(vf_grid* g, const float* verts, uint32_t nverts,
                      const uint32_t* faces, uint32_t nfaces);

/* Seeder::uniform (Seeder.cpp:154-208): n distinct occupied voxels, labels
 * 2..n+1 in (x,y,z) order.  out_xyzw: 4*n uint32, host. */
vf_status vf_sample_seeds(vf_grid* g, uint32_t n, uint64_t seed, int location,
                          uint32_t* out_xyzw);
/* Seeder::mergeSeeds (Seeder.cpp:115-152), host computation. */
vf_status vf_merge_seeds(const uint32_t* frags_xyzw, uint32_t nfrags,
                         uint32_t* seeds_xyzw, uint32_t nseeds, int distance);
/* CADScene::fractureModel seed assembly (CADScene.cpp:628-655):
 * uniform(main, location) [+ nearSeeds(num_impacts, bias_seeds, bias_focus)
 * when num_impacts > 0] [+ uniform(extra, BOTH) + mergeSeeds].  out holds
 * 4*(2*(num_seeds + bias_seeds) + num_extra_seeds) uint32; *nout gets the
 * count. */
vf_status vf_fracture_seeds(vf_grid* g, const vf_params* p, uint32_t* out_xyzw,
                            uint32_t* nout);

/* Fracturer::build (Fracturer.h:35): VF_FLOOD = FloodFracturer::build
 * (FloodFracturer.cpp:98-191: homogenize, seed, BFS waves, disjoint
 * cleanup, undoMask); VF_NAIVE = NaiveFracturer::build (CPU path
 * NaiveFracturer.cpp:26-68).  seeds_xyzw: 4*nseeds uint32, host.
 * Same-wave flood ties go to the lowest seed index.  Flood labels are
 * frag | prefix << 8 as Seeder::mergeSeeds makes them (Seeder.cpp:150): at
 * most 0x7FFF with a fragment id (low byte) of at least 2; others are
 * VF_ERR_INVALID. */
vf_status vf_fracture(vf_grid* g, int algorithm, int distance,
                      const uint32_t* seeds_xyzw, uint32_t nseeds);
/* reference-shaped flood: one kernel launch and one host read of the
 * frontier size per BFS wave, as FloodFracturer.cpp:143-158 does.  Same
 * result as vf_fracture(VF_FLOOD); used as the plain comparator. */
vf_status vf_fracture_plain(vf_grid* g, int distance, const uint32_t* seeds_xyzw,
                            uint32_t nseeds, uint32_t* waves_out);

/* Boundary perturbation by seeded 3-D value noise (no reference
 * counterpart): labelled voxels take the label found at v + round(A*n(v/P)). */
vf_status vf_perturb(vf_grid* g, float amplitude, uint32_t period, uint64_t seed);
/* RegularGrid::detectBoundaries (RegularGrid.cpp:64-80) */
vf_status vf_detect_boundaries(vf_grid* g, int boundary_size);
/* RegularGrid::erode (RegularGrid.cpp:82-159) incl. removeIsolatedRegions */
vf_status vf_erode(vf_grid* g, int type, uint32_t size, uint32_t iterations,
                   float probability, float threshold, uint64_t seed);
/* removeIsolatedRegionsGrid-comp.glsl:16-39 (RegularGrid.cpp:1006-1015) */
vf_status vf_remove_isolated(vf_grid* g);
/* RegularGrid::undoMask (RegularGrid.cpp:488-503): clear bit 15 */
vf_status vf_undo_mask(vf_grid* g);
/* RegularGrid::countValues (RegularGrid.cpp:601-625): counts[v] for values
 * v = label & 0x7FFF > 1.  counts: ncounts uint32 (host); *occupied = sum.
 * VF_ERR_RANGE if a label >= ncounts occurs (its count is dropped). */
vf_status vf_count_values(vf_grid* g, uint32_t* counts, uint32_t ncounts,
                          uint64_t* occupied);

/* ---- point clouds (CADModel::sampleCPU) ----------------------------------
 * CADModel::sampleCPU(max_samples) (CADModel.cpp:264-370) for every mesh of
 * the last vf_grid_triangulate, as the dataset generator samples each
 * fragment (CADScene.cpp:129-143, 340-372).  A mesh of T faces gets
 * min(P, S) points when S = max_samples > T (P = sum over faces of
 * max(ceil(area / sumArea * S), 1)), else S points on S distinct faces.
 * point_offsets (nmeshes + 1, may be NULL) and *npoints give the layout; the
 * points (x, y, z, 1) stay on the device for vf_grid_points.  The noise and
 * face draws come from `seed` and the mesh's fragment value (counter-based,
 * identical on every host); samples are in face order, and more than S
 * samples keep the systematic sample floor((i+1) S / P) > floor(i S / P)
 * (the reference shuffles with an unseeded generator).  VF_ERR_INVALID
 * without a triangulation. */
vf_status vf_grid_sample_meshes(vf_grid* g, uint32_t max_samples, uint64_t seed,
                                uint64_t* point_offsets, uint64_t* npoints);
/* the points of the last vf_grid_sample_meshes: 4 floats each, host */
vf_status vf_grid_points(vf_grid* g, float* points);
/* CADModel::sampleCPU of one host mesh (verts 3 floats, faces 3 uint32 per
 * element; mesh key 0): at most max_samples points (4 floats each) into
 * points, *npoints the count. */
vf_status vf_sample_mesh(vf_ctx* ctx, const float* verts, uint32_t nverts, const uint32_t* faces,
                         uint32_t nfaces, uint32_t max_samples, uint64_t seed, float* points,
                         uint64_t* npoints);

/* ---- impact path (CADScene::hit + Seeder::nearSeeds) ---------------------
 * RegularGrid::getClosestEntryVoxel -> rayTraversalAmanatidesWoo
 * (RegularGrid.cpp:265-270, 853-1004) for n rays on the GPU.  rays: 6 floats
 * per ray (origin xyz, direction xyz), host.  out: 3 uint32 per ray, the
 * reference's 1-based index of the first occupied (non-EMPTY) voxel along the
 * ray (voxel index + 1, which CADScene::hit uses as the impact seed), or
 * 0xFFFFFFFF x3 when the ray misses the box or every voxel on it is EMPTY.
 * VF_ERR_INVALID for a zero direction (the reference loops forever). */
vf_status vf_ray_entry_voxels(vf_grid* g, const float* rays, uint32_t n, uint32_t* out);
/* Seeder::nearSeeds (Seeder.cpp:49-113) on the GPU: num_impacts times, pick one
 * of the given seeds and place 1..pending new seeds on surface voxels
 * (occupied, an EMPTY voxel in the 3x3x3 box) within min(dims)/2 of it, at
 * offsets dims/2 - sum of `spreading` uniform draws in [0, dims/spreading)
 * (wrapped), at most num_seeds in all.  out_xyzw (4*(nfrags + num_seeds)
 * uint32) = the given seeds followed by the new ones in (x, y, z) order,
 * labelled on from the last given label; *nout = the count.  The draws come
 * from `seed` (counter-based, identical on every host).  VF_ERR_SEED_SEARCH
 * when an impact finds too few voxels in 2^20 candidates (the reference
 * loops forever); VF_ERR_INVALID for impacts without given seeds or
 * spreading outside [1, min(dims)]. */
vf_status vf_near_seeds(vf_grid* g, const uint32_t* frags_xyzw, uint32_t nfrags,
                        uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading,
                        uint64_t seed, uint32_t* out_xyzw, uint32_t* nout);

/* CADScene::fractureModel (CADScene.cpp:624-691) on an already voxelized
 * grid: seeds -> fracture -> [perturb] -> erode | detectBoundaries.  The
 * seeds used are returned when seeds_out (4*(2n+extra) uint32) is given. */
vf_status vf_fracture_model(vf_grid* g, const vf_params* p, uint32_t* seeds_out,
                            uint32_t* nseeds_out);

/* ---- jobs: whole pipeline from a mesh ------------------------------------ */
typedef struct vf_job {
  const float* verts;      /* host, 3 floats per vertex */
  uint32_t nverts;
  const uint32_t* faces;   /* host, 3 uint32 per triangle */
  uint32_t nfaces;
  uint32_t dims[3];        /* grid dims; all 0 => allocateMeshGrid(max_dim) */
  uint32_t max_dim;        /* used when dims are 0 */
  float aabb_min[3];       /* grid AABB; min == max => mesh AABB */
  float aabb_max[3];
  vf_params params;
  uint16_t* out_labels;    /* host X*Y*Z uint16 or NULL */
  uint32_t* out_counts;    /* host ncounts uint32 or NULL */
  uint32_t ncounts;
  uint64_t user_tag;       /* returned in the result */
} vf_job;

typedef struct vf_job_result {
  vf_status status;
  uint32_t dims[3];
  uint32_t nseeds;
  uint64_t voxels;         /* X*Y*Z */
  uint64_t occupied;       /* labelled voxels after the pipeline */
  uint32_t fragments;      /* distinct labels counted */
  uint32_t flood_passes;   /* brick passes (batched) or BFS waves (plain) */
  double submit_ms;        /* server: submit time, ms since server start */
  double done_ms;          /* server: result-on-host time */
  uint64_t user_tag;
} vf_job_result;

/* Batched path: all jobs packed into one brick work-queue per stage
 * (voxelize, seed, flood, perturb, erode/boundaries, count), persistent
 * kernels, labels and counts copied back to the jobs' host buffers. */
vf_status vf_batch_run(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs,
                       vf_job_result* results);
/* Resident mode: plan the jobs and upload their inputs once; then every
 * vf_batch_execute runs all stages on the HBM-resident inputs (download != 0
 * also copies labels and counts back).  The job structs and their host
 * buffers must stay valid until the next prepare or run. */
vf_status vf_batch_prepare(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs);
vf_status vf_batch_execute(vf_ctx* ctx, int download, vf_job_result* results);
/* Plain path: one job at a time, stage by stage, flood as one launch plus a
 * host read per BFS wave (the reference's execution shape). */
vf_status vf_plain_run(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs,
                       vf_job_result* results);
/* device bytes vf_batch_run needs for these jobs (admission control) */
size_t vf_job_footprint(const vf_job* job);

/* ---- serving: continuous batching ---------------------------------------
 * A server thread admits submitted jobs against hbm_budget, packs the
 * admitted ones into micro-batches on up to max_inflight streams, keeps
 * grids resident between stages and streams labels back.  The job's host
 * buffers must stay valid until its result is polled.  0 selects the
 * defaults: half the context's budget, 3 streams, 128 jobs per batch. */
vf_status vf_server_create(vf_ctx* ctx, size_t hbm_budget, uint32_t max_inflight,
                           uint32_t max_batch_jobs, vf_server** out);
vf_status vf_server_submit(vf_server* s, const vf_job* job, uint64_t* ticket);
/* waits up to wait_ms for results; *n = results written (<= max) */
vf_status vf_server_poll(vf_server* s, vf_job_result* out, uint32_t max,
                         uint32_t* n, int wait_ms);
vf_status vf_server_destroy(vf_server* s);

/* ---- pipelined batches ---------------------------------------------------
 * No counterpart in the reference.  A caller with a stream of batches keeps
 * up to `depth` (1..4) of them in flight, each with its own stream and device
 * memory: vf_pipeline_submit plans a batch, issues its uploads, stages and
 * downloads, and returns; vf_pipeline_collect waits for the oldest batch and
 * writes its results (vf_batch_run semantics per batch).  Labels are packed
 * on the device and copied to out_labels by the copy engine, so the download
 * of one batch runs while the next batch computes.  The jobs' host buffers
 * must stay valid until their batch is collected. */
vf_status vf_pipeline_create(vf_ctx* ctx, uint32_t depth, vf_pipeline** out);
/* VF_ERR_BUSY when `depth` batches are in flight: collect one first */
vf_status vf_pipeline_submit(vf_pipeline* p, const vf_job* jobs, uint32_t njobs);
/* results of the oldest batch, in job order; *njobs = its job count.
 * VF_ERR_INVALID when no batch is in flight or max < its job count (the
 * batch then stays in flight). */
vf_status vf_pipeline_collect(vf_pipeline* p, vf_job_result* results, uint32_t max,
                              uint32_t* njobs);
/* waits for the batches in flight (their results are dropped) */
vf_status vf_pipeline_destroy(vf_pipeline* p);

/* ---- flood without device allocation ------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory during this step (their memory is owned by a pool of their own, or
 * must not grow after start-up): FloodFracturer::build semantics on the
 * caller's device buffers -- d_grid (uint16, x-major X*Y*Z, 0 = EMPTY), the
 * seeds (device, 4 uint32 x,y,z,label per seed, labels 2..255) -- writing the
 * labels to d_labels (uint16, x-major X*Y*Z).  All scratch lives in one
 * file-scope device array of 32 MiB inside the library, held by every GPU
 * that loads it until exit; grids needing more (about 5 million voxels)
 * return VF_ERR_RANGE.  Calls share that array: calls that overlap on the
 * GPU race.  The flood inside is a cooperative launch with a grid-wide
 * barrier, so a call must not overlap a context's batched flood
 * (vf_batch_run, vf_pipeline_*, vf_server_*) on another stream either (the
 * barrier's bounded wait could run out: VF_ERR_TIMEOUT).  The first call on
 * a device looks up the array's address; make it before any stream capture.
 * Runs on `stream` (a cudaStream_t, NULL = default stream) and returns when
 * the labels are written.  nseeds = 0 labels every occupied voxel FREE (1).
 * On an error (VF_ERR_INVALID for a seed outside the grid or a label that is
 * not 2..255 in its low byte or carries a sub-seed prefix) the contents of
 * d_labels are unspecified. */
vf_status vf_flood_noalloc(const uint16_t* d_grid, uint16_t* d_labels, uint32_t X, uint32_t Y,
                           uint32_t Z, const uint32_t* d_seeds_xyzw, uint32_t nseeds,
                           int distance, void* stream);

/* ---- timing helpers for benchmarks (CUDA events on the context stream) --- */
vf_status vf_ctx_event_record(vf_ctx* ctx, int slot);
vf_status vf_ctx_event_elapsed(vf_ctx* ctx, int slot_a, int slot_b, float* ms);
/* per-kernel statistics of the last vf_batch_run: launches and device ms of
 * the flood relaxation kernel (for the roofline) */
vf_status vf_ctx_last_stats(vf_ctx* ctx, uint64_t* kernel_launches,
                            float* flood_ms, uint64_t* flood_bytes,
                            uint64_t* flood_brick_visits);

/* device ms of the stages of the last batched run: [0] input upload,
 * [1] tetrahedra, [2] parity raster, [3] shell SAT, [4] combine + live
 * bricks, [5] seeds, [6] fracture, [7] perturb, [8] erode/boundaries,
 * [9] counts, [10] download (n <= 11 entries written) */
vf_status vf_ctx_stage_ms(vf_ctx* ctx, float* ms, uint32_t n);
/* flood relaxation of the last batched run: passes (grid-wide rounds),
 * brick sweeps summed over all visits, visits that hit the sweep cap */
vf_status vf_ctx_flood_stats(vf_ctx* ctx, uint64_t* passes, uint64_t* sweeps,
                             uint64_t* maxit_hits);
/* raw flood counters of the last batched run: [0] brick visits, [1] passes,
 * [2] warps with work summed over sweeps (8 warps per brick), [3] barrier
 * timeouts, [4] sweeps, [5] visits at the sweep cap, [6] active rows summed
 * over sweeps, [7] voxel key changes, [8] 0, or the kind of the first
 * out-of-range access the relaxation skipped (1 brick id, 2 job id, 3 key
 * read, 4 queued brick id, 5 key write; the batch then fails with
 * VF_ERR_TIMEOUT) with [9], [10] its brick and index, [11..15] SM cycles / 256
 * summed over the relaxation CTAs in each phase of their work: [11] claiming
 * a brick, [12] staging its keys, [13] sweeps, [14] write-back and enqueue of
 * neighbours, [15] from the last claim of a pass through the pass barrier,
 * [16] visits that found no change around the brick and staged nothing
 * (included in [0]), [17] visits that staged their brick but changed no key.
 * n <= 20 are filled, the rest zeroed. */
vf_status vf_ctx_flood_counters(vf_ctx* ctx, uint64_t* out, uint32_t n);
/* bricks queued for each pass of the last batched flood (first 256 passes;
 * zero beyond the pass count). */
vf_status vf_ctx_flood_pass_sizes(vf_ctx* ctx, uint32_t* out, uint32_t n);
/* *replayed = 1 when the last vf_batch_execute ran its stage chain as a
 * CUDA graph (captured on the first execute after vf_batch_prepare, replayed
 * afterwards), 0 when it launched the stages directly. */
vf_status vf_ctx_last_graph(vf_ctx* ctx, int* replayed);

/* ---- tuning (no counterpart in the reference) ----------------------------
 * Launch settings of a context, in this order: [0] parity-fill CTAs per SM,
 * [1] shell-test CTAs per SM, [2] flood relaxation sweeps per brick visit
 * (BFS waves a brick advances per pass before it re-queues itself),
 * [3] flood CTAs per SM (0: as many as fit).  Results never depend on them. */
vf_status vf_ctx_set_tuning(vf_ctx* ctx, const int32_t* values, uint32_t n);
/* Spin limit of the flood relaxation's pass barrier on this context (polls
 * of about 64 ns each; 0 restores the default 2^26, about 4 s).  When the
 * limit runs out the kernel sets its error word and returns, and the call
 * fails with VF_ERR_TIMEOUT; the context stays usable.  A small limit makes
 * the bounded device wait run out on purpose (tests of the error path). */
vf_status vf_ctx_set_flood_wait_limit(vf_ctx* ctx, uint32_t spins);
vf_status vf_ctx_get_tuning(vf_ctx* ctx, int32_t* values, uint32_t n);
/* Autotuner: prepares `jobs` as a resident batch (as vf_batch_prepare, which
 * it replaces) and runs it under candidate settings, one knob at a time,
 * keeping for each knob the value with the lowest device time of its stage.
 * The chosen settings stay on ctx (n of them copied to `chosen`). */
vf_status vf_autotune(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs, int32_t* chosen,
                      uint32_t n);

#ifdef __cplusplus
}
#endif
#endif
