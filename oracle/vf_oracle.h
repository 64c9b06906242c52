/*
 * vf_oracle.h -- CPU oracle for the voxelize -> seed -> flood/Voronoi ->
 * perturb/erode -> count path of AlfonsoLRz/VoxelFragmentML.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The product
 * (voxelfragmentml_gb300/) never links, imports or calls it.
 *
 * Every function restates the reference algorithm it names (file:line of
 * the reference project).  Where the reference is racy or calls a graphics
 * pipeline, the restatement fixes one deterministic rule and says so.
 *
 * Parity pinning: the reference ships no tests and no golden vectors for
 * this path (its only fixture, docs/decompress/samples/AL_12B_grid_128r.rle,
 * pins the RLE grid format and the x-major voxel order).  The reference is
 * Windows/OpenGL/glm/boost/CGAL code and cannot be compiled here, and its
 * GL rasterizer cannot be run here.  Parity of the algorithm itself is
 * therefore UNPINNED against reference outputs; it is pinned against the
 * hand-worked known-answer cases in tests/golden/.
 *
 * Grid layout (RegularGrid.cpp:1031-1034): uint16 per voxel, index
 * x*Y*Z + y*Z + z.  Values: 0 EMPTY, 1 FREE, labels >1; bits 0-7 fragment
 * id, bits 8-14 sub-seed prefix, bit 15 boundary flag (voxelMask.glsl).
 *
 * Build with -ffp-contract=off: every float expression is evaluated in the
 * written order with separate rounding (no FMA), which the CUDA kernels
 * reproduce with -fmad=false.
 */
#ifndef VF_ORACLE_H
#define VF_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes shared with the product ABI (same numbers) */
#define VFO_OK 0
#define VFO_ERR_INVALID 1
#define VFO_ERR_SEED_SEARCH 4
#define VFO_ERR_RANGE 5

/* FractureParameters.h enums */
#define VFO_NAIVE 0
#define VFO_FLOOD 1
#define VFO_EUCLIDEAN 0
#define VFO_MANHATTAN 1
#define VFO_CHEBYSHEV 2
#define VFO_SQUARE 0
#define VFO_ELLIPSE 1
#define VFO_CROSS 2
/* Seeder::Location (Seeder.h:24) */
#define VFO_INNER 0
#define VFO_OUTER 1
#define VFO_BOTH 2

/* counter-based RNG streams */
#define VFO_STREAM_SEEDS 1u
#define VFO_STREAM_ERODE 2u
#define VFO_STREAM_NOISE 3u

uint64_t vfo_hash(uint64_t seed, uint32_t stream, uint64_t counter);
float vfo_u01(uint64_t h);

/* ---- voxelization (RegularGrid::fill(Model3D*) RegularGrid.cpp:173-212) ---- */
/* occupancy = tri-box SAT shell (Intersections3D.h:204-258) OR tetra-parity
 * interior (Tetravoxelizer.cpp:42-92,198-315).  grid is written with 0/1. */
int vfo_voxelize(const float* verts, uint32_t nverts, const uint32_t* faces,
                 uint32_t nfaces, uint32_t X, uint32_t Y, uint32_t Z,
                 const float aabb_min[3], const float aabb_max[3],
                 uint16_t* grid, int mode /*1 shell, 2 parity, 3 both*/);
/* the single SAT test, exposed for known-answer tests */
int vfo_tri_box(const float p0[3], const float p1[3], const float p2[3],
                const float box_min[3], const float box_max[3]);
/* allocateMeshGrid dims rule (CADScene.cpp:545-561) */
void vfo_grid_dims(const float aabb_min[3], const float aabb_max[3],
                   uint32_t max_voxels, uint32_t dims_out[3]);

/* ---- seeding (Seeder.cpp:115-208) ---- */
int vfo_seeder_uniform(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                       uint32_t n, uint64_t seed, int location,
                       uint32_t* out_xyzw);
int vfo_merge_seeds(const uint32_t* frags, uint32_t nfrags, uint32_t* seeds,
                    uint32_t nseeds, int dfunc);
/* CADScene::fractureModel seed assembly (CADScene.cpp:624-655):
 * uniform(main) [+ nearSeeds(num_impacts, bias_seeds, bias_focus) when
 * num_impacts > 0, the placed seeds joining the main ones] [+ uniform(extra,
 * BOTH) + mergeSeeds].  out must hold 4*(2*(n_main + bias_seeds) + n_extra)
 * entries; *nout receives the count. */
int vfo_fracture_seeds(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                       uint32_t n_main, uint32_t n_extra, int location,
                       int merge_dfunc, uint64_t seed, uint32_t num_impacts,
                       uint32_t bias_seeds, uint32_t bias_focus, uint32_t* out,
                       uint32_t* nout);

/* ---- fracturers ---- */
/* FloodFracturer::build (FloodFracturer.cpp:98-191).  Returns the number of
 * BFS waves run in *waves (may be NULL). */
int vfo_flood(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
              const uint32_t* seeds, uint32_t nseeds, int dfunc,
              uint32_t* waves);
/* NaiveFracturer::buildCPU (NaiveFracturer.cpp:26-68) */
int vfo_naive(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
              const uint32_t* seeds, uint32_t nseeds, int dfunc);

/* ---- boundary perturbation (no reference counterpart; defined here) ---- */
int vfo_perturb(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                float amplitude, uint32_t period, uint64_t seed);

/* ---- grid passes ---- */
void vfo_detect_boundaries(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                           int boundary_size);
void vfo_remove_isolated(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z);
int vfo_erode(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, int type,
              uint32_t size, uint32_t iterations, float probability,
              float threshold, uint64_t seed);
void vfo_undo_mask(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z);
/* RegularGrid::countValues (RegularGrid.cpp:601-625): counts[v] for
 * v = value & 0x7FFF over voxels with value > 1.  counts has ncounts
 * entries; returns VFO_ERR_RANGE if a value >= ncounts occurs. */
int vfo_count_values(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                     uint32_t* counts, uint32_t ncounts, uint64_t* occupied);

/* ---- whole job: fill -> seeds -> fracture -> perturb -> erode|boundaries ---- */
typedef struct vfo_params {
  int32_t algorithm, distance, num_seeds, num_extra_seeds, merge_distance,
      seed_location;
  uint64_t seed;
  float noise_amplitude;
  uint32_t noise_period;
  int32_t erode, erosion_type, erosion_size, erosion_iterations;
  float erosion_probability, erosion_threshold;
  int32_t boundary_size;
  int32_t num_impacts, bias_seeds, bias_focus; /* nearSeeds after the main seeds */
} vfo_params;

int vfo_run_job(const float* verts, uint32_t nverts, const uint32_t* faces,
                uint32_t nfaces, uint32_t X, uint32_t Y, uint32_t Z,
                const float aabb_min[3], const float aabb_max[3],
                const vfo_params* p, uint16_t* grid, uint32_t* counts,
                uint32_t ncounts, uint32_t* seeds_out, uint32_t* nseeds_out);

/* RLE export (RegularGrid.cpp:672-714): returns bytes written to out (or
 * needed when out is NULL). */
size_t vfo_rle_encode(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                      uint8_t* out, size_t cap);

/* RegularGrid::toTriangleMesh (RegularGrid.cpp:443-486): one smoothed
 * marching-cubes mesh per fragment value (label & 0x7FFF > 1, ascending),
 * vf_oracle_mesh.c.  Sizes go to *nmeshes / *nverts / *nfaces; with values
 * given, the meshes are written too: values[F], vert_off[F+1],
 * face_off[F+1], verts 4 floats (x, y, z, boundary) and faces 4 uint32
 * (three mesh-local vertex indices, boundary) per element. */
int vfo_triangulate(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                    const float amin[3], const float amax[3], uint32_t nb_iters,
                    float nb_weight, uint32_t b_iters, float b_weight,
                    uint32_t* nmeshes, uint64_t* nverts, uint64_t* nfaces,
                    uint16_t* values, uint64_t* vert_off, uint64_t* face_off,
                    float* verts, uint32_t* faces);

/* Impact path (vf_oracle_impact.c): the 1-based index of the first occupied
 * voxel a ray enters (RegularGrid::rayTraversalAmanatidesWoo, RegularGrid.cpp:
 * 900-1004; 0xFFFFFFFF x3 on a miss), and Seeder::nearSeeds (Seeder.cpp:
 * 49-113): out = frags followed by the new seeds, 4 uint32 each, *nout the
 * count (at most nfrags + num_seeds). */
/* CADModel::sampleCPU (vf_oracle_sample.c): at most S points (4 floats:
 * x, y, z, 1) on the mesh verts (4 floats per vertex) / faces (4 uint32 per
 * face: three vertex indices, unused); key: the mesh's draw key. */
int vfo_sample_mesh(const float* verts, const uint32_t* faces, uint32_t nfaces, uint32_t S,
                    uint64_t seed, uint32_t key, float* out, uint64_t* nout);

#define VFO_NEAR_MAX_CANDIDATES (1u << 20)
int vfo_ray_entry(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                  const float amin[3], const float amax[3], const float origin[3],
                  const float dir[3], uint32_t out[3]);
int vfo_ray_entry_batch(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                        const float amin[3], const float amax[3], const float* rays,
                        uint32_t n, uint32_t* out);
int vfo_near_seeds(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                   const uint32_t* frags, uint32_t nfrags, uint32_t num_impacts,
                   uint32_t num_seeds, uint32_t spreading, uint64_t seed,
                   uint32_t* out, uint32_t* nout);

#ifdef __cplusplus
}
#endif
#endif
