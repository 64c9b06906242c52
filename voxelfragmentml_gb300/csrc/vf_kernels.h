// vf_kernels.h -- host launchers of the device stages (internal).
//
// Every launcher takes a device array of JobDesc (one table per stage, see
// vf_runtime.cu) plus the per-job JobState array, and enqueues on `st`.
// Brick-parallel stages take the list of live bricks and brick_job map.
#pragma once
#include <string>
#include "vf_common.cuh"

namespace vfk {

// ---- voxelizer (Tetravoxelizer + tri-box SAT) ----
// flattened per-face work list (parity: slice planes crossing the face;
// shell: candidate columns): per-face counts and their exclusive prefix sums
// over the faces of all jobs
struct FaceScratch {
  uint32_t* pcnt;                // [total_faces]
  unsigned long long* pbase;     // [total_faces]
  unsigned long long* psums;     // [ceil(total_faces / 1024)]
  unsigned long long* ptotal;    // [1]
  float4* srec;                  // [6 * total_faces] per-face shell setup
};
void centroid_and_slices(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs);
void tetra_prep(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                uint32_t total_faces, const FaceScratch& fs);
void parity_raster(cudaStream_t st, const JobDesc* dj, const JobState* ds, int njobs,
                   uint32_t total_faces, const FaceScratch& fs, int num_sms, int grid_mult = 16);
// reuses the face scratch after the parity raster (counts, scan, runs)
void shell_sat(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces,
               const FaceScratch& fs, int num_sms, int grid_mult = 12);
// writes 0/1 labels (grid, and grid2 when dual) for every brick of every
// job and sets live[b]
void combine(cudaStream_t st, const JobDesc* dj, const uint32_t* brick_job,
             uint32_t total_bricks, uint8_t* live, int dual);
void mark_live(cudaStream_t st, const JobDesc* dj, const uint32_t* brick_job,
               uint32_t total_bricks, uint8_t* live);
void compact_live(cudaStream_t st, const uint8_t* live, uint32_t total_bricks,
                  uint32_t* list, uint32_t* count);

// labels of every job with a device-accessible `out` (T_CNT table: the
// final buffer) into `out`, rows of Z without the z padding
void pack_labels(cudaStream_t st, const JobDesc* dj, int njobs, uint64_t total_rows, int num_sms);

// exclusive prefix sum of n u32 into u64 (sums: ceil(n / 1024) + 1 scratch
// words); *total = the sum
void exclusive_scan(cudaStream_t st, const uint32_t* in, unsigned long long* out,
                    unsigned long long* sums, uint32_t n, unsigned long long* total);

// ---- RLE export (vf_rle.cu) ----
// run starts counted per (x, y) row of a grid [X][Y][Zp]
void rle_count(cudaStream_t st, const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, uint32_t Zp,
               uint32_t* row_cnt, int num_sms);
// records {u16 value, u32 repetitions} as 3 u16 per run, from the scanned
// row counts; starts: scratch of one u64 per run
void rle_write(cudaStream_t st, const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, uint32_t Zp,
               const unsigned long long* row_base, const unsigned long long* nruns,
               unsigned long long* starts, uint16_t* records, int num_sms);

// ---- marching cubes per fragment (vf_mesh.cu) ----
struct MeshGrid {
  const uint16_t* g;  // [X][Y][Zp] labels
  uint32_t X, Y, Z, Zp;
};
// the case table packed for the kernels: 4 bits per edge, triangle count
void mc_pack_table(unsigned long long tri[256], uint8_t ntri[256]);
// exposed-face masks (X*Y*Z bytes), vertices per grid row, present[value]
void mc_vertex_count(cudaStream_t st, const MeshGrid& G, uint8_t* mask, uint32_t* rcnt,
                     uint8_t* present, int num_sms);
// vertex id base per voxel, fragment key and (voxel * 8 + direction) per vertex
void mc_vertex_emit(cudaStream_t st, const MeshGrid& G, const uint8_t* mask,
                    const unsigned long long* rbase, const uint16_t* dense, uint32_t* vbase,
                    uint16_t* vkey, unsigned long long* vown, int num_sms);
// triangles per cell row ((X+1)*(Y+1) rows of Z+1 cells)
void mc_tri_count(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                  const uint8_t* ntri, uint32_t* rcnt, int num_sms);
void mc_tri_emit(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                 const uint8_t* ntri, const unsigned long long* rbase, const uint8_t* mask,
                 const uint32_t* vbase, const uint16_t* dense, uint16_t* tkey, uint4* tv,
                 uint32_t* vflag, uint32_t* err, int num_sms);
// stable order of items 0..n-1 by key[item] (< nkeys <= 65536) into out;
// tmp: n words (two passes), hist: split_hist_words(n) words, hbase the
// same count of u64, sums/tot: exclusive_scan scratch for that many words
size_t split_hist_words(uint64_t n);
void stable_split16(cudaStream_t st, const uint16_t* key, uint64_t n, uint32_t nkeys, uint32_t* tmp,
                    uint32_t* out, uint32_t* hist, unsigned long long* hbase,
                    unsigned long long* sums, unsigned long long* tot);
void mc_outputs(cudaStream_t st, const MeshGrid& G, const uint32_t* vperm,
                const unsigned long long* vown, const uint32_t* vflag, uint64_t V, const float s[3],
                const float c[3], uint32_t* vinv, float4* vert, const uint32_t* tperm,
                const uint4* tv, uint64_t T, uint4* gface, int num_sms);
// off[f] = first sorted position with key >= f, f = 0..F
void mc_offsets(cudaStream_t st, const uint16_t* key, const uint32_t* perm, uint64_t n, uint32_t F,
                unsigned long long* off);
// smoothSurface (MarchingCubes.cpp:489-510), in two steps.  mc_smooth_lists:
// per vertex, the distinct neighbours (with multiplicity) of the faces its
// pass sums, and meta; scratch deg V u32, start / ustart V + 1 u64, sums
// exclusive_scan scratch for V, ent / nbr one uint2 / u32 per counted face
// incidence (at most 3 T), meta V uint2, stats 2 u64 (boundary vertices,
// their neighbour entries); err bit 2 if a vertex has more incidences than
// its meta holds; needs V < 2^28.  mc_smooth_iterate: nb_iters over the
// non-boundary vertices, then b_iters over the boundary ones (tmp: V float4).
cudaError_t mc_smooth_lists(cudaStream_t st, const uint4* gface, uint64_t T, const float4* vert,
                            uint64_t V, uint32_t* deg, unsigned long long* start,
                            unsigned long long* ustart, unsigned long long* sums, uint2* ent,
                            uint32_t* nbr, uint2* meta, uint32_t* err, unsigned long long* stats,
                            int num_sms);
cudaError_t mc_smooth_iterate(cudaStream_t st, float4* vert, float4* tmp, uint64_t V,
                              const uint2* meta, const uint32_t* nbr, uint32_t nb_iters,
                              float nb_weight, uint32_t b_iters, float b_weight, int num_sms);
void mc_local_faces(cudaStream_t st, const uint4* gface, const uint32_t* tperm, const uint16_t* tkey,
                    const unsigned long long* voff, uint64_t T, uint4* out, int num_sms);

// ---- impact path (vf_impact.cu) ----
struct ImpactGrid {
  const uint16_t* g;  // [X][Y][Zp] labels
  uint32_t X, Y, Z, Zp;
  float amin[3], amax[3], cell[3];  // the grid's box and (amax - amin) / dims
};
// per ray (origin xyz, direction xyz): the 1-based index of the first
// occupied voxel, 0xFFFFFFFF x3 when none; zero directions are rejected by
// the caller.  bits (X * Y * ceil(Z / 32) words, or NULL): scratch for the
// packed occupancy the walks read instead of the labels
void ray_entry(cudaStream_t st, const ImpactGrid& G, const float* rays, uint32_t n, uint32_t* out,
               uint32_t* bits, int num_sms);
// Seeder::nearSeeds: the new seeds (4 uint32 each, labels label0 + 1, ...)
// in (x, y, z) order into out; status[0] = count, status[1] = 0 or
// VF_ERR_SEED_SEARCH.  Needs nfrags >= 1, num_seeds <= 4095 and
// 1 <= spreading <= min(dims) when num_impacts > 0.
void near_seeds(cudaStream_t st, const ImpactGrid& G, const uint32_t* frags, uint32_t nfrags,
                uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading, uint64_t seed,
                uint32_t label0, uint32_t* out, uint32_t* status);

// ---- point sampling of meshes (vf_sample.cu) ----
struct SampleMeshes {
  const float4* verts;  // x, y, z, (w)
  const uint4* faces;   // three vertex indices within the mesh, (w)
  const unsigned long long* vert_off;  // F + 1
  const unsigned long long* face_off;  // F + 1
  const uint32_t* keys;                // F: the noise and draw key of each mesh
  uint32_t F;
  uint64_t nfaces;
};
// areas, per-chunk sums (chunks of at most 1024 faces that start at each
// mesh's first face: cstart/cend, mchunk[m] = first chunk of mesh m, F + 1),
// per mesh sumArea (msum) and noise length (nb)
void pc_areas(cudaStream_t st, const SampleMeshes& M, float* area, const unsigned long long* cstart,
              const unsigned long long* cend, uint32_t nchunks, double* csum, float* cmax,
              const unsigned long long* mchunk, uint32_t S, float* msum, uint64_t* nb, int num_sms);
// for the meshes listed in sel (S <= T): S distinct faces into the bitmap
// chosen (one bit per global face, zeroed); err bit 0 if the draws run out
void pc_select(cudaStream_t st, const SampleMeshes& M, const uint32_t* sel, uint32_t nsel, uint32_t S,
               uint64_t seed, uint32_t* chosen, uint32_t* err);
// samples per face (cnt), their exclusive scan (soff, nfaces + 1), P per mesh
void pc_count(cudaStream_t st, const SampleMeshes& M, const float* area, const float* msum,
              const uint8_t* big, uint32_t S, const uint32_t* chosen, uint32_t* cnt,
              unsigned long long* P, unsigned long long* soff, unsigned long long* sums, int num_sms);
// the points (x, y, z, 1) of mesh m at out[out_off[m] ..]
void pc_points(cudaStream_t st, const SampleMeshes& M, const uint32_t* cnt, const unsigned long long* soff,
               const uint64_t* nb, const uint8_t* big, const unsigned long long* out_off, uint32_t S,
               uint64_t seed, float4* out, int num_sms);

// ---- seeds ----
void sample_seeds(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs);

// ---- fracturers ----
void naive(cudaStream_t st, const JobDesc* dj, const JobState* ds, const uint32_t* list,
           const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);

// ---- grid passes (brick kernels, live bricks only) ----
void lattice(cudaStream_t st, const JobDesc* dj, int njobs);
void perturb(cudaStream_t st, const JobDesc* dj, const uint32_t* list, const uint32_t* count,
             uint32_t max_count, const uint32_t* brick_job);
void detect_boundaries(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                       const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);
// boundary sizes 2..3
void detect_boundaries_wide(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                            const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);
void erode(cudaStream_t st, const JobDesc* dj, const uint32_t* list, const uint32_t* count,
           uint32_t max_count, const uint32_t* brick_job);
void remove_isolated(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                     const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);
void count_values(cudaStream_t st, const JobDesc* dj, JobState* ds, const uint32_t* list,
                  const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);

// ---- flood (vf_flood.cu) ----
// Words per brick of the flood's change record: [0] neighbour directions
// (bit dx*9 + dy*3 + dz: the brick at offset (dx-1, dy-1, dz-1) changed keys
// this brick reads; bit 13: every row), [1..8] rows whose key at z0-1 changed,
// [9..16] rows whose key at z0+32 changed (bit t & 31 of word t >> 5, row
// t = x * 16 + y within the brick).
constexpr uint32_t FLOOD_FDIR = 17;
// the current device, as an index into per-device caches of launch
// attributes (a kernel's shared-memory limit is set once per device)
inline int cur_dev() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) d = 0;
  return d & 63;
}

// TMA descriptor (CUtensorMap, 128 bytes, 64-byte aligned) of one job's
// flood keys uint32 [X][Y][Zk], encoded on the host for k_relax's tile
// loads: boxes of 36 x 18 x 18 keys (z, y, x), zeros outside the grid.
constexpr size_t KEYS_MAP_BYTES = 128;
// false (message in *err) when the driver cannot encode the map
bool encode_keys_map(void* map128, const uint32_t* keys, uint32_t X, uint32_t Y, uint32_t Zk,
                     std::string* err);

struct FloodScratch {
  uint32_t* queue[3];    // brick ids, capacity total_bricks each (rotating)
  uint32_t* qcount;      // [3]
  uint32_t* qhead;       // [3]
  uint32_t* epoch;       // [total_bricks]
  uint32_t* fdir;        // [total_bricks][FLOOD_FDIR] change record, zero between floods
  uint32_t* barrier;     // [2] count, generation
  uint32_t* err;         // [1] global error word
  uint32_t* stats;       // [4] brick visits, passes, overflow, timeout
  uint32_t max_passes;
  uint32_t total_bricks;
  uint32_t njobs = 1;    // job descriptors in the table
  int max_sweeps = 0;    // tuning: sweeps per brick visit (0: default cap)
  int ctas_per_sm = 0;   // tuning: resident CTAs per SM (0: as many as fit)
  uint32_t wait_spins = 0;  // spins of the pass barrier before it gives up (0: 2^26, ~4 s)
  const void* tmaps = nullptr;  // [njobs] keys tensor maps (KEYS_MAP_BYTES each, device)
  uint32_t* pass_sizes = nullptr;  // statistics: bricks queued per pass (256)
};
void flood_init_keys(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                     const uint32_t* count, uint32_t max_count, const uint32_t* brick_job,
                     const uint8_t* live);
void flood_seed_bricks(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs, uint8_t* live,
                       uint32_t* list, uint32_t* count);
void flood_seed(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                const FloodScratch& fs, const uint8_t* live);
// sets k_relax's shared-memory attribute and occupancy (once per process)
void flood_prepare(int num_sms);
cudaError_t flood_relax(cudaStream_t st, const JobDesc* dj, JobState* ds,
                        const uint32_t* brick_job, const uint8_t* live,
                        const FloodScratch& fs, int num_sms, int* blocks_used);
void flood_finalize(cudaStream_t st, const JobDesc* dj, const JobState* ds,
                    const uint32_t* list, const uint32_t* count, uint32_t max_count,
                    const uint32_t* brick_job, int pass2);
// sub-seed prefix competition and the disjoint cleanup
void flood_competition(cudaStream_t st, const JobDesc* dj, JobState* ds, const uint32_t* list,
                       const uint32_t* count, uint32_t max_count, const uint32_t* brick_job);
void flood_disjoint(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                    const uint32_t* list, const uint32_t* count, uint32_t max_count,
                    const uint32_t* brick_job, const FloodScratch& fs, const uint8_t* live);

// ---- plain (reference-shaped) per-voxel kernels for one job ----
void plain_init_keys(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_seed(cudaStream_t st, const JobDesc* dj, JobState* ds, uint32_t* frontier,
                uint32_t* fcount);
void plain_wave(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj,
                const uint32_t* cur, uint32_t ncur, uint32_t* next, uint32_t* ncount);
void plain_finalize(cudaStream_t st, const JobDesc* dj, const JobState* ds, const JobDesc& hj,
                    int pass2);
void plain_undo_mask(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_detect(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_erode(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_remove_isolated(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_perturb(cudaStream_t st, const JobDesc* dj, const JobDesc& hj);
void plain_naive(cudaStream_t st, const JobDesc* dj, const JobState* ds, const JobDesc& hj);
void plain_counts(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj);
void plain_competition(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj);
void plain_disjoint(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj,
                    uint32_t* frontier, uint32_t* fcount);

}  // namespace vfk
