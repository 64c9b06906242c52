// vf_common.cuh -- shared device/host definitions of the GB300 pipeline.
//
// Memory layout in HBM (per job):
//   grid, grid2 : uint16 [X][Y][Zp], Zp = roundup(Z, 8)   (labels, ping-pong)
//   keys        : uint32 [X][Y][Zk], Zk = roundup(Z, 4)   (flood state)
//   par, shell  : uint32 [X][Y][Zw], Zw = ceil(Z / 32)     (voxelizer bit planes,
//                 bit z&31 of word z>>5)
// Rows along z are contiguous, so every brick row is one coalesced segment.
// Padding (z >= Z) of a row that a kernel writes is written as zero.  The
// logical voxel index of the reference (x*Y*Z + y*Z + z,
// RegularGrid.cpp:1031-1034) is only used where the reference uses it as a
// value (erosion noise index, plain-path frontier entries).
//
// Bricks: VF_BX x VF_BY x VF_BZ voxels (x, y, z).  A global brick id indexes
// every brick of every job of a batch; brick_job[b] gives its job.  A brick
// is "live" when it holds an occupied voxel; every stage after the
// voxelizer touches live bricks only, and halo reads from bricks that are
// not live return EMPTY.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define VF_BX 16
#define VF_BY 16
#define VF_BZ 32
#define VF_BRICK_VOXELS (VF_BX * VF_BY * VF_BZ)

#define VOXEL_EMPTY 0u
#define VOXEL_FREE 1u

// flood key encoding: key = ~((dist << 12) | seed_slot); 0 = wall (EMPTY),
// 1 = occupied, not reached.  A larger key is closer (then a lower slot).
#define VF_KEY_WALL 0u
#define VF_KEY_UNREACHED 1u
#define VF_KEY_MIN_REACHED 4096u  // dist <= 0xFFFFE
#define VF_KEY_STEP 4096u

// per-job error bits (JobState::err)
#define VF_JERR_SEED_SEARCH 1u
#define VF_JERR_DIST_OVERFLOW 2u
#define VF_JERR_RANGE 4u
#define VF_JERR_TIMEOUT 8u
#define VF_JERR_INVALID 16u

#define VF_MAX_TRIES 1000000u   // Seeder.h:48
#define VF_FLOOD_NCOUNTERS 20    // raw flood relaxation counters (vf_ctx_flood_counters)
#define VF_NOISE_BUFFER 1000000u // RegularGrid.cpp:124

struct JobDesc {
  uint32_t X, Y, Z, Zp, Zk, Zw;
  uint32_t nbx, nby, nbz, brick_base, nbricks;
  uint16_t* grid;   // stage source (and in-place target)
  uint16_t* grid2;  // stage destination for double-buffered stages
  uint32_t* keys;
  uint32_t* par;
  uint32_t* shell;
  // mesh
  const float* verts;
  const uint32_t* faces;
  uint32_t nverts, nfaces;
  uint32_t face_base;   // first global face index of this job
  float amin[3], amax[3];
  float cs[3];          // cell size (amax - amin) / dims, IEEE division on the host
  float ics[3];         // 1 / cs (approximate: candidate bounds only)
  float4* tets;         // 3 float4 per face: its vertices in NDC sorted by y,
                        // (P0x,P0y,P0z,P1x) (P1y,P1z,P2x,P2y) (P2z,-,-,-)
  uint32_t* tet_range;  // first slice plane crossing the face (s0 | s1 << 16)
  float* ys;            // Y slice planes
  unsigned long long* etab;  // edge parity table: key lo << 32 | hi, bit 63 = odd
  uint32_t ecap;             // slots (power of two, >= 4 * nfaces)
  // seeds
  uint32_t* seeds;      // xyzw, capacity seeds_cap
  uint32_t seeds_cap;
  uint32_t seeds_given; // caller-provided seeds already in `seeds` (0: sample)
  // outputs
  uint32_t* counts;
  uint32_t ncounts;
  // params
  int32_t algorithm, distance, num_seeds, num_extra, merge_distance, seed_location;
  unsigned long long seed;
  float noise_amplitude;
  uint32_t noise_period;
  int32_t erode, erosion_type, erosion_size, erosion_iterations;
  float erosion_probability, erosion_threshold;
  int32_t boundary_size;
  int32_t num_impacts, bias_seeds, bias_focus;  // Seeder::nearSeeds after the main seeds
  float* lattice;       // perturbation lattice values, 3 per point
  uint32_t lat_nx, lat_ny, lat_nz;
  // label download: device-accessible destination (mapped pinned host memory
  // or device memory; null = copy-engine download) and first global row
  uint16_t* out;
  unsigned long long row_base;
  uint32_t out_dma;  // out is the device staging buffer of the DMA download
  // stage selection bits for the kernel that receives this table
  uint32_t active;
  float* emask;         // erosion mask (k^3 floats)
  float elimit;         // activations * threshold
  int32_t ek;           // erosion window size (odd)
};

struct JobState {
  float centroid[3];
  uint32_t nseeds;
  uint32_t err;
  uint32_t has_prefix;      // any seed label with a sub-seed prefix
  uint32_t disjoint;        // voxels reset by the disjoint cleanup
  uint32_t changed;         // generic convergence flag
  uint32_t minprefix[256];  // per fragment
  uint32_t rank_value[256]; // pass-2 slot -> label value
  uint32_t value_rank[256]; // fragment id -> pass-2 slot
  unsigned long long occupied;
  uint32_t passes;
  uint32_t nranks;
};

// ---------------------------------------------------------------------------
// Counter-based RNG (SplitMix64 finaliser, Steele/Lea/Flood 2014).  Replaces
// std::mt19937 + uniform_real_distribution (RandomUtilities.h:11-22).
__host__ __device__ __forceinline__ uint64_t vf_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t vf_hash(uint64_t seed, uint32_t stream,
                                                     uint64_t counter) {
  uint64_t k = vf_mix64(seed ^ ((uint64_t)stream * 0x9E3779B97F4A7C15ull));
  return vf_mix64(k + counter * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
}
__host__ __device__ __forceinline__ float vf_u01(uint64_t h) {
  return (float)(uint32_t)(h >> 40) * 5.9604644775390625e-8f;
}
#define VF_STREAM_SEEDS 1u
#define VF_STREAM_ERODE 2u
#define VF_STREAM_NOISE 3u
#define VF_STREAM_IMPACT 4u  // nearSeeds: fragment pick and seed count per impact
#define VF_STREAM_NEAR 5u    // nearSeeds: candidate offsets
#define VF_NEAR_MAX_CANDIDATES (1u << 20)  // candidates one impact may try
#define VF_STREAM_SAMPLE 6u       // point sampling: noise buffer
#define VF_STREAM_SAMPLE_FACE 7u  // point sampling: face draws

__host__ __device__ __forceinline__ uint32_t vf_roundup(uint32_t v, uint32_t m) {
  return (v + m - 1) / m * m;
}
__host__ __device__ __forceinline__ int vf_clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}
__host__ __device__ __forceinline__ size_t vf_gidx(const JobDesc& j, uint32_t x, uint32_t y,
                                                   uint32_t z) {
  return ((size_t)x * j.Y + y) * j.Zp + z;
}
__host__ __device__ __forceinline__ size_t vf_kidx(const JobDesc& j, uint32_t x, uint32_t y,
                                                   uint32_t z) {
  return ((size_t)x * j.Y + y) * j.Zk + z;
}
