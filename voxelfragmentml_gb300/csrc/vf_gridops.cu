// vf_gridops.cu -- seeding, naive Voronoi, perturbation, boundary detection,
// erosion, isolated-voxel removal and per-fragment counts on sm_103a.
//
// Brick kernels: one CTA (256 threads) per live brick, one thread per (x,y)
// row of VF_BZ = 32 voxels.  The brick plus an xy halo of H voxels and a z
// window [z0-8, z0+40) is staged in shared memory with 16-byte loads (rows
// are 16-byte aligned because Zp % 8 == 0), results are written back as
// 16-byte stores of whole rows (padding z >= Z written as 0).  Halo voxels
// outside the grid read as EMPTY; voxels of bricks that are not live are
// EMPTY in memory (both grid buffers start as the voxelizer output).
//
// The CTAs of a launch loop over the live-brick list (its length is read on
// the device, so launches need no host synchronisation).
#include <algorithm>

#include "vf_kernels.h"
#include "vf_near.cuh"

#include <cfloat>

namespace {

constexpr int ZW = VF_BZ + 16;  // z window of a staged tile (u16)

template <int H>
struct Tile {
  static constexpr int NX = VF_BX + 2 * H, NY = VF_BY + 2 * H;
  static constexpr int ROWS = NX * NY;
  static constexpr int BYTES = ROWS * ZW * 2;
};

__device__ __forceinline__ void brick_coords(const JobDesc& J, uint32_t b, uint32_t& x0,
                                             uint32_t& y0, uint32_t& z0) {
  const uint32_t lb = b - J.brick_base;
  const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
  x0 = bx * VF_BX;
  y0 = by * VF_BY;
  z0 = bz * VF_BZ;
}

// stage src rows [x0-H, x0+16+H) x [y0-H, y0+16+H) x [z0-8, z0+40) into tile
template <int H>
__device__ __forceinline__ void load_tile(const JobDesc& J, const uint16_t* src, uint32_t x0,
                                          uint32_t y0, uint32_t z0, uint16_t* tile) {
  using T = Tile<H>;
  uint4* t4 = reinterpret_cast<uint4*>(tile);
  constexpr int PER_ROW = ZW / 8;
  for (int q = threadIdx.x; q < T::ROWS * PER_ROW; q += blockDim.x) {
    const int row = q / PER_ROW, part = q % PER_ROW;
    const int x = (int)x0 - H + row / T::NY, y = (int)y0 - H + row % T::NY;
    const int z = (int)z0 - 8 + part * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (x >= 0 && y >= 0 && z >= 0 && x < (int)J.X && y < (int)J.Y && z < (int)J.Zp)
      v = __ldg(reinterpret_cast<const uint4*>(src + vf_gidx(J, x, y, z)));
    t4[q] = v;
  }
}
template <int H>
__device__ __forceinline__ uint16_t tval(const uint16_t* tile, int lx, int ly, int lz) {
  // lx, ly in [-H, 16+H), lz in [-8, 40) relative to the brick origin
  return tile[((lx + H) * Tile<H>::NY + (ly + H)) * ZW + (lz + 8)];
}

__device__ __forceinline__ void store_row(const JobDesc& J, uint16_t* dst, uint32_t x, uint32_t y,
                                          uint32_t z0, const uint16_t* v /*32*/) {
  const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);
  uint4* d = reinterpret_cast<uint4*>(dst + vf_gidx(J, x, y, z0));
  for (uint32_t q = 0; q < nz / 8; ++q) {
    uint4 w;
    w.x = (uint32_t)v[8 * q + 0] | ((uint32_t)v[8 * q + 1] << 16);
    w.y = (uint32_t)v[8 * q + 2] | ((uint32_t)v[8 * q + 3] << 16);
    w.z = (uint32_t)v[8 * q + 4] | ((uint32_t)v[8 * q + 5] << 16);
    w.w = (uint32_t)v[8 * q + 6] | ((uint32_t)v[8 * q + 7] << 16);
    d[q] = w;
  }
}

// ===========================================================================
// Seeding: Seeder::uniform (Seeder.cpp:154-208) + mergeSeeds (:115-152).
// One 1024-thread block per job.  Attempts are evaluated 1024 at a time in
// parallel; warp 0 then accepts them in attempt order (duplicates skipped),
// which is exactly the sequential rejection loop of the reference.
__device__ __forceinline__ bool occupied_at(const JobDesc& J, int x, int y, int z) {
  return J.grid[vf_gidx(J, x, y, z)] != VOXEL_EMPTY;
}
__device__ bool is_boundary(const JobDesc& J, int x, int y, int z) {
  // RegularGrid::isBoundary(x,y,z,1) (RegularGrid.cpp:543-559)
  const int x0 = vf_clampi(x - 1, 0, J.X - 1), x1 = vf_clampi(x + 1, 0, J.X - 1);
  const int y0 = vf_clampi(y - 1, 0, J.Y - 1), y1 = vf_clampi(y + 1, 0, J.Y - 1);
  const int z0 = vf_clampi(z - 1, 0, J.Z - 1), z1 = vf_clampi(z + 1, 0, J.Z - 1);
  for (int a = x0; a <= x1; ++a)
    for (int b = y0; b <= y1; ++b)
      for (int c = z0; c <= z1; ++c)
        if (J.grid[vf_gidx(J, a, b, c)] == VOXEL_EMPTY) return true;
  return false;
}

struct SeedSmem {
  unsigned long long acc[4096];
  unsigned long long cand[1024];
  uint16_t near_[4096];
  uint32_t idf[256];
  uint32_t cnt;
  uint32_t fail;
};

// returns false on SeederSearchError; out receives n xyzw entries
__device__ bool uniform_block(const JobDesc& J, SeedSmem& S, uint32_t n, uint64_t seed,
                              int location, uint32_t* out) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) { S.cnt = 0; S.fail = 0; }
  __syncthreads();
  const float fx = (float)(J.X - 1), fy = (float)(J.Y - 1), fz = (float)(J.Z - 1);
  for (uint32_t base = 0;; base += 1024) {
    if (S.cnt >= n || S.fail) break;
    if (base >= VF_MAX_TRIES) { if (t == 0) S.fail = 1; __syncthreads(); break; }
    const uint32_t a = base + t;
    unsigned long long key = ~0ull;
    if (a < VF_MAX_TRIES) {
      const int x = (int)__fmul_rn(fx, vf_u01(vf_hash(seed, VF_STREAM_SEEDS, 3ull * a + 0)));
      const int y = (int)__fmul_rn(fy, vf_u01(vf_hash(seed, VF_STREAM_SEEDS, 3ull * a + 1)));
      const int z = (int)__fmul_rn(fz, vf_u01(vf_hash(seed, VF_STREAM_SEEDS, 3ull * a + 2)));
      bool ok = occupied_at(J, x, y, z);
      if (ok && location != 2) ok = ((location == 1) == is_boundary(J, x, y, z));
      if (ok) key = ((unsigned long long)x << 24) | ((unsigned long long)y << 12) | (unsigned long long)z;
    }
    S.cand[t] = key;
    __syncthreads();
    if (warp == 0) {
      uint32_t cnt = S.cnt;
      for (int i = 0; i < 1024 && cnt < n; ++i) {
        const unsigned long long k = S.cand[i];
        if (k == ~0ull) continue;
        bool dup = false;
        for (uint32_t m = lane; m < cnt; m += 32) dup |= (S.acc[m] == k);
        dup = __any_sync(0xFFFFFFFFu, dup);
        if (!dup) {
          if (lane == 0) S.acc[cnt] = k;
          ++cnt;
        }
        __syncwarp();
      }
      if (lane == 0) S.cnt = cnt;
    }
    __syncthreads();
  }
  __syncthreads();
  if (S.fail || S.cnt < n) return false;
  // sort lexicographically (std::set<uvec3>), bitonic over the next power of 2
  uint32_t P = 1;
  while (P < n) P <<= 1;
  for (uint32_t i = n + t; i < P; i += blockDim.x) S.acc[i] = ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= P; k <<= 1)
    for (uint32_t jx = k >> 1; jx > 0; jx >>= 1) {
      for (uint32_t i = t; i < P; i += blockDim.x) {
        const uint32_t l = i ^ jx;
        if (l > i) {
          const unsigned long long a = S.acc[i], b = S.acc[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) { S.acc[i] = b; S.acc[l] = a; }
        }
      }
      __syncthreads();
    }
  for (uint32_t i = t; i < n; i += blockDim.x) {
    const unsigned long long k = S.acc[i];
    out[4 * i] = (uint32_t)(k >> 24);
    out[4 * i + 1] = (uint32_t)((k >> 12) & 0xFFF);
    out[4 * i + 2] = (uint32_t)(k & 0xFFF);
    out[4 * i + 3] = VOXEL_FREE + 1 + i;
  }
  __syncthreads();
  return true;
}

// Seeder::nearSeeds (vfnear::place) on the job's occupancy grid, after its nf
// main seeds in `seeds`: appends the placed seeds, labelled on from the last
// main seed; returns their count, or -1 when an impact runs out of candidates
struct JobGrid {
  const JobDesc& J;
  __device__ bool occupied(uint32_t x, uint32_t y, uint32_t z) const {
    return occupied_at(J, (int)x, (int)y, (int)z);
  }
  __device__ bool boundary(uint32_t x, uint32_t y, uint32_t z) const {
    return is_boundary(J, (int)x, (int)y, (int)z);
  }
};

__device__ int near_block(const JobDesc& J, SeedSmem& S, uint32_t* seeds, uint32_t nf) {
  return vfnear::place(JobGrid{J}, J.X, J.Y, J.Z, seeds, nf, (uint32_t)J.num_impacts,
                       (uint32_t)J.bias_seeds, (uint32_t)J.bias_focus, J.seed, seeds[4 * (nf - 1) + 3],
                       S.cand, S.acc, &S.cnt, seeds + 4 * (uint64_t)nf);
}

__device__ __forceinline__ float seed_dist(int dfunc, const uint32_t* s, const uint32_t* f) {
  const float dx = __fsub_rn((float)s[0], (float)f[0]), dy = __fsub_rn((float)s[1], (float)f[1]),
              dz = __fsub_rn((float)s[2], (float)f[2]);
  if (dfunc == 0)
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  if (dfunc == 1) return __fadd_rn(__fadd_rn(fabsf(dx), fabsf(dy)), fabsf(dz));
  return fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)));
}

__global__ void __launch_bounds__(1024) k_seeds(const JobDesc* jobs, JobState* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SeedSmem& S = *reinterpret_cast<SeedSmem*>(smem_raw);
  const JobDesc& J = jobs[blockIdx.x];
  JobState& js = st[blockIdx.x];
  const int t = threadIdx.x;
  if (!J.active) return;
  if (J.seeds_given) {
    if (t == 0) {
      js.nseeds = J.seeds_given;
      uint32_t hp = 0;
      for (uint32_t i = 0; i < J.seeds_given; ++i) hp |= J.seeds[4 * i + 3] > 0xFFu;
      js.has_prefix = hp;
    }
    return;
  }
  uint32_t nm = (uint32_t)J.num_seeds;
  const uint32_t ne = (uint32_t)J.num_extra;
  if (J.X < 2 || J.Y < 2 || J.Z < 2 || nm > 254 || 2 * nm + ne > J.seeds_cap) {
    if (t == 0) { js.err |= VF_JERR_INVALID; js.nseeds = 0; }
    return;
  }
  if (!uniform_block(J, S, nm, J.seed, J.seed_location, J.seeds)) {
    if (t == 0) { js.err |= VF_JERR_SEED_SEARCH; js.nseeds = 0; }
    return;
  }
  if (J.num_impacts > 0 && nm > 0 && J.bias_seeds > 0) {
    // CADScene.cpp:636-638: nearSeeds(seeds, numImpacts, biasSeeds, biasFocus)
    if (J.bias_focus < 1 || (uint32_t)J.bias_focus > min(J.X, min(J.Y, J.Z))) {
      if (t == 0) { js.err |= VF_JERR_INVALID; js.nseeds = 0; }
      return;
    }
    const int placed = near_block(J, S, J.seeds, nm);
    if (placed < 0) {
      if (t == 0) { js.err |= VF_JERR_SEED_SEARCH; js.nseeds = 0; }
      return;
    }
    nm += (uint32_t)placed;
    if (nm > 254) {  // 8-bit fragment ids 2..255
      if (t == 0) { js.err |= VF_JERR_RANGE; js.nseeds = 0; }
      return;
    }
  }
  uint32_t total = nm;
  if (ne > 0 && nm > 0) {
    // extraSeeds = uniform(BOTH) after a copy of the main seeds, merged
    // (CADScene.cpp:647-655); seed value seed + golden ratio
    uint32_t* list = J.seeds + 4 * (size_t)nm;
    for (uint32_t i = t; i < 4 * nm; i += blockDim.x) list[i] = J.seeds[i];
    __syncthreads();
    if (!uniform_block(J, S, ne, J.seed + 0x9E3779B97F4A7C15ull, 2, list + 4 * (size_t)nm)) {
      if (t == 0) { js.err |= VF_JERR_SEED_SEARCH; js.nseeds = 0; }
      return;
    }
    const uint32_t nl = nm + ne;
    for (uint32_t k = t; k < nl; k += blockDim.x) {
      float best = FLT_MAX;
      int nearest = 0;
      for (uint32_t i = 0; i < nm; ++i) {
        const float d = seed_dist(J.merge_distance, list + 4 * k, J.seeds + 4 * i);
        if (d < best) { best = d; nearest = (int)i; }
      }
      S.near_[k] = (uint16_t)nearest;
    }
    for (uint32_t i = t; i < 256; i += blockDim.x) S.idf[i] = 0;
    __syncthreads();
    if (t == 0) {
      for (uint32_t k = 0; k < nl; ++k) {
        const uint32_t w = J.seeds[4 * S.near_[k] + 3];
        const uint32_t pre = ++S.idf[w & 0xFFu];
        if (pre > 127) js.err |= VF_JERR_RANGE;
        list[4 * k + 3] = w | (pre << 8);
      }
    }
    total = 2 * nm + ne;
  }
  __syncthreads();
  if (t == 0) {
    js.nseeds = total;
    uint32_t hp = 0;
    for (uint32_t i = 0; i < total; ++i) hp |= J.seeds[4 * i + 3] > 0xFFu;
    js.has_prefix = hp;
  }
}

// ===========================================================================
// NaiveFracturer::buildCPU (NaiveFracturer.cpp:26-68): every occupied voxel
// takes the label of the nearest seed; strict '<' keeps the lowest index.
__global__ void __launch_bounds__(256) k_naive(const JobDesc* jobs, const JobState* st,
                                               const uint32_t* list, const uint32_t* count,
                                               const uint32_t* brick_job) {
  __shared__ uint4 sd[512];
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active) continue;
    const uint32_t ns = st[j].nseeds;
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    const uint32_t x = x0 + threadIdx.x / VF_BY, y = y0 + threadIdx.x % VF_BY;
    const bool row_ok = x < J.X && y < J.Y;
    uint16_t v[VF_BZ];
    float best[VF_BZ];
    if (row_ok) {
      const uint4* src = reinterpret_cast<const uint4*>(J.grid + vf_gidx(J, x, y, z0));
      const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);
#pragma unroll
      for (int q = 0; q < VF_BZ / 8; ++q) {
        uint4 w = (q * 8 < (int)nz) ? src[q] : make_uint4(0, 0, 0, 0);
        v[8 * q + 0] = w.x & 0xFFFF; v[8 * q + 1] = w.x >> 16;
        v[8 * q + 2] = w.y & 0xFFFF; v[8 * q + 3] = w.y >> 16;
        v[8 * q + 4] = w.z & 0xFFFF; v[8 * q + 5] = w.z >> 16;
        v[8 * q + 6] = w.w & 0xFFFF; v[8 * q + 7] = w.w >> 16;
      }
    }
#pragma unroll
    for (int z = 0; z < VF_BZ; ++z) best[z] = FLT_MAX;
    for (uint32_t c0 = 0; c0 < ns; c0 += 512) {
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < 512 && c0 + i < ns; i += blockDim.x)
        sd[i] = reinterpret_cast<const uint4*>(J.seeds)[c0 + i];
      __syncthreads();
      if (!row_ok) continue;
      const uint32_t cn = min(512u, ns - c0);
      for (uint32_t s = 0; s < cn; ++s) {
        const uint4 sp = sd[s];
        const int dx = (int)x - (int)sp.x, dy = (int)y - (int)sp.y;
#pragma unroll
        for (int z = 0; z < VF_BZ; ++z) {
          const int dz = (int)(z0 + z) - (int)sp.z;
          float d;
          if (J.distance == 0) {
            const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz)));
          } else if (J.distance == 1) {
            d = (float)(abs(dx) + abs(dy) + abs(dz));
          } else {
            d = (float)max(abs(dx), max(abs(dy), abs(dz)));
          }
          if (v[z] != VOXEL_EMPTY && d < best[z]) { best[z] = d; v[z] = (uint16_t)sp.w; }
        }
      }
    }
    if (row_ok) {
      // padding voxels stay 0 (they are EMPTY and never labelled)
      store_row(J, J.grid, x, y, z0, v);
    }
  }
}

// ===========================================================================
// Boundary perturbation (no reference counterpart).  Lattice values are
// precomputed per job; per voxel the 3-channel trilinear noise gives the
// offset of the voxel whose label is taken.  Reads src, writes dst.
__global__ void k_lattice(const JobDesc* jobs) {
  const JobDesc& J = jobs[blockIdx.y];
  if (!J.active) return;
  const uint32_t n = J.lat_nx * J.lat_ny * J.lat_nz * 3;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t c = i % 3, p = i / 3;
    const uint32_t iz = p % J.lat_nz, iy = (p / J.lat_nz) % J.lat_ny, ix = p / (J.lat_nz * J.lat_ny);
    const uint64_t ctr = (((uint64_t)ix << 40) | ((uint64_t)iy << 20) | iz) * 4u + c;
    J.lattice[i] = __fsub_rn(__fmul_rn(vf_u01(vf_hash(J.seed, VF_STREAM_NOISE, ctr)), 2.0f), 1.0f);
  }
}

__device__ __forceinline__ float lerp_(float a, float b, float t) {
  return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}

__global__ void __launch_bounds__(256) k_perturb(const JobDesc* jobs, const uint32_t* list,
                                                 const uint32_t* count, const uint32_t* brick_job) {
  // per brick: the lattice index and in-cell coordinate of its 16 x, 16 y
  // and 32 z values, t = (c mod P) / P rounded as the oracle divides
  __shared__ float t0s[VF_BX], t1s[VF_BY], t2s[VF_BZ];
  __shared__ uint32_t i0s[VF_BX], i1s[VF_BY], i2s[VF_BZ];
  // the thread's row of labels (34-u16 pitch: the u16 of one z from 32
  // threads falls on 32 distinct banks)
  __shared__ __align__(16) uint16_t vrows[256 * 34];
  // the brick's labelled voxels (row << 5 | z), dealt to all threads: the
  // labelled voxels of a thin wall are few and uneven per row
  __shared__ uint16_t vq[256 * VF_BZ];
  __shared__ uint32_t wq[8];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint16_t* v = vrows + t * 34;
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;  // uniform across the CTA
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    const uint32_t P = J.noise_period;
    const float fp = (float)P;
    __syncthreads();  // the previous brick is done with the tables, rows and queue
    if (t < VF_BZ) {
      const uint32_t gz = z0 + t;
      t2s[t] = __fdiv_rn((float)(gz % P), fp);
      i2s[t] = gz / P;
    } else if (t < VF_BZ + VF_BX) {
      const uint32_t gx = x0 + (t - VF_BZ);
      t0s[t - VF_BZ] = __fdiv_rn((float)(gx % P), fp);
      i0s[t - VF_BZ] = gx / P;
    } else if (t < VF_BZ + VF_BX + VF_BY) {
      const uint32_t gy = y0 + (t - VF_BZ - VF_BX);
      t1s[t - VF_BZ - VF_BX] = __fdiv_rn((float)(gy % P), fp);
      i1s[t - VF_BZ - VF_BX] = gy / P;
    }
    const uint32_t x = x0 + t / VF_BY, y = y0 + t % VF_BY;
    const bool rowok = x < J.X && y < J.Y;
    const uint16_t* src = J.grid;
    // the brick's label rows into shared memory, 4 lanes per row along z (a
    // warp instruction reads 8 whole 64-byte rows); chunks at or past Zp are
    // zero
    const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);
    {
      uint4 w[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t u = i * 256 + t, row = u >> 2, q = u & 3;
        const uint32_t xr = x0 + row / VF_BY, yr = y0 + row % VF_BY;
        w[i] = (xr < J.X && yr < J.Y && 8 * q < nz)
                   ? *reinterpret_cast<const uint4*>(src + vf_gidx(J, xr, yr, z0 + 8 * q))
                   : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t u = i * 256 + t, row = u >> 2, q = u & 3;
        // 4-byte aligned: 68-byte row pitch, 16-byte chunks
        uint32_t* d = reinterpret_cast<uint32_t*>(vrows + row * 34 + 8 * q);
        d[0] = w[i].x; d[1] = w[i].y; d[2] = w[i].z; d[3] = w[i].w;
      }
    }
    __syncthreads();
    uint32_t m = 0;  // labelled z of this row
    if (rowok) {
#pragma unroll
      for (int z = 0; z < VF_BZ; ++z) m |= (uint32_t)(v[z] > VOXEL_FREE) << z;
    }
    const uint32_t c = (uint32_t)__popc(m);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) wq[warp] = incl;
    __syncthreads();
    uint32_t base = incl - c, total = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      base += w < warp ? wq[w] : 0u;
      total += wq[w];
    }
    while (m) {
      const uint32_t z = (uint32_t)__ffs(m) - 1;
      m &= m - 1;
      vq[base++] = (uint16_t)((t << 5) | z);
    }
    __syncthreads();
    // Per labelled voxel: a 3-channel trilinear value noise n(v / P) from the
    // lattice (lerp along z, then y, then x, as the oracle), offset
    // floor(A * n + 0.5) per axis, and the label found there if it is labelled.
    const uint32_t sy = J.lat_nz * 3, sx = J.lat_ny * sy;
    const float amp = J.noise_amplitude;
    for (uint32_t i = t; i < total; i += blockDim.x) {
      const uint32_t e = vq[i], row = e >> 5, z = e & 31u;
      const uint32_t lx = row / VF_BY, ly = row % VF_BY;
      const uint32_t xr = x0 + lx, yr = y0 + ly, gz = z0 + z;
      const float t0 = t0s[lx], t1 = t1s[ly], t2 = t2s[z];
      const float* L = J.lattice + (size_t)i0s[lx] * sx + (size_t)i1s[ly] * sy + (size_t)i2s[z] * 3;
      int o[3];
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const float c00 = lerp_(L[ch], L[3 + ch], t2), c01 = lerp_(L[sy + ch], L[sy + 3 + ch], t2);
        const float c10 = lerp_(L[sx + ch], L[sx + 3 + ch], t2),
                    c11 = lerp_(L[sx + sy + ch], L[sx + sy + 3 + ch], t2);
        const float c0 = lerp_(c00, c01, t1), c1 = lerp_(c10, c11, t1);
        const float nzv = lerp_(c0, c1, t0);
        o[ch] = (int)floorf(__fadd_rn(__fmul_rn(amp, nzv), 0.5f));
      }
      const long ux = (long)xr + o[0], uy = (long)yr + o[1], uz = (long)gz + o[2];
      if (ux < 0 || uy < 0 || uz < 0 || ux >= (long)J.X || uy >= (long)J.Y || uz >= (long)J.Z) continue;
      const uint16_t u = src[vf_gidx(J, (uint32_t)ux, (uint32_t)uy, (uint32_t)uz)];
      if (u > VOXEL_FREE) vrows[row * 34 + z] = u;
    }
    __syncthreads();
    // rows back out as they came in, 4 lanes per row
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t u = i * 256 + t, row = u >> 2, q = u & 3;
      const uint32_t xr = x0 + row / VF_BY, yr = y0 + row % VF_BY;
      if (xr < J.X && yr < J.Y && 8 * q < nz) {
        const uint32_t* r32 = reinterpret_cast<const uint32_t*>(vrows + row * 34 + 8 * q);
        *reinterpret_cast<uint4*>(J.grid2 + vf_gidx(J, xr, yr, z0 + 8 * q)) =
            make_uint4(r32[0], r32[1], r32[2], r32[3]);
      }
    }
  }
}

// ===========================================================================
// detectBoundaries-comp.glsl:18-43 (in place; neighbour reads clear bit 15,
// so concurrent updates of neighbours cannot change the outcome).
template <int H>
__global__ void __launch_bounds__(256) k_detect(const JobDesc* jobs, const uint32_t* list,
                                                const uint32_t* count, const uint32_t* brick_job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t* tile = reinterpret_cast<uint16_t*>(smem_raw);
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;  // uniform across the CTA
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    __syncthreads();
    load_tile<H>(J, J.grid, x0, y0, z0, tile);
    __syncthreads();
    const int lx = threadIdx.x / VF_BY, ly = threadIdx.x % VF_BY;
    const uint32_t x = x0 + lx, y = y0 + ly;
    if (x >= J.X || y >= J.Y) continue;
    const int bs = J.boundary_size;
    uint16_t v[VF_BZ];
    bool any = false;
    for (int z = 0; z < VF_BZ; ++z) {
      const uint16_t g = tval<H>(tile, lx, ly, z);
      v[z] = g;
      const int gz = (int)z0 + z;
      if (g <= VOXEL_FREE || gz >= (int)J.Z) continue;
      const int xa = max((int)x - bs, 0) - (int)x0, xb = min((int)x + bs, (int)J.X - 1) - (int)x0;
      const int ya = max((int)y - bs, 0) - (int)y0, yb = min((int)y + bs, (int)J.Y - 1) - (int)y0;
      const int za = max(gz - bs, 0) - (int)z0, zb = min(gz + bs, (int)J.Z - 1) - (int)z0;
      bool bd = false;
      for (int a = xa; a <= xb && !bd; ++a)
        for (int c = ya; c <= yb && !bd; ++c)
          for (int d = za; d <= zb && !bd; ++d) {
            const uint16_t u = tval<H>(tile, a, c, d) & 0x7FFFu;
            bd = u > VOXEL_FREE && u != g;
          }
      if (bd) { v[z] = g | 0x8000u; any = true; }
    }
    if (any) store_row(J, J.grid, x, y, z0, v);
  }
}

// detectBoundaries with boundary size <= 1, by window extrema.  Over the
// labelled voxels of the clamped 3x3x3 window (masked value u = w & 0x7FFF,
// labelled when u > 1; voxels outside the grid or the live bricks are 0),
// let mn / mx be the smallest / largest u.  A voxel g > 1 is a boundary in
// the reference's test (some labelled u != g) exactly when a labelled voxel
// exists and not all of them equal g: mn != none and (mn != g or mx != g).
// The window extrema are separable: phase 1 takes the z-window of every
// staged row (brick + 1-voxel halo) into two u16x2 planes, phase 2 the 3x3
// rows around each brick row, both with paired 16-bit min/max.
constexpr int D1_ROWS = (VF_BX + 2) * (VF_BY + 2);
constexpr int D1_W = VF_BZ / 2;  // u16 pairs per row
constexpr int D1_BYTES = Tile<1>::BYTES + 2 * D1_ROWS * D1_W * 4;
// 16-byte chunk c of window row r is stored at chunk c ^ ((r >> 1) & 3): the
// chunk-q loads of any 8 consecutive rows then fall on 8 distinct bank groups
__device__ __forceinline__ int d1_swz(int r, int c) { return c ^ ((r >> 1) & 3); }

__global__ void __launch_bounds__(256, 3) k_detect1(const JobDesc* jobs, const uint32_t* list,
                                                 const uint32_t* count, const uint32_t* brick_job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t* tile = reinterpret_cast<uint16_t*>(smem_raw);
  uint32_t* zmin = reinterpret_cast<uint32_t*>(smem_raw + Tile<1>::BYTES);
  uint32_t* zmax = zmin + D1_ROWS * D1_W;
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;  // uniform across the CTA
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    __syncthreads();
    load_tile<1>(J, J.grid, x0, y0, z0, tile);
    __syncthreads();
    const bool self_only = J.boundary_size <= 0;  // uniform across the CTA
    if (!self_only) {
      // phase 1: z-window extrema of every staged row.  A thread takes a
      // quarter row (4 u32 words = u16 pairs p = 4c .. 4c + 3) and the words
      // either side of it.  The window of pair p is (2p-1, 2p), (2p, 2p+1)
      // and (2p+1, 2p+2); labelled halves keep u = w & 0x7FFF, the others
      // become 0xFFFF (min) / 0 (max).  The masks act on each 16-bit half
      // alone, so they are taken once per word and the shifted windows are
      // byte permutes of the masked words.
      auto lo = [](uint32_t w) {
        const uint32_t u = w & 0x7FFF7FFFu;
        return u | ~__vcmpgtu2(u, 0x00010001u);
      };
      auto hi = [](uint32_t w) {
        const uint32_t u = w & 0x7FFF7FFFu;
        return u & __vcmpgtu2(u, 0x00010001u);
      };
      for (int i = threadIdx.x; i < D1_ROWS * 4; i += blockDim.x) {
        const int r = i >> 2, c = i & 3;
        const uint32_t* rw = reinterpret_cast<const uint32_t*>(tile + r * ZW + 8) + 4 * c;
        const uint4 m = *reinterpret_cast<const uint4*>(rw);
        const uint32_t w[6] = {rw[-1], m.x, m.y, m.z, m.w, rw[4]};
        uint32_t L[6], H[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) { L[k] = lo(w[k]); H[k] = hi(w[k]); }
        uint32_t mn[4], mx[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          mn[k] = __vminu2(__vminu2(__byte_perm(L[k], L[k + 1], 0x5432), L[k + 1]),
                           __byte_perm(L[k + 1], L[k + 2], 0x5432));
          mx[k] = __vmaxu2(__vmaxu2(__byte_perm(H[k], H[k + 1], 0x5432), H[k + 1]),
                           __byte_perm(H[k + 1], H[k + 2], 0x5432));
        }
        const int o = r * D1_W + (d1_swz(r, c) << 2);
        *reinterpret_cast<uint4*>(zmin + o) = make_uint4(mn[0], mn[1], mn[2], mn[3]);
        *reinterpret_cast<uint4*>(zmax + o) = make_uint4(mx[0], mx[1], mx[2], mx[3]);
      }
      __syncthreads();
    }
    const int lx = threadIdx.x / VF_BY, ly = threadIdx.x % VF_BY;
    const uint32_t x = x0 + lx, y = y0 + ly;
    if (x >= J.X || y >= J.Y) continue;
    const uint16_t* own = tile + ((lx + 1) * Tile<1>::NY + (ly + 1)) * ZW + 8;
    // rows are written 8 voxels (16 bytes) at a time, and only where a voxel
    // was marked; z >= Zp is outside the row
    uint4* dst = reinterpret_cast<uint4*>(J.grid + vf_gidx(J, x, y, z0));
    const uint32_t nq = min((uint32_t)VF_BZ, J.Zp - z0) / 8;
#pragma unroll 1
    for (uint32_t q = 0; q < nq; ++q) {
      uint32_t out[4];
      bool any = false;
      // the row's 8 voxels of this chunk, one 16-byte load
      const uint4 gq = *reinterpret_cast<const uint4*>(own + 8 * q);
      const uint32_t gw[4] = {gq.x, gq.y, gq.z, gq.w};
      if (self_only) {
        // the window is the voxel itself: only a marked voxel can differ from
        // its own masked value
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const uint16_t g = (uint16_t)(gw[h >> 1] >> (16 * (h & 1)));
          const uint32_t u = g & 0x7FFFu;
          const bool bd = g > VOXEL_FREE && u > VOXEL_FREE && u != g;
          const uint32_t o = bd ? (uint32_t)(g | 0x8000u) : (uint32_t)g;
          if (h & 1) out[h >> 1] |= o << 16; else out[h >> 1] = o;
          any |= bd;
        }
      } else {
        // phase 2: the 3x3 rows around this row
        uint4 mn = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
        uint4 mx = make_uint4(0, 0, 0, 0);
#pragma unroll 3
        for (int r = 0; r < 9; ++r) {
          const int row = (lx + r / 3) * Tile<1>::NY + (ly + r % 3);
          const uint4 a = reinterpret_cast<const uint4*>(zmin + row * D1_W)[d1_swz(row, q)];
          const uint4 c = reinterpret_cast<const uint4*>(zmax + row * D1_W)[d1_swz(row, q)];
          mn.x = __vminu2(mn.x, a.x); mn.y = __vminu2(mn.y, a.y);
          mn.z = __vminu2(mn.z, a.z); mn.w = __vminu2(mn.w, a.w);
          mx.x = __vmaxu2(mx.x, c.x); mx.y = __vmaxu2(mx.y, c.y);
          mx.z = __vmaxu2(mx.z, c.z); mx.w = __vmaxu2(mx.w, c.w);
        }
        // per 16-bit half: marked when g > FREE, some labelled voxel is in
        // the window (min != 0xFFFF) and the window is not uniformly g
        const uint32_t mns[4] = {mn.x, mn.y, mn.z, mn.w}, mxs[4] = {mx.x, mx.y, mx.z, mx.w};
        uint32_t marked = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint32_t bd = __vcmpgtu2(gw[k], 0x00010001u) & __vcmpne2(mns[k], 0xFFFFFFFFu) &
                              (__vcmpne2(mns[k], gw[k]) | __vcmpne2(mxs[k], gw[k]));
          out[k] = gw[k] | (bd & 0x80008000u);
          marked |= bd;
        }
        any = marked != 0;
      }
      if (any) dst[q] = make_uint4(out[0], out[1], out[2], out[3]);
    }
  }
}

// erodeGrid-comp.glsl:26-59: src -> dst.  Gate bool(unmaskedBit(v,15)) holds
// for every labelled voxel; full 16-bit equality; globalCount = clamped
// window size; noise[idx % 1e6] from the counter RNG.
template <int H>
__global__ void __launch_bounds__(256) k_erode(const JobDesc* jobs, const uint32_t* list,
                                               const uint32_t* count, const uint32_t* brick_job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t* tile = reinterpret_cast<uint16_t*>(smem_raw);
  float* mask = reinterpret_cast<float*>(smem_raw + Tile<H>::BYTES);
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    const int k = J.ek, m2 = k / 2;
    __syncthreads();
    load_tile<H>(J, J.grid, x0, y0, z0, tile);
    for (int i = threadIdx.x; i < k * k * k; i += blockDim.x) mask[i] = J.emask[i];
    __syncthreads();
    const int lx = threadIdx.x / VF_BY, ly = threadIdx.x % VF_BY;
    const uint32_t x = x0 + lx, y = y0 + ly;
    if (x >= J.X || y >= J.Y) continue;
    uint16_t v[VF_BZ];
    const unsigned long long rowlin = ((unsigned long long)x * J.Y + y) * J.Z;
    for (int z = 0; z < VF_BZ; ++z) {
      const uint16_t g = tval<H>(tile, lx, ly, z);
      v[z] = g;
      const int gz = (int)z0 + z;
      if (gz >= (int)J.Z) continue;
      if (!(g > VOXEL_FREE && (g & 0x7FFFu) != 0)) continue;
      const uint32_t nidx = (uint32_t)((rowlin + gz) % VF_NOISE_BUFFER);
      if (!(vf_u01(vf_hash(J.seed, VF_STREAM_ERODE, nidx)) < J.erosion_probability)) continue;
      const int mnx = (int)x - m2, mny = (int)y - m2, mnz = gz - m2;
      const int xa = max(mnx, 0), xb = min((int)x + m2, (int)J.X - 1);
      const int ya = max(mny, 0), yb = min((int)y + m2, (int)J.Y - 1);
      const int za = max(mnz, 0), zb = min(gz + m2, (int)J.Z - 1);
      uint32_t cnt = 0, global = 0;
      for (int a = xa; a <= xb; ++a)
        for (int c = ya; c <= yb; ++c)
          for (int d = za; d <= zb; ++d) {
            const float m = mask[(a - mnx) * k * k + (c - mny) * k + (d - mnz)];
            const float eq = (float)(tval<H>(tile, a - (int)x0, c - (int)y0, d - (int)z0) == g);
            cnt += (uint32_t)__fmul_rn(eq, m);
            ++global;
          }
      const float act = __fdiv_rn((float)cnt, (float)global);
      if (act < J.elimit) v[z] = VOXEL_EMPTY;
    }
    store_row(J, J.grid2, x, y, z0, v);
  }
}

// removeIsolatedRegionsGrid-comp.glsl:16-39, src -> dst (Jacobi)
__global__ void __launch_bounds__(256) k_isolated(const JobDesc* jobs, const uint32_t* list,
                                                  const uint32_t* count, const uint32_t* brick_job) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t* tile = reinterpret_cast<uint16_t*>(smem_raw);
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    __syncthreads();
    load_tile<1>(J, J.grid, x0, y0, z0, tile);
    __syncthreads();
    const int lx = threadIdx.x / VF_BY, ly = threadIdx.x % VF_BY;
    const uint32_t x = x0 + lx, y = y0 + ly;
    if (x >= J.X || y >= J.Y) continue;
    uint16_t v[VF_BZ];
    const int xa = ((int)x > 0 ? -1 : 0) + lx, xb = ((int)x + 1 < (int)J.X ? 1 : 0) + lx;
    const int ya = ((int)y > 0 ? -1 : 0) + ly, yb = ((int)y + 1 < (int)J.Y ? 1 : 0) + ly;
    for (int z = 0; z < VF_BZ; ++z) {
      const uint16_t g = tval<1>(tile, lx, ly, z);
      v[z] = g;
      const int gz = (int)z0 + z;
      if (gz >= (int)J.Z || g == VOXEL_EMPTY) continue;  // EMPTY stays EMPTY
      const int za = (gz > 0 ? -1 : 0) + z, zb = (gz + 1 < (int)J.Z ? 1 : 0) + z;
      int c = -1;
      for (int a = xa; a <= xb; ++a)
        for (int q = ya; q <= yb; ++q)
          for (int d = za; d <= zb; ++d) c += tval<1>(tile, a, q, d) == g;
      if (c < 6) v[z] = VOXEL_EMPTY;
    }
    store_row(J, J.grid2, x, y, z0, v);
  }
}

// RegularGrid::countValues (RegularGrid.cpp:601-625)
__global__ void __launch_bounds__(256) k_counts(const JobDesc* jobs, JobState* st,
                                                const uint32_t* list, const uint32_t* count,
                                                const uint32_t* brick_job) {
  __shared__ uint32_t hist[256];
  __shared__ unsigned long long occ;
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active) continue;
    uint32_t x0, y0, z0;
    brick_coords(J, b, x0, y0, z0);
    __syncthreads();
    hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) occ = 0;
    __syncthreads();
    // four lanes per row, each 16 bytes (8 voxels) of the row's 64: a warp
    // reads 8 rows as contiguous segments; 4 passes cover the brick's 256 rows
    uint32_t mine = 0, err = 0;
    const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);
    const uint32_t part = threadIdx.x & 3u;
    uint4 wv[4];
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) {
      const uint32_t row = (threadIdx.x >> 2) + 64u * pass;
      const uint32_t x = x0 + row / VF_BY, y = y0 + row % VF_BY;
      wv[pass] = make_uint4(0, 0, 0, 0);
      if (x < J.X && y < J.Y && 8u * part < nz)
        wv[pass] = *reinterpret_cast<const uint4*>(J.grid + vf_gidx(J, x, y, z0 + 8u * part));
    }
#pragma unroll
    for (int pass = 0; pass < 4; ++pass) {
      const uint32_t ww[4] = {wv[pass].x, wv[pass].y, wv[pass].z, wv[pass].w};
#pragma unroll
      for (int h = 0; h < 8; ++h) {
        const uint32_t g = (ww[h >> 1] >> (16 * (h & 1))) & 0xFFFFu;
        if (g > VOXEL_FREE) {
          const uint32_t val = g & 0x7FFFu;
          ++mine;
          if (val < 256) atomicAdd(&hist[val], 1u);
          else if (val < J.ncounts) atomicAdd(&J.counts[val], 1u);
          else err = 1;
        }
      }
    }
    if (mine) atomicAdd(&occ, (unsigned long long)mine);
    if (err) atomicOr(&st[j].err, VF_JERR_RANGE);
    __syncthreads();
    const uint32_t h = hist[threadIdx.x];
    if (h) {
      if (threadIdx.x < J.ncounts) atomicAdd(&J.counts[threadIdx.x], h);
      else atomicOr(&st[j].err, VF_JERR_RANGE);
    }
    if (threadIdx.x == 0 && occ) atomicAdd(&st[j].occupied, occ);
  }
}


// ---------------------------------------------------------------------------
// label download, 16-byte path (Z % 4 == 0, destination 16-byte aligned):
// the job's output is a flat array of X*Y*Z labels written in 16-byte units
// (8 labels); each unit is two 8-byte halves, and a half never crosses a row
// (Z % 4 == 0), so it is one 8-byte load from row (e / Z) at z = e % Z.  Units
// go to consecutive lanes, so every warp store is 512 contiguous bytes.
// Labels into a caller's buffer the GPU writes directly (mapped pinned host
// memory): 16-byte units that may straddle rows (Z a multiple of 4), one
// 32-bit division per unit.
__global__ void __launch_bounds__(256) k_pack16(const JobDesc* jobs, int njobs) {
  for (int j = blockIdx.y; j < njobs; j += gridDim.y) {
    const JobDesc& J = jobs[j];
    if (!J.out || J.out_dma || (J.Z & 3u) || (reinterpret_cast<uintptr_t>(J.out) & 15u)) continue;
    const unsigned long long total = (unsigned long long)J.X * J.Y * J.Z;
    const unsigned long long units = total / 8;
    uint4* d = reinterpret_cast<uint4*>(J.out);
    const uint32_t Z = J.Z;
    if (total < (1ull << 32)) {
      // one 32-bit division per unit; the second half's row follows from the first
      for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < (uint32_t)units;
           u += gridDim.x * blockDim.x) {
        const uint32_t e0 = 8 * u;
        const uint32_t r0 = e0 / Z, o0 = e0 - r0 * Z;
        const uint32_t r1 = o0 + 4 < Z ? r0 : r0 + 1, o1 = o0 + 4 < Z ? o0 + 4 : o0 + 4 - Z;
        const uint2 a = *reinterpret_cast<const uint2*>(J.grid + (size_t)r0 * J.Zp + o0);
        const uint2 b = *reinterpret_cast<const uint2*>(J.grid + (size_t)r1 * J.Zp + o1);
        d[u] = make_uint4(a.x, a.y, b.x, b.y);
      }
    } else {
      for (unsigned long long u = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; u < units;
           u += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long e0 = 8 * u, e1 = e0 + 4;
        const unsigned long long r0 = e0 / Z, r1 = e1 / Z;
        const uint2 a = *reinterpret_cast<const uint2*>(J.grid + r0 * J.Zp + (e0 - r0 * Z));
        const uint2 b = *reinterpret_cast<const uint2*>(J.grid + r1 * J.Zp + (e1 - r1 * Z));
        d[u] = make_uint4(a.x, a.y, b.x, b.y);
      }
    }
    // the last total % 8 labels (a multiple of 4)
    if (blockIdx.x == 0 && threadIdx.x == 0 && (total & 7u)) {
      const unsigned long long e = total - 4, r = e / J.Z;
      *reinterpret_cast<uint2*>(J.out + e) = *reinterpret_cast<const uint2*>(J.grid + r * J.Zp + (e - r * J.Z));
    }
  }
}

// label download: one warp per (x, y) row, the final grid (row pitch Zp) into
// the caller's buffer (row pitch Z); 8-byte stores when Z % 4 == 0 and the
// destination is 8-byte aligned
// Labels without the z padding into J.out (a device staging buffer, or a
// caller's buffer k_pack16 does not take): one warp per (x, y) row of any job (rows of all jobs are
// numbered consecutively, row_base per job), copied with the widest access
// the row's alignment allows.
// Packs each row's labels (z padded to Zp) into the job's staging buffer
// (J.out, Z per row).  A warp takes 4 consecutive rows of the batch, 8 lanes
// per row (rows are 64..384 labels: 8..48 16-byte units), so a warp has four
// rows' loads in flight.  A warp's rows only increase, so its job is found by
// walking forward from the previous one.
__global__ void __launch_bounds__(256) k_pack(const JobDesc* jobs, int njobs,
                                              unsigned long long total_rows) {
  const int lane = threadIdx.x & 31, sub = lane & 7;
  const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  int j = 0;
  for (unsigned long long r0 = (((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 4;
       r0 < total_rows; r0 += nw * 4) {
    const unsigned long long r = r0 + (lane >> 3);
    if (r >= total_rows) continue;
    while (j + 1 < njobs && jobs[j + 1].row_base <= r) ++j;
    const JobDesc& J = jobs[j];
    if (!J.out) continue;
    if (!J.out_dma && (J.Z & 3u) == 0u && (reinterpret_cast<uintptr_t>(J.out) & 15u) == 0u) continue;  // k_pack16
    const unsigned long long lr = r - J.row_base;
    const uint16_t* src = J.grid + lr * J.Zp;  // 16-byte aligned (Zp is a multiple of 8)
    uint16_t* dst = J.out + lr * J.Z;
    const uintptr_t da = reinterpret_cast<uintptr_t>(dst);
    const uint32_t Z = J.Z;
    if ((Z & 7u) == 0u && (da & 15u) == 0u) {
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      uint4* d4 = reinterpret_cast<uint4*>(dst);
#pragma unroll 2
      for (uint32_t q = sub; q < Z / 8; q += 8) d4[q] = __ldcs(s4 + q);
    } else if ((Z & 3u) == 0u && (da & 7u) == 0u) {
      const uint2* s2 = reinterpret_cast<const uint2*>(src);
      uint2* d2 = reinterpret_cast<uint2*>(dst);
      for (uint32_t q = sub; q < Z / 4; q += 8) d2[q] = __ldcs(s2 + q);
    } else if ((Z & 1u) == 0u && (da & 3u) == 0u) {
      const uint32_t* s1 = reinterpret_cast<const uint32_t*>(src);
      uint32_t* d1 = reinterpret_cast<uint32_t*>(dst);
      for (uint32_t q = sub; q < Z / 2; q += 8) d1[q] = __ldcs(s1 + q);
    } else {
      for (uint32_t q = sub; q < Z; q += 8) dst[q] = src[q];
    }
  }
}
}  // namespace

namespace vfk {

static inline int brick_grid(uint32_t max_count) {
  uint32_t g = max_count ? max_count : 1;
  return (int)(g > (1u << 20) ? (1u << 20) : g);
}

void sample_seeds(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs) {
  static bool attr[64] = {};  // per device
  const int dv = cur_dev();
  if (!attr[dv]) {
    cudaFuncSetAttribute(k_seeds, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SeedSmem));
    attr[dv] = true;
  }
  if (njobs > 0) k_seeds<<<njobs, 1024, sizeof(SeedSmem), st>>>(dj, ds);
}

void naive(cudaStream_t st, const JobDesc* dj, const JobState* ds, const uint32_t* list,
           const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  if (max_count) k_naive<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job);
}

void lattice(cudaStream_t st, const JobDesc* dj, int njobs) {
  if (njobs > 0) k_lattice<<<dim3(64, njobs), 256, 0, st>>>(dj);
}
void perturb(cudaStream_t st, const JobDesc* dj, const uint32_t* list, const uint32_t* count,
             uint32_t max_count, const uint32_t* brick_job) {
  if (max_count) k_perturb<<<brick_grid(max_count), 256, 0, st>>>(dj, list, count, brick_job);
}

template <int H>
static void detect_h(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                     const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  static bool attr[64] = {};  // per device
  const int dv = cur_dev();
  if (!attr[dv]) {
    cudaFuncSetAttribute(k_detect<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, Tile<H>::BYTES);
    attr[dv] = true;
  }
  k_detect<H><<<brick_grid(max_count), 256, Tile<H>::BYTES, st>>>(dj, list, count, brick_job);
}
void detect_boundaries(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                       const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  // boundary sizes 0..1 (the default): window extrema; 2..3: detect_boundaries_wide
  if (!max_count) return;
  static bool attr[64] = {};  // per device
  const int dv = cur_dev();
  if (!attr[dv]) {
    cudaFuncSetAttribute(k_detect1, cudaFuncAttributeMaxDynamicSharedMemorySize, D1_BYTES);
    attr[dv] = true;
  }
  k_detect1<<<brick_grid(max_count), 256, D1_BYTES, st>>>(dj, list, count, brick_job);
}
void detect_boundaries_wide(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                            const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  if (!max_count) return;
  detect_h<3>(st, dj, list, count, max_count, brick_job);
}

template <int H>
static void erode_h(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                    const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  static bool attr[64] = {};  // per device
  const int dv = cur_dev();
  const int bytes = Tile<H>::BYTES + 343 * 4;
  if (!attr[dv]) {
    cudaFuncSetAttribute(k_erode<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    attr[dv] = true;
  }
  k_erode<H><<<brick_grid(max_count), 256, bytes, st>>>(dj, list, count, brick_job);
}
void erode(cudaStream_t st, const JobDesc* dj, const uint32_t* list, const uint32_t* count,
           uint32_t max_count, const uint32_t* brick_job) {
  if (!max_count) return;
  erode_h<3>(st, dj, list, count, max_count, brick_job);
}
void remove_isolated(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                     const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  static bool attr[64] = {};  // per device
  const int dv = cur_dev();
  if (!attr[dv]) {
    cudaFuncSetAttribute(k_isolated, cudaFuncAttributeMaxDynamicSharedMemorySize, Tile<1>::BYTES);
    attr[dv] = true;
  }
  if (max_count)
    k_isolated<<<brick_grid(max_count), 256, Tile<1>::BYTES, st>>>(dj, list, count, brick_job);
}
void count_values(cudaStream_t st, const JobDesc* dj, JobState* ds, const uint32_t* list,
                  const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  if (max_count) k_counts<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job);
}

void pack_labels(cudaStream_t st, const JobDesc* dj, int njobs, uint64_t total_rows, int num_sms) {
  if (njobs <= 0 || !total_rows) return;
  const int per_job = std::max(1, num_sms * 8 / njobs);
  k_pack16<<<dim3(per_job, std::min(njobs, 65535)), 256, 0, st>>>(dj, njobs);
  k_pack<<<num_sms * 8, 256, 0, st>>>(dj, njobs, (unsigned long long)total_rows);
}

}  // namespace vfk
