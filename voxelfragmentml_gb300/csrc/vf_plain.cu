// vf_plain.cu -- reference-shaped GPU path for one job at a time.
//
// Same shape as the reference's GL compute path (ComputeShader.cpp:96-99,
// FloodFracturer.cpp:143-158): one thread per voxel over the whole grid for
// every grid pass, and the flood as one launch per BFS wave over a frontier
// stack of voxel indices with a host read of the next stack size after every
// wave.  Claims are deterministic (atomicMax on the flood key, so the lowest
// seed index wins a same-wave tie) and the results equal the brick path's.
// This path is the "plain per-instance" comparator of the benchmarks and a
// second, independent GPU implementation for the parity tests.
#include "vf_kernels.h"

#include <cfloat>

namespace {

__device__ __forceinline__ bool voxel_of(const JobDesc& J, uint64_t i, uint32_t& x, uint32_t& y,
                                         uint32_t& z) {
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  if (i >= N) return false;
  z = (uint32_t)(i % J.Z);
  y = (uint32_t)((i / J.Z) % J.Y);
  x = (uint32_t)(i / ((uint64_t)J.Z * J.Y));
  return true;
}

__global__ void kp_init_keys(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const uint64_t n = (uint64_t)J.X * J.Y * J.Zk;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t z = (uint32_t)(i % J.Zk);
    const uint64_t row = i / J.Zk;
    uint32_t k = 0;
    if (z < J.Z) k = J.grid[row * J.Zp + z] ? VF_KEY_UNREACHED : VF_KEY_WALL;
    J.keys[i] = k;
  }
}

__global__ void kp_seed(const JobDesc* jobs, JobState* st, uint32_t* frontier, uint32_t* fcount) {
  const JobDesc& J = jobs[0];
  JobState& s = st[0];
  for (int f = 0; f < 256; ++f) s.minprefix[f] = 0xFFFFFFFFu;
  s.passes = 0;
  s.disjoint = 0;
  uint32_t n = 0;
  for (uint32_t i = 0; i < s.nseeds; ++i) {
    const uint32_t x = J.seeds[4 * i], y = J.seeds[4 * i + 1], z = J.seeds[4 * i + 2],
                   w = J.seeds[4 * i + 3];
    // label = frag | prefix << 8 (Seeder.cpp:150), fragment id >= 2
    if (x >= J.X || y >= J.Y || z >= J.Z || w > 0x7FFFu || (w & 0xFFu) <= VOXEL_FREE) {
      s.err |= VF_JERR_INVALID;
      continue;
    }
    J.keys[vf_kidx(J, x, y, z)] = ~i;
    frontier[n++] = (x * J.Y + y) * J.Z + z;  // RegularGrid::getPositionIndex
  }
  *fcount = n;
}

// floodFracturer-comp.glsl:24-64 shape: thread = (frontier entry, offset)
__global__ void kp_wave(const JobDesc* jobs, JobState* st, const uint32_t* cur, uint32_t ncur,
                        uint32_t* next, uint32_t* ncount) {
  const JobDesc& J = jobs[0];
  const int nn = J.distance == 1 ? 6 : 26;
  const uint64_t total = (uint64_t)ncur * nn;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t f = cur[i / nn];
    int o = (int)(i % nn);
    int dx, dy, dz;
    if (nn == 6) {
      const int t6[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
      dx = t6[o][0]; dy = t6[o][1]; dz = t6[o][2];
    } else {
      if (o >= 13) ++o;  // skip the centre
      dx = o / 9 - 1; dy = (o / 3) % 3 - 1; dz = o % 3 - 1;
    }
    const uint32_t fz = f % J.Z, fy = (f / J.Z) % J.Y, fx = f / (J.Z * J.Y);
    const int x = (int)fx + dx, y = (int)fy + dy, z = (int)fz + dz;
    if (x < 0 || y < 0 || z < 0 || x >= (int)J.X || y >= (int)J.Y || z >= (int)J.Z) continue;
    const uint32_t kf = *(volatile uint32_t*)(J.keys + vf_kidx(J, fx, fy, fz));
    if (kf < 2u * VF_KEY_STEP) {
      if (kf >= VF_KEY_MIN_REACHED) atomicOr(&st[0].err, VF_JERR_DIST_OVERFLOW);
      continue;
    }
    const uint32_t cand = kf - VF_KEY_STEP;
    uint32_t* kn = J.keys + vf_kidx(J, x, y, z);
    const uint32_t cur_k = *(volatile uint32_t*)kn;
    if (cur_k == VF_KEY_WALL || cur_k >= cand) continue;
    const uint32_t old = atomicMax(kn, cand);
    if (old == VF_KEY_UNREACHED) next[atomicAdd(ncount, 1u)] = ((uint32_t)x * J.Y + y) * J.Z + z;
  }
}

__global__ void kp_finalize(const JobDesc* jobs, const JobState* st, int pass2) {
  const JobDesc& J = jobs[0];
  const JobState& s = st[0];
  const bool keep_prefix = !pass2 && s.has_prefix;
  const uint64_t n = (uint64_t)J.X * J.Y * J.Zp;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t z = (uint32_t)(i % J.Zp);
    const uint64_t row = i / J.Zp;
    uint32_t v = 0;
    if (z < J.Z) {
      const uint32_t key = J.keys[row * J.Zk + z];
      if (key >= VF_KEY_MIN_REACHED) {
        const uint32_t slot = (~key) & 0xFFFu;
        v = pass2 ? s.rank_value[slot] : J.seeds[4 * slot + 3];
        if (!keep_prefix) v &= 0xFFu;
      } else {
        v = key;
      }
    }
    J.grid[i] = (uint16_t)v;
  }
}

// detectBoundaries-comp.glsl:18-43, one thread per voxel, in place
__global__ void kp_detect(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const int b = J.boundary_size;
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    uint16_t* gp = J.grid + vf_gidx(J, x, y, z);
    const uint16_t g = *gp;
    if (g <= VOXEL_FREE) continue;
    const int x0 = vf_clampi((int)x - b, 0, J.X - 1), x1 = vf_clampi((int)x + b, 0, J.X - 1);
    const int y0 = vf_clampi((int)y - b, 0, J.Y - 1), y1 = vf_clampi((int)y + b, 0, J.Y - 1);
    const int z0 = vf_clampi((int)z - b, 0, J.Z - 1), z1 = vf_clampi((int)z + b, 0, J.Z - 1);
    bool bd = false;
    for (int a = x0; a <= x1 && !bd; ++a)
      for (int c = y0; c <= y1 && !bd; ++c)
        for (int d = z0; d <= z1 && !bd; ++d) {
          const uint16_t u = *(volatile uint16_t*)(J.grid + vf_gidx(J, a, c, d)) & 0x7FFFu;
          bd = u > VOXEL_FREE && u != g;
        }
    if (bd) *gp = g | 0x8000u;
  }
}

// erodeGrid-comp.glsl:26-59, grid -> grid2
__global__ void kp_erode(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const int k = J.ek, m2 = k / 2;
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    const uint16_t g = J.grid[vf_gidx(J, x, y, z)];
    uint16_t out = g;
    if (g > VOXEL_FREE && (g & 0x7FFFu) != 0 &&
        vf_u01(vf_hash(J.seed, VF_STREAM_ERODE, (uint32_t)(i % VF_NOISE_BUFFER))) < J.erosion_probability) {
      const int mnx = (int)x - m2, mny = (int)y - m2, mnz = (int)z - m2;
      const int xa = max(mnx, 0), xb = min((int)x + m2, (int)J.X - 1);
      const int ya = max(mny, 0), yb = min((int)y + m2, (int)J.Y - 1);
      const int za = max(mnz, 0), zb = min((int)z + m2, (int)J.Z - 1);
      uint32_t cnt = 0, global = 0;
      for (int a = xa; a <= xb; ++a)
        for (int c = ya; c <= yb; ++c)
          for (int d = za; d <= zb; ++d) {
            const float m = J.emask[(a - mnx) * k * k + (c - mny) * k + (d - mnz)];
            cnt += (uint32_t)__fmul_rn((float)(J.grid[vf_gidx(J, a, c, d)] == g), m);
            ++global;
          }
      if (__fdiv_rn((float)cnt, (float)global) < J.elimit) out = VOXEL_EMPTY;
    }
    J.grid2[vf_gidx(J, x, y, z)] = out;
  }
}

// removeIsolatedRegionsGrid-comp.glsl:16-39, grid -> grid2 (Jacobi)
__global__ void kp_isolated(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    const uint16_t g = J.grid[vf_gidx(J, x, y, z)];
    int c = -1;
    for (int a = max((int)x - 1, 0); a <= min((int)x + 1, (int)J.X - 1); ++a)
      for (int b = max((int)y - 1, 0); b <= min((int)y + 1, (int)J.Y - 1); ++b)
        for (int d = max((int)z - 1, 0); d <= min((int)z + 1, (int)J.Z - 1); ++d)
          c += J.grid[vf_gidx(J, a, b, d)] == g;
    J.grid2[vf_gidx(J, x, y, z)] = c < 6 ? (uint16_t)VOXEL_EMPTY : g;
  }
}

__device__ __forceinline__ float lerp_(float a, float b, float t) {
  return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}

// perturbation, grid -> grid2
__global__ void kp_perturb(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  const uint32_t P = J.noise_period;
  const float fp = (float)P;
  const uint32_t sy = J.lat_nz * 3, sx = J.lat_ny * sy;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    const uint16_t g = J.grid[vf_gidx(J, x, y, z)];
    uint16_t out = g;
    if (g > VOXEL_FREE) {
      const float t0 = __fdiv_rn((float)(x % P), fp), t1 = __fdiv_rn((float)(y % P), fp),
                  t2 = __fdiv_rn((float)(z % P), fp);
      const float* L = J.lattice + (size_t)(x / P) * sx + (size_t)(y / P) * sy + (size_t)(z / P) * 3;
      int o[3];
      for (int ch = 0; ch < 3; ++ch) {
        const float c00 = lerp_(L[ch], L[3 + ch], t2), c01 = lerp_(L[sy + ch], L[sy + 3 + ch], t2);
        const float c10 = lerp_(L[sx + ch], L[sx + 3 + ch], t2),
                    c11 = lerp_(L[sx + sy + ch], L[sx + sy + 3 + ch], t2);
        const float n = lerp_(lerp_(c00, c01, t1), lerp_(c10, c11, t1), t0);
        o[ch] = (int)floorf(__fadd_rn(__fmul_rn(J.noise_amplitude, n), 0.5f));
      }
      const long ux = (long)x + o[0], uy = (long)y + o[1], uz = (long)z + o[2];
      if (ux >= 0 && uy >= 0 && uz >= 0 && ux < (long)J.X && uy < (long)J.Y && uz < (long)J.Z) {
        const uint16_t u = J.grid[vf_gidx(J, (uint32_t)ux, (uint32_t)uy, (uint32_t)uz)];
        if (u > VOXEL_FREE) out = u;
      }
    }
    J.grid2[vf_gidx(J, x, y, z)] = out;
  }
}

// naiveFracturer-comp.glsl:19-43 shape with the CPU path's semantics
__global__ void kp_naive(const JobDesc* jobs, const JobState* st) {
  const JobDesc& J = jobs[0];
  const uint32_t ns = st[0].nseeds;
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    uint16_t* gp = J.grid + vf_gidx(J, x, y, z);
    if (*gp == VOXEL_EMPTY) continue;
    float best = FLT_MAX;
    uint16_t lab = *gp;
    for (uint32_t s = 0; s < ns; ++s) {
      const int dx = (int)x - (int)J.seeds[4 * s], dy = (int)y - (int)J.seeds[4 * s + 1],
                dz = (int)z - (int)J.seeds[4 * s + 2];
      float d;
      if (J.distance == 0) {
        const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
        d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz)));
      } else if (J.distance == 1) {
        d = (float)(abs(dx) + abs(dy) + abs(dz));
      } else {
        d = (float)max(abs(dx), max(abs(dy), abs(dz)));
      }
      if (d < best) { best = d; lab = (uint16_t)J.seeds[4 * s + 3]; }
    }
    *gp = lab;
  }
}

__global__ void kp_counts(const JobDesc* jobs, JobState* st) {
  const JobDesc& J = jobs[0];
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    const uint16_t g = J.grid[vf_gidx(J, x, y, z)];
    if (g <= VOXEL_FREE) continue;
    const uint32_t v = g & 0x7FFFu;
    atomicAdd(&st[0].occupied, 1ull);
    if (v < J.ncounts) atomicAdd(&J.counts[v], 1u);
    else atomicOr(&st[0].err, VF_JERR_RANGE);
  }
}

__global__ void kp_competition(const JobDesc* jobs, JobState* st) {
  const JobDesc& J = jobs[0];
  const bool six = J.distance == 1;
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    volatile uint16_t* gv = J.grid + vf_gidx(J, x, y, z);
    const uint32_t g = *gv;
    if (g <= VOXEL_FREE) continue;
    const uint32_t f = g & 0xFFu;
    uint32_t p = g >> 8;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const int nz = (dx != 0) + (dy != 0) + (dz != 0);
          if (nz == 0 || (six && nz != 1)) continue;
          const int ux = (int)x + dx, uy = (int)y + dy, uz = (int)z + dz;
          if (ux < 0 || uy < 0 || uz < 0 || ux >= (int)J.X || uy >= (int)J.Y || uz >= (int)J.Z) continue;
          const uint32_t u = *(volatile uint16_t*)(J.grid + vf_gidx(J, ux, uy, uz));
          if (u > VOXEL_FREE && (u & 0xFFu) == f && (u >> 8) < p) p = u >> 8;
        }
    if (p != (g >> 8)) { *gv = (uint16_t)(f | (p << 8)); st[0].changed = 1; }
  }
}

__global__ void kp_minprefix(const JobDesc* jobs, JobState* st) {
  const JobDesc& J = jobs[0];
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    const uint32_t g = J.grid[vf_gidx(J, x, y, z)];
    if (g > VOXEL_FREE) atomicMin(&st[0].minprefix[g & 0xFFu], g >> 8);
  }
}

__global__ void kp_ranks(JobState* st) {
  JobState& s = st[0];
  uint32_t nr = 0;
  for (uint32_t f = 0; f < 256; ++f)
    if (s.minprefix[f] != 0xFFFFFFFFu) s.rank_value[nr++] = f | (s.minprefix[f] << 8);
  for (uint32_t a = 1; a < nr; ++a) {
    const uint32_t v = s.rank_value[a];
    uint32_t b = a;
    while (b > 0 && s.rank_value[b - 1] > v) { s.rank_value[b] = s.rank_value[b - 1]; --b; }
    s.rank_value[b] = v;
  }
  for (uint32_t r = 0; r < nr; ++r) s.value_rank[s.rank_value[r] & 0xFFu] = r;
  s.nranks = nr;
}

// disjointSetStack-comp.glsl:20-37: the survivors become the next frontier
__global__ void kp_disjoint_reset(const JobDesc* jobs, JobState* st, uint32_t* frontier,
                                  uint32_t* fcount) {
  const JobDesc& J = jobs[0];
  JobState& s = st[0];
  const uint64_t N = (uint64_t)J.X * J.Y * J.Z;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x, y, z;
    voxel_of(J, i, x, y, z);
    uint16_t* gp = J.grid + vf_gidx(J, x, y, z);
    const uint32_t g = *gp;
    uint32_t key = g ? VF_KEY_UNREACHED : VF_KEY_WALL;
    if (g > VOXEL_FREE) {
      if ((g >> 8) != s.minprefix[g & 0xFFu]) {
        *gp = VOXEL_FREE;
        atomicAdd(&s.disjoint, 1u);
      } else {
        key = ~s.value_rank[g & 0xFFu];
        frontier[atomicAdd(fcount, 1u)] = (uint32_t)i;
      }
    }
    J.keys[vf_kidx(J, x, y, z)] = key;
  }
}

// RegularGrid::undoMask / undoMask-comp.glsl unmaskBit: clear bit 15
__global__ void kp_undo_mask(const JobDesc* jobs) {
  const JobDesc& J = jobs[0];
  const uint64_t n = (uint64_t)J.X * J.Y * J.Zp;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    J.grid[i] &= 0x7FFFu;
}

inline int gridsz(uint64_t n) {
  uint64_t g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 65535ull * 16) g = 65535ull * 16;
  return (int)g;
}

}  // namespace

namespace vfk {

void plain_init_keys(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_init_keys<<<gridsz((uint64_t)hj.X * hj.Y * hj.Zk), 256, 0, st>>>(dj);
}
void plain_seed(cudaStream_t st, const JobDesc* dj, JobState* ds, uint32_t* frontier,
                uint32_t* fcount) {
  kp_seed<<<1, 1, 0, st>>>(dj, ds, frontier, fcount);
}
void plain_wave(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj,
                const uint32_t* cur, uint32_t ncur, uint32_t* next, uint32_t* ncount) {
  const int nn = hj.distance == 1 ? 6 : 26;
  kp_wave<<<gridsz((uint64_t)ncur * nn), 256, 0, st>>>(dj, ds, cur, ncur, next, ncount);
}
void plain_finalize(cudaStream_t st, const JobDesc* dj, const JobState* ds, const JobDesc& hj,
                    int pass2) {
  kp_finalize<<<gridsz((uint64_t)hj.X * hj.Y * hj.Zp), 256, 0, st>>>(dj, ds, pass2);
}
void plain_undo_mask(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_undo_mask<<<gridsz((uint64_t)hj.X * hj.Y * hj.Zp), 256, 0, st>>>(dj);
}
void plain_detect(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_detect<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj);
}
void plain_erode(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_erode<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj);
}
void plain_remove_isolated(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_isolated<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj);
}
void plain_perturb(cudaStream_t st, const JobDesc* dj, const JobDesc& hj) {
  kp_perturb<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj);
}
void plain_naive(cudaStream_t st, const JobDesc* dj, const JobState* ds, const JobDesc& hj) {
  kp_naive<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj, ds);
}
void plain_counts(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj) {
  kp_counts<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj, ds);
}
void plain_competition(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj) {
  kp_competition<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj, ds);
}
void plain_disjoint(cudaStream_t st, const JobDesc* dj, JobState* ds, const JobDesc& hj,
                    uint32_t* frontier, uint32_t* fcount) {
  kp_minprefix<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj, ds);
  kp_ranks<<<1, 1, 0, st>>>(ds);
  cudaMemsetAsync(fcount, 0, sizeof(uint32_t), st);
  kp_disjoint_reset<<<gridsz((uint64_t)hj.X * hj.Y * hj.Z), 256, 0, st>>>(dj, ds, frontier, fcount);
}

}  // namespace vfk
