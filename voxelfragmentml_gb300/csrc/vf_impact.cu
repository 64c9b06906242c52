// vf_impact.cu -- the impact path on sm_103a: the voxel a ray enters first
// (RegularGrid::getClosestEntryVoxel -> rayTraversalAmanatidesWoo,
// RegularGrid.cpp:265-270, 853-1004) for a batch of rays, and the seeds
// placed around impacts (Seeder::nearSeeds, Seeder.cpp:49-113), as
// CADScene::hit and CADScene::fractureModel use them (CADScene.cpp:508-520,
// 629-645).
//
//   k_ray_entry   one thread per ray: the reference's slab test and
//                 Amanatides-Woo walk in its operation order (every float
//                 step rounded as written); the walk is bounded by
//                 X + Y + Z + 3 steps, more than a ray can take
//   k_near_seeds  one CTA: impacts in order; per impact, rounds of 256
//                 candidates drawn from the counter-based hash and tested in
//                 parallel (distance to the impact's fragment seed, occupied,
//                 an EMPTY voxel in the clamped 3x3x3 box, not chosen
//                 before); the first valid ones in candidate order are kept;
//                 at the end the chosen voxels are ranked in (x, y, z) order
//                 (the reference's std::set) and labelled
#include <cfloat>

#include "vf.h"
#include "vf_kernels.h"

namespace {

constexpr uint32_t EMPTY = 0u;

__device__ __forceinline__ uint16_t gat(const vfk::ImpactGrid& G, uint32_t x, uint32_t y, uint32_t z) {
  return G.g[((uint64_t)x * G.Y + y) * G.Zp + z];
}

__device__ bool ray_box(const float o[3], const float d[3], const float mn[3], const float mx[3],
                        float& tmin, float& tmax) {
  float tMin, tMax, tYMin, tYMax, tZMin, tZMax;
  const float xi = __fdiv_rn(1.0f, d[0]);
  if (xi >= 0) {
    tMin = __fmul_rn(__fsub_rn(mn[0], o[0]), xi);
    tMax = __fmul_rn(__fsub_rn(mx[0], o[0]), xi);
  } else {
    tMin = __fmul_rn(__fsub_rn(mx[0], o[0]), xi);
    tMax = __fmul_rn(__fsub_rn(mn[0], o[0]), xi);
  }
  const float yi = __fdiv_rn(1.0f, d[1]);
  if (yi >= 0) {
    tYMin = __fmul_rn(__fsub_rn(mn[1], o[1]), yi);
    tYMax = __fmul_rn(__fsub_rn(mx[1], o[1]), yi);
  } else {
    tYMin = __fmul_rn(__fsub_rn(mx[1], o[1]), yi);
    tYMax = __fmul_rn(__fsub_rn(mn[1], o[1]), yi);
  }
  if (tMin > tYMax || tYMin > tMax) return false;
  if (tYMin > tMin) tMin = tYMin;
  if (tYMax < tMax) tMax = tYMax;
  const float zi = __fdiv_rn(1.0f, d[2]);
  if (zi >= 0) {
    tZMin = __fmul_rn(__fsub_rn(mn[2], o[2]), zi);
    tZMax = __fmul_rn(__fsub_rn(mx[2], o[2]), zi);
  } else {
    tZMin = __fmul_rn(__fsub_rn(mx[2], o[2]), zi);
    tZMax = __fmul_rn(__fsub_rn(mn[2], o[2]), zi);
  }
  if (tMin > tZMax || tZMin > tMax) return false;
  if (tZMin > tMin) tMin = tZMin;
  if (tZMax < tMax) tMax = tZMax;
  tmin = tMin;
  tmax = tMax;
  return tMin < FLT_MAX && tMax > 0.0f;
}

__global__ void __launch_bounds__(256) k_ray_entry(vfk::ImpactGrid G, const float* rays, uint32_t n,
                                                   uint32_t* out) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const float o[3] = {rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]};
    const float d[3] = {rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]};
    uint32_t res[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    float tMin = 0.0f, tMax = 0.0f;
    const bool zero = d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f;  // rejected by the caller
    if (!zero && ray_box(o, d, G.amin, G.amax, tMin, tMax)) {
      if (tMin < 0.0f) tMin = 0.0f;
      const uint32_t dims[3] = {G.X, G.Y, G.Z};
      float start[3], tNext[3], tDelta[3];
      int step[3];
      uint32_t cur[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) start[a] = __fadd_rn(o[a], __fmul_rn(d[a], tMin));
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float c = ceilf(__fdiv_rn(__fsub_rn(start[a], G.amin[a]), G.cell[a]));
        cur[a] = (uint32_t)(c > 1.0f ? c : 1.0f);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (d[a] > 0.0f) {
          step[a] = 1;
          tDelta[a] = __fdiv_rn(G.cell[a], d[a]);
          tNext[a] = __fadd_rn(
              tMin, __fdiv_rn(__fsub_rn(__fadd_rn(G.amin[a], __fmul_rn((float)cur[a], G.cell[a])), start[a]),
                              d[a]));
        } else if (d[a] < 0.0f) {
          step[a] = -1;
          tDelta[a] = __fdiv_rn(G.cell[a], -d[a]);
          tNext[a] = __fadd_rn(
              tMin,
              __fdiv_rn(__fsub_rn(__fadd_rn(G.amin[a], __fmul_rn((float)(cur[a] - 1u), G.cell[a])), start[a]),
                        d[a]));
        } else {
          step[a] = 0;
          tDelta[a] = FLT_MAX;
          tNext[a] = FLT_MAX;
        }
      }
      const uint64_t limit = (uint64_t)dims[0] + dims[1] + dims[2] + 3;
      for (uint64_t it = 0; it < limit; ++it) {
        if (!(cur[0] <= dims[0] && cur[1] <= dims[1] && cur[2] <= dims[2] && cur[0] > 0 && cur[1] > 0 &&
              cur[2] > 0))
          break;
        if (gat(G, cur[0] - 1, cur[1] - 1, cur[2] - 1) != EMPTY) {
          res[0] = cur[0];
          res[1] = cur[1];
          res[2] = cur[2];
          break;
        }
        const int a = (tNext[0] < tNext[1] && tNext[0] < tNext[2]) ? 0 : (tNext[1] < tNext[2] ? 1 : 2);
        cur[a] = (uint32_t)((int64_t)cur[a] + step[a]);
        tNext[a] = __fadd_rn(tNext[a], tDelta[a]);
      }
    }
    out[3 * r + 0] = res[0];
    out[3 * r + 1] = res[1];
    out[3 * r + 2] = res[2];
  }
}

__device__ bool is_boundary(const vfk::ImpactGrid& G, int x, int y, int z) {
  const int lo0 = max(x - 1, 0), lo1 = max(y - 1, 0), lo2 = max(z - 1, 0);
  const int hi0 = min(x + 1, (int)G.X - 1), hi1 = min(y + 1, (int)G.Y - 1), hi2 = min(z + 1, (int)G.Z - 1);
  for (int i = lo0; i <= hi0; ++i)
    for (int j = lo1; j <= hi1; ++j)
      for (int k = lo2; k <= hi2; ++k)
        if (gat(G, (uint32_t)i, (uint32_t)j, (uint32_t)k) == EMPTY) return true;
  return false;
}

__device__ __forceinline__ uint32_t biased(uint64_t seed, uint32_t impact, uint64_t cand, int axis,
                                           uint32_t n, uint32_t spreading) {
  const uint32_t m = n / spreading;
  uint32_t s = 0;
  for (uint32_t j = 0; j < spreading; ++j) {
    const uint64_t ctr = ((uint64_t)impact << 44) + (cand * 3u + (uint64_t)axis) * spreading + j;
    s += (uint32_t)(vf_hash(seed, VF_STREAM_NEAR, ctr) >> 33) % m;
  }
  return s;
}

// status[0] = chosen count, status[1] = 0 or VF_ERR_SEED_SEARCH
__global__ void __launch_bounds__(256) k_near_seeds(vfk::ImpactGrid G, const uint32_t* frags,
                                                    uint32_t nfrags, uint32_t num_impacts,
                                                    uint32_t num_seeds, uint32_t spreading,
                                                    uint64_t seed, uint32_t label0, uint32_t* chosen,
                                                    uint32_t* out, uint32_t* status) {
  __shared__ uint32_t cand[256][3];
  __shared__ uint8_t ok[256];
  __shared__ uint32_t s_nch, s_got, s_fail;
  const uint32_t t = threadIdx.x;
  if (t == 0) {
    s_nch = 0;
    s_fail = 0;
  }
  __syncthreads();
  const uint32_t dims[3] = {G.X, G.Y, G.Z}, half[3] = {G.X / 2, G.Y / 2, G.Z / 2};
  const uint32_t mind = min(G.X, min(G.Y, G.Z));
  const float minDiv = (float)(mind / 2);
  uint32_t pending = num_seeds;
  for (uint32_t i = 0; i < num_impacts; ++i) {
    const uint32_t fi = (uint32_t)__fmul_rn(vf_u01(vf_hash(seed, VF_STREAM_IMPACT, 2ull * i)), (float)nfrags);
    const uint32_t* f = frags + 4 * (uint64_t)min(fi, nfrags - 1);
    if (!pending) continue;
    uint32_t want =
        1u + (uint32_t)__fmul_rn(vf_u01(vf_hash(seed, VF_STREAM_IMPACT, 2ull * i + 1)), (float)pending);
    if (want > pending) want = pending;
    if (t == 0) s_got = 0;
    __syncthreads();
    for (uint64_t k0 = 0; k0 < VF_NEAR_MAX_CANDIDATES; k0 += 256) {
      const uint64_t k = k0 + t;
      uint32_t v[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int64_t off = (int64_t)half[a] - (int64_t)biased(seed, i, k, a, dims[a], spreading);
        v[a] = (uint32_t)(((int64_t)f[a] + off + (int64_t)dims[a]) % (int64_t)dims[a]);
      }
      const float dx = __fsub_rn((float)f[0], (float)v[0]), dy = __fsub_rn((float)f[1], (float)v[1]),
                  dz = __fsub_rn((float)f[2], (float)v[2]);
      const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
      bool good = k < VF_NEAR_MAX_CANDIDATES && !(dist > minDiv) && gat(G, v[0], v[1], v[2]) != EMPTY;
      const uint32_t nprev = s_nch;
      for (uint32_t c = 0; c < nprev && good; ++c)
        good = !(chosen[3 * c] == v[0] && chosen[3 * c + 1] == v[1] && chosen[3 * c + 2] == v[2]);
      if (good) good = is_boundary(G, (int)v[0], (int)v[1], (int)v[2]);
      cand[t][0] = v[0];
      cand[t][1] = v[1];
      cand[t][2] = v[2];
      ok[t] = good ? 1 : 0;
      __syncthreads();
      if (t == 0) {
        // candidate order; a repeat within this round counts once
        uint32_t nch = s_nch, got = s_got;
        for (uint32_t j = 0; j < 256 && got < want; ++j) {
          if (!ok[j]) continue;
          bool dup = false;
          for (uint32_t c = nprev; c < nch && !dup; ++c)
            dup = chosen[3 * c] == cand[j][0] && chosen[3 * c + 1] == cand[j][1] &&
                  chosen[3 * c + 2] == cand[j][2];
          if (dup) continue;
          chosen[3 * nch] = cand[j][0];
          chosen[3 * nch + 1] = cand[j][1];
          chosen[3 * nch + 2] = cand[j][2];
          ++nch;
          ++got;
        }
        s_nch = nch;
        s_got = got;
      }
      __syncthreads();
      if (s_got >= want) break;
    }
    if (s_got < want) {
      if (t == 0) s_fail = 1;
      break;
    }
    pending -= want;
    __syncthreads();
  }
  __syncthreads();
  const uint32_t nch = s_nch;
  if (!s_fail) {
    // rank in (x, y, z) order; chosen voxels are distinct
    for (uint32_t c = t; c < nch; c += blockDim.x) {
      const uint32_t x = chosen[3 * c], y = chosen[3 * c + 1], z = chosen[3 * c + 2];
      uint32_t rank = 0;
      for (uint32_t e = 0; e < nch; ++e) {
        const uint32_t ex = chosen[3 * e], ey = chosen[3 * e + 1], ez = chosen[3 * e + 2];
        rank += (ex < x || (ex == x && (ey < y || (ey == y && ez < z)))) ? 1u : 0u;
      }
      uint32_t* o = out + 4 * (uint64_t)rank;
      o[0] = x;
      o[1] = y;
      o[2] = z;
      o[3] = label0 + rank + 1;
    }
  }
  if (t == 0) {
    status[0] = nch;
    status[1] = s_fail ? (uint32_t)VF_ERR_SEED_SEARCH : 0u;
  }
}

}  // namespace

namespace vfk {

void ray_entry(cudaStream_t st, const ImpactGrid& G, const float* rays, uint32_t n, uint32_t* out,
               int num_sms) {
  if (!n) return;
  const int blocks = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms * 8);
  k_ray_entry<<<blocks, 256, 0, st>>>(G, rays, n, out);
}

void near_seeds(cudaStream_t st, const ImpactGrid& G, const uint32_t* frags, uint32_t nfrags,
                uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading, uint64_t seed,
                uint32_t label0, uint32_t* chosen, uint32_t* out, uint32_t* status) {
  k_near_seeds<<<1, 256, 0, st>>>(G, frags, nfrags, num_impacts, num_seeds, spreading, seed, label0,
                                  chosen, out, status);
}

}  // namespace vfk
