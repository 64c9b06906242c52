// vf_impact.cu -- the impact path on sm_103a: the voxel a ray enters first
// (RegularGrid::getClosestEntryVoxel -> rayTraversalAmanatidesWoo,
// RegularGrid.cpp:265-270, 853-1004) for a batch of rays, and the seeds
// placed around impacts (Seeder::nearSeeds, Seeder.cpp:49-113), as
// CADScene::hit and CADScene::fractureModel use them (CADScene.cpp:508-520,
// 629-645).
//
//   k_occ_bits    (batches of rays) the grid's occupancy packed 1 bit per
//                 voxel, so the walks read an L2-resident bitmap
//   k_ray_entry   one thread per ray: the reference's slab test and
//                 Amanatides-Woo walk in its operation order (every float
//                 step rounded as written); the walk is bounded by
//                 X + Y + Z + 3 steps, more than a ray can take
//   k_near_seeds  one CTA running vfnear::place (vf_near.cuh): impacts in
//                 order, rounds of 256 candidates tested in parallel, the
//                 first valid ones in candidate order kept, then sorted in
//                 (x, y, z) order (the reference's std::set) and labelled
#include <cfloat>

#include "vf.h"
#include "vf_kernels.h"
#include "vf_near.cuh"

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

// occupancy bits (label != EMPTY) of grid row r: word r * Zw + z / 32
__global__ void __launch_bounds__(256) k_occ_bits(vfk::ImpactGrid G, uint32_t Zw, uint32_t* bits) {
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)G.X * G.Y;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const uint16_t* row = G.g + r * G.Zp;
    for (uint32_t z0 = 0; z0 < G.Z; z0 += 32) {
      const uint32_t z = z0 + lane;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, z < G.Z && row[z] != EMPTY);
      if (lane == 0) bits[r * Zw + (z0 >> 5)] = m;
    }
  }
}

// Occupancy of a voxel: from the label grid, or (many rays) from the packed
// bits, which stay in L2 while the rays walk.
struct LabelOcc {
  const vfk::ImpactGrid& G;
  __device__ bool operator()(uint32_t x, uint32_t y, uint32_t z) const { return gat(G, x, y, z) != EMPTY; }
};
struct BitOcc {
  const uint32_t* bits;
  uint32_t Y, Zw;
  __device__ bool operator()(uint32_t x, uint32_t y, uint32_t z) const {
    return (__ldg(bits + ((uint64_t)x * Y + y) * Zw + (z >> 5)) >> (z & 31u)) & 1u;
  }
};

template <typename Occ>
__global__ void __launch_bounds__(256) k_ray_entry(vfk::ImpactGrid G, Occ occ, const float* rays, uint32_t n,
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
        if (occ(cur[0] - 1, cur[1] - 1, cur[2] - 1)) {
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

struct ImpactView {
  const vfk::ImpactGrid& G;
  __device__ bool occupied(uint32_t x, uint32_t y, uint32_t z) const { return gat(G, x, y, z) != EMPTY; }
  // RegularGrid::isBoundary(x, y, z, 1) (RegularGrid.cpp:543-559)
  __device__ bool boundary(uint32_t x, uint32_t y, uint32_t z) const {
    const int lo0 = max((int)x - 1, 0), lo1 = max((int)y - 1, 0), lo2 = max((int)z - 1, 0);
    const int hi0 = min((int)x + 1, (int)G.X - 1), hi1 = min((int)y + 1, (int)G.Y - 1),
              hi2 = min((int)z + 1, (int)G.Z - 1);
    for (int i = lo0; i <= hi0; ++i)
      for (int j = lo1; j <= hi1; ++j)
        for (int k = lo2; k <= hi2; ++k)
          if (gat(G, (uint32_t)i, (uint32_t)j, (uint32_t)k) == EMPTY) return true;
    return false;
  }
};

// status[0] = count placed, status[1] = 0 or VF_ERR_SEED_SEARCH
__global__ void __launch_bounds__(256) k_near_seeds(vfk::ImpactGrid G, const uint32_t* frags,
                                                    uint32_t nfrags, uint32_t num_impacts,
                                                    uint32_t num_seeds, uint32_t spreading,
                                                    uint64_t seed, uint32_t label0, uint32_t* out,
                                                    uint32_t* status) {
  __shared__ unsigned long long cand[256];
  __shared__ unsigned long long acc[4096];
  __shared__ uint32_t cnt;
  const int n = vfnear::place(ImpactView{G}, G.X, G.Y, G.Z, frags, nfrags, num_impacts, num_seeds,
                              spreading, seed, label0, cand, acc, &cnt, out);
  if (threadIdx.x == 0) {
    status[0] = n < 0 ? 0u : (uint32_t)n;
    status[1] = n < 0 ? (uint32_t)VF_ERR_SEED_SEARCH : 0u;
  }
}

}  // namespace

namespace vfk {

void ray_entry(cudaStream_t st, const ImpactGrid& G, const float* rays, uint32_t n, uint32_t* out,
               uint32_t* bits, int num_sms) {
  if (!n) return;
  const int blocks = (int)std::min<uint32_t>((n + 255) / 256, (uint32_t)num_sms * 8);
  if (bits) {
    const uint32_t Zw = (G.Z + 31) / 32;
    const uint64_t rows = (uint64_t)G.X * G.Y;
    const int bb = (int)std::max<uint64_t>(1, std::min<uint64_t>((rows * 32 + 255) / 256, (uint64_t)num_sms * 8));
    k_occ_bits<<<bb, 256, 0, st>>>(G, Zw, bits);
    k_ray_entry<<<blocks, 256, 0, st>>>(G, BitOcc{bits, G.Y, Zw}, rays, n, out);
  } else {
    k_ray_entry<<<blocks, 256, 0, st>>>(G, LabelOcc{G}, rays, n, out);
  }
}

void near_seeds(cudaStream_t st, const ImpactGrid& G, const uint32_t* frags, uint32_t nfrags,
                uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading, uint64_t seed,
                uint32_t label0, uint32_t* out, uint32_t* status) {
  k_near_seeds<<<1, 256, 0, st>>>(G, frags, nfrags, num_impacts, num_seeds, spreading, seed, label0,
                                  out, status);
}

}  // namespace vfk
