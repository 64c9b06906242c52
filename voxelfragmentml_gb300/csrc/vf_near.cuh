// vf_near.cuh -- Seeder::nearSeeds (Seeder.cpp:49-113) for one CTA, shared by
// vf_near_seeds (vf_impact.cu) and the batched seeding stage (vf_gridops.cu).
//
// Per impact i: a given seed f picked by the hash; nseeds drawn in
// [1, pending]; candidates v = (f + dims/2 - biased(dims, spreading) + dims)
// mod dims per axis, biased(n, s) = the sum of s draws r % (n / s); a
// candidate counts when its distance to f is at most min(dims)/2, the voxel is
// occupied, not chosen before, and its clamped 3x3x3 box holds an EMPTY voxel.
// Each round tests blockDim.x candidates in parallel and warp 0 keeps the
// first valid ones in candidate order, so the result equals the sequential
// sampler's.  The chosen voxels are written in (x, y, z) order with labels
// label0 + 1, label0 + 2, ...
#pragma once
#include "vf_common.cuh"

namespace vfnear {

// Grid: occupied(x, y, z) and boundary(x, y, z) (an EMPTY voxel in the
// clamped 3x3x3 box).  cand: blockDim.x words; acc: a power of two >= the
// seeds placed (at most 4096).  Returns the count placed, -1 when an impact
// runs out of its 2^20 candidates.
template <typename Grid>
__device__ int place(const Grid& G, uint32_t X, uint32_t Y, uint32_t Z, const uint32_t* frags,
                     uint32_t nf, uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading,
                     uint64_t seed, uint32_t label0, unsigned long long* cand,
                     unsigned long long* acc, uint32_t* s_cnt, uint32_t* out) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t nt = blockDim.x;
  const uint32_t dims[3] = {X, Y, Z}, half[3] = {X / 2, Y / 2, Z / 2};
  const float minDiv = (float)(min(X, min(Y, Z)) / 2);
  if (t == 0) *s_cnt = 0;
  __syncthreads();
  uint32_t pending = num_seeds;
  for (uint32_t i = 0; i < num_impacts; ++i) {
    const uint32_t fi = (uint32_t)__fmul_rn(vf_u01(vf_hash(seed, VF_STREAM_IMPACT, 2ull * i)), (float)nf);
    const uint32_t* f = frags + 4 * (uint64_t)min(fi, nf - 1);
    if (!pending) continue;
    uint32_t want =
        1u + (uint32_t)__fmul_rn(vf_u01(vf_hash(seed, VF_STREAM_IMPACT, 2ull * i + 1)), (float)pending);
    if (want > pending) want = pending;
    const uint32_t goal = *s_cnt + want;
    for (uint64_t k0 = 0; k0 < VF_NEAR_MAX_CANDIDATES; k0 += nt) {
      const uint64_t k = k0 + (uint64_t)t;
      uint32_t v[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const uint32_t m = dims[a] / spreading;
        uint32_t bsum = 0;
        for (uint32_t j = 0; j < spreading; ++j) {
          const uint64_t ctr = ((uint64_t)i << 44) + (k * 3u + (uint64_t)a) * spreading + j;
          bsum += (uint32_t)(vf_hash(seed, VF_STREAM_NEAR, ctr) >> 33) % m;
        }
        const int64_t off = (int64_t)half[a] - (int64_t)bsum;
        v[a] = (uint32_t)(((int64_t)f[a] + off + (int64_t)dims[a]) % (int64_t)dims[a]);
      }
      const float dx = __fsub_rn((float)f[0], (float)v[0]), dy = __fsub_rn((float)f[1], (float)v[1]),
                  dz = __fsub_rn((float)f[2], (float)v[2]);
      const float dist =
          __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
      bool good = k < VF_NEAR_MAX_CANDIDATES && !(dist > minDiv) && G.occupied(v[0], v[1], v[2]);
      if (good) good = G.boundary(v[0], v[1], v[2]);
      cand[t] = good ? (((unsigned long long)v[0] << 24) | ((unsigned long long)v[1] << 12) | v[2]) : ~0ull;
      __syncthreads();
      if (warp == 0) {
        uint32_t cnt = *s_cnt;
        for (uint32_t c = 0; c < nt && cnt < goal; ++c) {
          const unsigned long long key = cand[c];
          if (key == ~0ull) continue;
          bool dup = false;
          for (uint32_t m = lane; m < cnt; m += 32) dup |= (acc[m] == key);
          dup = __any_sync(0xFFFFFFFFu, dup);
          if (!dup) {
            if (lane == 0) acc[cnt] = key;
            ++cnt;
          }
          __syncwarp();
        }
        if (lane == 0) *s_cnt = cnt;
      }
      __syncthreads();
      if (*s_cnt >= goal) break;
    }
    if (*s_cnt < goal) return -1;
    pending -= want;
  }
  const uint32_t n = *s_cnt;
  // (x, y, z) order: bitonic over the next power of two
  uint32_t P = 1;
  while (P < n) P <<= 1;
  for (uint32_t q = n + t; q < P; q += nt) acc[q] = ~0ull;
  __syncthreads();
  for (uint32_t kk = 2; kk <= P; kk <<= 1)
    for (uint32_t jx = kk >> 1; jx > 0; jx >>= 1) {
      for (uint32_t q = t; q < P; q += nt) {
        const uint32_t l = q ^ jx;
        if (l > q) {
          const unsigned long long a = acc[q], b = acc[l];
          const bool up = (q & kk) == 0;
          if ((a > b) == up) { acc[q] = b; acc[l] = a; }
        }
      }
      __syncthreads();
    }
  for (uint32_t q = t; q < n; q += nt) {
    const unsigned long long key = acc[q];
    out[4 * q] = (uint32_t)(key >> 24);
    out[4 * q + 1] = (uint32_t)((key >> 12) & 0xFFF);
    out[4 * q + 2] = (uint32_t)(key & 0xFFF);
    out[4 * q + 3] = label0 + 1 + q;
  }
  __syncthreads();
  return (int)n;
}

}  // namespace vfnear
