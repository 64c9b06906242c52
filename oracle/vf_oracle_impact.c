/*
 * vf_oracle_impact.c -- CPU oracle of the impact path: the voxel a ray enters
 * first (RegularGrid::getClosestEntryVoxel / rayTraversalAmanatidesWoo,
 * RegularGrid.cpp:265-270, 853-1004) and the seeds placed around impacts
 * (Seeder::nearSeeds, Seeder.cpp:49-113), the seeding CADScene::hit and
 * CADScene::fractureModel use for user impacts (CADScene.cpp:508-520,
 * 629-645).
 *
 * TEST INFRASTRUCTURE ONLY (see vf_oracle.h).
 *
 * Ray traversal, in the reference's operation order: slab test against the
 * grid's box (1/d per axis, t0 = 0, t1 = FLT_MAX); tMin = max(tMin, 0); the
 * entry point o + d*tMin; the starting index max(1, ceil((p - min) / cell))
 * (1-based); per axis the step, tDelta = cell / |d| and the first boundary
 * crossing; then Amanatides-Woo steps (x when tMaxX < tMaxY and tMaxX < tMaxZ,
 * else y when tMaxY < tMaxZ, else z) until the index leaves [1, dims] or the
 * voxel index - 1 is not EMPTY.  The result is that 1-based index, which
 * CADScene::hit uses as the impact seed as is.  The walk is bounded here by
 * X + Y + Z + 3 steps (it can take no more); a zero direction is rejected
 * (the reference would loop forever).
 *
 * nearSeeds, per impact i: a fragment seed f picked uniformly; nseeds drawn in
 * [1, pending]; candidates v = (f + dims/2 - biased(dims, spreading) + dims)
 * mod dims per axis, biased(n, s) = sum of s draws r % (n / s); a candidate
 * counts when its distance to f is at most min(dims)/2, it is occupied (not
 * EMPTY), not chosen before, and some voxel of its clamped 3x3x3 box is EMPTY
 * (RegularGrid::isBoundary(.., 1), RegularGrid.cpp:543-559).  The chosen
 * voxels, in (x, y, z) order (the reference's std::set), follow the given
 * seeds with labels counting on from the last one's.
 * Fixed here: the draws come from the counter-based hash (the reference uses
 * rand() and std::mt19937, whose streams are implementation specific); an
 * impact tries at most VFO_NEAR_MAX_CANDIDATES candidates and then fails
 * with VFO_ERR_SEED_SEARCH (the reference loops forever); impacts after the
 * pending count reaches 0 place no seed (the reference would draw from an
 * empty range).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "vf_oracle.h"

#define VOXEL_EMPTY 0u
#define VFO_STREAM_IMPACT 4u
#define VFO_STREAM_NEAR 5u

static inline uint16_t gat(const uint16_t* g, uint32_t Y, uint32_t Z, uint32_t x, uint32_t y,
                           uint32_t z) {
  return g[((size_t)x * Y + y) * Z + z];
}

/* RegularGrid::rayBoxIntersection (RegularGrid.cpp:853-898) */
static int ray_box(const float o[3], const float d[3], const float mn[3], const float mx[3],
                   float* tmin, float* tmax, float t0, float t1) {
  float tMin, tMax;
  const float xi = 1.0f / d[0];
  if (xi >= 0) {
    tMin = (mn[0] - o[0]) * xi;
    tMax = (mx[0] - o[0]) * xi;
  } else {
    tMin = (mx[0] - o[0]) * xi;
    tMax = (mn[0] - o[0]) * xi;
  }
  const float yi = 1.0f / d[1];
  float tYMin, tYMax;
  if (yi >= 0) {
    tYMin = (mn[1] - o[1]) * yi;
    tYMax = (mx[1] - o[1]) * yi;
  } else {
    tYMin = (mx[1] - o[1]) * yi;
    tYMax = (mn[1] - o[1]) * yi;
  }
  if (tMin > tYMax || tYMin > tMax) return 0;
  if (tYMin > tMin) tMin = tYMin;
  if (tYMax < tMax) tMax = tYMax;
  const float zi = 1.0f / d[2];
  float tZMin, tZMax;
  if (zi >= 0) {
    tZMin = (mn[2] - o[2]) * zi;
    tZMax = (mx[2] - o[2]) * zi;
  } else {
    tZMin = (mx[2] - o[2]) * zi;
    tZMax = (mn[2] - o[2]) * zi;
  }
  if (tMin > tZMax || tZMin > tMax) return 0;
  if (tZMin > tMin) tMin = tZMin;
  if (tZMax < tMax) tMax = tZMax;
  *tmin = tMin;
  *tmax = tMax;
  return tMin < t1 && tMax > t0;
}

int vfo_ray_entry(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, const float amin[3],
                  const float amax[3], const float origin[3], const float dir[3], uint32_t out[3]) {
  out[0] = out[1] = out[2] = 0xFFFFFFFFu;
  if (dir[0] == 0.0f && dir[1] == 0.0f && dir[2] == 0.0f) return VFO_ERR_INVALID;
  const uint32_t dims[3] = {X, Y, Z};
  float cell[3];
  for (int a = 0; a < 3; ++a) cell[a] = (amax[a] - amin[a]) / (float)dims[a];
  float tMin = 0.0f, tMax = 0.0f;
  if (!ray_box(origin, dir, amin, amax, &tMin, &tMax, 0.0f, FLT_MAX)) return 0;
  if (tMin < 0.0f) tMin = 0.0f;
  float start[3], tNext[3], tDelta[3];
  int step[3];
  uint32_t cur[3];
  for (int a = 0; a < 3; ++a) start[a] = origin[a] + dir[a] * tMin;
  for (int a = 0; a < 3; ++a) {
    const float c = ceilf((start[a] - amin[a]) / cell[a]);
    cur[a] = (uint32_t)(c > 1.0f ? c : 1.0f);
  }
  /* tMax of the reference becomes FLT_MAX (glm::max(tMax, t1)) */
  const float tEnd = FLT_MAX;
  for (int a = 0; a < 3; ++a) {
    if (dir[a] > 0.0f) {
      step[a] = 1;
      tDelta[a] = cell[a] / dir[a];
      tNext[a] = tMin + (amin[a] + (float)cur[a] * cell[a] - start[a]) / dir[a];
    } else if (dir[a] < 0.0f) {
      step[a] = -1;
      tDelta[a] = cell[a] / -dir[a];
      tNext[a] = tMin + (amin[a] + (float)(cur[a] - 1) * cell[a] - start[a]) / dir[a];
    } else {
      step[a] = 0;
      tDelta[a] = tEnd;
      tNext[a] = tEnd;
    }
  }
  const uint64_t limit = (uint64_t)X + Y + Z + 3;
  for (uint64_t it = 0; it < limit; ++it) {
    if (!(cur[0] <= X && cur[1] <= Y && cur[2] <= Z && cur[0] > 0 && cur[1] > 0 && cur[2] > 0))
      break;
    if (gat(grid, Y, Z, cur[0] - 1, cur[1] - 1, cur[2] - 1) != VOXEL_EMPTY) {
      memcpy(out, cur, sizeof(cur));
      return 0;
    }
    int a;
    if (tNext[0] < tNext[1] && tNext[0] < tNext[2]) a = 0;
    else if (tNext[1] < tNext[2]) a = 1;
    else a = 2;
    cur[a] = (uint32_t)((int64_t)cur[a] + step[a]);
    tNext[a] += tDelta[a];
  }
  return 0;
}

/* n rays (6 floats each) -> 3 uint32 each; OpenMP over rays (independent) */
int vfo_ray_entry_batch(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                        const float amin[3], const float amax[3], const float* rays, uint32_t n,
                        uint32_t* out) {
  int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
  for (int64_t r = 0; r < (int64_t)n; ++r)
    err |= vfo_ray_entry(grid, X, Y, Z, amin, amax, rays + 6 * r, rays + 6 * r + 3, out + 3 * r);
  return err;
}

static int is_boundary(const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, int x, int y, int z) {
  const int lo[3] = {x - 1 < 0 ? 0 : x - 1, y - 1 < 0 ? 0 : y - 1, z - 1 < 0 ? 0 : z - 1};
  const int hi[3] = {x + 1 > (int)X - 1 ? (int)X - 1 : x + 1, y + 1 > (int)Y - 1 ? (int)Y - 1 : y + 1,
                     z + 1 > (int)Z - 1 ? (int)Z - 1 : z + 1};
  for (int i = lo[0]; i <= hi[0]; ++i)
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int k = lo[2]; k <= hi[2]; ++k)
        if (gat(g, Y, Z, (uint32_t)i, (uint32_t)j, (uint32_t)k) == VOXEL_EMPTY) return 1;
  return 0;
}

static int cmp_xyz3(const void* pa, const void* pb) {
  const uint32_t* a = (const uint32_t*)pa;
  const uint32_t* b = (const uint32_t*)pb;
  for (int i = 0; i < 3; ++i)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

/* biased(n, s) = sum over j < s of r_j % (n / s) for the candidate's axis */
static uint32_t biased(uint64_t seed, uint32_t impact, uint64_t cand, int axis, uint32_t n,
                       uint32_t spreading) {
  const uint32_t m = n / spreading;
  uint32_t s = 0;
  for (uint32_t j = 0; j < spreading; ++j) {
    const uint64_t ctr = ((uint64_t)impact << 44) + (cand * 3u + (uint64_t)axis) * spreading + j;
    s += (uint32_t)(vfo_hash(seed, VFO_STREAM_NEAR, ctr) >> 33) % m;
  }
  return s;
}

int vfo_near_seeds(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, const uint32_t* frags,
                   uint32_t nfrags, uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading,
                   uint64_t seed, uint32_t* out, uint32_t* nout) {
  if (!grid || !out || !nout || (nfrags && !frags)) return VFO_ERR_INVALID;
  const uint32_t mind = (X < Y ? (X < Z ? X : Z) : (Y < Z ? Y : Z));
  if (num_impacts && (!nfrags || spreading < 1 || spreading > mind)) return VFO_ERR_INVALID;
  const uint32_t dims[3] = {X, Y, Z}, half[3] = {X / 2, Y / 2, Z / 2};
  const float minDiv = (float)(mind / 2);
  uint32_t* chosen = (uint32_t*)malloc(3 * (size_t)(num_seeds ? num_seeds : 1) * sizeof(uint32_t));
  if (!chosen) return VFO_ERR_RANGE;
  uint32_t nch = 0, pending = num_seeds;
  int st = 0;
  for (uint32_t i = 0; i < num_impacts && !st; ++i) {
    const uint32_t fi =
        (uint32_t)(vfo_u01(vfo_hash(seed, VFO_STREAM_IMPACT, 2ull * i)) * (float)nfrags);
    const uint32_t* f = frags + 4 * (size_t)(fi < nfrags ? fi : nfrags - 1);
    if (!pending) continue;
    uint32_t want = 1u + (uint32_t)(vfo_u01(vfo_hash(seed, VFO_STREAM_IMPACT, 2ull * i + 1)) * (float)pending);
    if (want > pending) want = pending;
    uint32_t got = 0;
    uint64_t k = 0;
    for (; got < want && k < VFO_NEAR_MAX_CANDIDATES; ++k) {
      uint32_t v[3];
      for (int a = 0; a < 3; ++a) {
        const int64_t off = (int64_t)half[a] - (int64_t)biased(seed, i, k, a, dims[a], spreading);
        v[a] = (uint32_t)(((int64_t)f[a] + off + (int64_t)dims[a]) % (int64_t)dims[a]);
      }
      const float dx = (float)f[0] - (float)v[0], dy = (float)f[1] - (float)v[1],
                  dz = (float)f[2] - (float)v[2];
      if (sqrtf(dx * dx + dy * dy + dz * dz) > minDiv) continue;
      if (gat(grid, Y, Z, v[0], v[1], v[2]) == VOXEL_EMPTY) continue;
      int dup = 0;
      for (uint32_t c = 0; c < nch && !dup; ++c)
        dup = chosen[3 * c] == v[0] && chosen[3 * c + 1] == v[1] && chosen[3 * c + 2] == v[2];
      if (dup) continue;
      if (!is_boundary(grid, X, Y, Z, (int)v[0], (int)v[1], (int)v[2])) continue;
      memcpy(chosen + 3 * (size_t)nch, v, sizeof(v));
      ++nch;
      ++got;
    }
    if (got < want) st = VFO_ERR_SEED_SEARCH;
    pending -= want;
  }
  if (!st) {
    qsort(chosen, nch, 3 * sizeof(uint32_t), cmp_xyz3);
    memcpy(out, frags, 4 * (size_t)nfrags * sizeof(uint32_t));
    uint32_t label = nfrags ? frags[4 * (size_t)(nfrags - 1) + 3] : 1u;
    for (uint32_t c = 0; c < nch; ++c) {
      uint32_t* o = out + 4 * ((size_t)nfrags + c);
      o[0] = chosen[3 * c];
      o[1] = chosen[3 * c + 1];
      o[2] = chosen[3 * c + 2];
      o[3] = ++label;
    }
    *nout = nfrags + nch;
  }
  free(chosen);
  return st;
}
