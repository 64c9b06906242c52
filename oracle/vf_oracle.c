/*
 * vf_oracle.c -- CPU oracle (restatement) of the VoxelFragmentML hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * Never linked into the product library.  See vf_oracle.h for the layout,
 * the value encoding and the parity-pinning status ("parity unpinned"
 * against reference outputs: the reference has no tests or golden vectors
 * for this path and cannot be built or run here).
 *
 * Compile with: -O2 -ffp-contract=off -fopenmp (see oracle/Makefile).
 * OpenMP is only used where the result cannot depend on the schedule.
 */
#include "vf_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define VOXEL_EMPTY 0u
#define VOXEL_FREE 1u
#define MAX_TRIES 1000000u /* Seeder.h:48 */
#define NOISE_BUFFER 1000000u /* RegularGrid.cpp:124 fillNoiseBuffer(.., 1e6) */
#define MAX_SEEDS 4095u

static inline size_t lin(uint32_t x, uint32_t y, uint32_t z, uint32_t Y,
                         uint32_t Z) {
  /* RegularGrid::getPositionIndex (RegularGrid.cpp:1031-1034), 64-bit */
  return ((size_t)x * Y + y) * Z + z;
}
static inline int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

/* ------------------------------------------------------------------------ */
/* Counter-based RNG.  Replaces std::mt19937 + uniform_real_distribution
 * (RandomUtilities.h:11-22), whose float distribution is implementation
 * specific.  Finaliser: SplitMix64 (Steele, Lea, Flood 2014). */
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t vfo_hash(uint64_t seed, uint32_t stream, uint64_t counter) {
  uint64_t k = mix64(seed ^ ((uint64_t)stream * 0x9E3779B97F4A7C15ull));
  return mix64(k + counter * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
}
/* 24 random bits -> float in [0,1), exact */
float vfo_u01(uint64_t h) { return (float)(uint32_t)(h >> 40) * 5.9604644775390625e-8f; }

/* ------------------------------------------------------------------------ */
/* Triangle / AABB separating-axis test, Intersections3D.h:204-258 with the
 * helpers at :260-420, in the reference's operation order. */
typedef struct { float x, y, z; } v3;
static inline v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }

typedef struct {
  v3 v0, v1, v2, r; /* triangle relative to box centre, box radius */
  float mn, mx, rad;
} satd;

static int axis_x01(satd* d, float a, float b, float fa, float fb) {
  float p0 = a * d->v0.y - b * d->v0.z;
  float p2 = a * d->v2.y - b * d->v2.z;
  if (p0 < p2) { d->mn = p0; d->mx = p2; } else { d->mn = p2; d->mx = p0; }
  d->rad = fa * d->r.y + fb * d->r.z;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static int axis_x2(satd* d, float a, float b, float fa, float fb) {
  float p0 = a * d->v0.y - b * d->v0.z;
  float p1 = a * d->v1.y - b * d->v1.z;
  if (p0 < p1) { d->mn = p0; d->mx = p1; } else { d->mn = p1; d->mx = p0; }
  d->rad = fa * d->r.y + fb * d->r.z;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static int axis_y02(satd* d, float a, float b, float fa, float fb) {
  float p0 = -a * d->v0.x + b * d->v0.z;
  float p2 = -a * d->v2.x + b * d->v2.z;
  if (p0 < p2) { d->mn = p0; d->mx = p2; } else { d->mn = p2; d->mx = p0; }
  d->rad = fa * d->r.x + fb * d->r.z;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static int axis_y1(satd* d, float a, float b, float fa, float fb) {
  float p0 = -a * d->v0.x + b * d->v0.z;
  float p1 = -a * d->v1.x + b * d->v1.z;
  if (p0 < p1) { d->mn = p0; d->mx = p1; } else { d->mn = p1; d->mx = p0; }
  d->rad = fa * d->r.x + fb * d->r.z;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static int axis_z12(satd* d, float a, float b, float fa, float fb) {
  float p1 = a * d->v1.x - b * d->v1.y;
  float p2 = a * d->v2.x - b * d->v2.y;
  if (p2 < p1) { d->mn = p2; d->mx = p1; } else { d->mn = p1; d->mx = p2; }
  d->rad = fa * d->r.x + fb * d->r.y;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static int axis_z0(satd* d, float a, float b, float fa, float fb) {
  float p0 = a * d->v0.x - b * d->v0.y;
  float p1 = a * d->v1.x - b * d->v1.y;
  if (p0 < p1) { d->mn = p0; d->mx = p1; } else { d->mn = p1; d->mx = p0; }
  d->rad = fa * d->r.x + fb * d->r.y;
  return !(d->mn > d->rad || d->mx < -d->rad);
}
static void minmax3(float a, float b, float c, float* mn, float* mx) {
  *mn = *mx = a;
  if (b < *mn) *mn = b;
  if (b > *mx) *mx = b;
  if (c < *mn) *mn = c;
  if (c > *mx) *mx = c;
}
static int plane_box(v3 n, v3 v, v3 mb) {
  /* planeBoxOverlap, Intersections3D.h:268-293 */
  float nv[3] = {n.x, n.y, n.z}, vv[3] = {v.x, v.y, v.z}, m[3] = {mb.x, mb.y, mb.z};
  float vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    if (nv[q] > 0.0f) { vmin[q] = -m[q] - vv[q]; vmax[q] = m[q] - vv[q]; }
    else { vmin[q] = m[q] - vv[q]; vmax[q] = -m[q] - vv[q]; }
  }
  /* glm::dot(vec3) = (x*x' + y*y') + z*z' */
  if (nv[0] * vmin[0] + nv[1] * vmin[1] + nv[2] * vmin[2] > 0.0f) return 0;
  if (nv[0] * vmax[0] + nv[1] * vmax[1] + nv[2] * vmax[2] >= 0.0f) return 1;
  return 0;
}
static int tri_box_c(v3 p0, v3 p1, v3 p2, v3 c, v3 r) {
  satd d;
  d.r = r;
  d.v0 = v3sub(p0, c);
  d.v1 = v3sub(p1, c);
  d.v2 = v3sub(p2, c);
  v3 e0 = v3sub(d.v1, d.v0), e1 = v3sub(d.v2, d.v1), e2 = v3sub(d.v0, d.v2);
  float fx = fabsf(e0.x), fy = fabsf(e0.y), fz = fabsf(e0.z);
  if (!axis_x01(&d, e0.z, e0.y, fz, fy)) return 0;
  if (!axis_y02(&d, e0.z, e0.x, fz, fx)) return 0;
  if (!axis_z12(&d, e0.y, e0.x, fy, fx)) return 0;
  fx = fabsf(e1.x); fy = fabsf(e1.y); fz = fabsf(e1.z);
  if (!axis_x01(&d, e1.z, e1.y, fz, fy)) return 0;
  if (!axis_y02(&d, e1.z, e1.x, fz, fx)) return 0;
  if (!axis_z0(&d, e1.y, e1.x, fy, fx)) return 0;
  fx = fabsf(e2.x); fy = fabsf(e2.y); fz = fabsf(e2.z);
  if (!axis_x2(&d, e2.z, e2.y, fz, fy)) return 0;
  if (!axis_y1(&d, e2.z, e2.x, fz, fx)) return 0;
  if (!axis_z12(&d, e2.y, e2.x, fy, fx)) return 0;
  float mn, mx;
  minmax3(d.v0.x, d.v1.x, d.v2.x, &mn, &mx);
  if (mn > d.r.x || mx < -d.r.x) return 0;
  minmax3(d.v0.y, d.v1.y, d.v2.y, &mn, &mx);
  if (mn > d.r.y || mx < -d.r.y) return 0;
  minmax3(d.v0.z, d.v1.z, d.v2.z, &mn, &mx);
  if (mn > d.r.z || mx < -d.r.z) return 0;
  /* glm::cross(e0, e1) */
  v3 n = {e0.y * e1.z - e1.y * e0.z, e0.z * e1.x - e1.z * e0.x, e0.x * e1.y - e1.x * e0.y};
  return plane_box(n, d.v0, d.r);
}
/* box from (min,max) via AABB::center() = (max+min)/2 and extent() = max -
 * center (AABB.h:41,51) */
static void box_cr(v3 bmin, v3 bmax, v3* c, v3* r) {
  c->x = (bmax.x + bmin.x) / 2.0f; c->y = (bmax.y + bmin.y) / 2.0f; c->z = (bmax.z + bmin.z) / 2.0f;
  r->x = bmax.x - c->x; r->y = bmax.y - c->y; r->z = bmax.z - c->z;
}
int vfo_tri_box(const float p0[3], const float p1[3], const float p2[3],
                const float box_min[3], const float box_max[3]) {
  v3 a = {p0[0], p0[1], p0[2]}, b = {p1[0], p1[1], p1[2]}, c = {p2[0], p2[1], p2[2]};
  v3 mn = {box_min[0], box_min[1], box_min[2]}, mx = {box_max[0], box_max[1], box_max[2]};
  v3 bc, br;
  box_cr(mn, mx, &bc, &br);
  return tri_box_c(a, b, c, bc, br);
}

static int float_cell(float f, int n) {
  /* floor of a cell coordinate, clamped before the int conversion */
  if (!(f > -1.0e9f)) f = -1.0e9f;
  if (f > 1.0e9f) f = 1.0e9f;
  return clampi((int)floorf(f), -2, n + 1);
}

/* Surface shell: every voxel whose box the triangle overlaps (SAT).
 * Voxel box: min = aabbMin + cellSize*i, max = min + cellSize
 * (RegularGrid::getAABBs, RegularGrid.cpp:246-262); cellSize = size/dims
 * (RegularGrid.cpp:426-441). Candidates: the triangle's cell bbox grown by
 * one cell on each side. */
static void vox_shell(const float* V, const uint32_t* F, uint32_t nf,
                      uint32_t X, uint32_t Y, uint32_t Z, const float* amin,
                      const float* amax, uint8_t* shell) {
  const uint32_t dims[3] = {X, Y, Z};
  float cs[3];
  for (int a = 0; a < 3; ++a) cs[a] = (amax[a] - amin[a]) / (float)dims[a];
#pragma omp parallel for schedule(dynamic, 256)
  for (long f = 0; f < (long)nf; ++f) {
    const float* q[3] = {V + 3 * (size_t)F[3 * f], V + 3 * (size_t)F[3 * f + 1],
                         V + 3 * (size_t)F[3 * f + 2]};
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      float tmn, tmx;
      minmax3(q[0][a], q[1][a], q[2][a], &tmn, &tmx);
      lo[a] = clampi(float_cell((tmn - amin[a]) / cs[a], (int)dims[a]) - 1, 0, (int)dims[a] - 1);
      hi[a] = clampi(float_cell((tmx - amin[a]) / cs[a], (int)dims[a]) + 1, 0, (int)dims[a] - 1);
    }
    v3 p0 = {q[0][0], q[0][1], q[0][2]}, p1 = {q[1][0], q[1][1], q[1][2]},
       p2 = {q[2][0], q[2][1], q[2][2]};
    for (int i = lo[0]; i <= hi[0]; ++i)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int k = lo[2]; k <= hi[2]; ++k) {
          v3 bmin = {amin[0] + cs[0] * (float)i, amin[1] + cs[1] * (float)j,
                     amin[2] + cs[2] * (float)k};
          v3 bmax = {bmin.x + cs[0], bmin.y + cs[1], bmin.z + cs[2]};
          v3 c, r;
          box_cr(bmin, bmax, &c, &r);
          if (tri_box_c(p0, p1, p2, c, r))
            __atomic_store_n(&shell[lin(i, j, k, Y, Z)], 1, __ATOMIC_RELAXED);
        }
  }
}

/* ------------------------------------------------------------------------ */
/* Tetra-parity solid fill: Tetravoxelizer (Tetravoxelizer.cpp:42-92 GS,
 * :198-247 initializeModel, :264-315 compute).  Each face plus the mesh
 * centroid is a tetrahedron; slice plane y_s is cut through every
 * tetrahedron; the 1-2 cross-section triangles are rasterised with XOR so
 * that the covered parity at pixel centre (x,z) is the inside bit.
 *
 * Raster rule (the GL rasteriser cannot run here; this restates it):
 * vertices go to window coordinates x_w = x*w/2 + w/2 (GL viewport
 * transform), are snapped to 1/256 pixel (8 sub-pixel bits), and pixel
 * centres are tested with exact integer edge functions; samples exactly on
 * an edge belong to the triangle for which the edge is a "top-left" edge
 * (equivalent to nudging every sample by (+e, +e^2)), which keeps shared
 * edges and vertices single-owned so XOR parity is watertight. */
typedef struct { float x, y, z; } tv;

static inline float interp_c(float a, float b, float t) {
  /* GLSL mix(a,b,t) = a*(1-t) + b*t, no contraction */
  float omt = 1.0f - t;
  float l = a * omt;
  float r = b * t;
  return l + r;
}
static inline void interp(tv A, tv B, float s, float* ox, float* oz) {
  /* INTERP(A,B,s) = mix(A, B, (s - A.y) / (B.y - A.y))  (Tetravoxelizer.cpp:45) */
  float t = (s - A.y) / (B.y - A.y);
  *ox = interp_c(A.x, B.x, t);
  *oz = interp_c(A.z, B.z, t);
}
static inline int32_t to_fixed(float ndc, float half) {
  float w = ndc * half + half; /* separate mul and add (-ffp-contract=off) */
  return (int32_t)rintf(w * 256.0f);
}
static inline int64_t edge_fn(int32_t ax, int32_t az, int32_t bx, int32_t bz,
                              int64_t px, int64_t pz) {
  return (int64_t)(bx - ax) * (pz - az) - (int64_t)(bz - az) * (px - ax);
}
static inline int owns_edge(int32_t ax, int32_t az, int32_t bx, int32_t bz) {
  int32_t dz = bz - az, dx = bx - ax;
  return (dz < 0) || (dz == 0 && dx > 0);
}
static inline int64_t fdiv_floor(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}
/* rasterise one triangle (NDC x,z) into an X x Z byte plane with XOR */
static void raster_xor(float ax, float az, float bx, float bz, float cx,
                       float cz, uint32_t W, uint32_t H, float hw, float hh,
                       uint8_t* plane /* [z][x] */) {
  int32_t x0 = to_fixed(ax, hw), z0 = to_fixed(az, hh);
  int32_t x1 = to_fixed(bx, hw), z1 = to_fixed(bz, hh);
  int32_t x2 = to_fixed(cx, hw), z2 = to_fixed(cz, hh);
  int64_t area = edge_fn(x0, z0, x1, z1, x2, z2);
  if (area == 0) return;
  if (area < 0) { /* orient counter-clockwise */
    int32_t tx = x1, tz = z1;
    x1 = x2; z1 = z2; x2 = tx; z2 = tz;
  }
  int32_t mnx = x0 < x1 ? (x0 < x2 ? x0 : x2) : (x1 < x2 ? x1 : x2);
  int32_t mxx = x0 > x1 ? (x0 > x2 ? x0 : x2) : (x1 > x2 ? x1 : x2);
  int32_t mnz = z0 < z1 ? (z0 < z2 ? z0 : z2) : (z1 < z2 ? z1 : z2);
  int32_t mxz = z0 > z1 ? (z0 > z2 ? z0 : z2) : (z1 > z2 ? z1 : z2);
  int64_t ilo = fdiv_floor((int64_t)mnx - 128 + 255, 256), ihi = fdiv_floor((int64_t)mxx - 128, 256);
  int64_t klo = fdiv_floor((int64_t)mnz - 128 + 255, 256), khi = fdiv_floor((int64_t)mxz - 128, 256);
  if (ilo < 0) ilo = 0;
  if (klo < 0) klo = 0;
  if (ihi > (int64_t)W - 1) ihi = (int64_t)W - 1;
  if (khi > (int64_t)H - 1) khi = (int64_t)H - 1;
  int o01 = owns_edge(x0, z0, x1, z1), o12 = owns_edge(x1, z1, x2, z2),
      o20 = owns_edge(x2, z2, x0, z0);
  for (int64_t k = klo; k <= khi; ++k) {
    int64_t pz = k * 256 + 128;
    for (int64_t i = ilo; i <= ihi; ++i) {
      int64_t px = i * 256 + 128;
      int64_t e0 = edge_fn(x0, z0, x1, z1, px, pz);
      int64_t e1 = edge_fn(x1, z1, x2, z2, px, pz);
      int64_t e2 = edge_fn(x2, z2, x0, z0, px, pz);
      int in = (e0 > 0 || (e0 == 0 && o01)) && (e1 > 0 || (e1 == 0 && o12)) &&
               (e2 > 0 || (e2 == 0 && o20));
      if (in) plane[(size_t)k * W + (size_t)i] ^= 1u;
    }
  }
}

static void sort4_by_y(tv* v) {
  /* sort4Vec3ByLowerY (Tetravoxelizer.h:75-81) */
  tv t;
#define SW(a, b) if (v[a].y > v[b].y) { t = v[a]; v[a] = v[b]; v[b] = t; }
  SW(0, 1) SW(2, 3) SW(0, 2) SW(1, 3) SW(1, 2)
#undef SW
}

/* centroid of all vertices.  Summed per component in 1024 interleaved
 * lanes (lane t adds vertices t, t+1024, ... in order) followed by a
 * pairwise tree over the lanes (512, 256, ..., 1), then divided by
 * (float)n.  The reference sums sequentially (Tetravoxelizer.cpp:206-212);
 * the lane order lets the device compute the same bits in parallel. */
static void centroid_lanes(const float* V, uint32_t nv, float out[3]) {
  float (*lane)[3] = (float(*)[3])calloc(1024, sizeof(float[3]));
  for (uint32_t t = 0; t < 1024; ++t)
    for (uint64_t i = t; i < nv; i += 1024)
      for (int a = 0; a < 3; ++a) lane[t][a] = lane[t][a] + V[3 * i + a];
  for (uint32_t s = 512; s >= 1; s >>= 1)
    for (uint32_t t = 0; t < s; ++t)
      for (int a = 0; a < 3; ++a) lane[t][a] = lane[t][a] + lane[t + s][a];
  for (int a = 0; a < 3; ++a) out[a] = lane[0][a] / (float)nv;
  free(lane);
}

static void vox_parity(const float* V, uint32_t nv, const uint32_t* F,
                       uint32_t nf, uint32_t X, uint32_t Y, uint32_t Z,
                       const float* amin, const float* amax, uint8_t* par) {
  float cen[3], ctr[3], dim[3];
  centroid_lanes(V, nv, cen);
  for (int a = 0; a < 3; ++a) {
    dim[a] = amax[a] - amin[a];          /* aabb.size() */
    ctr[a] = 0.5f * (amin[a] + amax[a]); /* centerBBox */
  }
  /* scaleToNDC: 2*(v - c)/dim (Tetravoxelizer.h:70-72) */
#define NDC(dst, src)                                        \
  do {                                                       \
    float d0 = (src)[0] - ctr[0], d1 = (src)[1] - ctr[1], d2 = (src)[2] - ctr[2]; \
    (dst).x = (2.0f * d0) / dim[0];                          \
    (dst).y = (2.0f * d1) / dim[1];                          \
    (dst).z = (2.0f * d2) / dim[2];                          \
  } while (0)
  tv c;
  NDC(c, cen);
  tv* tet = (tv*)malloc(sizeof(tv) * 4 * (size_t)(nf ? nf : 1));
  for (uint32_t f = 0; f < nf; ++f) {
    for (int k = 0; k < 3; ++k) NDC(tet[4 * (size_t)f + k], V + 3 * (size_t)F[3 * f + k]);
    tet[4 * (size_t)f + 3] = c;
    sort4_by_y(tet + 4 * (size_t)f);
  }
#undef NDC
  /* slice planes: ySlice = -1, ySlice += 2/res.y per slice (float
   * accumulation, Tetravoxelizer.cpp:280-293) */
  float* ys = (float*)malloc(sizeof(float) * Y);
  float step = 2.0f / (float)Y, acc = -1.0f;
  for (uint32_t s = 0; s < Y; ++s) { ys[s] = acc; acc = acc + step; }
  const float hw = 0.5f * (float)X, hh = 0.5f * (float)Z;
#pragma omp parallel for schedule(dynamic, 1)
  for (long s = 0; s < (long)Y; ++s) {
    const float sl = ys[s];
    uint8_t* plane = par + (size_t)s * X * Z; /* [y][z][x] as glReadPixels */
    for (uint32_t f = 0; f < nf; ++f) {
      const tv* t = tet + 4 * (size_t)f;
      tv A = t[0], B = t[1], C = t[2], D = t[3];
      if (!(A.y < sl && sl <= D.y)) continue;
      float p0x, p0z, v1x, v1z, v2x, v2z;
      interp(A, D, sl, &p0x, &p0z);
      if (sl <= B.y) interp(A, B, sl, &v1x, &v1z); else interp(B, D, sl, &v1x, &v1z);
      if (sl <= C.y) interp(A, C, sl, &v2x, &v2z); else interp(C, D, sl, &v2x, &v2z);
      raster_xor(p0x, p0z, v1x, v1z, v2x, v2z, X, Z, hw, hh, plane);
      if (B.y < sl && sl <= C.y) {
        float bx, bz;
        interp(B, C, sl, &bx, &bz);
        raster_xor(bx, bz, v2x, v2z, v1x, v1z, X, Z, hw, hh, plane);
      }
    }
  }
  free(ys);
  free(tet);
}

int vfo_voxelize(const float* verts, uint32_t nverts, const uint32_t* faces,
                 uint32_t nfaces, uint32_t X, uint32_t Y, uint32_t Z,
                 const float aabb_min[3], const float aabb_max[3],
                 uint16_t* grid, int mode) {
  if (!grid || X == 0 || Y == 0 || Z == 0 || (nfaces && (!verts || !faces)))
    return VFO_ERR_INVALID;
  for (uint64_t i = 0; i < 3ull * nfaces; ++i)
    if (faces[i] >= nverts) return VFO_ERR_INVALID;
  const size_t N = (size_t)X * Y * Z;
  memset(grid, 0, N * sizeof(uint16_t));
  if (nfaces == 0) return VFO_OK;
  if (mode & 1) {
    uint8_t* shell = (uint8_t*)calloc(N, 1);
    vox_shell(verts, faces, nfaces, X, Y, Z, aabb_min, aabb_max, shell);
    for (size_t i = 0; i < N; ++i)
      if (shell[i]) grid[i] = VOXEL_FREE;
    free(shell);
  }
  if (mode & 2) {
    uint8_t* par = (uint8_t*)calloc(N, 1);
    vox_parity(verts, nverts, faces, nfaces, X, Y, Z, aabb_min, aabb_max, par);
    /* y-major GL layout -> x-major grid (RegularGrid.cpp:185-201) */
#pragma omp parallel for
    for (long y = 0; y < (long)Y; ++y)
      for (uint32_t x = 0; x < X; ++x)
        for (uint32_t z = 0; z < Z; ++z)
          if (par[((size_t)y * Z + z) * X + x] & 1u) grid[lin(x, y, z, Y, Z)] = VOXEL_FREE;
    free(par);
  }
  return VFO_OK;
}

void vfo_grid_dims(const float aabb_min[3], const float aabb_max[3],
                   uint32_t max_voxels, uint32_t dims_out[3]) {
  /* CADScene::allocateMeshGrid (CADScene.cpp:545-561) */
  float size[3];
  for (int a = 0; a < 3; ++a) size[a] = aabb_max[a] - aabb_min[a];
  float mx = fmaxf(size[0], fmaxf(size[1], size[2]));
  for (int a = 0; a < 3; ++a) {
    float v = ((float)max_voxels * size[a]) / mx;
    int d = (int)floorf(v);
    while (d % 4 != 0) ++d;
    while (d % 4 != 0 || d > (int)max_voxels) --d;
    dims_out[a] = (uint32_t)(d < 0 ? 0 : d);
  }
}

/* ------------------------------------------------------------------------ */
/* Seeder::isBoundary (RegularGrid.cpp:543-559) with neighbourhoodSize 1 */
static int is_boundary(const uint16_t* g, int x, int y, int z, uint32_t X,
                       uint32_t Y, uint32_t Z) {
  int x0 = clampi(x - 1, 0, X - 1), x1 = clampi(x + 1, 0, X - 1);
  int y0 = clampi(y - 1, 0, Y - 1), y1 = clampi(y + 1, 0, Y - 1);
  int z0 = clampi(z - 1, 0, Z - 1), z1 = clampi(z + 1, 0, Z - 1);
  for (int a = x0; a <= x1; ++a)
    for (int b = y0; b <= y1; ++b)
      for (int c = z0; c <= z1; ++c)
        if (g[lin(a, b, c, Y, Z)] == VOXEL_EMPTY) return 1;
  return 0;
}

static int cmp_xyz(const void* pa, const void* pb) {
  const uint32_t* a = (const uint32_t*)pa;
  const uint32_t* b = (const uint32_t*)pb;
  for (int i = 0; i < 3; ++i)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

/* Seeder::uniform (Seeder.cpp:154-208).  Attempt i draws
 * c = int((float)(dim-1) * U) per axis (getUniformRandomInt(0, dim-1),
 * RandomUtilities.h), U from the counter RNG at counter 3*i + axis. */
int vfo_seeder_uniform(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                       uint32_t n, uint64_t seed, int location,
                       uint32_t* out_xyzw) {
  if (n == 0) return VFO_OK;
  if (!grid || !out_xyzw || X < 2 || Y < 2 || Z < 2 || n > MAX_SEEDS ||
      location < VFO_INNER || location > VFO_BOTH)
    return VFO_ERR_INVALID;
  uint32_t cnt = 0;
  const float fx = (float)(X - 1), fy = (float)(Y - 1), fz = (float)(Z - 1);
  for (uint32_t attempt = 0; cnt != n; ++attempt) {
    if (attempt == MAX_TRIES) return VFO_ERR_SEED_SEARCH;
    int x = (int)(fx * vfo_u01(vfo_hash(seed, VFO_STREAM_SEEDS, 3ull * attempt + 0)));
    int y = (int)(fy * vfo_u01(vfo_hash(seed, VFO_STREAM_SEEDS, 3ull * attempt + 1)));
    int z = (int)(fz * vfo_u01(vfo_hash(seed, VFO_STREAM_SEEDS, 3ull * attempt + 2)));
    if (grid[lin(x, y, z, Y, Z)] == VOXEL_EMPTY) continue;
    int dup = 0;
    for (uint32_t i = 0; i < cnt && !dup; ++i)
      dup = out_xyzw[4 * i] == (uint32_t)x && out_xyzw[4 * i + 1] == (uint32_t)y &&
            out_xyzw[4 * i + 2] == (uint32_t)z;
    if (dup) continue;
    if (location != VFO_BOTH) {
      int b = is_boundary(grid, x, y, z, X, Y, Z);
      if ((location == VFO_OUTER) != (b != 0)) continue;
    }
    out_xyzw[4 * cnt] = x;
    out_xyzw[4 * cnt + 1] = y;
    out_xyzw[4 * cnt + 2] = z;
    ++cnt;
  }
  /* std::set<uvec3> order, labels 2,3,... (Seeder.cpp:198-205) */
  qsort(out_xyzw, n, 4 * sizeof(uint32_t), cmp_xyz);
  for (uint32_t i = 0; i < n; ++i) out_xyzw[4 * i + 3] = VOXEL_FREE + 1 + i;
  return VFO_OK;
}

static float seed_dist(int dfunc, const uint32_t* s, const uint32_t* f) {
  float dx = (float)s[0] - (float)f[0], dy = (float)s[1] - (float)f[1],
        dz = (float)s[2] - (float)f[2];
  switch (dfunc) {
    case VFO_EUCLIDEAN: return sqrtf(dx * dx + dy * dy + dz * dz);
    case VFO_MANHATTAN: return fabsf(dx) + fabsf(dy) + fabsf(dz);
    default: return fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)));
  }
}

/* Seeder::mergeSeeds (Seeder.cpp:115-152) */
int vfo_merge_seeds(const uint32_t* frags, uint32_t nfrags, uint32_t* seeds,
                    uint32_t nseeds, int dfunc) {
  if (nseeds == 0) return VFO_OK;
  if (nfrags == 0 || !frags || !seeds) return VFO_ERR_INVALID;
  uint32_t idf[256] = {0};
  for (uint32_t k = 0; k < nseeds; ++k) {
    float best = FLT_MAX;
    int nearest = -1;
    for (uint32_t i = 0; i < nfrags; ++i) {
      float d = seed_dist(dfunc, seeds + 4 * k, frags + 4 * i);
      if (d < best) { best = d; nearest = (int)i; }
    }
    if (nearest < 0) return VFO_ERR_INVALID;
    uint32_t w = frags[4 * nearest + 3];
    if (w > 255) return VFO_ERR_RANGE;
    uint32_t pre = ++idf[w];
    if (pre > 127) return VFO_ERR_RANGE; /* would reach the boundary bit */
    seeds[4 * k + 3] = w | (pre << 8);
  }
  return VFO_OK;
}

int vfo_fracture_seeds(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                       uint32_t n_main, uint32_t n_extra, int location,
                       int merge_dfunc, uint64_t seed, uint32_t num_impacts,
                       uint32_t bias_seeds, uint32_t bias_focus, uint32_t* out,
                       uint32_t* nout) {
  if (n_main > 254) return VFO_ERR_RANGE; /* 8-bit fragment ids 2..255 */
  const uint32_t bias = num_impacts ? bias_seeds : 0u;
  if ((uint64_t)2 * (n_main + bias) + n_extra > MAX_SEEDS) return VFO_ERR_RANGE;
  int st = vfo_seeder_uniform(grid, X, Y, Z, n_main, seed, location, out);
  if (st) return st;
  if (num_impacts && n_main && bias_seeds) {
    /* CADScene.cpp:636-638: seeds = nearSeeds(seeds, numImpacts, biasSeeds,
     * biasFocus); the placed seeds become main seeds */
    uint32_t* tmp = (uint32_t*)malloc(4 * sizeof(uint32_t) * (size_t)(n_main + bias_seeds));
    if (!tmp) return VFO_ERR_RANGE;
    uint32_t nn = 0;
    st = vfo_near_seeds(grid, X, Y, Z, out, n_main, num_impacts, bias_seeds, bias_focus, seed, tmp, &nn);
    if (!st) {
      memcpy(out, tmp, 4 * sizeof(uint32_t) * (size_t)nn);
      n_main = nn;
    }
    free(tmp);
    if (st) return st;
    if (n_main > 254) return VFO_ERR_RANGE;
  }
  uint32_t total = n_main;
  if (n_extra > 0 && n_main > 0) {
    /* extraSeeds = uniform(BOTH); insert(begin, seeds); mergeSeeds(seeds,
     * extraSeeds); seeds.insert(end, extraSeeds) (CADScene.cpp:647-655).
     * The extra draw uses the derived seed value seed + golden ratio. */
    uint32_t* list = out + 4 * (size_t)n_main;
    memcpy(list, out, 4 * sizeof(uint32_t) * n_main);
    st = vfo_seeder_uniform(grid, X, Y, Z, n_extra, seed + 0x9E3779B97F4A7C15ull,
                            VFO_BOTH, list + 4 * (size_t)n_main);
    if (st) return st;
    st = vfo_merge_seeds(out, n_main, list, n_main + n_extra, merge_dfunc);
    if (st) return st;
    total = 2 * n_main + n_extra;
  }
  if (nout) *nout = total;
  return VFO_OK;
}

/* ------------------------------------------------------------------------ */
/* Neighbourhoods: VON_NEUMANN (6) and MOORE (26), FloodFracturer.cpp:8-27.
 * Manhattan uses 6, Euclidean and Chebyshev use 26 (FloodFracturer.cpp:114).
 */
static const int VN[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static int MOORE_N[26][3];
static void init_moore(void) {
  int k = 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c)
        if (a || b || c) { MOORE_N[k][0] = a; MOORE_N[k][1] = b; MOORE_N[k][2] = c; ++k; }
}

/* FloodFracturer::build (FloodFracturer.cpp:98-191) with the kernels
 * floodFracturer-comp.glsl:24-64, disjointSet-comp.glsl:17-24,
 * disjointSetStack-comp.glsl:20-37 and undoMask-comp.glsl:25-29.
 *
 * Deterministic restatement: each BFS wave is evaluated against the grid as
 * it was at the start of the wave (Jacobi).  A FREE voxel adjacent to
 * several frontier voxels takes the claim of the one with the lowest seed
 * index (first pass) or the lowest 16-bit label (re-flood passes after the
 * disjoint cleanup); the reference leaves this to the last writer.  The
 * sub-seed prefix competition (glsl:49-62) lets the lower prefix of the same
 * fragment overwrite the higher one; several proposals on one voxel take
 * the lowest.  Seeds that share a voxel: the later seed in the list wins,
 * as grid.set in list order does (FloodFracturer.cpp:101-103). */
int vfo_flood(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
              const uint32_t* seeds, uint32_t nseeds, int dfunc,
              uint32_t* waves_out) {
  if (!grid || X == 0 || Y == 0 || Z == 0 || nseeds > MAX_SEEDS ||
      (nseeds && !seeds))
    return VFO_ERR_INVALID;
  init_moore();
  const size_t N = (size_t)X * Y * Z;
  const int nn = dfunc == VFO_MANHATTAN ? 6 : 26;
  const int(*off)[3] = dfunc == VFO_MANHATTAN ? VN : (const int(*)[3])MOORE_N;
  for (uint32_t i = 0; i < nseeds; ++i) {
    if (seeds[4 * i] >= X || seeds[4 * i + 1] >= Y || seeds[4 * i + 2] >= Z)
      return VFO_ERR_INVALID;
    /* a label is frag | prefix << 8 (Seeder.cpp:150): its fragment id (low
     * byte) is a label itself, >= 2; the reference never makes others */
    if (seeds[4 * i + 3] > 0x7FFF || (seeds[4 * i + 3] & 0xFFu) <= VOXEL_FREE) return VFO_ERR_INVALID;
  }
  /* homogenize (RegularGrid.cpp:533-541) */
  for (size_t i = 0; i < N; ++i)
    if (grid[i] != VOXEL_EMPTY) grid[i] = VOXEL_FREE;
  int32_t* rank = (int32_t*)malloc(N * sizeof(int32_t));
  uint64_t* prop = (uint64_t*)malloc(N * sizeof(uint64_t));
  uint8_t* mark = (uint8_t*)calloc(N, 1);
  size_t* cur = (size_t*)malloc(N * sizeof(size_t));
  size_t* nxt = (size_t*)malloc(N * sizeof(size_t));
  size_t* touched = (size_t*)malloc(N * sizeof(size_t));
  if (!rank || !prop || !mark || !cur || !nxt || !touched) {
    free(rank); free(prop); free(mark); free(cur); free(nxt); free(touched);
    return VFO_ERR_INVALID;
  }
  for (size_t i = 0; i < N; ++i) { rank[i] = INT32_MAX; prop[i] = UINT64_MAX; }
  size_t ncur = 0;
  for (uint32_t i = 0; i < nseeds; ++i) {
    size_t v = lin(seeds[4 * i], seeds[4 * i + 1], seeds[4 * i + 2], Y, Z);
    grid[v] = (uint16_t)seeds[4 * i + 3];
    rank[v] = (int32_t)i;
    if (!mark[v]) { mark[v] = 1; cur[ncur++] = v; }
  }
  for (size_t i = 0; i < ncur; ++i) mark[cur[i]] = 0;
  uint32_t waves = 0;
  for (int pass = 0;; ++pass) {
    while (ncur > 0) {
      size_t ntouched = 0;
      for (size_t q = 0; q < ncur; ++q) {
        size_t f = cur[q];
        int fx = (int)(f / ((size_t)Y * Z)), fy = (int)((f / Z) % Y), fz = (int)(f % Z);
        uint16_t gf = grid[f];
        for (int o = 0; o < nn; ++o) {
          int x = fx + off[o][0], y = fy + off[o][1], z = fz + off[o][2];
          if (x < 0 || y < 0 || z < 0 || x >= (int)X || y >= (int)Y || z >= (int)Z) continue;
          size_t n = lin(x, y, z, Y, Z);
          uint16_t gn = grid[n];
          uint64_t key;
          size_t tgt;
          if (gn == VOXEL_FREE) {
            key = ((uint64_t)(uint32_t)rank[f] << 16) | gf;
            tgt = n;
          } else if ((gn & 0xFFu) == (gf & 0xFFu)) {
            uint16_t pf = gf >> 8, pn = gn >> 8;
            if (pf > pn) { key = gn; tgt = f; }
            else if (pn > pf) { key = gf; tgt = n; }
            else continue;
          } else {
            continue;
          }
          if (prop[tgt] == UINT64_MAX) touched[ntouched++] = tgt;
          if (key < prop[tgt]) prop[tgt] = key;
        }
      }
      size_t nnext = 0;
      for (size_t q = 0; q < ntouched; ++q) {
        size_t v = touched[q];
        uint64_t key = prop[v];
        prop[v] = UINT64_MAX;
        if (grid[v] == VOXEL_FREE) {
          grid[v] = (uint16_t)(key & 0xFFFFu);
          rank[v] = (int32_t)(key >> 16);
        } else {
          grid[v] = (uint16_t)(key & 0xFFFFu);
        }
        nxt[nnext++] = v;
      }
      size_t* t = cur; cur = nxt; nxt = t;
      ncur = nnext;
      ++waves;
    }
    /* disjointSet: per-fragment minimum prefix; disjointSetStack: the rest
     * go back to FREE, the survivors become the next frontier */
    uint32_t minp[256];
    for (int i = 0; i < 256; ++i) minp[i] = UINT32_MAX;
    for (size_t v = 0; v < N; ++v)
      if (grid[v] > VOXEL_FREE) {
        uint32_t fr = grid[v] & 0xFFu, p = grid[v] >> 8;
        if (p < minp[fr]) minp[fr] = p;
      }
    size_t disjoint = 0;
    ncur = 0;
    for (size_t v = 0; v < N; ++v)
      if (grid[v] > VOXEL_FREE) {
        if ((uint32_t)(grid[v] >> 8) != minp[grid[v] & 0xFFu]) {
          grid[v] = VOXEL_FREE;
          ++disjoint;
        } else {
          cur[ncur++] = v;
          rank[v] = grid[v]; /* re-flood ties: lowest label */
        }
      }
    if (disjoint == 0) break;
  }
  /* undoMask(unmaskRightMost): value & 0xFF (FloodFracturer.cpp:180-186) */
  for (size_t v = 0; v < N; ++v) grid[v] &= 0xFFu;
  free(rank); free(prop); free(mark); free(cur); free(nxt); free(touched);
  if (waves_out) *waves_out = waves;
  return VFO_OK;
}

/* NaiveFracturer::buildCPU (NaiveFracturer.cpp:26-68): nearest seed, strict
 * '<' so the lowest seed index wins ties; Euclidean = sqrt in float. */
int vfo_naive(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
              const uint32_t* seeds, uint32_t nseeds, int dfunc) {
  if (!grid || (nseeds && !seeds)) return VFO_ERR_INVALID;
#pragma omp parallel for
  for (long x = 0; x < (long)X; ++x)
    for (uint32_t y = 0; y < Y; ++y)
      for (uint32_t z = 0; z < Z; ++z) {
        size_t v = lin(x, y, z, Y, Z);
        if (grid[v] == VOXEL_EMPTY) continue;
        float best = FLT_MAX;
        for (uint32_t s = 0; s < nseeds; ++s) {
          int dx = (int)x - (int)seeds[4 * s], dy = (int)y - (int)seeds[4 * s + 1],
              dz = (int)z - (int)seeds[4 * s + 2];
          float d;
          if (dfunc == VFO_EUCLIDEAN) {
            float fx = (float)dx, fy = (float)dy, fz = (float)dz;
            d = sqrtf(fx * fx + fy * fy + fz * fz);
          } else if (dfunc == VFO_MANHATTAN) {
            d = (float)(abs(dx) + abs(dy) + abs(dz));
          } else {
            int m = abs(dx) > abs(dy) ? abs(dx) : abs(dy);
            d = (float)(m > abs(dz) ? m : abs(dz));
          }
          if (d < best) { best = d; grid[v] = (uint16_t)seeds[4 * s + 3]; }
        }
      }
  return VFO_OK;
}

/* ------------------------------------------------------------------------ */
/* Boundary perturbation.  The reference has no such step (its only noise
 * is the erosion gate, erodeGrid-comp.glsl:34).  Definition used here:
 * per labelled voxel v, a 3-channel trilinear value noise n(v/P) in
 * [-1,1) from lattice values L = 2*U - 1 (counter RNG, stream NOISE,
 * counter ((ix<<40)|(iy<<20)|iz)*4 + channel), offset
 * o = floor(A*n + 0.5) per axis; v takes the label at v+o when that voxel
 * is inside the grid and labelled (>1), else keeps its own.  All reads come
 * from the unperturbed grid. */
static float lattice(uint64_t seed, uint32_t ix, uint32_t iy, uint32_t iz, int c) {
  uint64_t ctr = (((uint64_t)ix << 40) | ((uint64_t)iy << 20) | iz) * 4u + (uint64_t)c;
  return vfo_u01(vfo_hash(seed, VFO_STREAM_NOISE, ctr)) * 2.0f - 1.0f;
}
static inline float lerpf_(float a, float b, float t) {
  float d = b - a;
  float m = t * d;
  return a + m;
}
int vfo_perturb(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                float amplitude, uint32_t period, uint64_t seed) {
  if (!grid || period == 0 || !(amplitude >= 0.0f) || amplitude > 64.0f)
    return VFO_ERR_INVALID;
  const size_t N = (size_t)X * Y * Z;
  uint16_t* src = (uint16_t*)malloc(N * sizeof(uint16_t));
  memcpy(src, grid, N * sizeof(uint16_t));
  const float fp = (float)period;
#pragma omp parallel for
  for (long x = 0; x < (long)X; ++x)
    for (uint32_t y = 0; y < Y; ++y)
      for (uint32_t z = 0; z < Z; ++z) {
        size_t v = lin(x, y, z, Y, Z);
        if (src[v] <= VOXEL_FREE) continue;
        uint32_t c[3] = {(uint32_t)x, y, z}, i[3];
        float t[3];
        for (int a = 0; a < 3; ++a) {
          i[a] = c[a] / period;
          t[a] = (float)(c[a] % period) / fp;
        }
        int o[3];
        for (int ch = 0; ch < 3; ++ch) {
          float c000 = lattice(seed, i[0], i[1], i[2], ch), c001 = lattice(seed, i[0], i[1], i[2] + 1, ch);
          float c010 = lattice(seed, i[0], i[1] + 1, i[2], ch), c011 = lattice(seed, i[0], i[1] + 1, i[2] + 1, ch);
          float c100 = lattice(seed, i[0] + 1, i[1], i[2], ch), c101 = lattice(seed, i[0] + 1, i[1], i[2] + 1, ch);
          float c110 = lattice(seed, i[0] + 1, i[1] + 1, i[2], ch), c111 = lattice(seed, i[0] + 1, i[1] + 1, i[2] + 1, ch);
          float c00 = lerpf_(c000, c001, t[2]), c01 = lerpf_(c010, c011, t[2]);
          float c10 = lerpf_(c100, c101, t[2]), c11 = lerpf_(c110, c111, t[2]);
          float c0 = lerpf_(c00, c01, t[1]), c1 = lerpf_(c10, c11, t[1]);
          float n = lerpf_(c0, c1, t[0]);
          float s = amplitude * n;
          o[ch] = (int)floorf(s + 0.5f);
        }
        long ux = x + o[0], uy = (long)y + o[1], uz = (long)z + o[2];
        if (ux < 0 || uy < 0 || uz < 0 || ux >= (long)X || uy >= (long)Y || uz >= (long)Z) continue;
        uint16_t g = src[lin(ux, uy, uz, Y, Z)];
        if (g > VOXEL_FREE) grid[v] = g;
      }
  free(src);
  return VFO_OK;
}

/* RegularGrid::detectBoundaries (RegularGrid.cpp:64-80) +
 * detectBoundaries-comp.glsl:18-43.  The shader updates in place, but every
 * neighbour read clears bit 15 first, so reading a snapshot is the same. */
void vfo_detect_boundaries(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                           int b) {
  const size_t N = (size_t)X * Y * Z;
  uint16_t* src = (uint16_t*)malloc(N * sizeof(uint16_t));
  memcpy(src, grid, N * sizeof(uint16_t));
#pragma omp parallel for
  for (long x = 0; x < (long)X; ++x)
    for (int y = 0; y < (int)Y; ++y)
      for (int z = 0; z < (int)Z; ++z) {
        size_t v = lin(x, y, z, Y, Z);
        uint16_t g = src[v];
        if (g <= VOXEL_FREE) continue;
        int x0 = clampi(x - b, 0, X - 1), x1 = clampi(x + b, 0, X - 1);
        int y0 = clampi(y - b, 0, Y - 1), y1 = clampi(y + b, 0, Y - 1);
        int z0 = clampi(z - b, 0, Z - 1), z1 = clampi(z + b, 0, Z - 1);
        int bd = 0;
        for (int a = x0; a <= x1 && !bd; ++a)
          for (int c = y0; c <= y1 && !bd; ++c)
            for (int d = z0; d <= z1 && !bd; ++d) {
              uint16_t u = src[lin(a, c, d, Y, Z)] & 0x7FFFu;
              bd = u > VOXEL_FREE && u != g;
            }
        if (bd) grid[v] = g | 0x8000u;
      }
  free(src);
}

/* removeIsolatedRegionsGrid-comp.glsl:16-39: a voxel with fewer than 6
 * equal values among its clamped 26-neighbourhood becomes EMPTY.  The shader
 * runs in place (racy); this reads a snapshot (Jacobi). */
void vfo_remove_isolated(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z) {
  const size_t N = (size_t)X * Y * Z;
  uint16_t* src = (uint16_t*)malloc(N * sizeof(uint16_t));
  memcpy(src, grid, N * sizeof(uint16_t));
#pragma omp parallel for
  for (long x = 0; x < (long)X; ++x)
    for (int y = 0; y < (int)Y; ++y)
      for (int z = 0; z < (int)Z; ++z) {
        size_t v = lin(x, y, z, Y, Z);
        int count = -1;
        int x0 = clampi(x - 1, 0, X - 1), x1 = clampi(x + 1, 0, X - 1);
        int y0 = clampi(y - 1, 0, Y - 1), y1 = clampi(y + 1, 0, Y - 1);
        int z0 = clampi(z - 1, 0, Z - 1), z1 = clampi(z + 1, 0, Z - 1);
        for (int a = x0; a <= x1; ++a)
          for (int c = y0; c <= y1; ++c)
            for (int d = z0; d <= z1; ++d) count += src[lin(a, c, d, Y, Z)] == src[v];
        if (count < 6) grid[v] = VOXEL_EMPTY;
      }
  free(src);
}

/* RegularGrid::erode (RegularGrid.cpp:82-159) + erodeGrid-comp.glsl:26-59 +
 * copyGrid + removeIsolatedRegions.  Quirks kept: the gate
 * bool(unmaskedBit(v, 15)) holds for every labelled voxel; equality
 * compares all 16 bits; activations is normalised by k^3; globalCount is the
 * clamped window size.  The noise buffer (1e6 uniform floats) comes from
 * the counter RNG, stream ERODE, counter j. */
int vfo_erode(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, int type,
              uint32_t k, uint32_t iterations, float probability,
              float threshold, uint64_t seed) {
  if (!grid || k == 0 || k > 15 || type < VFO_SQUARE || type > VFO_CROSS) return VFO_ERR_INVALID;
  if (!(k % 2)) ++k;
  const uint32_t msz = k * k * k;
  const int cc = (int)floorf((float)k / 2.0f);
  float* mask = (float*)calloc(msz, sizeof(float));
  float activations = 0.0f;
  if (type == VFO_SQUARE) {
    for (uint32_t i = 0; i < msz; ++i) mask[i] = 1.0f;
    activations = (float)msz;
  } else if (type == VFO_CROSS) {
    for (uint32_t x = 0; x < k; ++x) mask[x * k * k + cc * k + cc] = 1.0f;
    for (uint32_t y = 0; y < k; ++y) mask[cc * k * k + y * k + cc] = 1.0f;
    for (uint32_t z = 0; z < k; ++z) mask[cc * k * k + cc * k + z] = 1.0f;
    activations = 1.0f / 3.0f * (float)msz;
  } else {
    for (uint32_t x = 0; x < k; ++x)
      for (uint32_t y = 0; y < k; ++y)
        for (uint32_t z = 0; z < k; ++z) {
          float dx = (float)x - (float)cc, dy = (float)y - (float)cc, dz = (float)z - (float)cc;
          float d = sqrtf(dx * dx + dy * dy + dz * dz);
          if (d < (float)cc + FLT_EPSILON) {
            mask[x * k * k + y * k + z] = 1.0f;
            activations = activations + 1.0f;
          }
        }
  }
  activations = activations / (float)msz;
  const float limit = activations * threshold;
  float* noise = (float*)malloc(sizeof(float) * NOISE_BUFFER);
  for (uint32_t j = 0; j < NOISE_BUFFER; ++j) noise[j] = vfo_u01(vfo_hash(seed, VFO_STREAM_ERODE, j));
  const size_t N = (size_t)X * Y * Z;
  uint16_t* src = (uint16_t*)malloc(N * sizeof(uint16_t));
  const int m2 = (int)floorf((float)k / 2.0f);
  for (uint32_t it = 0; it < iterations; ++it) {
    vfo_detect_boundaries(grid, X, Y, Z, 1);
    memcpy(src, grid, N * sizeof(uint16_t));
#pragma omp parallel for
    for (long x = 0; x < (long)X; ++x)
      for (int y = 0; y < (int)Y; ++y)
        for (int z = 0; z < (int)Z; ++z) {
          size_t v = lin(x, y, z, Y, Z);
          uint16_t g = src[v];
          if (!(g > VOXEL_FREE && (g & 0x7FFFu) != 0 && noise[v % NOISE_BUFFER] < probability)) continue;
          int mnx = (int)x - m2, mny = y - m2, mnz = z - m2;
          int x0 = clampi(mnx, 0, X - 1), x1 = clampi((int)x + m2, 0, X - 1);
          int y0 = clampi(mny, 0, Y - 1), y1 = clampi(y + m2, 0, Y - 1);
          int z0 = clampi(mnz, 0, Z - 1), z1 = clampi(z + m2, 0, Z - 1);
          uint32_t count = 0, global = 0;
          for (int a = x0; a <= x1; ++a)
            for (int c = y0; c <= y1; ++c)
              for (int d = z0; d <= z1; ++d) {
                float m = mask[(a - mnx) * k * k + (c - mny) * k + (d - mnz)];
                count += (uint32_t)((float)(src[lin(a, c, d, Y, Z)] == g) * m);
                ++global;
              }
          float act = (float)count / (float)global;
          if (act < limit) grid[v] = VOXEL_EMPTY;
        }
  }
  vfo_remove_isolated(grid, X, Y, Z);
  free(src);
  free(noise);
  free(mask);
  return VFO_OK;
}

/* RegularGrid::undoMask (RegularGrid.cpp:488-503): clear bit 15 */
void vfo_undo_mask(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z) {
  const size_t N = (size_t)X * Y * Z;
  for (size_t i = 0; i < N; ++i) grid[i] &= 0x7FFFu;
}

int vfo_count_values(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                     uint32_t* counts, uint32_t ncounts, uint64_t* occupied) {
  const size_t N = (size_t)X * Y * Z;
  if (counts) memset(counts, 0, sizeof(uint32_t) * ncounts);
  uint64_t occ = 0;
  int st = VFO_OK;
  for (size_t i = 0; i < N; ++i)
    if (grid[i] > VOXEL_FREE) {
      uint32_t v = grid[i] & 0x7FFFu;
      ++occ;
      if (v < ncounts) { if (counts) ++counts[v]; }
      else st = VFO_ERR_RANGE;
    }
  if (occupied) *occupied = occ;
  return st;
}

int vfo_run_job(const float* verts, uint32_t nverts, const uint32_t* faces,
                uint32_t nfaces, uint32_t X, uint32_t Y, uint32_t Z,
                const float aabb_min[3], const float aabb_max[3],
                const vfo_params* p, uint16_t* grid, uint32_t* counts,
                uint32_t ncounts, uint32_t* seeds_out, uint32_t* nseeds_out) {
  int st = vfo_voxelize(verts, nverts, faces, nfaces, X, Y, Z, aabb_min, aabb_max, grid, 3);
  if (st) return st;
  const uint32_t bias = p->num_impacts > 0 ? (uint32_t)p->bias_seeds : 0u;
  uint32_t cap = 2 * ((uint32_t)p->num_seeds + bias) + (uint32_t)p->num_extra_seeds;
  uint32_t* seeds = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (cap ? cap : 1));
  uint32_t ns = 0;
  st = vfo_fracture_seeds(grid, X, Y, Z, (uint32_t)p->num_seeds,
                          (uint32_t)p->num_extra_seeds, p->seed_location,
                          p->merge_distance, p->seed, (uint32_t)(p->num_impacts > 0 ? p->num_impacts : 0),
                          (uint32_t)p->bias_seeds, (uint32_t)p->bias_focus, seeds, &ns);
  if (!st) {
    if (p->algorithm == VFO_FLOOD) st = vfo_flood(grid, X, Y, Z, seeds, ns, p->distance, NULL);
    else if (p->algorithm == VFO_NAIVE) st = vfo_naive(grid, X, Y, Z, seeds, ns, p->distance);
    else st = VFO_ERR_INVALID;
  }
  if (!st && p->noise_amplitude > 0.0f)
    st = vfo_perturb(grid, X, Y, Z, p->noise_amplitude, p->noise_period, p->seed);
  if (!st) {
    if (p->erode)
      st = vfo_erode(grid, X, Y, Z, p->erosion_type, (uint32_t)p->erosion_size,
                     (uint32_t)p->erosion_iterations, p->erosion_probability,
                     p->erosion_threshold, p->seed);
    else
      vfo_detect_boundaries(grid, X, Y, Z, p->boundary_size);
  }
  if (!st && counts) st = vfo_count_values(grid, X, Y, Z, counts, ncounts, NULL);
  if (seeds_out && !st) memcpy(seeds_out, seeds, sizeof(uint32_t) * 4 * ns);
  if (nseeds_out) *nseeds_out = ns;
  free(seeds);
  return st;
}

size_t vfo_rle_encode(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z,
                      uint8_t* out, size_t cap) {
  /* RegularGrid::exportRLE (RegularGrid.cpp:672-714): uvec3 dims, then
   * {u16 value, u32 repetitions} runs over the x-major grid, little endian */
  const size_t N = (size_t)X * Y * Z;
  size_t pos = 0;
#define PUT(byte) do { if (out && pos < cap) out[pos] = (uint8_t)(byte); ++pos; } while (0)
  uint32_t d[3] = {X, Y, Z};
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 4; ++b) PUT(d[a] >> (8 * b));
  size_t i = 0;
  while (i < N) {
    uint16_t v = grid[i];
    size_t j = i;
    while (j < N && grid[j] == v && j - i < 0xFFFFFFFFu) ++j;
    uint32_t r = (uint32_t)(j - i);
    PUT(v); PUT(v >> 8);
    for (int b = 0; b < 4; ++b) PUT(r >> (8 * b));
    i = j;
  }
#undef PUT
  return pos;
}
