/*
 * vf_oracle_mesh.c -- CPU oracle of RegularGrid::toTriangleMesh
 * (RegularGrid.cpp:443-486): one marching-cubes mesh per fragment value,
 * with vertex fusion and Laplacian smoothing (MarchingCubes.cpp:364-436,
 * 480-510; marchingCubes-comp.glsl, findSameVertices_01/02-comp.glsl,
 * buildMarchingCubesFaces-comp.glsl, markBoundaryTriangles-comp.glsl,
 * laplacianSmoothing-comp.glsl, finishLaplacianSmoothing-comp.glsl).
 *
 * TEST INFRASTRUCTURE ONLY (see vf_oracle.h).
 *
 * What the reference does, per fragment value v (ascending):
 *  - the grid is copied into a lattice padded by one FREE voxel on every
 *    side (MarchingCubes::setGrid, MarchingCubes.cpp:512-530);
 *  - every lattice point c with c.x > 0, c.y < Yp-1, c.z < Zp-1 marches one
 *    cell whose corners are c + VF_MC_CORNER[i]; corner i is "outside" (bit
 *    i of the configuration) when its label without bit 15 differs from v
 *    (marchingCubes-comp.glsl:105-120); the field is 0/1 and the isolevel
 *    0.5, so every vertex is the exact midpoint of its edge (findVertex,
 *    :72-89); triangle t of the case table is emitted as edges (3t, 3t+2,
 *    3t+1) with w = bit 15 of the voxel at c (:140-156);
 *  - vertices with equal positions are fused (Morton sort + run merge,
 *    MarchingCubes.cpp:420-475) and moved into the grid's box by
 *    translate(-s) * translate(min) * scale(s), s = aabb.size() / dims
 *    (RegularGrid.cpp:478-480), applied as s*p + (min - s);
 *  - face w = max of its vertices' w (markBoundaryTriangles-comp.glsl);
 *  - smoothSurface runs nb_iters Jacobi iterations over the non-boundary
 *    vertices (faces whose three vertices have w == 0), then b_iters over
 *    the boundary vertices (all faces): every face adds each vertex's
 *    position, truncated to int32 after *10000, to its two other vertices
 *    with int32 atomics and 1 to their counts; a vertex of the target type
 *    with a count moves to mix(p, sum / count / 10000, weight).
 *
 * Deterministic rules fixed here (the reference leaves them to GPU atomics):
 *  - vertex order within a mesh: by the fragment voxel the vertex's edge
 *    leaves (x-major), then by the edge's direction -x,+x,-y,+y,-z,+z;
 *  - face order: by marched cell (x-major lattice order), then by the
 *    triangle's place in the case table;
 *  - a fused vertex's w is 1 when any triangle using it has w 1 (the
 *    reference keeps the w of whichever copy its sort leaves first);
 *  - the affine map and mix() round every product and sum separately
 *    (mix(a, b, t) = a*(1-t) + b*t, the GLSL definition).
 * The fusion here is exact; the reference's Morton codes keep 10 bits per
 * axis, so on lattices wider than 512 two positions can share a code and its
 * run merge can then leave duplicates.
 */
#include <stdlib.h>
#include <string.h>

#include "vf_oracle.h"
#include "../voxelfragmentml_gb300/csrc/vf_mc_table.h"

#define VOXEL_FREE 1u

static int mc_tri[256][16];
static int mc_ntri[256];
static int mc_ready;

static void mc_init(void) {
  if (mc_ready) return;
  for (int c = 0; c < 256; ++c) {
    const char* s = VF_MC_TRIANGLES[c];
    int n = 0;
    for (; s[n]; ++n) {
      const char ch = s[n];
      mc_tri[c][n] = ch <= '9' ? ch - '0' : ch - 'a' + 10;
    }
    mc_ntri[c] = n / 3;
  }
  mc_ready = 1;
}

/* label of padded lattice point (i, j, k): the grid voxel (i-1, j-1, k-1),
 * FREE outside it (MarchingCubes.cpp:512-530) */
static inline uint16_t lat(const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, int64_t i,
                           int64_t j, int64_t k) {
  if (i < 1 || j < 1 || k < 1 || i > (int64_t)X || j > (int64_t)Y || k > (int64_t)Z)
    return (uint16_t)VOXEL_FREE;
  return g[((size_t)(i - 1) * Y + (size_t)(j - 1)) * Z + (size_t)(k - 1)];
}

/* float -> int32 like the GPU conversion: toward zero, saturating, NaN -> 0 */
static inline int32_t f2i_rz(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

typedef struct {
  uint16_t value;
  uint32_t nv, nt;
  float* v;     /* 4 per vertex */
  uint32_t* f;  /* 4 per face */
} mmesh;

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y);
}

static uint32_t find_key(const uint64_t* keys, uint32_t n, uint64_t k) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (keys[mid] < k) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* owner key of the vertex on the edge between lattice points A and B (one of
 * them carries v): the grid voxel with label v and the direction to the other */
static uint64_t edge_key(const int64_t A[3], const int64_t B[3], int a_is_v, uint32_t Y,
                         uint32_t Z) {
  const int64_t* o = a_is_v ? A : B;
  const int64_t* t = a_is_v ? B : A;
  int dir = 0;
  for (int ax = 0; ax < 3; ++ax)
    if (t[ax] != o[ax]) dir = 2 * ax + (t[ax] > o[ax]);
  const uint64_t lin = ((uint64_t)(o[0] - 1) * Y + (uint64_t)(o[1] - 1)) * Z + (uint64_t)(o[2] - 1);
  return lin * 6u + (uint64_t)dir;
}

static void smooth(mmesh* m, uint32_t iters, float weight, int boundary) {
  const uint32_t nv = m->nv, nt = m->nt;
  if (!nv || !iters) return;
  int32_t* acc = (int32_t*)calloc((size_t)nv * 4, sizeof(int32_t));
  const float target = boundary ? 1.0f : 0.0f;
  const float omw = 1.0f - weight;
  for (uint32_t it = 0; it < iters; ++it) {
    memset(acc, 0, (size_t)nv * 4 * sizeof(int32_t));
    for (uint32_t t = 0; t < nt; ++t) {
      const uint32_t* f = m->f + 4 * (size_t)t;
      int valid = 1;
      if (!boundary)
        for (int i = 0; i < 3 && valid; ++i) valid = m->v[4 * (size_t)f[i] + 3] == target;
      if (!valid) continue;
      for (int i = 0; i < 3; ++i) {
        const float* p = m->v + 4 * (size_t)f[i];
        const int32_t q[3] = {f2i_rz(p[0] * 10000.0f), f2i_rz(p[1] * 10000.0f),
                              f2i_rz(p[2] * 10000.0f)};
        const uint32_t i1 = f[(i + 1) % 3], i2 = f[(i + 2) % 3];
        for (int a = 0; a < 3; ++a) {
          acc[4 * (size_t)i1 + a] = (int32_t)((uint32_t)acc[4 * (size_t)i1 + a] + (uint32_t)q[a]);
          acc[4 * (size_t)i2 + a] = (int32_t)((uint32_t)acc[4 * (size_t)i2 + a] + (uint32_t)q[a]);
        }
        acc[4 * (size_t)i1 + 3] += 1;
        acc[4 * (size_t)i2 + 3] += 1;
      }
    }
    for (uint32_t i = 0; i < nv; ++i) {
      float* p = m->v + 4 * (size_t)i;
      const int32_t* a = acc + 4 * (size_t)i;
      if (p[3] != target || a[3] <= 0) continue;
      const float cnt = (float)a[3];
      for (int ax = 0; ax < 3; ++ax) {
        const float avg = ((float)a[ax] / cnt) / 10000.0f;
        p[ax] = p[ax] * omw + avg * weight;
      }
    }
  }
  free(acc);
}

/* the mesh of one fragment value; returns 0 or VFO_ERR_RANGE (allocation) */
static int mesh_one(const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, uint16_t v,
                    const int64_t lo[3], const int64_t hi[3], const float s[3], const float c0[3],
                    uint32_t nb_iters, float nb_weight, uint32_t b_iters, float b_weight,
                    mmesh* out) {
  /* pass 1: triangles as owner keys, in marched-cell order */
  size_t cap = 1024, nt = 0;
  uint64_t* tk = (uint64_t*)malloc(cap * 3 * sizeof(uint64_t));
  uint32_t* tw = (uint32_t*)malloc(cap * sizeof(uint32_t));
  if (!tk || !tw) { free(tk); free(tw); return VFO_ERR_RANGE; }
  /* cells whose corners can carry v: lattice points c with c.x in
   * [lo.x, hi.x+1], c.y in [lo.y-1, hi.y], c.z in [lo.z-1, hi.z] (lo/hi:
   * the value's lattice box), clipped to the marched range */
  const int64_t Xp = (int64_t)X + 2, Yp = (int64_t)Y + 2, Zp = (int64_t)Z + 2;
  const int64_t x0 = lo[0] > 1 ? lo[0] : 1, x1 = hi[0] + 1 < Xp - 1 ? hi[0] + 1 : Xp - 1;
  const int64_t y0 = lo[1] - 1 > 0 ? lo[1] - 1 : 0, y1 = hi[1] < Yp - 2 ? hi[1] : Yp - 2;
  const int64_t z0 = lo[2] - 1 > 0 ? lo[2] - 1 : 0, z1 = hi[2] < Zp - 2 ? hi[2] : Zp - 2;
  for (int64_t cx = x0; cx <= x1; ++cx)
    for (int64_t cy = y0; cy <= y1; ++cy)
      for (int64_t cz = z0; cz <= z1; ++cz) {
        int64_t P[8][3];
        int in[8];
        int conf = 0;
        for (int i = 0; i < 8; ++i) {
          P[i][0] = cx + VF_MC_CORNER[i][0];
          P[i][1] = cy + VF_MC_CORNER[i][1];
          P[i][2] = cz + VF_MC_CORNER[i][2];
          in[i] = (uint16_t)(lat(g, X, Y, Z, P[i][0], P[i][1], P[i][2]) & 0x7FFFu) == v;
          if (!in[i]) conf |= 1 << i;
        }
        const int n = mc_ntri[conf];
        if (!n) continue;
        const uint32_t w = (uint32_t)(lat(g, X, Y, Z, cx, cy, cz) >> 15);
        for (int t = 0; t < n; ++t) {
          if (nt == cap) {
            cap *= 2;
            uint64_t* k2 = (uint64_t*)realloc(tk, cap * 3 * sizeof(uint64_t));
            uint32_t* w2 = (uint32_t*)realloc(tw, cap * sizeof(uint32_t));
            if (k2) tk = k2;
            if (w2) tw = w2;
            if (!k2 || !w2) { free(tk); free(tw); return VFO_ERR_RANGE; }
          }
          static const int order[3] = {0, 2, 1};
          for (int j = 0; j < 3; ++j) {
            const int e = mc_tri[conf][3 * t + order[j]];
            const int a = VF_MC_EDGE[e][0], b = VF_MC_EDGE[e][1];
            tk[3 * nt + j] = edge_key(P[a], P[b], in[a], Y, Z);
          }
          tw[nt] = w;
          ++nt;
        }
      }
  /* pass 2: fusion -- one vertex per distinct position (owner key) */
  uint64_t* keys = (uint64_t*)malloc((nt * 3 + 1) * sizeof(uint64_t));
  if (!keys) { free(tk); free(tw); return VFO_ERR_RANGE; }
  memcpy(keys, tk, nt * 3 * sizeof(uint64_t));
  qsort(keys, nt * 3, sizeof(uint64_t), cmp_u64);
  size_t nv = 0;
  for (size_t i = 0; i < nt * 3; ++i)
    if (!i || keys[i] != keys[i - 1]) keys[nv++] = keys[i];
  out->value = v;
  out->nv = (uint32_t)nv;
  out->nt = (uint32_t)nt;
  out->v = (float*)calloc(nv * 4 + 4, sizeof(float));
  out->f = (uint32_t*)calloc(nt * 4 + 4, sizeof(uint32_t));
  if (!out->v || !out->f) { free(keys); free(tk); free(tw); return VFO_ERR_RANGE; }
  for (size_t t = 0; t < nt; ++t)
    for (int j = 0; j < 3; ++j) {
      const uint32_t id = find_key(keys, (uint32_t)nv, tk[3 * t + j]);
      out->f[4 * t + j] = id;
      if (tw[t]) out->v[4 * (size_t)id + 3] = 1.0f;
    }
  for (size_t i = 0; i < nv; ++i) {
    const uint64_t lin = keys[i] / 6u;
    const int dir = (int)(keys[i] % 6u);
    const uint64_t ox = lin / ((uint64_t)Y * Z), oy = (lin / Z) % Y, oz = lin % Z;
    /* lattice position of the midpoint: owner voxel + 1 (padding) +- 0.5 */
    float p[3] = {(float)(ox + 1), (float)(oy + 1), (float)(oz + 1)};
    p[dir >> 1] += (dir & 1) ? 0.5f : -0.5f;
    for (int a = 0; a < 3; ++a) out->v[4 * i + a] = s[a] * p[a] + c0[a];
  }
  for (size_t t = 0; t < nt; ++t) {
    const uint32_t* f = out->f + 4 * t;
    const float w = out->v[4 * (size_t)f[0] + 3] > out->v[4 * (size_t)f[1] + 3]
                        ? out->v[4 * (size_t)f[0] + 3]
                        : out->v[4 * (size_t)f[1] + 3];
    out->f[4 * t + 3] = (uint32_t)(w > out->v[4 * (size_t)f[2] + 3] ? w : out->v[4 * (size_t)f[2] + 3]);
  }
  free(keys);
  free(tk);
  free(tw);
  smooth(out, nb_iters, nb_weight, 0);
  smooth(out, b_iters, b_weight, 1);
  return 0;
}

int vfo_triangulate(const uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, const float amin[3],
                    const float amax[3], uint32_t nb_iters, float nb_weight, uint32_t b_iters,
                    float b_weight, uint32_t* nmeshes, uint64_t* nverts, uint64_t* nfaces,
                    uint16_t* values, uint64_t* vert_off, uint64_t* face_off, float* verts,
                    uint32_t* faces) {
  if (!grid || !nmeshes || !nverts || !nfaces || !X || !Y || !Z) return VFO_ERR_INVALID;
  mc_init();
  /* fragment values (countValues: label & 0x7FFF > 1) and their lattice boxes */
  int64_t* box = (int64_t*)malloc(32768 * 6 * sizeof(int64_t));
  if (!box) return VFO_ERR_RANGE;
  for (int v = 0; v < 32768; ++v) {
    box[6 * v + 0] = box[6 * v + 1] = box[6 * v + 2] = INT64_MAX;
    box[6 * v + 3] = box[6 * v + 4] = box[6 * v + 5] = -1;
  }
  for (uint32_t x = 0; x < X; ++x)
    for (uint32_t y = 0; y < Y; ++y)
      for (uint32_t z = 0; z < Z; ++z) {
        const uint32_t v = grid[((size_t)x * Y + y) * Z + z] & 0x7FFFu;
        if (v <= VOXEL_FREE) continue;
        const int64_t p[3] = {(int64_t)x + 1, (int64_t)y + 1, (int64_t)z + 1};
        for (int a = 0; a < 3; ++a) {
          if (p[a] < box[6 * v + a]) box[6 * v + a] = p[a];
          if (p[a] > box[6 * v + 3 + a]) box[6 * v + 3 + a] = p[a];
        }
      }
  uint16_t vals[32768];
  uint32_t F = 0;
  for (int v = 2; v < 32768; ++v)
    if (box[6 * v + 3] >= 0) vals[F++] = (uint16_t)v;
  /* s = aabb.size() / dims; translation min - s */
  const uint32_t dims[3] = {X, Y, Z};
  float s[3], c0[3];
  for (int a = 0; a < 3; ++a) {
    const float size = amax[a] - amin[a];
    s[a] = size / (float)dims[a];
    c0[a] = amin[a] - s[a];
  }
  mmesh* ms = (mmesh*)calloc(F ? F : 1, sizeof(mmesh));
  int err = 0;
  if (!ms) err = VFO_ERR_RANGE;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int i = 0; i < (int)F; ++i) {
    if (err) continue;
    const uint16_t v = vals[i];
    err |= mesh_one(grid, X, Y, Z, v, box + 6 * v, box + 6 * v + 3, s, c0, nb_iters, nb_weight,
                    b_iters, b_weight, &ms[i]);
  }
  uint64_t NV = 0, NT = 0;
  if (!err) {
    for (uint32_t i = 0; i < F; ++i) {
      NV += ms[i].nv;
      NT += ms[i].nt;
    }
    *nmeshes = F;
    *nverts = NV;
    *nfaces = NT;
    if (values) {
      uint64_t ov = 0, of = 0;
      for (uint32_t i = 0; i < F; ++i) {
        values[i] = ms[i].value;
        if (vert_off) vert_off[i] = ov;
        if (face_off) face_off[i] = of;
        if (verts) memcpy(verts + 4 * ov, ms[i].v, (size_t)ms[i].nv * 4 * sizeof(float));
        if (faces) memcpy(faces + 4 * of, ms[i].f, (size_t)ms[i].nt * 4 * sizeof(uint32_t));
        ov += ms[i].nv;
        of += ms[i].nt;
      }
      if (vert_off) vert_off[F] = ov;
      if (face_off) face_off[F] = of;
    }
  }
  if (ms)
    for (uint32_t i = 0; i < F; ++i) {
      free(ms[i].v);
      free(ms[i].f);
    }
  free(ms);
  free(box);
  return err;
}
