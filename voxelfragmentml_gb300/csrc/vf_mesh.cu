// vf_mesh.cu -- RegularGrid::toTriangleMesh (RegularGrid.cpp:443-486) on
// sm_103a: one smoothed marching-cubes mesh per fragment value, for all
// fragments in one pass over the grid.
//
// The reference runs MarchingCubes::triangulateFieldGPU (MarchingCubes.cpp:
// 364-412) once per fragment value: marching cubes over the whole padded grid
// with the 0/1 field "label == value" and isolevel 0.5, Morton-sort + run
// merge of equal vertex positions, faces, boundary flags and Laplacian
// smoothing.  With a 0/1 field every vertex is the exact midpoint of a
// lattice edge whose two ends differ, and the case table uses every such
// edge of a cell, so the fused vertices of fragment v are exactly the pairs
// (voxel of v, face direction) whose neighbour across the face is not v.
// That turns fusion into enumeration:
//
//   k_mc_vcount   warp per grid row, 16 voxels per lane: exposed-face mask
//                 (6 bits) per voxel, vertex count per row, fragment values
//                 present
//   scan          row counts -> first vertex of each row
//   k_mc_vemit    warp per row: vertex id base per voxel, one record (owner
//                 voxel, direction) and fragment key per vertex, in voxel
//                 order then direction -x,+x,-y,+y,-z,+z
//   k_mc_tcount   warp per cell row: triangles of every fragment present
//                 among the cell's 8 corners (case table in shared memory)
//   scan          cell-row counts -> first triangle of each row
//   k_mc_temit    warp per cell row: cells with triangles queued in shared
//                 memory and dealt to the lanes; triangles as three vertex
//                 ids, looked up from the owner voxel's id base and face
//                 mask; cell boundary flags OR-ed into the vertices
//   k_ms_hist/k_ms_scatter  stable split of vertices and of triangles by
//                 fragment (LSD, 8-bit digits, one or two passes)
//   k_mc_vout     vertex positions through the grid's affine map
//   k_mc_fout     faces in sorted vertex ids, face flag = OR of vertex flags
//   k_inc_count / k_inc_fill / k_inc_unique / k_inc_compact  per vertex, the
//                 distinct neighbours (with multiplicity) of the faces its
//                 smoothing pass sums
//   k_lap_gather  one Laplacian iteration per launch (laplacianSmoothing +
//                 finishLaplacianSmoothing-comp.glsl) as a per-vertex gather
//                 of the same int32 fixed-point sums
//   k_mc_local    face indices relative to their mesh
//
// Vertex and face orders are fixed (the reference leaves them to atomics):
// vertices by owner voxel then direction, faces by cell (x-major) then by
// case-table triangle; a vertex is a boundary vertex when any triangle using
// it comes from a cell whose voxel has bit 15.
#include "vf_kernels.h"
#include "vf_mc_table.h"

namespace {

constexpr uint32_t FREE = 1u;
constexpr uint32_t MS_ITEMS = 8;                 // items per lane in a split chunk
constexpr uint32_t MS_CHUNK = 256 * MS_ITEMS;    // items per CTA

constexpr unsigned FULL = 0xFFFFFFFFu;

// Grid rows have a pitch Zp = roundup(Z, 8), so 8 labels starting at a
// multiple of 8 are one aligned 16-byte load.  Labels at z >= Z, and rows
// outside the grid, read as FREE.
__device__ __forceinline__ void load8(const uint16_t* row, uint32_t z0, uint32_t Z, uint32_t Zp,
                                      uint32_t out[8]) {
  if (row && z0 < Zp) {
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(row + z0));
    out[0] = q.x & 0xFFFFu; out[1] = q.x >> 16; out[2] = q.y & 0xFFFFu; out[3] = q.y >> 16;
    out[4] = q.z & 0xFFFFu; out[5] = q.z >> 16; out[6] = q.w & 0xFFFFu; out[7] = q.w >> 16;
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (z0 + e >= Z) out[e] = FREE;
  } else {
#pragma unroll
    for (int e = 0; e < 8; ++e) out[e] = FREE;
  }
}

// the same 8 labels packed two per word, as loaded (no unpacking)
__device__ __forceinline__ uint4 load8w(const uint16_t* row, uint32_t z0, uint32_t Z, uint32_t Zp) {
  constexpr uint32_t FF = FREE | (FREE << 16);
  if (!row || z0 >= Zp) return make_uint4(FF, FF, FF, FF);
  uint4 q = __ldg(reinterpret_cast<const uint4*>(row + z0));
  if (z0 + 8 > Z) {  // the row's last labels: FREE past Z
    uint32_t wd[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (z0 + e >= Z)
        wd[e >> 1] = (e & 1) ? ((wd[e >> 1] & 0xFFFFu) | (FREE << 16)) : ((wd[e >> 1] & 0xFFFF0000u) | FREE);
    q = make_uint4(wd[0], wd[1], wd[2], wd[3]);
  }
  return q;
}

// label e (0..7, a compile-time index after unrolling) of a packed load
__device__ __forceinline__ uint32_t lab_of(const uint4& q, int e) {
  const uint32_t wd = e < 2 ? q.x : (e < 4 ? q.y : (e < 6 ? q.z : q.w));
  return (e & 1) ? (wd >> 16) : (wd & 0xFFFFu);
}

// every label of the packed load equals l0 (bit 15 ignored)
__device__ __forceinline__ bool all_equal(const uint4& q, uint32_t l0) {
  const uint32_t L = l0 | (l0 << 16);
  return ((q.x & 0x7FFF7FFFu) == L) & ((q.y & 0x7FFF7FFFu) == L) & ((q.z & 0x7FFF7FFFu) == L) &
         ((q.w & 0x7FFF7FFFu) == L);
}

__device__ __forceinline__ const uint16_t* row_ptr(const vfk::MeshGrid& G, int64_t x, int64_t y) {
  return (x >= 0 && y >= 0 && x < (int64_t)G.X && y < (int64_t)G.Y)
             ? G.g + ((uint64_t)x * G.Y + (uint64_t)y) * G.Zp
             : nullptr;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__device__ __forceinline__ uint32_t byte_of(uint2 m, int e) {
  return ((e < 4 ? m.x : m.y) >> (8 * (e & 3))) & 0xFFu;
}

// warp per grid row, 16 voxels per lane: face masks (bit d: the neighbour in
// direction -x,+x,-y,+y,-z,+z carries another label), stored at the grid's
// pitch into a zeroed buffer (all-FREE lanes store nothing); vertices per
// row; present[value] for every fragment value
__global__ void __launch_bounds__(256) k_mc_vcount(vfk::MeshGrid G, uint8_t* mask, uint32_t* rcnt,
                                                   uint8_t* present) {
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)G.X * G.Y;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t x = (int64_t)(r / G.Y), y = (int64_t)(r % G.Y);
    const uint16_t* rc = G.g + r * G.Zp;
    const uint16_t* nb[4] = {row_ptr(G, x - 1, y), row_ptr(G, x + 1, y), row_ptr(G, x, y - 1),
                             row_ptr(G, x, y + 1)};
    uint32_t carry = FREE, n = 0;
    for (uint32_t z0 = 0; z0 < G.Z; z0 += 512) {
      const uint32_t zb = z0 + 16 * lane;
      const uint4 qa = load8w(rc, zb, G.Z, G.Zp), qb = load8w(rc, zb + 8, G.Z, G.Zp);
      const uint32_t last = qb.w >> 16;
      const uint32_t before = __shfl_up_sync(FULL, last, 1);
      uint32_t after = __shfl_down_sync(FULL, qa.x & 0xFFFFu, 1);
      const uint32_t zm1 = (lane == 0 ? carry : before) & 0x7FFFu;
      if (lane == 31) after = (z0 + 512 < G.Z) ? (uint32_t)__ldg(rc + z0 + 512) : FREE;
      after &= 0x7FFFu;
      carry = __shfl_sync(FULL, last, 31);
      uint32_t cnt = 0;
      // a label >= 2 somewhere in the lane's 16 voxels (bits 1..14 of a half)
      if (((qa.x | qa.y | qa.z | qa.w | qb.x | qb.y | qb.z | qb.w) & 0x7FFE7FFEu) != 0u) {
        uint32_t c[16], mk[16];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          c[e] = lab_of(qa, e) & 0x7FFFu;
          c[8 + e] = lab_of(qb, e) & 0x7FFFu;
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const uint32_t zl = e ? c[e - 1] : zm1, zh = e < 15 ? c[e + 1] : after;
          mk[e] = c[e] > FREE ? (((uint32_t)(zl != c[e]) << 4) | ((uint32_t)(zh != c[e]) << 5)) : 0u;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint4 oa = load8w(nb[k], zb, G.Z, G.Zp), ob = load8w(nb[k], zb + 8, G.Z, G.Zp);
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const uint32_t o = lab_of(e < 8 ? oa : ob, e & 7) & 0x7FFFu;
            if (c[e] > FREE) mk[e] |= (uint32_t)(o != c[e]) << k;
          }
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          cnt += (uint32_t)__popc(mk[e]);
          // every fragment has a voxel exposed towards -x (its lowest-x voxel)
          if ((mk[e] & 1u) && (e == 0 || c[e - 1] != c[e])) present[c[e]] = 1;
        }
        uint8_t* dst = mask + r * G.Zp + zb;
        if (zb < G.Zp)
          *reinterpret_cast<uint2*>(dst) =
              make_uint2(mk[0] | (mk[1] << 8) | (mk[2] << 16) | (mk[3] << 24),
                         mk[4] | (mk[5] << 8) | (mk[6] << 16) | (mk[7] << 24));
        if (zb + 8 < G.Zp)
          *reinterpret_cast<uint2*>(dst + 8) =
              make_uint2(mk[8] | (mk[9] << 8) | (mk[10] << 16) | (mk[11] << 24),
                         mk[12] | (mk[13] << 8) | (mk[14] << 16) | (mk[15] << 24));
      }
      n += __reduce_add_sync(FULL, cnt);
    }
    if (lane == 0) rcnt[r] = n;
  }
}

// warp per row, 8 voxels per lane: first vertex id of every voxel (at the
// grid's pitch) and one record per vertex, in voxel order then direction
__global__ void __launch_bounds__(256) k_mc_vemit(vfk::MeshGrid G, const uint8_t* mask,
                                                  const unsigned long long* rbase,
                                                  const uint16_t* dense, uint32_t* vbase,
                                                  uint16_t* vkey, unsigned long long* vown) {
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)G.X * G.Y;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    uint64_t base = rbase[r];
    const uint16_t* rc = G.g + r * G.Zp;
    for (uint32_t z0 = 0; z0 < G.Z; z0 += 256) {
      const uint32_t zb = z0 + 8 * lane;
      uint2 mm = make_uint2(0u, 0u);
      if (zb < G.Zp) mm = *reinterpret_cast<const uint2*>(mask + r * G.Zp + zb);
      const uint32_t tot = (uint32_t)(__popc(mm.x) + __popc(mm.y));
      const uint32_t incl = warp_incl_scan(tot, lane);
      const uint64_t vb = base + (incl - tot);
      if (tot) {  // id bases are read only for voxels with faces
        uint32_t b[8], run = 0;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          b[e] = (uint32_t)(vb + run);
          run += (uint32_t)__popc(byte_of(mm, e));
        }
        uint4* dst = reinterpret_cast<uint4*>(vbase + r * G.Zp + zb);
        dst[0] = make_uint4(b[0], b[1], b[2], b[3]);
        dst[1] = make_uint4(b[4], b[5], b[6], b[7]);
      }
      if (tot) {
        uint32_t c[8];
        load8(rc, zb, G.Z, G.Zp, c);
        uint64_t o = vb;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          uint32_t m = byte_of(mm, e);
          if (!m) continue;
          const uint16_t key = dense[c[e] & 0x7FFFu];
          const unsigned long long lin = r * G.Zp + zb + e;
          while (m) {
            const uint32_t d = (uint32_t)__ffs(m) - 1;
            m &= m - 1;
            vkey[o] = key;
            vown[o] = lin * 8ull + d;
            ++o;
          }
        }
      }
      base += __shfl_sync(FULL, incl, 31);
    }
  }
}

struct McShared {
  unsigned long long tri[256];  // 15 nibbles: edges of up to five triangles
  uint8_t ntri[256];
};

__device__ __forceinline__ void load_table(McShared& S, const unsigned long long* tri,
                                           const uint8_t* ntri) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    S.tri[i] = tri[i];
    S.ntri[i] = ntri[i];
  }
  __syncthreads();
}

// Cells: the reference marches every padded-lattice point (a+1, b, c),
// a in [0, X], b in [0, Y], c in [0, Z]; corner i of that cell is grid voxel
// (a + dx, b - 1 + dy, c - 1 + dz) for VF_MC_CORNER[i] = (dx, dy, dz), so a
// row of cells (a, b) reads the four grid rows (a, b-1), (a-1, b-1), (a, b),
// (a-1, b) at z = c-1 and z = c.  A warp takes 256 cells per step, 8 per lane:
// lane l loads z = c0 + 8l .. +7 of each row and gets z = c0 + 8l - 1 from
// lane l-1 (lane 0 from the previous step).
struct CellRows {
  const uint16_t* r[4];
  uint32_t carry[4];  // z = c0 - 1 of each row
};

__device__ __forceinline__ void cell_rows_init(const vfk::MeshGrid& G, int64_t a, int64_t b,
                                               CellRows& R) {
  R.r[0] = row_ptr(G, a, b - 1);
  R.r[1] = row_ptr(G, a - 1, b - 1);
  R.r[2] = row_ptr(G, a, b);
  R.r[3] = row_ptr(G, a - 1, b);
#pragma unroll
  for (int k = 0; k < 4; ++k) R.carry[k] = FREE;
}

__device__ __forceinline__ void cell_rows_load(const vfk::MeshGrid& G, CellRows& R, uint32_t c0,
                                               int lane, uint32_t cur[4][8], uint32_t prv0[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    load8(R.r[k], c0 + 8 * lane, G.Z, G.Zp, cur[k]);
    prv0[k] = __shfl_up_sync(FULL, cur[k][7], 1);
    if (lane == 0) prv0[k] = R.carry[k];
    R.carry[k] = __shfl_sync(FULL, cur[k][7], 31);
  }
}

// corner labels (bit 15 cleared) in VF_MC_CORNER order from the previous (z =
// c-1) and current (z = c) label of each row
__device__ __forceinline__ void corners(const uint32_t prv[4], const uint32_t cur[4], uint32_t v[8]) {
  v[0] = prv[0] & 0x7FFFu;  // ( 0,0,0): (a,   b-1, c-1)
  v[1] = cur[0] & 0x7FFFu;  // ( 0,0,1): (a,   b-1, c)
  v[2] = cur[1] & 0x7FFFu;  // (-1,0,1): (a-1, b-1, c)
  v[3] = prv[1] & 0x7FFFu;  // (-1,0,0): (a-1, b-1, c-1)
  v[4] = prv[2] & 0x7FFFu;  // ( 0,1,0): (a,   b,   c-1)
  v[5] = cur[2] & 0x7FFFu;  // ( 0,1,1): (a,   b,   c)
  v[6] = cur[3] & 0x7FFFu;  // (-1,1,1): (a-1, b,   c)
  v[7] = prv[3] & 0x7FFFu;  // (-1,1,0): (a-1, b,   c-1)
}

__device__ __forceinline__ bool uniform8(const uint32_t v[8]) {
  bool u = true;
#pragma unroll
  for (int j = 1; j < 8; ++j) u &= v[j] == v[0];
  return u;
}

__device__ __forceinline__ uint32_t config_of(const uint32_t v[8], uint32_t t) {
  uint32_t conf = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) conf |= (uint32_t)(v[j] != t) << j;
  return conf;
}

__device__ __forceinline__ bool first_of(const uint32_t v[8], int i) {
  bool first = v[i] > FREE;
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (j < i && v[j] == v[i]) first = false;
  return first;
}

__device__ __forceinline__ uint32_t cell_triangles(const McShared& S, const uint32_t v[8]) {
  if (uniform8(v)) return 0;  // one label on all corners: configuration 0 or 255
  uint32_t k = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if (first_of(v, i)) k += S.ntri[config_of(v, v[i])];
  return k;
}

// per warp: the step's four rows (index 7: z = c0 - 1, 8 + j: z = c0 + j),
// the queue of its cells whose corners are not all one label, and per queued
// cell its triangle count, then its first triangle
struct CellShared {
  McShared T;
  uint16_t rows[8][4][264];
  uint16_t qcell[8][256];
  uint32_t qtri[8][256];
};

// Stage one step (256 cells) of cell row (a, b) in shared memory and queue
// its mixed cells (corners not all one label) in cell order; uniform cells
// have no triangles.  Returns the queue length.
__device__ __forceinline__ uint32_t stage_cells(const vfk::MeshGrid& G, CellRows& R, CellShared& S,
                                                int w, int lane, uint32_t c0) {
  uint4 q[4];
  uint32_t prv0[4], old[4];
  __syncwarp();  // the previous step's rows and queue are consumed
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    q[k] = load8w(R.r[k], c0 + 8 * lane, G.Z, G.Zp);
    const uint32_t last = q[k].w >> 16;
    const uint32_t p = __shfl_up_sync(FULL, last, 1);
    old[k] = R.carry[k];
    prv0[k] = lane == 0 ? old[k] : p;
    R.carry[k] = __shfl_sync(FULL, last, 31);
  }
  // one label on all 36 lattice points of the lane's 8 cells: nothing mixed
  const uint32_t l0 = prv0[0] & 0x7FFFu;
  bool same = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) same &= all_equal(q[k], l0) & ((prv0[k] & 0x7FFFu) == l0);
  if (__all_sync(FULL, same)) return 0;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) S.rows[w][k][7] = (uint16_t)old[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) *reinterpret_cast<uint4*>(&S.rows[w][k][8 + 8 * lane]) = q[k];
  uint32_t mixed = 0;
  if (!same) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      uint32_t pr[4], cu[4], v[8];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        pr[k] = e ? lab_of(q[k], e - 1) : prv0[k];
        cu[k] = lab_of(q[k], e);
      }
      corners(pr, cu, v);
      if (!uniform8(v) && c0 + 8 * lane + e <= G.Z) mixed |= 1u << e;
    }
  }
  const uint32_t na = (uint32_t)__popc(mixed);
  const uint32_t incl = warp_incl_scan(na, lane);
  uint32_t qp = incl - na;
  while (mixed) {
    const uint32_t e = (uint32_t)__ffs(mixed) - 1;
    mixed &= mixed - 1;
    S.qcell[w][qp++] = (uint16_t)(8 * lane + e);
  }
  __syncwarp();
  return __shfl_sync(FULL, incl, 31);
}

// corner labels of queued cell j of the warp's staged step
__device__ __forceinline__ void staged_corners(const CellShared& S, int w, uint32_t j, uint32_t v[8],
                                               uint32_t& raw0) {
  uint32_t pr[4], cu[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    pr[q] = S.rows[w][q][7 + j];
    cu[q] = S.rows[w][q][8 + j];
  }
  raw0 = pr[0];
  corners(pr, cu, v);
}

__global__ void __launch_bounds__(256) k_mc_tcount(vfk::MeshGrid G, const unsigned long long* tri,
                                                   const uint8_t* ntri, uint32_t* rcnt) {
  __shared__ __align__(16) CellShared S;
  load_table(S.T, tri, ntri);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t a = (int64_t)(r / (G.Y + 1)), b = (int64_t)(r % (G.Y + 1));
    CellRows R;
    cell_rows_init(G, a, b, R);
    uint32_t n = 0;
    for (uint32_t c0 = 0; c0 <= G.Z; c0 += 256) {
      const uint32_t nq = stage_cells(G, R, S, w, lane, c0);
      uint32_t k = 0;
      for (uint32_t i = lane; i < nq; i += 32) {
        uint32_t v[8], raw0;
        staged_corners(S, w, S.qcell[w][i], v, raw0);
        k += cell_triangles(S.T, v);
      }
      n += __reduce_add_sync(FULL, k);
    }
    if (lane == 0) rcnt[r] = n;
  }
}

// offset (dx, dy, dz) of corner i, packed: bit 0 dx == -1, bit 1 dy, bit 2 dz
__device__ __forceinline__ uint32_t corner_bits(uint32_t i) {
  return (0x3762'1540u >> (4 * i)) & 7u;  // 0:000 1:100 2:101 3:001 4:010 5:110 6:111 7:011
}

// Mixed cells are queued per step and dealt to the lanes (count, prefix,
// emit), so the work follows the surface cells rather than the grid.
__global__ void __launch_bounds__(256, 2) k_mc_temit(vfk::MeshGrid G, const unsigned long long* tri,
                                                     const uint8_t* ntri,
                                                     const unsigned long long* rbase,
                                                     const uint8_t* mask, const uint32_t* vbase,
                                                     const uint16_t* dense, uint16_t* tkey, uint4* tv,
                                                     uint32_t* vflag, uint32_t* err) {
  __shared__ __align__(16) CellShared S;
  load_table(S.T, tri, ntri);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t a = (int64_t)(r / (G.Y + 1)), b = (int64_t)(r % (G.Y + 1));
    CellRows R;
    cell_rows_init(G, a, b, R);
    uint64_t base = rbase[r];
    for (uint32_t c0 = 0; c0 <= G.Z; c0 += 256) {
      const uint32_t nq = stage_cells(G, R, S, w, lane, c0);
      if (!nq) continue;
      // triangles per queued cell, then their exclusive prefix (8 entries per lane)
      for (uint32_t i = lane; i < nq; i += 32) {
        uint32_t v[8], raw0;
        staged_corners(S, w, S.qcell[w][i], v, raw0);
        S.qtri[w][i] = cell_triangles(S.T, v);
      }
      __syncwarp();
      uint32_t part[8], sum = 0;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const uint32_t i = 8 * lane + e;
        part[e] = i < nq ? S.qtri[w][i] : 0u;
        sum += part[e];
      }
      const uint32_t incl = warp_incl_scan(sum, lane);
      uint32_t run = incl - sum;
      __syncwarp();
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const uint32_t i = 8 * lane + e;
        if (i < nq) S.qtri[w][i] = run;
        run += part[e];
      }
      __syncwarp();
      // one triangle per lane: triangle k of the step belongs to the last
      // queued cell whose first triangle is <= k (cells without triangles
      // share their successor's prefix), then to the fragment and case-table
      // row found by counting the cell's triangles in order
      const uint32_t ntot = __shfl_sync(FULL, incl, 31);
      for (uint32_t k = lane; k < ntot; k += 32) {
        uint32_t lo = 0, hi = nq;
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (S.qtri[w][mid] <= k) lo = mid; else hi = mid;
        }
        const uint32_t j = S.qcell[w][lo];
        const int64_t c = (int64_t)c0 + j;
        uint32_t r = k - S.qtri[w][lo];  // triangle within the cell
        const uint64_t tt = base + k;
        uint32_t v[8], raw0;
        staged_corners(S, w, j, v, raw0);
        const uint32_t wb = raw0 >> 15;  // bit 15 of the voxel at the cell's lattice point
        uint32_t fm = 0;  // corners that hold the first copy of a fragment label
#pragma unroll
        for (int q = 0; q < 8; ++q) fm |= (uint32_t)first_of(v, q) << q;
        uint32_t target = 0, conf = 0, nt = 0;
        while (fm) {
          const int i0 = __ffs(fm) - 1;
          fm &= fm - 1;
          target = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (q == i0) target = v[q];
          conf = config_of(v, target);
          nt = S.T.ntri[conf];
          if (r < nt) break;
          r -= nt;
        }
        const unsigned long long edges = S.T.tri[conf];
        const uint32_t q = r;
        uint32_t id[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          const int slot = 3 * (int)q + (jj == 0 ? 0 : (jj == 1 ? 2 : 1));
          const uint32_t e = (uint32_t)(edges >> (4 * slot)) & 15u;
          // edge endpoints (VF_MC_EDGE); the owner is the end inside the fragment
          const uint32_t pa = (uint32_t)(0x3210'7654'3210ull >> (4 * e)) & 15u;
          const uint32_t pb = (uint32_t)(0x7654'4765'0321ull >> (4 * e)) & 15u;
          const bool a_own = ((conf >> pa) & 1u) == 0u;
          const uint32_t own = a_own ? pa : pb, oth = a_own ? pb : pa;
          const uint32_t ob = corner_bits(own), tb = corner_bits(oth);
          const int64_t ox = a - (int64_t)(ob & 1u), oy = b - 1 + (int64_t)((ob >> 1) & 1u),
                        oz = c - 1 + (int64_t)((ob >> 2) & 1u);
          const uint32_t diff = ob ^ tb;  // one bit: the axis
          const uint32_t axis = diff == 1u ? 0u : (diff == 2u ? 1u : 2u);
          // x: bit set = dx -1, so the other end lies at larger x when its bit is clear
          const uint32_t up = axis == 0u ? ((tb & 1u) == 0u) : ((tb >> axis) & 1u);
          const uint32_t d = 2u * axis + up;
          const uint64_t lin = ((uint64_t)ox * G.Y + (uint64_t)oy) * G.Zp + (uint64_t)oz;
          const uint32_t mk = mask[lin];
          if ((mk >> d) & 1u) {
            id[jj] = vbase[lin] + (uint32_t)__popc(mk & ((1u << d) - 1u));
            if (wb) atomicOr(vflag + (id[jj] >> 5), 1u << (id[jj] & 31u));
          } else {  // the owner's face mask must hold the edge's direction
            atomicOr(err, 1u);
            id[jj] = 0;
          }
        }
        tkey[tt] = dense[target];
        tv[tt] = make_uint4(id[0], id[1], id[2], 0u);
      }
      base += __shfl_sync(FULL, incl, 31);
    }
  }
}

// ---- stable split by a 16-bit key, 8 bits per pass -----------------------
__device__ __forceinline__ uint32_t ms_item(const uint32_t* in, uint64_t i) {
  return in ? in[i] : (uint32_t)i;
}

__global__ void __launch_bounds__(256) k_ms_hist(const uint16_t* key, const uint32_t* in, uint64_t n,
                                                 int shift, uint32_t nchunks, uint32_t* hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t c0 = (uint64_t)blockIdx.x * MS_CHUNK;
  for (uint32_t k = 0; k < MS_ITEMS; ++k) {
    const uint64_t i = c0 + (uint64_t)k * 256 + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[ms_item(in, i)] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nchunks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_ms_scatter(const uint16_t* key, const uint32_t* in,
                                                    uint64_t n, int shift, uint32_t nchunks,
                                                    const unsigned long long* hbase, uint32_t* out) {
  __shared__ uint32_t cnt[8][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = lane; d < 256; d += 32) cnt[w][d] = 0;
  __syncwarp();
  const uint64_t wbase = (uint64_t)blockIdx.x * MS_CHUNK + (uint64_t)w * (32 * MS_ITEMS);
  uint32_t item[MS_ITEMS], dig[MS_ITEMS], rank[MS_ITEMS];
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (uint32_t k = 0; k < MS_ITEMS; ++k) {
    const uint64_t i = wbase + (uint64_t)k * 32 + lane;
    const bool ok = i < n;
    item[k] = ok ? ms_item(in, i) : 0u;
    dig[k] = ok ? ((uint32_t)(key[item[k]] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, dig[k]);
    uint32_t before = 0;
    if (ok) before = cnt[w][dig[k]];
    rank[k] = before + (uint32_t)__popc(peers & lt);
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) cnt[w][dig[k]] = before + (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    // per digit: exclusive prefix over the warps + the chunk's base
    const uint32_t d = threadIdx.x;
    uint64_t run = hbase[(uint64_t)d * nchunks + blockIdx.x];
    for (int ww = 0; ww < 8; ++ww) {
      const uint32_t c = cnt[ww][d];
      cnt[ww][d] = (uint32_t)run;  // final positions fit 32 bits (n < 2^32)
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (uint32_t k = 0; k < MS_ITEMS; ++k)
    if (dig[k] < 256u) out[cnt[w][dig[k]] + rank[k]] = item[k];
}

// ---- outputs ---------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mc_vout(vfk::MeshGrid G, const uint32_t* vperm,
                                                 const unsigned long long* vown,
                                                 const uint32_t* vflag, uint64_t V, float sx,
                                                 float sy, float sz, float cx, float cy, float cz,
                                                 uint32_t* vinv, float4* out) {
  const uint64_t YZ = (uint64_t)G.Y * G.Zp;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < V;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t gv = vperm[s];
    vinv[gv] = (uint32_t)s;
    const unsigned long long own = vown[gv];
    const uint64_t lin = own >> 3;
    const uint32_t d = (uint32_t)(own & 7ull);
    float p[3] = {(float)(lin / YZ + 1), (float)((lin / G.Zp) % G.Y + 1), (float)(lin % G.Zp + 1)};
    p[d >> 1] += (d & 1u) ? 0.5f : -0.5f;
    float4 o;
    o.x = __fadd_rn(__fmul_rn(sx, p[0]), cx);
    o.y = __fadd_rn(__fmul_rn(sy, p[1]), cy);
    o.z = __fadd_rn(__fmul_rn(sz, p[2]), cz);
    o.w = (float)((vflag[gv >> 5] >> (gv & 31u)) & 1u);
    out[s] = o;
  }
}

__global__ void __launch_bounds__(256) k_mc_fout(const uint32_t* tperm, const uint4* tv,
                                                 const uint32_t* vinv, const uint32_t* vflag,
                                                 uint64_t T, uint4* gface) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < T;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 t = tv[tperm[s]];
    const uint32_t w = ((vflag[t.x >> 5] >> (t.x & 31u)) | (vflag[t.y >> 5] >> (t.y & 31u)) |
                        (vflag[t.z >> 5] >> (t.z & 31u))) & 1u;
    gface[s] = make_uint4(vinv[t.x], vinv[t.y], vinv[t.z], w);
  }
}

// first sorted position of every key 0..F (F: one past the last mesh)
__global__ void k_mc_offsets(const uint16_t* key, const uint32_t* perm, uint64_t n, uint32_t F,
                             unsigned long long* off) {
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f <= F; f += gridDim.x * blockDim.x) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo) / 2;
      if ((uint32_t)key[perm[mid]] < f) lo = mid + 1; else hi = mid;
    }
    off[f] = lo;
  }
}

// Laplacian smoothing as a gather.  Each vertex is smoothed in one pass only
// (non-boundary vertices in the first, boundary vertices in the second) and
// sums the other two vertices of the faces that pass counts for it: every
// incident face for a boundary vertex, the faces without boundary vertices
// for a non-boundary one.  Those incidences are listed once per vertex
// (counting sort); the sums are integers, so their order does not matter.
__device__ __forceinline__ bool counts_for(const uint4& f, const float* vw, uint32_t u) {
  return f.w == 0u || vw[4 * (uint64_t)u] == 1.0f;
}

__global__ void __launch_bounds__(256) k_inc_count(const uint4* gface, const float4* vert, uint64_t T,
                                                   uint32_t* deg) {
  const float* vw = reinterpret_cast<const float*>(vert) + 3;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < T;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 f = gface[s];
    if (counts_for(f, vw, f.x)) atomicAdd(deg + f.x, 1u);
    if (counts_for(f, vw, f.y)) atomicAdd(deg + f.y, 1u);
    if (counts_for(f, vw, f.z)) atomicAdd(deg + f.z, 1u);
  }
}

__global__ void __launch_bounds__(256) k_inc_fill(const uint4* gface, const float4* vert, uint64_t T,
                                                  const unsigned long long* start, uint32_t* cursor,
                                                  uint2* ent) {
  const float* vw = reinterpret_cast<const float*>(vert) + 3;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < T;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 f = gface[s];
    if (counts_for(f, vw, f.x)) ent[start[f.x] + atomicAdd(cursor + f.x, 1u)] = make_uint2(f.y, f.z);
    if (counts_for(f, vw, f.y)) ent[start[f.y] + atomicAdd(cursor + f.y, 1u)] = make_uint2(f.z, f.x);
    if (counts_for(f, vw, f.z)) ent[start[f.z] + atomicAdd(cursor + f.z, 1u)] = make_uint2(f.x, f.y);
  }
}

// the incidence pairs of vertex u folded in place into distinct neighbours,
// each entry (neighbour << 4 | multiplicity): on a closed surface every edge
// lies in two faces, so this halves the entries and the gathers
__global__ void __launch_bounds__(256) k_inc_unique(const unsigned long long* start, uint2* ent,
                                                    uint64_t V, uint32_t* ucnt, uint32_t* err) {
  for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < V;
       u += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t* w = reinterpret_cast<uint32_t*>(ent + start[u]);
    const uint32_t n2 = (uint32_t)(2 * (start[u + 1] - start[u]));
    uint32_t out = 0;
    for (uint32_t i = 0; i < n2; ++i) {
      const uint32_t n = w[i];  // every slot below i was read already
      uint32_t j = 0;
      while (j < out && (w[j] >> 4) != n) ++j;
      if (j < out) {
        if ((w[j] & 15u) == 15u) atomicOr(err, 2u); else ++w[j];
      } else {
        w[out++] = (n << 4) | 1u;
      }
    }
    ucnt[u] = out;
  }
}

// dense neighbour lists and per-vertex meta: x = first entry, y = count of
// summed positions (2 per face incidence, 16 bits) | entries << 16 (15 bits)
// | boundary type << 31
// stats: [0] boundary vertices, [1] neighbour entries of boundary vertices
__global__ void __launch_bounds__(256) k_inc_compact(const unsigned long long* start,
                                                     const uint2* ent,
                                                     const unsigned long long* ustart,
                                                     const float4* vert, uint64_t V,
                                                     uint32_t* nbr, uint2* meta, uint32_t* err,
                                                     unsigned long long* stats) {
  const float* vw = reinterpret_cast<const float*>(vert) + 3;
  const uint64_t n = (V + 31) & ~31ull;  // whole warps, for the reductions
  for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t type = 0, len = 0;
    if (u < V) {
      const uint32_t* w = reinterpret_cast<const uint32_t*>(ent + start[u]);
      const uint64_t b = ustart[u];
      len = (uint32_t)(ustart[u + 1] - b);
      const uint64_t cnt = 2 * (start[u + 1] - start[u]);
      if (cnt > 0xFFFFu || len > 0x7FFFu) atomicOr(err, 2u);
      for (uint32_t k = 0; k < len; ++k) nbr[b + k] = w[k];
      type = vw[4 * u] == 1.0f ? 1u : 0u;
      meta[u] = make_uint2((uint32_t)b,
                           (uint32_t)(cnt & 0xFFFFu) | ((len & 0x7FFFu) << 16) | (type << 31));
    }
    const uint32_t nb = __reduce_add_sync(FULL, type), ne = __reduce_add_sync(FULL, type ? len : 0u);
    if ((threadIdx.x & 31) == 0 && nb) {
      atomicAdd(stats + 0, (unsigned long long)nb);
      atomicAdd(stats + 1, (unsigned long long)ne);
    }
  }
}

__device__ __forceinline__ uint32_t to_fixed(float p) {
  return (uint32_t)__float2int_rz(__fmul_rn(p, 10000.0f));  // saturating, NaN -> 0
}

// one Jacobi iteration (laplacianSmoothing + finishLaplacianSmoothing) for the
// vertices of type `target`; other vertices are read from src, never written
// (both buffers hold them)
__global__ void __launch_bounds__(256) k_lap_gather(const float4* src, float4* dst, const uint2* meta,
                                                    const uint32_t* nbr, uint64_t V, uint32_t target,
                                                    float omw, float weight) {
  for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < V;
       u += (uint64_t)gridDim.x * blockDim.x) {
    const uint2 m = meta[u];
    if ((m.y >> 31) != target) continue;
    float4 p = src[u];
    const uint32_t cnt = m.y & 0xFFFFu, len = (m.y >> 16) & 0x7FFFu;
    if (cnt) {
      uint32_t sx = 0, sy = 0, sz = 0;
      // four entries, then their four positions, in flight at a time
      for (uint32_t k = 0; k < len; k += 4) {
        uint32_t e[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) e[j] = k + j < len ? __ldg(nbr + m.x + k + j) : 0u;
        float4 a[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) a[j] = e[j] ? src[e[j] >> 4] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t mult = e[j] & 15u;  // 0 for the padding slots
          sx += mult * to_fixed(a[j].x);
          sy += mult * to_fixed(a[j].y);
          sz += mult * to_fixed(a[j].z);
        }
      }
      const float c = __int2float_rn((int)cnt);
      const float ax = __fdiv_rn(__fdiv_rn(__int2float_rn((int)sx), c), 10000.0f);
      const float ay = __fdiv_rn(__fdiv_rn(__int2float_rn((int)sy), c), 10000.0f);
      const float az = __fdiv_rn(__fdiv_rn(__int2float_rn((int)sz), c), 10000.0f);
      p.x = __fadd_rn(__fmul_rn(p.x, omw), __fmul_rn(ax, weight));
      p.y = __fadd_rn(__fmul_rn(p.y, omw), __fmul_rn(ay, weight));
      p.z = __fadd_rn(__fmul_rn(p.z, omw), __fmul_rn(az, weight));
    }
    dst[u] = p;
  }
}

__global__ void __launch_bounds__(256) k_mc_local(const uint4* gface, const uint32_t* tperm,
                                                  const uint16_t* tkey,
                                                  const unsigned long long* voff, uint64_t T,
                                                  uint4* out) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < T;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 f = gface[s];
    const uint32_t b = (uint32_t)voff[tkey[tperm[s]]];
    out[s] = make_uint4(f.x - b, f.y - b, f.z - b, f.w);
  }
}

inline int grid_for(uint64_t n, int num_sms, int per_sm = 8) {
  const uint64_t need = (n + 255) / 256;
  const uint64_t cap = (uint64_t)num_sms * per_sm;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, cap));
}

// one wave of a grid-stride row kernel: the CTAs that fit on the GPU at
// once, so no CTA waits for a second wave
template <typename K>
int one_wave(K kernel, uint64_t rows, int num_sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1)
    per_sm = 2;
  return grid_for(rows * 32, num_sms, per_sm);
}

}  // namespace

namespace vfk {

void mc_pack_table(unsigned long long tri[256], uint8_t ntri[256]) {
  for (int c = 0; c < 256; ++c) {
    const char* s = VF_MC_TRIANGLES[c];
    unsigned long long w = 0;
    int n = 0;
    for (; s[n]; ++n) {
      const unsigned long long e = (unsigned long long)(s[n] <= '9' ? s[n] - '0' : s[n] - 'a' + 10);
      w |= e << (4 * n);
    }
    tri[c] = w;
    ntri[c] = (uint8_t)(n / 3);
  }
}

void mc_vertex_count(cudaStream_t st, const MeshGrid& G, uint8_t* mask, uint32_t* rcnt,
                     uint8_t* present, int num_sms) {
  const uint64_t rows = (uint64_t)G.X * G.Y;
  if (rows) k_mc_vcount<<<one_wave(k_mc_vcount, rows, num_sms), 256, 0, st>>>(G, mask, rcnt, present);
}

void mc_vertex_emit(cudaStream_t st, const MeshGrid& G, const uint8_t* mask,
                    const unsigned long long* rbase, const uint16_t* dense, uint32_t* vbase,
                    uint16_t* vkey, unsigned long long* vown, int num_sms) {
  const uint64_t rows = (uint64_t)G.X * G.Y;
  if (rows)
    k_mc_vemit<<<one_wave(k_mc_vemit, rows, num_sms), 256, 0, st>>>(G, mask, rbase, dense, vbase, vkey,
                                                                     vown);
}

void mc_tri_count(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                  const uint8_t* ntri, uint32_t* rcnt, int num_sms) {
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  k_mc_tcount<<<one_wave(k_mc_tcount, rows, num_sms), 256, 0, st>>>(G, tri, ntri, rcnt);
}

void mc_tri_emit(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                 const uint8_t* ntri, const unsigned long long* rbase, const uint8_t* mask,
                 const uint32_t* vbase, const uint16_t* dense, uint16_t* tkey, uint4* tv,
                 uint32_t* vflag, uint32_t* err, int num_sms) {
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  k_mc_temit<<<one_wave(k_mc_temit, rows, num_sms), 256, 0, st>>>(G, tri, ntri, rbase, mask, vbase, dense,
                                                           tkey, tv, vflag, err);
}

size_t split_hist_words(uint64_t n) { return 256 * std::max<uint64_t>(1, (n + MS_CHUNK - 1) / MS_CHUNK); }

void stable_split16(cudaStream_t st, const uint16_t* key, uint64_t n, uint32_t nkeys, uint32_t* tmp,
                    uint32_t* out, uint32_t* hist, unsigned long long* hbase,
                    unsigned long long* sums, unsigned long long* tot) {
  if (!n) return;
  const uint32_t nchunks = (uint32_t)((n + MS_CHUNK - 1) / MS_CHUNK);
  const int passes = nkeys > 256 ? 2 : 1;
  const uint32_t* in = nullptr;
  for (int p = 0; p < passes; ++p) {
    uint32_t* dst = (p == passes - 1) ? out : tmp;
    k_ms_hist<<<nchunks, 256, 0, st>>>(key, in, n, 8 * p, nchunks, hist);
    exclusive_scan(st, hist, hbase, sums, 256u * nchunks, tot);
    k_ms_scatter<<<nchunks, 256, 0, st>>>(key, in, n, 8 * p, nchunks, hbase, dst);
    in = dst;
  }
}

void mc_outputs(cudaStream_t st, const MeshGrid& G, const uint32_t* vperm,
                const unsigned long long* vown, const uint32_t* vflag, uint64_t V, const float s[3],
                const float c[3], uint32_t* vinv, float4* vert, const uint32_t* tperm,
                const uint4* tv, uint64_t T, uint4* gface, int num_sms) {
  if (V)
    k_mc_vout<<<grid_for(V, num_sms), 256, 0, st>>>(G, vperm, vown, vflag, V, s[0], s[1], s[2], c[0],
                                                    c[1], c[2], vinv, vert);
  if (T) k_mc_fout<<<grid_for(T, num_sms), 256, 0, st>>>(tperm, tv, vinv, vflag, T, gface);
}

void mc_offsets(cudaStream_t st, const uint16_t* key, const uint32_t* perm, uint64_t n, uint32_t F,
                unsigned long long* off) {
  k_mc_offsets<<<(F + 256) / 256, 256, 0, st>>>(key, perm, n, F, off);
}

cudaError_t mc_smooth_lists(cudaStream_t st, const uint4* gface, uint64_t T, const float4* vert,
                            uint64_t V, uint32_t* deg, unsigned long long* start,
                            unsigned long long* ustart, unsigned long long* sums, uint2* ent,
                            uint32_t* nbr, uint2* meta, uint32_t* err, unsigned long long* stats,
                            int num_sms) {
  if (!V || !T) return cudaSuccess;
  cudaError_t e;
  const int gv = grid_for(V, num_sms), gt = grid_for(T, num_sms);
  if ((e = cudaMemsetAsync(deg, 0, V * 4, st))) return e;
  if ((e = cudaMemsetAsync(stats, 0, 16, st))) return e;
  k_inc_count<<<gt, 256, 0, st>>>(gface, vert, T, deg);
  exclusive_scan(st, deg, start, sums, (uint32_t)V, start + V);
  if ((e = cudaMemsetAsync(deg, 0, V * 4, st))) return e;
  k_inc_fill<<<gt, 256, 0, st>>>(gface, vert, T, start, deg, ent);
  k_inc_unique<<<gv, 256, 0, st>>>(start, ent, V, deg, err);
  exclusive_scan(st, deg, ustart, sums, (uint32_t)V, ustart + V);
  k_inc_compact<<<gv, 256, 0, st>>>(start, ent, ustart, vert, V, nbr, meta, err, stats);
  return cudaGetLastError();
}

cudaError_t mc_smooth_iterate(cudaStream_t st, float4* vert, float4* tmp, uint64_t V,
                              const uint2* meta, const uint32_t* nbr, uint32_t nb_iters,
                              float nb_weight, uint32_t b_iters, float b_weight, int num_sms) {
  if (!V || (!nb_iters && !b_iters)) return cudaSuccess;
  cudaError_t e;
  const int gv = grid_for(V, num_sms);
  // both buffers hold every position; each iteration rewrites the target
  // vertices only
  if ((e = cudaMemcpyAsync(tmp, vert, V * sizeof(float4), cudaMemcpyDeviceToDevice, st))) return e;
  float4* cur = vert;
  float4* nxt = tmp;
  for (uint32_t pass = 0; pass < 2; ++pass) {
    const uint32_t iters = pass ? b_iters : nb_iters;
    const float weight = pass ? b_weight : nb_weight;
    const float omw = 1.0f - weight;
    for (uint32_t it = 0; it < iters; ++it) {
      k_lap_gather<<<gv, 256, 0, st>>>(cur, nxt, meta, nbr, V, pass, omw, weight);
      std::swap(cur, nxt);
    }
    // the finished type must match in both buffers before the other pass
    if (pass == 0 && nb_iters && b_iters)
      if ((e = cudaMemcpyAsync(nxt, cur, V * sizeof(float4), cudaMemcpyDeviceToDevice, st))) return e;
  }
  if (cur != vert) return cudaMemcpyAsync(vert, cur, V * sizeof(float4), cudaMemcpyDeviceToDevice, st);
  return cudaGetLastError();
}

void mc_local_faces(cudaStream_t st, const uint4* gface, const uint32_t* tperm, const uint16_t* tkey,
                    const unsigned long long* voff, uint64_t T, uint4* out, int num_sms) {
  if (T) k_mc_local<<<grid_for(T, num_sms), 256, 0, st>>>(gface, tperm, tkey, voff, T, out);
}

}  // namespace vfk
