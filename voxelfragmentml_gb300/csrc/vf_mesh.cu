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
//   k_mc_vcount   warp per grid row: exposed-face mask (6 bits) per voxel,
//                 vertex count per row, fragment values present
//   scan          row counts -> first vertex of each row
//   k_mc_vemit    warp per row: vertex id base per voxel, one record (owner
//                 voxel, direction) and fragment key per vertex, in voxel
//                 order then direction -x,+x,-y,+y,-z,+z
//   k_mc_tcount   warp per cell row: triangles of every fragment present
//                 among the cell's 8 corners (case table in shared memory)
//   scan          cell-row counts -> first triangle of each row
//   k_mc_temit    warp per cell row: triangles as three vertex ids, looked up
//                 from the owner voxel's id base and face mask; cell boundary
//                 flags OR-ed into the vertices
//   k_ms_hist/k_ms_scatter  stable split of vertices and of triangles by
//                 fragment (LSD, 8-bit digits, one or two passes)
//   k_mc_vout     vertex positions through the grid's affine map
//   k_mc_fout     faces in sorted vertex ids, face flag = OR of vertex flags
//   k_lap_faces / k_lap_finish   Laplacian iterations, int32 atomics as
//                 laplacianSmoothing-comp.glsl / finishLaplacianSmoothing
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

__device__ __forceinline__ uint32_t glab(const vfk::MeshGrid& G, int64_t x, int64_t y, int64_t z) {
  if (x < 0 || y < 0 || z < 0 || x >= (int64_t)G.X || y >= (int64_t)G.Y || z >= (int64_t)G.Z)
    return FREE;
  return __ldg(G.g + ((uint64_t)x * G.Y + (uint64_t)y) * G.Zp + (uint64_t)z);
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__global__ void __launch_bounds__(256) k_mc_vcount(vfk::MeshGrid G, uint8_t* mask, uint32_t* rcnt,
                                                   uint8_t* present) {
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)G.X * G.Y;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t x = (int64_t)(r / G.Y), y = (int64_t)(r % G.Y);
    uint32_t n = 0;
    for (uint32_t z0 = 0; z0 < G.Z; z0 += 32) {
      const int64_t z = z0 + lane;
      uint32_t mk = 0, v = 0;
      if (z < G.Z) {
        v = glab(G, x, y, z) & 0x7FFFu;
        if (v > FREE) {
          const uint32_t nb[6] = {glab(G, x - 1, y, z), glab(G, x + 1, y, z), glab(G, x, y - 1, z),
                                  glab(G, x, y + 1, z), glab(G, x, y, z - 1), glab(G, x, y, z + 1)};
#pragma unroll
          for (int d = 0; d < 6; ++d) mk |= (uint32_t)((nb[d] & 0x7FFFu) != v) << d;
        }
        mask[r * G.Z + (uint64_t)z] = (uint8_t)mk;
      }
      // every fragment has a voxel exposed towards -x (its lowest-x voxel)
      const uint32_t key = (mk & 1u) ? v : 0xFFFFFFFFu;
      const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
      if (key != 0xFFFFFFFFu && lane == __ffs(peers) - 1) present[v] = 1;
      n += __reduce_add_sync(0xFFFFFFFFu, (uint32_t)__popc(mk));
    }
    if (lane == 0) rcnt[r] = n;
  }
}

__global__ void __launch_bounds__(256) k_mc_vemit(vfk::MeshGrid G, const uint8_t* mask,
                                                  const unsigned long long* rbase,
                                                  const uint16_t* dense, uint32_t* vbase,
                                                  uint16_t* vkey, unsigned long long* vown) {
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)G.X * G.Y;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    uint64_t base = rbase[r];
    const uint16_t* row = G.g + r * G.Zp;
    for (uint32_t z0 = 0; z0 < G.Z; z0 += 32) {
      const uint32_t z = z0 + lane;
      const uint64_t lin = r * G.Z + z;
      const uint32_t mk = z < G.Z ? (uint32_t)mask[lin] : 0u;
      const uint32_t c = (uint32_t)__popc(mk);
      const uint32_t incl = warp_incl_scan(c, lane);
      const uint64_t vb = base + (incl - c);
      if (z < G.Z) vbase[lin] = (uint32_t)vb;
      if (mk) {
        const uint16_t key = dense[row[z] & 0x7FFFu];
        uint32_t m = mk;
        for (uint32_t k = 0; m; ++k) {
          const uint32_t d = (uint32_t)__ffs(m) - 1;
          m &= m - 1;
          vkey[vb + k] = key;
          vown[vb + k] = (unsigned long long)lin * 8ull + d;
        }
      }
      base += __shfl_sync(0xFFFFFFFFu, incl, 31);
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

// the 8 corner labels (bit 15 cleared) of cell (a, b, c): corner i is grid
// voxel (a + dx, b - 1 + dy, c - 1 + dz) for VF_MC_CORNER[i] = (dx, dy, dz)
__device__ __forceinline__ void cell_corners(const vfk::MeshGrid& G, int64_t a, int64_t b, int64_t c,
                                             uint32_t v[8]) {
  const uint32_t l00 = glab(G, a, b - 1, c - 1), l01 = glab(G, a, b - 1, c);
  const uint32_t m00 = glab(G, a - 1, b - 1, c - 1), m01 = glab(G, a - 1, b - 1, c);
  const uint32_t l10 = glab(G, a, b, c - 1), l11 = glab(G, a, b, c);
  const uint32_t m10 = glab(G, a - 1, b, c - 1), m11 = glab(G, a - 1, b, c);
  v[0] = l00 & 0x7FFFu;  // ( 0,0,0)
  v[1] = l01 & 0x7FFFu;  // ( 0,0,1)
  v[2] = m01 & 0x7FFFu;  // (-1,0,1)
  v[3] = m00 & 0x7FFFu;  // (-1,0,0)
  v[4] = l10 & 0x7FFFu;  // ( 0,1,0)
  v[5] = l11 & 0x7FFFu;  // ( 0,1,1)
  v[6] = m11 & 0x7FFFu;  // (-1,1,1)
  v[7] = m10 & 0x7FFFu;  // (-1,1,0)
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

__global__ void __launch_bounds__(256) k_mc_tcount(vfk::MeshGrid G, const unsigned long long* tri,
                                                   const uint8_t* ntri, uint32_t* rcnt) {
  __shared__ McShared S;
  load_table(S, tri, ntri);
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t a = (int64_t)(r / (G.Y + 1)), b = (int64_t)(r % (G.Y + 1));
    uint32_t n = 0;
    for (uint32_t c0 = 0; c0 <= G.Z; c0 += 32) {
      const int64_t c = c0 + lane;
      uint32_t k = 0;
      if (c <= (int64_t)G.Z) {
        uint32_t v[8];
        cell_corners(G, a, b, c, v);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (first_of(v, i)) k += S.ntri[config_of(v, v[i])];
      }
      n += __reduce_add_sync(0xFFFFFFFFu, k);
    }
    if (lane == 0) rcnt[r] = n;
  }
}

// offset (dx, dy, dz) of corner i, packed: bit 0 dx == -1, bit 1 dy, bit 2 dz
__device__ __forceinline__ uint32_t corner_bits(int i) {
  return (uint32_t)(0x3762'1540u >> (4 * i)) & 7u;  // 0:000 1:100 2:101 3:001 4:010 5:110 6:111 7:011
}

__global__ void __launch_bounds__(256) k_mc_temit(vfk::MeshGrid G, const unsigned long long* tri,
                                                  const uint8_t* ntri,
                                                  const unsigned long long* rbase,
                                                  const uint8_t* mask, const uint32_t* vbase,
                                                  const uint16_t* dense, uint16_t* tkey, uint4* tv,
                                                  uint32_t* vflag, uint32_t* err) {
  __shared__ McShared S;
  load_table(S, tri, ntri);
  const int lane = threadIdx.x & 31;
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const int64_t a = (int64_t)(r / (G.Y + 1)), b = (int64_t)(r % (G.Y + 1));
    uint64_t base = rbase[r];
    for (uint32_t c0 = 0; c0 <= G.Z; c0 += 32) {
      const int64_t c = c0 + lane;
      const bool in = c <= (int64_t)G.Z;
      uint32_t v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      uint32_t k = 0;
      if (in) {
        cell_corners(G, a, b, c, v);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (first_of(v, i)) k += S.ntri[config_of(v, v[i])];
      }
      const uint32_t incl = warp_incl_scan(k, lane);
      uint64_t t = base + (incl - k);
      if (k) {
        // boundary flag: bit 15 of the voxel at the cell's lattice point
        const uint32_t w = glab(G, a, b - 1, c - 1) >> 15;
        for (int i = 0; i < 8; ++i) {
          if (!first_of(v, i)) continue;
          const uint32_t tv_ = v[i];
          const uint32_t conf = config_of(v, tv_);
          const uint32_t nt = S.ntri[conf];
          const unsigned long long edges = S.tri[conf];
          const uint16_t key = dense[tv_];
          for (uint32_t q = 0; q < nt; ++q, ++t) {
            uint32_t id[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int slot = 3 * (int)q + (j == 0 ? 0 : (j == 1 ? 2 : 1));
              const uint32_t e = (uint32_t)(edges >> (4 * slot)) & 15u;
              // edge endpoints (VF_MC_EDGE)
              const uint32_t pa = (uint32_t)(0x3210'7654'3210ull >> (4 * e)) & 15u;
              const uint32_t pb = (uint32_t)(0x7654'4765'0321ull >> (4 * e)) & 15u;
              const bool a_own = v[pa] == tv_;
              const uint32_t own = a_own ? pa : pb, oth = a_own ? pb : pa;
              const uint32_t ob = corner_bits((int)own), tb = corner_bits((int)oth);
              const int64_t ox = a - (int64_t)(ob & 1u), oy = b - 1 + (int64_t)((ob >> 1) & 1u),
                            oz = c - 1 + (int64_t)((ob >> 2) & 1u);
              const uint32_t diff = ob ^ tb;  // one bit: the axis
              const uint32_t axis = diff == 1u ? 0u : (diff == 2u ? 1u : 2u);
              // +x is dx 0 vs -1: the other end is at larger x when its dx bit is clear
              const uint32_t up = axis == 0u ? ((tb & 1u) == 0u) : ((tb >> axis) & 1u);
              const uint32_t d = 2u * axis + up;
              const uint64_t lin = ((uint64_t)ox * G.Y + (uint64_t)oy) * G.Z + (uint64_t)oz;
              const uint32_t mk = mask[lin];
              if ((mk >> d) & 1u) {
                id[j] = vbase[lin] + (uint32_t)__popc(mk & ((1u << d) - 1u));
                if (w) atomicOr(vflag + (id[j] >> 5), 1u << (id[j] & 31u));
              } else {  // the owner's face mask must hold the edge's direction
                atomicOr(err, 1u);
                id[j] = 0;
              }
            }
            tkey[t] = key;
            tv[t] = make_uint4(id[0], id[1], id[2], 0u);
          }
        }
      }
      base += __shfl_sync(0xFFFFFFFFu, incl, 31);
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
  const uint64_t YZ = (uint64_t)G.Y * G.Z;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < V;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t gv = vperm[s];
    vinv[gv] = (uint32_t)s;
    const unsigned long long own = vown[gv];
    const uint64_t lin = own >> 3;
    const uint32_t d = (uint32_t)(own & 7ull);
    float p[3] = {(float)(lin / YZ + 1), (float)((lin / G.Z) % G.Y + 1), (float)(lin % G.Z + 1)};
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

__device__ __forceinline__ int32_t to_fixed(float p) {
  return __float2int_rz(__fmul_rn(p, 10000.0f));  // saturating, NaN -> 0
}

__global__ void __launch_bounds__(256) k_lap_faces(const uint4* gface, const float4* vert, uint64_t T,
                                                   int boundary, int4* acc) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < T;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 f = gface[s];
    const float4 p0 = vert[f.x], p1 = vert[f.y], p2 = vert[f.z];
    if (!boundary && !(p0.w == 0.0f && p1.w == 0.0f && p2.w == 0.0f)) continue;
    const uint32_t id[3] = {f.x, f.y, f.z};
    const float4 p[3] = {p0, p1, p2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int32_t qx = to_fixed(p[i].x), qy = to_fixed(p[i].y), qz = to_fixed(p[i].z);
#pragma unroll
      for (int j = 1; j <= 2; ++j) {
        int* a = reinterpret_cast<int*>(acc + id[(i + j) % 3]);
        atomicAdd(a + 0, qx);
        atomicAdd(a + 1, qy);
        atomicAdd(a + 2, qz);
        atomicAdd(a + 3, 1);
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_lap_finish(const int4* acc, uint64_t V, float target,
                                                    float omw, float weight, float4* vert) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < V;
       s += (uint64_t)gridDim.x * blockDim.x) {
    float4 p = vert[s];
    const int4 a = acc[s];
    if (p.w != target || a.w <= 0) continue;
    const float cnt = __int2float_rn(a.w);
    const float ax = __fdiv_rn(__fdiv_rn(__int2float_rn(a.x), cnt), 10000.0f);
    const float ay = __fdiv_rn(__fdiv_rn(__int2float_rn(a.y), cnt), 10000.0f);
    const float az = __fdiv_rn(__fdiv_rn(__int2float_rn(a.z), cnt), 10000.0f);
    p.x = __fadd_rn(__fmul_rn(p.x, omw), __fmul_rn(ax, weight));
    p.y = __fadd_rn(__fmul_rn(p.y, omw), __fmul_rn(ay, weight));
    p.z = __fadd_rn(__fmul_rn(p.z, omw), __fmul_rn(az, weight));
    vert[s] = p;
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
  if (rows) k_mc_vcount<<<grid_for(rows * 32, num_sms), 256, 0, st>>>(G, mask, rcnt, present);
}

void mc_vertex_emit(cudaStream_t st, const MeshGrid& G, const uint8_t* mask,
                    const unsigned long long* rbase, const uint16_t* dense, uint32_t* vbase,
                    uint16_t* vkey, unsigned long long* vown, int num_sms) {
  const uint64_t rows = (uint64_t)G.X * G.Y;
  if (rows)
    k_mc_vemit<<<grid_for(rows * 32, num_sms), 256, 0, st>>>(G, mask, rbase, dense, vbase, vkey, vown);
}

void mc_tri_count(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                  const uint8_t* ntri, uint32_t* rcnt, int num_sms) {
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  k_mc_tcount<<<grid_for(rows * 32, num_sms), 256, 0, st>>>(G, tri, ntri, rcnt);
}

void mc_tri_emit(cudaStream_t st, const MeshGrid& G, const unsigned long long* tri,
                 const uint8_t* ntri, const unsigned long long* rbase, const uint8_t* mask,
                 const uint32_t* vbase, const uint16_t* dense, uint16_t* tkey, uint4* tv,
                 uint32_t* vflag, uint32_t* err, int num_sms) {
  const uint64_t rows = (uint64_t)(G.X + 1) * (G.Y + 1);
  k_mc_temit<<<grid_for(rows * 32, num_sms), 256, 0, st>>>(G, tri, ntri, rbase, mask, vbase, dense,
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

void mc_smooth(cudaStream_t st, const uint4* gface, uint64_t T, float4* vert, uint64_t V, int4* acc,
               uint32_t iters, float weight, int boundary, int num_sms) {
  if (!V || !T) return;
  const float omw = 1.0f - weight;
  for (uint32_t it = 0; it < iters; ++it) {
    cudaMemsetAsync(acc, 0, V * sizeof(int4), st);
    k_lap_faces<<<grid_for(T, num_sms), 256, 0, st>>>(gface, vert, T, boundary, acc);
    k_lap_finish<<<grid_for(V, num_sms), 256, 0, st>>>(acc, V, boundary ? 1.0f : 0.0f, omw, weight,
                                                       vert);
  }
}

void mc_local_faces(cudaStream_t st, const uint4* gface, const uint32_t* tperm, const uint16_t* tkey,
                    const unsigned long long* voff, uint64_t T, uint4* out, int num_sms) {
  if (T) k_mc_local<<<grid_for(T, num_sms), 256, 0, st>>>(gface, tperm, tkey, voff, T, out);
}

}  // namespace vfk
