// vf_voxelize.cu -- solid voxelization of triangle meshes on sm_103a.
//
// Occupancy of a voxel = (some triangle overlaps the voxel box: FP32 SAT in
// the operation order of Intersections3D.h:204-258) OR (the voxel sample
// point is inside the mesh by tetra parity: Tetravoxelizer.cpp:42-92, 198-315).
//
// Stages, all batched over every job of a batch:
//   centroid_and_slices : one 1024-thread block per job; fixed-order
//                         lane sums of the vertices + the slice planes
//   tetra_prep          : one thread per face -> its vertices in NDC sorted
//                         by y, the slice planes crossing it, one use of each
//                         edge in the job's edge parity table
//   parity_raster       : the tetra-parity fill computed from edge crossings
//                         (derivation above k_tetra): (face, slice) segments
//                         flattened by a prefix sum over the faces and run in
//                         warp-interleaved runs, the internal faces of edges
//                         used an odd number of times, then a prefix XOR
//                         along x turns the per-row crossing markers into the
//                         parity plane
//   shell_sat           : per-face work items (columns of the triangle's
//                         footprint) flattened by a prefix sum; warps test
//                         runs of items with the exact SAT
//   combine             : one CTA per brick; bit planes -> uint16 0/1 rows,
//                         brick liveness
// All float arithmetic uses the _rn intrinsics (and the file is compiled
// with -fmad=false): every result is bit-identical to the CPU oracle.
#include "vf_kernels.h"

namespace {

__device__ __forceinline__ int job_of_face(const JobDesc* J, int njobs, uint32_t f) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (J[mid].face_base <= f) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_centroid(const JobDesc* jobs, JobState* st) {
  const JobDesc& J = jobs[blockIdx.x];
  __shared__ float sx[1024], sy[1024], sz[1024];
  const int t = threadIdx.x;
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
  for (uint32_t i = t; i < J.nverts; i += 1024) {
    a0 = __fadd_rn(a0, J.verts[3 * (size_t)i]);
    a1 = __fadd_rn(a1, J.verts[3 * (size_t)i + 1]);
    a2 = __fadd_rn(a2, J.verts[3 * (size_t)i + 2]);
  }
  sx[t] = a0; sy[t] = a1; sz[t] = a2;
  for (int s = 512; s >= 1; s >>= 1) {
    __syncthreads();
    if (t < s) {
      sx[t] = __fadd_rn(sx[t], sx[t + s]);
      sy[t] = __fadd_rn(sy[t], sy[t + s]);
      sz[t] = __fadd_rn(sz[t], sz[t + s]);
    }
  }
  __syncthreads();
  if (t == 0) {
    float n = (float)J.nverts;
    st[blockIdx.x].centroid[0] = __fdiv_rn(sx[0], n);
    st[blockIdx.x].centroid[1] = __fdiv_rn(sy[0], n);
    st[blockIdx.x].centroid[2] = __fdiv_rn(sz[0], n);
    // ySlice = -1; ySlice += 2/res.y (Tetravoxelizer.cpp:280-293)
    float step = __fdiv_rn(2.0f, (float)J.Y), acc = -1.0f;
    for (uint32_t s = 0; s < J.Y; ++s) {
      J.ys[s] = acc;
      acc = __fadd_rn(acc, step);
    }
  }
}

struct tv { float x, y, z; };

__device__ __forceinline__ tv to_ndc(const float* v, const float* ctr, const float* dim) {
  // scaleToNDC: 2*(v - c)/dim (Tetravoxelizer.h:70-72)
  tv r;
  r.x = __fdiv_rn(__fmul_rn(2.0f, __fsub_rn(v[0], ctr[0])), dim[0]);
  r.y = __fdiv_rn(__fmul_rn(2.0f, __fsub_rn(v[1], ctr[1])), dim[1]);
  r.z = __fdiv_rn(__fmul_rn(2.0f, __fsub_rn(v[2], ctr[2])), dim[2]);
  return r;
}

__device__ __forceinline__ uint32_t upper_bound_f(const float* a, uint32_t n, float v) {
  uint32_t lo = 0, hi = n;  // first index with a[i] > v
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] > v) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// ---- parity by edge crossings ---------------------------------------------
// The reference rasterises, for every slice plane, the cross-section of every
// tetrahedron (face + centroid) with XOR at pixel centres (GL rules: 8
// sub-pixel bits, top-left ownership of samples on edges).  With that rule a
// sample p is inside a cross-section triangle exactly when the point
// p + (e, e^2) (e -> 0) is inside the open triangle, and that point lies on
// no edge and no vertex line.  A ray from it towards -x therefore crosses the
// triangle's boundary an odd number of times exactly when p is inside; for a
// zero-area triangle (never rasterised) the crossings are even.  Hence the
// XOR of all rasterised triangles at p is the parity of the number of
// cross-section EDGES that the ray crosses, and an edge's crossing depends
// only on its two snapped end points:
//   edge (u, v), u.z < v.z (fixed point), crosses at pixel centre
//   p = (256 i + 128, 256 k + 128)  iff  u.z <= p.z < v.z  and
//   (v.x - u.x)(p.z - u.z) - (v.z - u.z)(p.x - u.x) <= 0.
// Each cross-section edge lies on one face of its tetrahedron and its end
// points are INTERP on two tetrahedron edges (lower-y vertex first).  An
// internal face (mesh edge + centroid) is shared by every tetrahedron whose
// mesh face holds that edge, and each computes the same end points, so the
// copies cancel in pairs: only the mesh faces' own segments and the internal
// faces of mesh edges used an odd number of times (open or non-manifold
// meshes) contribute.  Per segment and pixel row the first crossed pixel
// gets a marker bit; a prefix XOR along x then yields the parity plane.
// The quad split's diagonal belongs to both of its triangles and cancels.

// slot value of an edge parity table: lo << 32 | hi (lo < hi < 2^31), bit 63
// toggled once per use of the edge; an empty slot is all ones
#define VF_EDGE_EMPTY 0xFFFFFFFFFFFFFFFFull
#define VF_EDGE_ODD 0x8000000000000000ull

__device__ __forceinline__ void edge_use(const JobDesc& J, uint32_t a, uint32_t b) {
  if (a == b) return;  // a degenerate edge bounds a zero-area face: no crossing
  const unsigned long long key =
      a < b ? ((unsigned long long)a << 32 | b) : ((unsigned long long)b << 32 | a);
  const uint32_t mask = J.ecap - 1;
  uint32_t h = (uint32_t)vf_mix64(key) & mask;
  for (uint32_t probe = 0; probe < J.ecap; ++probe) {
    const unsigned long long old = atomicCAS(J.etab + h, VF_EDGE_EMPTY, key);
    if (old == VF_EDGE_EMPTY || (old & ~VF_EDGE_ODD) == key) {
      atomicXor(J.etab + h, VF_EDGE_ODD);
      return;
    }
    h = (h + 1) & mask;
  }
}

__device__ __forceinline__ void sort3_y(tv* v) {
  tv t;
#define SW(a, b) if (v[a].y > v[b].y) { t = v[a]; v[a] = v[b]; v[b] = t; }
  SW(0, 1) SW(1, 2) SW(0, 1)
#undef SW
}

// per face: NDC vertices sorted by y, the slice planes crossing the face
// (P0.y < ys[s] <= P2.y), and one use of each of its edges
__global__ void k_tetra(const JobDesc* jobs, JobState* st, int njobs, uint32_t total,
                        uint32_t* pcnt) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += gridDim.x * blockDim.x) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    const uint32_t f = g - J.face_base;
    const uint32_t i0 = J.faces[3 * (size_t)f], i1 = J.faces[3 * (size_t)f + 1],
                   i2 = J.faces[3 * (size_t)f + 2];
    if (i0 >= J.nverts || i1 >= J.nverts || i2 >= J.nverts) {
      atomicOr(&st[j].err, VF_JERR_INVALID);  // bad face: never dereferenced
      J.tet_range[f] = 0xFFFFu;
      pcnt[g] = 0;
      continue;
    }
    float ctr[3], dim[3];
    for (int a = 0; a < 3; ++a) {
      ctr[a] = __fmul_rn(0.5f, __fadd_rn(J.amin[a], J.amax[a]));
      dim[a] = __fsub_rn(J.amax[a], J.amin[a]);
    }
    tv v[3];
    v[0] = to_ndc(J.verts + 3 * (size_t)i0, ctr, dim);
    v[1] = to_ndc(J.verts + 3 * (size_t)i1, ctr, dim);
    v[2] = to_ndc(J.verts + 3 * (size_t)i2, ctr, dim);
    sort3_y(v);
    float4* o = J.tets + 3 * (size_t)f;
    o[0] = make_float4(v[0].x, v[0].y, v[0].z, v[1].x);
    o[1] = make_float4(v[1].y, v[1].z, v[2].x, v[2].y);
    o[2] = make_float4(v[2].z, 0.0f, 0.0f, 0.0f);
    const uint32_t s0 = upper_bound_f(J.ys, J.Y, v[0].y);
    const uint32_t s1e = upper_bound_f(J.ys, J.Y, v[2].y);
    J.tet_range[f] = (s1e > s0) ? (s0 | ((s1e - 1) << 16)) : 0xFFFFu;
    pcnt[g] = s1e > s0 ? s1e - s0 : 0u;  // (face, slice) items
    edge_use(J, i0, i1);
    edge_use(J, i1, i2);
    edge_use(J, i2, i0);
  }
}

// ---- exact segment arithmetic (INTERP and the raster rule of the oracle) ---
__device__ __forceinline__ float interp_c(float a, float b, float t) {
  return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t));
}
__device__ __forceinline__ void interp(const tv& A, const tv& B, float s, float& ox, float& oz) {
  float t = __fdiv_rn(__fsub_rn(s, A.y), __fsub_rn(B.y, A.y));
  ox = interp_c(A.x, B.x, t);
  oz = interp_c(A.z, B.z, t);
}
__device__ __forceinline__ int32_t to_fixed(float ndc, float half) {
  float w = __fadd_rn(__fmul_rn(ndc, half), half);
  return __float2int_rn(__fmul_rn(w, 256.0f));
}
__device__ __forceinline__ int ceil_div_i(int a, int b) {  // b > 0
  return a >= 0 ? (a + b - 1) / b : -((-a) / b);
}
__device__ __forceinline__ long long ceil_div_ll(long long a, long long b) {  // b > 0
  return a >= 0 ? (a + b - 1) / b : -((-a) / b);
}

// markers of one snapped segment in the parity plane of `slice`: per pixel
// row k it crosses, the first pixel column i whose centre the -x ray from
// (centre + (e, e^2)) sees the segment from
__device__ void segment_markers(const JobDesc& J, uint32_t slice, int ax, int az, int bx, int bz) {
  if (az == bz) return;  // horizontal: the ray at z + e^2 never meets it
  int ux = ax, uz = az, vx = bx, vz = bz;
  if (uz > vz) { ux = bx; uz = bz; vx = ax; vz = az; }
  const int klo = max(ceil_div_i(uz - 128, 256), 0);
  const int khi = min(ceil_div_i(vz - 128, 256) - 1, (int)J.Z - 1);
  if (klo > khi) return;
  const long long dz = vz - uz, dx = vx - ux;
  const long long den = 256 * dz;
  uint32_t* const col = J.par + (size_t)slice * J.Zw;
  const size_t istride = (size_t)J.Y * J.Zw;
  for (int k = klo; k <= khi; ++k) {
    // pixel centre x >= u.x + dx (pz - u.z) / dz
    const long long num = dz * ux + dx * ((long long)k * 256 + 128 - uz) - 128 * dz;
    long long i = ceil_div_ll(num, den);
    if (i < 0) i = 0;
    if (i >= (long long)J.X) continue;
    atomicXor(col + (size_t)i * istride + (k >> 5), 1u << (k & 31));
  }
}

// the segment of triangle P (sorted by y, P0.y < sl <= P2.y) in plane sl:
// INTERP on P0-P2 and on P0-P1 or P1-P2 (Tetravoxelizer.cpp:45-89)
__device__ __forceinline__ void face_segment(const JobDesc& J, const tv& P0, const tv& P1,
                                             const tv& P2, uint32_t s) {
  const float sl = J.ys[s];
  float ax, az, bx, bz;
  interp(P0, P2, sl, ax, az);
  const bool lo = sl <= P1.y;
  interp(lo ? P0 : P1, lo ? P1 : P2, sl, bx, bz);
  const float hw = __fmul_rn(0.5f, (float)J.X), hh = __fmul_rn(0.5f, (float)J.Z);
  segment_markers(J, s, to_fixed(ax, hw), to_fixed(az, hh), to_fixed(bx, hw), to_fixed(bz, hh));
}

// ---- exclusive scan of the per-face pair counts (1024 faces per block) -----
__device__ __forceinline__ unsigned long long warp_incl_scan(unsigned long long v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}
// block-wide exclusive scan of one value per thread (blockDim 1024)
__device__ unsigned long long block_excl_scan(unsigned long long v, unsigned long long* total) {
  __shared__ unsigned long long ws[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned long long inc = warp_incl_scan(v);
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    const unsigned long long x = ws[lane];
    ws[lane] = warp_incl_scan(x) - x;
  }
  __syncthreads();
  const unsigned long long r = ws[w] + inc - v;
  if (total && threadIdx.x == blockDim.x - 1) *total = r + v;
  __syncthreads();
  return r;
}
__global__ void __launch_bounds__(1024) k_scan_local(const uint32_t* in, unsigned long long* out,
                                                     unsigned long long* sums, uint32_t n) {
  const uint32_t i = blockIdx.x * 1024u + threadIdx.x;
  const unsigned long long v = i < n ? in[i] : 0ull;
  __shared__ unsigned long long tot;
  const unsigned long long r = block_excl_scan(v, &tot);
  if (i < n) out[i] = r;
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}
__global__ void __launch_bounds__(1024) k_scan_sums(unsigned long long* sums, uint32_t nb,
                                                    unsigned long long* grand) {
  // one block: each thread owns a contiguous chunk of block sums
  const uint32_t per = (nb + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per, b1 = min(b0 + per, nb);
  unsigned long long acc = 0;
  for (uint32_t b = b0; b < b1; ++b) acc += sums[b];
  __shared__ unsigned long long tot;
  unsigned long long base = block_excl_scan(acc, &tot);
  for (uint32_t b = b0; b < b1; ++b) {
    const unsigned long long t = sums[b];
    sums[b] = base;
    base += t;
  }
  if (threadIdx.x == 0) *grand = tot;
}
__global__ void k_scan_add(unsigned long long* out, const unsigned long long* sums, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / 1024u];
}

// Warp-interleaved runs over a flattened work list (faces in batch order,
// items of a face contiguous): a warp owns WARP_RUN consecutive items and
// lane l takes items base + l, base + l + 32, ...  Neighbouring lanes work on
// neighbouring items of the same face, so control flow stays coherent and no
// lane idles when a face has few items.  One binary search per warp run; each
// lane then steps its face cursor forward.
constexpr uint32_t WARP_RUN = 32 * 16;

__device__ __forceinline__ uint32_t face_of_item(const unsigned long long* base, uint32_t nfaces,
                                                 unsigned long long p) {
  uint32_t lo = 0, hi = nfaces - 1;  // last face whose first item is <= p
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (base[mid] <= p) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_parity_flat(const JobDesc* jobs, int njobs,
                                                  const uint32_t* pcnt,
                                                  const unsigned long long* pbase,
                                                  const unsigned long long* ptotal,
                                                  uint32_t total_faces) {
  const unsigned long long total = *ptotal;
  const int lane = threadIdx.x & 31;
  const unsigned long long nwruns = (total + WARP_RUN - 1) / WARP_RUN;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  for (unsigned long long wr = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
       wr < nwruns; wr += nwarps) {
    const unsigned long long base = wr * WARP_RUN;
    const unsigned long long end = min(base + WARP_RUN, total);
    uint32_t g = 0;
    if (lane == 0) g = face_of_item(pbase, total_faces, base);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    uint32_t cached = 0xFFFFFFFFu;
    tv P0, P1, P2;
    const JobDesc* J = nullptr;
    uint32_t s0 = 0;
    unsigned long long fb = 0;
    for (unsigned long long p = base + lane; p < end; p += 32) {
      // advance the face cursor (faces with no item have pbase equal to the next)
      while (p >= pbase[g] + pcnt[g]) ++g;
      if (g != cached) {
        cached = g;
        J = &jobs[job_of_face(jobs, njobs, g)];
        const uint32_t f = g - J->face_base;
        const float4* o = J->tets + 3 * (size_t)f;
        const float4 q0 = o[0], q1 = o[1], q2 = o[2];
        P0 = {q0.x, q0.y, q0.z};
        P1 = {q0.w, q1.x, q1.y};
        P2 = {q1.z, q1.w, q2.x};
        s0 = J->tet_range[f] & 0xFFFFu;
        fb = pbase[g];
      }
      face_segment(*J, P0, P1, P2, s0 + (uint32_t)(p - fb));
    }
  }
}

// internal faces (mesh edge + centroid) of the edges used an odd number of
// times: one warp per table word of 32 slots, lanes over the slice planes
__global__ void __launch_bounds__(256) k_odd_edges(const JobDesc* jobs, const JobState* st,
                                                   int njobs) {
  const int lane = threadIdx.x & 31;
  for (int j = blockIdx.y; j < njobs; j += gridDim.y) {
    const JobDesc& J = jobs[j];
    if (!J.nfaces || !J.ecap) continue;
    float ctr[3], dim[3];
    for (int a = 0; a < 3; ++a) {
      ctr[a] = __fmul_rn(0.5f, __fadd_rn(J.amin[a], J.amax[a]));
      dim[a] = __fsub_rn(J.amax[a], J.amin[a]);
    }
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < J.ecap / 32;
         w += (gridDim.x * blockDim.x) >> 5) {
      const unsigned long long v = J.etab[w * 32 + lane];
      unsigned m = __ballot_sync(0xFFFFFFFFu, v != VF_EDGE_EMPTY && (v & VF_EDGE_ODD));
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const unsigned long long key = __shfl_sync(0xFFFFFFFFu, v, src) & ~VF_EDGE_ODD;
        tv p[3];
        p[0] = to_ndc(J.verts + 3 * (size_t)(uint32_t)(key >> 32), ctr, dim);
        p[1] = to_ndc(J.verts + 3 * (size_t)(uint32_t)key, ctr, dim);
        p[2] = to_ndc(st[j].centroid, ctr, dim);
        sort3_y(p);
        const uint32_t s0 = upper_bound_f(J.ys, J.Y, p[0].y);
        const uint32_t s1e = upper_bound_f(J.ys, J.Y, p[2].y);
        for (uint32_t s = s0 + lane; s < s1e; s += 32) face_segment(J, p[0], p[1], p[2], s);
      }
    }
  }
}

// markers -> parity: prefix XOR along x of every (y, z-word) column
__global__ void __launch_bounds__(256) k_prefix_x(const JobDesc* jobs, int njobs) {
  for (int j = blockIdx.y; j < njobs; j += gridDim.y) {
    const JobDesc& J = jobs[j];
    if (!J.nfaces) continue;
    const uint32_t cols = J.Y * J.Zw;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
      uint32_t* p = J.par + c;
      uint32_t run = 0;
      uint32_t x = 0;
      for (; x + 8 <= J.X; x += 8) {
        uint32_t w[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) w[q] = p[(size_t)(x + q) * cols];
#pragma unroll
        for (int q = 0; q < 8; ++q) { run ^= w[q]; p[(size_t)(x + q) * cols] = run; }
      }
      for (; x < J.X; ++x) { run ^= p[(size_t)x * cols]; p[(size_t)x * cols] = run; }
    }
  }
}

// ---- SAT (Intersections3D.h:204-420), FP32 without contraction -----------
struct satd { tv v0, v1, v2, r; };

__device__ __forceinline__ bool ax_test(float pa, float pb, float rad) {
  float mn = pa < pb ? pa : pb, mx = pa < pb ? pb : pa;
  return !(mn > rad || mx < -rad);
}
#define MUL __fmul_rn
#define ADD __fadd_rn
#define SUB __fsub_rn
__device__ __forceinline__ bool x01(const satd& d, float a, float b, float fa, float fb) {
  float p0 = SUB(MUL(a, d.v0.y), MUL(b, d.v0.z)), p2 = SUB(MUL(a, d.v2.y), MUL(b, d.v2.z));
  return ax_test(p0, p2, ADD(MUL(fa, d.r.y), MUL(fb, d.r.z)));
}
__device__ __forceinline__ bool x2(const satd& d, float a, float b, float fa, float fb) {
  float p0 = SUB(MUL(a, d.v0.y), MUL(b, d.v0.z)), p1 = SUB(MUL(a, d.v1.y), MUL(b, d.v1.z));
  return ax_test(p0, p1, ADD(MUL(fa, d.r.y), MUL(fb, d.r.z)));
}
__device__ __forceinline__ bool y02(const satd& d, float a, float b, float fa, float fb) {
  float p0 = ADD(MUL(-a, d.v0.x), MUL(b, d.v0.z)), p2 = ADD(MUL(-a, d.v2.x), MUL(b, d.v2.z));
  return ax_test(p0, p2, ADD(MUL(fa, d.r.x), MUL(fb, d.r.z)));
}
__device__ __forceinline__ bool y1(const satd& d, float a, float b, float fa, float fb) {
  float p0 = ADD(MUL(-a, d.v0.x), MUL(b, d.v0.z)), p1 = ADD(MUL(-a, d.v1.x), MUL(b, d.v1.z));
  return ax_test(p0, p1, ADD(MUL(fa, d.r.x), MUL(fb, d.r.z)));
}
__device__ __forceinline__ bool z12(const satd& d, float a, float b, float fa, float fb) {
  float p1 = SUB(MUL(a, d.v1.x), MUL(b, d.v1.y)), p2 = SUB(MUL(a, d.v2.x), MUL(b, d.v2.y));
  // zAxisTest_12 orders (p2, p1): same min/max
  return ax_test(p1, p2, ADD(MUL(fa, d.r.x), MUL(fb, d.r.y)));
}
__device__ __forceinline__ bool z0(const satd& d, float a, float b, float fa, float fb) {
  float p0 = SUB(MUL(a, d.v0.x), MUL(b, d.v0.y)), p1 = SUB(MUL(a, d.v1.x), MUL(b, d.v1.y));
  return ax_test(p0, p1, ADD(MUL(fa, d.r.x), MUL(fb, d.r.y)));
}
__device__ __forceinline__ void mm3(float a, float b, float c, float& mn, float& mx) {
  mn = mx = a;
  if (b < mn) mn = b;
  if (b > mx) mx = b;
  if (c < mn) mn = c;
  if (c > mx) mx = c;
}
// The SAT as a conjunction of tests, each evaluated exactly as
// Intersections3D.h:204-258 does; MASK selects which run (a separating axis
// makes the result false whatever the order).  Bits 0-8: the edge-cross-axis
// tests (edge e0: x01 y02 z12; e1: x01 y02 z0; e2: x2 y1 z12), bits 9-11: the
// box axes x, y, z, bit 12: the plane-box test.
constexpr uint32_t SAT_ALL = 0x1FFFu;
// tests that use only the two axes other than C: the same for every cell of
// a column along C (the x-axis family uses y, z; the box axes other than C)
__host__ __device__ constexpr uint32_t sat_column_mask(int C) {
  return C == 0 ? ((1u << 0) | (1u << 3) | (1u << 6) | (1u << 10) | (1u << 11))
       : C == 1 ? ((1u << 1) | (1u << 4) | (1u << 7) | (1u << 9) | (1u << 11))
                : ((1u << 2) | (1u << 5) | (1u << 8) | (1u << 9) | (1u << 10));
}

template <uint32_t MASK>
__device__ __forceinline__ bool tri_box_sel(const tv& p0, const tv& p1, const tv& p2, const tv& c,
                                            const tv& r) {
  satd d;
  d.r = r;
  d.v0 = {SUB(p0.x, c.x), SUB(p0.y, c.y), SUB(p0.z, c.z)};
  d.v1 = {SUB(p1.x, c.x), SUB(p1.y, c.y), SUB(p1.z, c.z)};
  d.v2 = {SUB(p2.x, c.x), SUB(p2.y, c.y), SUB(p2.z, c.z)};
  tv e0 = {SUB(d.v1.x, d.v0.x), SUB(d.v1.y, d.v0.y), SUB(d.v1.z, d.v0.z)};
  tv e1 = {SUB(d.v2.x, d.v1.x), SUB(d.v2.y, d.v1.y), SUB(d.v2.z, d.v1.z)};
  tv e2 = {SUB(d.v0.x, d.v2.x), SUB(d.v0.y, d.v2.y), SUB(d.v0.z, d.v2.z)};
  float fx = fabsf(e0.x), fy = fabsf(e0.y), fz = fabsf(e0.z);
  if ((MASK & (1u << 0)) && !x01(d, e0.z, e0.y, fz, fy)) return false;
  if ((MASK & (1u << 1)) && !y02(d, e0.z, e0.x, fz, fx)) return false;
  if ((MASK & (1u << 2)) && !z12(d, e0.y, e0.x, fy, fx)) return false;
  fx = fabsf(e1.x); fy = fabsf(e1.y); fz = fabsf(e1.z);
  if ((MASK & (1u << 3)) && !x01(d, e1.z, e1.y, fz, fy)) return false;
  if ((MASK & (1u << 4)) && !y02(d, e1.z, e1.x, fz, fx)) return false;
  if ((MASK & (1u << 5)) && !z0(d, e1.y, e1.x, fy, fx)) return false;
  fx = fabsf(e2.x); fy = fabsf(e2.y); fz = fabsf(e2.z);
  if ((MASK & (1u << 6)) && !x2(d, e2.z, e2.y, fz, fy)) return false;
  if ((MASK & (1u << 7)) && !y1(d, e2.z, e2.x, fz, fx)) return false;
  if ((MASK & (1u << 8)) && !z12(d, e2.y, e2.x, fy, fx)) return false;
  float mn, mx;
  if (MASK & (1u << 9)) {
    mm3(d.v0.x, d.v1.x, d.v2.x, mn, mx);
    if (mn > d.r.x || mx < -d.r.x) return false;
  }
  if (MASK & (1u << 10)) {
    mm3(d.v0.y, d.v1.y, d.v2.y, mn, mx);
    if (mn > d.r.y || mx < -d.r.y) return false;
  }
  if (MASK & (1u << 11)) {
    mm3(d.v0.z, d.v1.z, d.v2.z, mn, mx);
    if (mn > d.r.z || mx < -d.r.z) return false;
  }
  if (!(MASK & (1u << 12))) return true;
  tv n = {SUB(MUL(e0.y, e1.z), MUL(e1.y, e0.z)), SUB(MUL(e0.z, e1.x), MUL(e1.z, e0.x)),
          SUB(MUL(e0.x, e1.y), MUL(e1.x, e0.y))};
  // planeBoxOverlap
  float nv[3] = {n.x, n.y, n.z}, vv[3] = {d.v0.x, d.v0.y, d.v0.z}, m[3] = {r.x, r.y, r.z};
  float vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    if (nv[q] > 0.0f) { vmin[q] = SUB(-m[q], vv[q]); vmax[q] = SUB(m[q], vv[q]); }
    else { vmin[q] = SUB(m[q], vv[q]); vmax[q] = SUB(-m[q], vv[q]); }
  }
  if (ADD(ADD(MUL(nv[0], vmin[0]), MUL(nv[1], vmin[1])), MUL(nv[2], vmin[2])) > 0.0f) return false;
  if (ADD(ADD(MUL(nv[0], vmax[0]), MUL(nv[1], vmax[1])), MUL(nv[2], vmax[2])) >= 0.0f) return true;
  return false;
}

// the voxel box of cell (i, j, k) as RegularGrid::getAABBs builds it
__device__ __forceinline__ void cell_box(const JobDesc& J, const float* cs, int i, int jj, int k,
                                         tv& ce, tv& r) {
  tv bmin = {ADD(J.amin[0], MUL(cs[0], (float)i)), ADD(J.amin[1], MUL(cs[1], (float)jj)),
             ADD(J.amin[2], MUL(cs[2], (float)k))};
  tv bmax = {ADD(bmin.x, cs[0]), ADD(bmin.y, cs[1]), ADD(bmin.z, cs[2])};
  // (max + min) / 2: x * 0.5 and x / 2 are the same correctly rounded value
  ce = {MUL(ADD(bmax.x, bmin.x), 0.5f), MUL(ADD(bmax.y, bmin.y), 0.5f),
        MUL(ADD(bmax.z, bmin.z), 0.5f)};
  r = {SUB(bmax.x, ce.x), SUB(bmax.y, ce.y), SUB(bmax.z, ce.z)};
}

__device__ __forceinline__ int float_cell(float f, int n) {
  if (!(f > -1.0e9f)) f = -1.0e9f;
  if (f > 1.0e9f) f = 1.0e9f;
  return vf_clampi((int)floorf(f), -2, n + 1);
}

// the exact test of one voxel (reference operation order) and the mark.
// column_done: the column tests of axis c already passed for this cell's
// column, so only the rest of the SAT runs; c < 0: the whole SAT
__device__ __forceinline__ void test_cell(const JobDesc& J, const float* cs, const tv& p0,
                                          const tv& p1, const tv& p2, int i, int jj, int k, int c) {
  tv ce, r;
  cell_box(J, cs, i, jj, k, ce, r);
  bool hit;
  if (c == 0) hit = tri_box_sel<SAT_ALL ^ sat_column_mask(0)>(p0, p1, p2, ce, r);
  else if (c == 1) hit = tri_box_sel<SAT_ALL ^ sat_column_mask(1)>(p0, p1, p2, ce, r);
  else if (c == 2) hit = tri_box_sel<SAT_ALL ^ sat_column_mask(2)>(p0, p1, p2, ce, r);
  else hit = tri_box_sel<SAT_ALL>(p0, p1, p2, ce, r);
  if (hit) atomicOr(J.shell + ((size_t)i * J.Y + jj) * J.Zw + (k >> 5), 1u << (k & 31));
}

// Per-face setup of the shell test.  Candidates: the cells touching the
// triangle's bounding box (widened by 0.01 cell + 256 ulp of the largest
// coordinate: any cell further out fails the exact box-axis tests), as
// columns along the dominant normal axis c.  Per
// column, (1) the SAT tests that do not involve axis c (the c-family edge
// axes and the two other box axes) run exactly, once: they are the same for
// every cell of the column, and a column they reject holds no hit; (2) the
// plane slab along c bounds the cells, with a margin (2% of a cell + 64 ulp
// of the largest coordinate) far beyond the rounding of the float SAT, so no
// cell the exact test accepts is dropped.  Each remaining cell then runs the
// rest of the SAT.  The marked set equals testing the full bbox.
// Work items: columns (a, b) when pruning, else every bbox cell (whole SAT).
struct ShellSetup {
  float cs[3];                 // cell size (x, y, z)
  tv p0, p1, p2;               // the triangle
  // pruning, in the axes (a, b, c) = (c+1, c+2, c) mod 3; without pruning
  // (a, b, c) = (x, y, z) and every bbox cell is an item
  float amin_a, amin_b, amin_c, cs_a, cs_b, q0_a, q0_b, q0_c, nr_a, nr_b;
  float Pa1, Pb1, Pa2, Pb2;    // projected triangle relative to p0 (ccw)
  float ha, hb, w, inr, ics;
  int lo_a, lo_b, lo_c, n_b, n_c, hi_c;
  int c;
  bool prune;
  uint32_t items;
};

__device__ bool shell_setup(const JobDesc& J, uint32_t f, ShellSetup& S) {
  const uint32_t dims[3] = {J.X, J.Y, J.Z};
  for (int a = 0; a < 3; ++a) S.cs[a] = J.cs[a];
  const uint32_t* fi = J.faces + 3 * (size_t)f;
  if (fi[0] >= J.nverts || fi[1] >= J.nverts || fi[2] >= J.nverts) return false;
  const float* q0 = J.verts + 3 * (size_t)fi[0];
  const float* q1 = J.verts + 3 * (size_t)fi[1];
  const float* q2 = J.verts + 3 * (size_t)fi[2];
  // The largest coordinate in play sets the rounding scale of the float SAT
  // (box bounds, centres, vertex offsets): its errors are a few ulp of M.
  float M = 0.0f;
  for (int a = 0; a < 3; ++a) {
    M = fmaxf(M, fmaxf(fabsf(J.amin[a]), fabsf(J.amax[a])));
    M = fmaxf(M, fmaxf(fabsf(q0[a]), fmaxf(fabsf(q1[a]), fabsf(q2[a]))));
  }
  const float ulp64 = M * 7.62939453125e-6f;  // 64 * 2^-23 * M
  int lo[3], n[3];
  for (int a = 0; a < 3; ++a) {
    float mn, mx;
    mm3(q0[a], q1[a], q2[a], mn, mx);
    // Cells that touch the triangle's extent along a, widened by 0.01 cell +
    // 256 ulp of M: a cell further out fails the exact SAT's box-axis test,
    // whose roundings are a few ulp of M; the 0.01 cell covers the rounding
    // of these index computations (below 2^-11 cell for 4096 cells).
    const float mc = 0.01f + 4.0f * ulp64 * J.ics[a];
    lo[a] = vf_clampi(float_cell(SUB(mn, J.amin[a]) * J.ics[a] - mc, dims[a]), 0, dims[a] - 1);
    const int hi = vf_clampi(float_cell(SUB(mx, J.amin[a]) * J.ics[a] + mc, dims[a]), 0, dims[a] - 1);
    n[a] = hi - lo[a] + 1;
  }
  S.p0 = {q0[0], q0[1], q0[2]};
  S.p1 = {q1[0], q1[1], q1[2]};
  S.p2 = {q2[0], q2[1], q2[2]};
  const float e1[3] = {q1[0] - q0[0], q1[1] - q0[1], q1[2] - q0[2]};
  const float e2[3] = {q2[0] - q0[0], q2[1] - q0[1], q2[2] - q0[2]};
  const float nr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                       e1[0] * e2[1] - e1[1] * e2[0]};
  int c = fabsf(nr[1]) > fabsf(nr[0]) ? 1 : 0;
  if (fabsf(nr[2]) > fabsf(c ? nr[1] : nr[0])) c = 2;
  const float e1n = fabsf(e1[0]) + fabsf(e1[1]) + fabsf(e1[2]);
  const float e2n = fabsf(e2[0]) + fabsf(e2[1]) + fabsf(e2[2]);
  const float nrc_abs = fabsf(c == 0 ? nr[0] : (c == 1 ? nr[1] : nr[2]));
  S.prune = nrc_abs > 1e-3f * e1n * e2n && nrc_abs > 0.0f;
  if (!S.prune) {
    S.c = 2;
    S.lo_a = lo[0]; S.lo_b = lo[1]; S.lo_c = lo[2];
    S.n_b = n[1]; S.n_c = n[2]; S.hi_c = lo[2] + n[2] - 1;
    S.nr_a = S.nr_b = S.inr = S.Pa1 = S.Pb1 = S.Pa2 = S.Pb2 = S.ha = S.hb = S.w = 0.0f;
    S.items = (uint32_t)(n[0] * n[1] * n[2]);
    return true;
  }
  const int ax = (c + 1) % 3, bx = (c + 2) % 3;
  // register selects instead of dynamic indexing (keeps the arrays out of
  // local memory)
#define SEL(v, i) ((i) == 0 ? (v)[0] : ((i) == 1 ? (v)[1] : (v)[2]))
  S.c = c;
  S.lo_a = SEL(lo, ax); S.lo_b = SEL(lo, bx); S.lo_c = SEL(lo, c);
  const int n_a = SEL(n, ax);
  S.n_b = SEL(n, bx); S.n_c = SEL(n, c); S.hi_c = S.lo_c + S.n_c - 1;
  S.amin_a = SEL(J.amin, ax); S.amin_b = SEL(J.amin, bx); S.amin_c = SEL(J.amin, c);
  S.cs_a = SEL(S.cs, ax); S.cs_b = SEL(S.cs, bx);
  const float cs_c = SEL(S.cs, c);
  S.q0_a = SEL(q0, ax); S.q0_b = SEL(q0, bx); S.q0_c = SEL(q0, c);
  S.nr_a = SEL(nr, ax); S.nr_b = SEL(nr, bx);
  const float nr_c = SEL(nr, c);
  float P1a = SEL(e1, ax), P1b = SEL(e1, bx), P2a = SEL(e2, ax), P2b = SEL(e2, bx);
#define SEL2(v, i) ((i) == 0 ? (v)[0] : ((i) == 1 ? (v)[1] : (v)[2]))
#undef SEL
  if (nr_c < 0.0f) { float t = P1a; P1a = P2a; P2a = t; t = P1b; P1b = P2b; P2b = t; }
  S.Pa1 = P1a; S.Pb1 = P1b; S.Pa2 = P2a; S.Pb2 = P2b;
  // half cell + margin.  The margin (2% of a cell + 64 ulp of the largest
  // coordinate in play) is far above the rounding of the exact float SAT and
  // of these bounds, so no cell the exact test accepts is dropped.
  S.ha = 0.52f * S.cs_a + ulp64;
  S.hb = 0.52f * S.cs_b + ulp64;
  const float hc = 0.52f * cs_c + ulp64;
  S.inr = __frcp_rn(nr_c);
  S.w = hc + (fabsf(S.nr_a) * S.ha + fabsf(S.nr_b) * S.hb) * fabsf(S.inr);
  S.ics = SEL2(J.ics, c);
#undef SEL2
  S.items = (uint32_t)(n_a * S.n_b);
  return true;
}

// the candidate cells of work item q: column (ia, ib) along c, cells
// klo .. klo + n - 1 (n = 0: the column is pruned).  Items of a face without
// pruning are single cells (ia, ib, klo) = (i, j, k) with c = z.
__device__ __forceinline__ void shell_column(const ShellSetup& S, uint32_t q, int& ia, int& ib,
                                             int& klo, int& n) {
  n = 0;
  if (!S.prune) {
    klo = S.lo_c + (int)(q % S.n_c);
    ib = S.lo_b + (int)((q / S.n_c) % S.n_b);
    ia = S.lo_a + (int)(q / (S.n_c * S.n_b));
    n = 1;
    return;
  }
  ia = S.lo_a + (int)(q / S.n_b);
  ib = S.lo_b + (int)(q % S.n_b);
  // the SAT tests that do not involve axis c, exactly, once per column: the
  // box of every cell of the column has the same extent along a and b
  {
    const float bmin_a = ADD(S.amin_a, MUL(S.cs_a, (float)ia)), bmax_a = ADD(bmin_a, S.cs_a);
    const float bmin_b = ADD(S.amin_b, MUL(S.cs_b, (float)ib)), bmax_b = ADD(bmin_b, S.cs_b);
    const float ce_a = MUL(ADD(bmax_a, bmin_a), 0.5f), ce_b = MUL(ADD(bmax_b, bmin_b), 0.5f);
    const float r_a = SUB(bmax_a, ce_a), r_b = SUB(bmax_b, ce_b);
    bool keep;
    if (S.c == 0) keep = tri_box_sel<sat_column_mask(0)>(S.p0, S.p1, S.p2, tv{0.0f, ce_a, ce_b}, tv{0.0f, r_a, r_b});
    else if (S.c == 1) keep = tri_box_sel<sat_column_mask(1)>(S.p0, S.p1, S.p2, tv{ce_b, 0.0f, ce_a}, tv{r_b, 0.0f, r_a});
    else keep = tri_box_sel<sat_column_mask(2)>(S.p0, S.p1, S.p2, tv{ce_a, ce_b, 0.0f}, tv{r_a, r_b, 0.0f});
    if (!keep) return;
  }
  const float ca = (S.amin_a + S.cs_a * ((float)ia + 0.5f)) - S.q0_a;
  const float cb = (S.amin_b + S.cs_b * ((float)ib + 0.5f)) - S.q0_b;
  // slab bounds (conservative: the margin is far above these roundings)
  const float tc = S.q0_c - (S.nr_a * ca + S.nr_b * cb) * S.inr;
  // cells whose centre is within w of the plane along c
  klo = max(S.lo_c, (int)ceilf((tc - S.w - S.amin_c) * S.ics - 0.5f));
  const int khi = min(S.hi_c, (int)floorf((tc + S.w - S.amin_c) * S.ics - 0.5f));
  n = max(khi - klo + 1, 0);
}

// Per-face setup packed into 6 float4 (computed once per face here, then
// read by every lane that takes an item of the face):
//   (p0.xyz, p1.x) (p1.yz, p2.xy) (p2.z, nr_a, nr_b, 1/nr_c) (Pa1, Pb1, Pa2, Pb2)
//   (ha, hb, w, job) (c | prune << 2, lo_a | lo_b << 16, lo_c | hi_c << 16, n_b | n_c << 16)
__global__ void k_shell_count(const JobDesc* jobs, int njobs, uint32_t total, uint32_t* scnt,
                              float4* srec) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    ShellSetup S;
    if (!shell_setup(J, g - J.face_base, S)) {
      scnt[g] = 0u;
      continue;
    }
    scnt[g] = S.items;
    float4* r = srec + 6 * (size_t)g;
    r[0] = make_float4(S.p0.x, S.p0.y, S.p0.z, S.p1.x);
    r[1] = make_float4(S.p1.y, S.p1.z, S.p2.x, S.p2.y);
    r[2] = make_float4(S.p2.z, S.nr_a, S.nr_b, S.inr);
    r[3] = make_float4(S.Pa1, S.Pb1, S.Pa2, S.Pb2);
    r[4] = make_float4(S.ha, S.hb, S.w, __int_as_float(j));
    r[5] = make_float4(__int_as_float(S.c | (S.prune ? 4 : 0)), __int_as_float(S.lo_a | (S.lo_b << 16)),
                       __int_as_float(S.lo_c | (S.hi_c << 16)), __int_as_float(S.n_b | (S.n_c << 16)));
  }
}

__device__ __forceinline__ int shell_unpack(const JobDesc* jobs, const float4* rec, ShellSetup& S) {
  const float4 r0 = rec[0], r1 = rec[1], r2 = rec[2], r3 = rec[3], r4 = rec[4], r5 = rec[5];
  S.p0 = {r0.x, r0.y, r0.z};
  S.p1 = {r0.w, r1.x, r1.y};
  S.p2 = {r1.z, r1.w, r2.x};
  S.nr_a = r2.y; S.nr_b = r2.z; S.inr = r2.w;
  S.Pa1 = r3.x; S.Pb1 = r3.y; S.Pa2 = r3.z; S.Pb2 = r3.w;
  S.ha = r4.x; S.hb = r4.y; S.w = r4.z;
  const int j = __float_as_int(r4.w);
  const int cp = __float_as_int(r5.x), lab = __float_as_int(r5.y), lch = __float_as_int(r5.z),
            nbc = __float_as_int(r5.w);
  S.c = cp & 3;
  S.prune = (cp & 4) != 0;
  S.lo_a = lab & 0xFFFF; S.lo_b = lab >> 16;
  S.lo_c = lch & 0xFFFF; S.hi_c = lch >> 16;
  S.n_b = nbc & 0xFFFF; S.n_c = nbc >> 16;
  const JobDesc& J = jobs[j];
  const int c = S.c, ax = c == 2 ? 0 : c + 1, bx = c == 0 ? 2 : (c == 1 ? 0 : 1);
#define SEL(v, i) ((i) == 0 ? (v)[0] : ((i) == 1 ? (v)[1] : (v)[2]))
  const float p0[3] = {S.p0.x, S.p0.y, S.p0.z};
  S.cs[0] = J.cs[0]; S.cs[1] = J.cs[1]; S.cs[2] = J.cs[2];
  S.amin_a = SEL(J.amin, ax); S.amin_b = SEL(J.amin, bx); S.amin_c = SEL(J.amin, c);
  S.cs_a = SEL(J.cs, ax); S.cs_b = SEL(J.cs, bx);
  S.ics = SEL(J.ics, c);
  S.q0_a = SEL(p0, ax); S.q0_b = SEL(p0, bx); S.q0_c = SEL(p0, c);
#undef SEL
  return j;
}

// Warp-interleaved runs over the (face, column) items.  Each lane prunes its
// column to a range of candidate cells; the cells of all 32 columns are then
// dealt out to the lanes, one exact SAT per lane per round, so lanes with
// pruned or short columns do not idle while others test.
__global__ void __launch_bounds__(256, 3) k_shell_flat(const JobDesc* jobs, const uint32_t* scnt,
                                                       const unsigned long long* sbase,
                                                       const unsigned long long* stotal,
                                                       uint32_t total_faces, const float4* srec) {
  const unsigned long long total = *stotal;
  const int lane = threadIdx.x & 31;
  const unsigned long long nwruns = (total + WARP_RUN - 1) / WARP_RUN;
  const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
  for (unsigned long long wr = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
       wr < nwruns; wr += nwarps) {
    const unsigned long long base = wr * WARP_RUN;
    const unsigned long long end = min(base + WARP_RUN, total);
    uint32_t g = 0;
    if (lane == 0) g = face_of_item(sbase, total_faces, base);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    uint32_t cached = 0xFFFFFFFFu;
    ShellSetup S;
    S.c = 2;
    S.p0 = S.p1 = S.p2 = {0.0f, 0.0f, 0.0f};
    S.cs[0] = S.cs[1] = S.cs[2] = 0.0f;
    int jidx = 0;
    unsigned long long fb = 0;
    for (unsigned long long p0 = base; p0 < end; p0 += 32) {
      const unsigned long long p = p0 + lane;
      int ia = 0, ib = 0, klo = 0, n = 0;
      if (p < end) {
        while (p >= sbase[g] + scnt[g]) ++g;
        if (g != cached) {
          cached = g;
          jidx = shell_unpack(jobs, srec + 6 * (size_t)g, S);
          fb = sbase[g];
        }
        shell_column(S, (uint32_t)(p - fb), ia, ib, klo, n);
      }
      // exclusive scan of the lanes' cell counts
      int incl = n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += t;
      }
      const int ncells = __shfl_sync(0xFFFFFFFFu, incl, 31);
      const int excl = incl - n;
      for (int t0 = 0; t0 < ncells; t0 += 32) {
        const int t = t0 + lane;
        // owner: the last lane whose first cell is <= t
        int src = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const int e = __shfl_sync(0xFFFFFFFFu, excl, src + step);
          if (e <= t) src += step;
        }
        const tv q0 = {__shfl_sync(0xFFFFFFFFu, S.p0.x, src), __shfl_sync(0xFFFFFFFFu, S.p0.y, src),
                       __shfl_sync(0xFFFFFFFFu, S.p0.z, src)};
        const tv q1 = {__shfl_sync(0xFFFFFFFFu, S.p1.x, src), __shfl_sync(0xFFFFFFFFu, S.p1.y, src),
                       __shfl_sync(0xFFFFFFFFu, S.p1.z, src)};
        const tv q2 = {__shfl_sync(0xFFFFFFFFu, S.p2.x, src), __shfl_sync(0xFFFFFFFFu, S.p2.y, src),
                       __shfl_sync(0xFFFFFFFFu, S.p2.z, src)};
        const float cs[3] = {__shfl_sync(0xFFFFFFFFu, S.cs[0], src),
                             __shfl_sync(0xFFFFFFFFu, S.cs[1], src),
                             __shfl_sync(0xFFFFFFFFu, S.cs[2], src)};
        const int sj = __shfl_sync(0xFFFFFFFFu, jidx, src);
        // test mode: the face's axis c (column tests already passed) or -1
        // (faces without pruning: every item is one cell, whole SAT)
        const int mode = __shfl_sync(0xFFFFFFFFu, S.prune ? S.c : -1, src);
        const int sc = mode < 0 ? 2 : mode;
        const int sa = __shfl_sync(0xFFFFFFFFu, ia, src);
        const int sb = __shfl_sync(0xFFFFFFFFu, ib, src);
        const int sk = __shfl_sync(0xFFFFFFFFu, klo, src) + t - __shfl_sync(0xFFFFFFFFu, excl, src);
        if (t < ncells) {
          // (a, b, c) -> (x, y, z): c = 0: (k, a, b); c = 1: (b, k, a); c = 2: (a, b, k)
          const int x = sc == 0 ? sk : (sc == 1 ? sb : sa);
          const int y = sc == 0 ? sa : (sc == 1 ? sk : sb);
          const int z = sc == 0 ? sb : (sc == 1 ? sa : sk);
          test_cell(jobs[sj], cs, q0, q1, q2, x, y, z, mode);
        }
      }
    }
  }
}
#undef MUL
#undef ADD
#undef SUB

// one CTA per brick, one thread per (x,y) row of 32 z voxels = one word.
// grid2 (the second label buffer) needs zeros in bricks that are not live:
// stencil tiles read their halo from them.  Live bricks of grid2 are written
// in full by the first stage that targets it, so only non-live bricks are
// cleared there (dual != 0).
__global__ void __launch_bounds__(256) k_combine(const JobDesc* jobs, const uint32_t* brick_job,
                                                 uint32_t total, uint8_t* live, int dual) {
  // One CTA per column of bricks along z (the CTA of the column's first
  // brick; the others skip it), a warp per (x, y) row with the lanes along z:
  // the row's bit-plane words load coalesced, and each store instruction
  // writes 32 consecutive 16-byte label units.
  __shared__ uint32_t colmask[4];  // bricks of the column with an occupied voxel (bit bz)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t b = blockIdx.x; b < total; b += gridDim.x) {
    const JobDesc& J = jobs[brick_job[b]];
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz;
    if (bz != 0) continue;  // uniform across the CTA
    const uint32_t by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    if (threadIdx.x < 4) colmask[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t nw = J.Zw;      // words per row = bricks per column (<= 128)
    const uint32_t nq = J.Zp / 8;  // 16-byte label units of the row
    uint32_t m[4] = {0, 0, 0, 0};  // this warp's rows: bricks with an occupied voxel
    for (uint32_t row = warp; row < VF_BX * VF_BY; row += 8) {
      const uint32_t x = bx * VF_BX + row / VF_BY, y = by * VF_BY + row % VF_BY;
      if (x >= J.X || y >= J.Y) continue;  // uniform across the warp
      const size_t w0 = ((size_t)x * J.Y + y) * nw;
      uint4* dst = reinterpret_cast<uint4*>(J.grid + vf_gidx(J, x, y, 0));
      for (uint32_t wb = 0; wb < nw; wb += 32) {
        const uint32_t w = wb + lane;
        const uint32_t word = w < nw ? (J.par[w0 + w] | J.shell[w0 + w]) : 0u;
        m[wb >> 5] |= __ballot_sync(0xFFFFFFFFu, word != 0u);
        // units q = 4 wb + 32 k + lane take byte (q & 3) of word q >> 2 (lane
        // (8 k + lane / 4) of this group); bits at z >= Z are never set, so the
        // row padding is written as 0
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k) {
          const uint32_t src = __shfl_sync(0xFFFFFFFFu, word, (int)(8 * k + (uint32_t)lane / 4));
          const uint32_t q = 4 * wb + 32 * k + (uint32_t)lane;
          if (q < nq) {
            const uint32_t bits = src >> (8 * (lane & 3));
            uint4 v;
            v.x = (bits & 1u) | ((bits >> 1) & 1u) << 16;
            v.y = ((bits >> 2) & 1u) | ((bits >> 3) & 1u) << 16;
            v.z = ((bits >> 4) & 1u) | ((bits >> 5) & 1u) << 16;
            v.w = ((bits >> 6) & 1u) | ((bits >> 7) & 1u) << 16;
            dst[q] = v;
          }
        }
      }
    }
    if (lane == 0)
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (m[i]) atomicOr(&colmask[i], m[i]);
    __syncthreads();
    for (uint32_t w = threadIdx.x; w < J.nbz; w += blockDim.x)
      live[b + w] = (colmask[w >> 5] >> (w & 31)) & 1u;
    if (dual) {
      // the second label buffer needs zeros in the bricks that are not live
      // (stencil tiles read their halo there); live bricks are written in
      // full by the first stage that targets it
      for (uint32_t row = warp; row < VF_BX * VF_BY; row += 8) {
        const uint32_t x = bx * VF_BX + row / VF_BY, y = by * VF_BY + row % VF_BY;
        if (x >= J.X || y >= J.Y) continue;
        uint4* dst2 = reinterpret_cast<uint4*>(J.grid2 + vf_gidx(J, x, y, 0));
        for (uint32_t q = lane; q < nq; q += 32) {
          const uint32_t w = q >> 2;  // the brick (word) of this unit
          if (!((colmask[w >> 5] >> (w & 31)) & 1u)) dst2[q] = make_uint4(0, 0, 0, 0);
        }
      }
    }
    __syncthreads();  // colmask is reused by the next column
  }
}
__global__ void __launch_bounds__(256) k_mark_live(const JobDesc* jobs, const uint32_t* brick_job,
                                                   uint32_t total, uint8_t* live) {
  for (uint32_t b = blockIdx.x; b < total; b += gridDim.x) {
    const JobDesc& J = jobs[brick_job[b]];
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t x = bx * VF_BX + threadIdx.x / VF_BY, y = by * VF_BY + threadIdx.x % VF_BY;
    const uint32_t z0 = bz * VF_BZ;
    int any = 0;
    if (x < J.X && y < J.Y) {
      const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);
      const uint4* src = reinterpret_cast<const uint4*>(J.grid + vf_gidx(J, x, y, z0));
      for (uint32_t q = 0; q < nz / 8; ++q) {
        uint4 v = src[q];
        any |= (v.x | v.y | v.z | v.w) != 0;
      }
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) live[b] = any ? 1 : 0;
  }
}

__global__ void k_compact(const uint8_t* live, uint32_t total, uint32_t* list, uint32_t* count) {
  const int lane = threadIdx.x & 31;
  // grid-stride over bricks, warp-aggregated append (ballot + popc)
  for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < total;
       i0 += gridDim.x * blockDim.x) {
    const uint32_t i = i0 + lane;
    const bool keep = i < total && live[i];
    const unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (keep) list[base + __popc(m & ((1u << lane) - 1u))] = i;
  }
}

}  // namespace

namespace vfk {

static inline int grid_for(uint32_t n, int per, int cap) {
  uint64_t g = (n + (uint64_t)per - 1) / per;
  if (g < 1) g = 1;
  if (g > (uint64_t)cap) g = cap;
  return (int)g;
}

void centroid_and_slices(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs) {
  if (njobs > 0) k_centroid<<<njobs, 1024, 0, st>>>(dj, ds);
}
void tetra_prep(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                uint32_t total_faces, const FaceScratch& fs) {
  if (total_faces)
    k_tetra<<<grid_for(total_faces, 256, 65535), 256, 0, st>>>(dj, ds, njobs, total_faces, fs.pcnt);
}
void parity_raster(cudaStream_t st, const JobDesc* dj, const JobState* ds, int njobs,
                   uint32_t total_faces, const FaceScratch& fs, int num_sms, int grid_mult) {
  if (!total_faces) return;
  const uint32_t nb = (total_faces + 1023) / 1024;
  k_scan_local<<<nb, 1024, 0, st>>>(fs.pcnt, fs.pbase, fs.psums, total_faces);
  k_scan_sums<<<1, 1024, 0, st>>>(fs.psums, nb, fs.ptotal);
  k_scan_add<<<(total_faces + 255) / 256, 256, 0, st>>>(fs.pbase, fs.psums, total_faces);
  k_parity_flat<<<num_sms * grid_mult, 256, 0, st>>>(dj, njobs, fs.pcnt, fs.pbase, fs.ptotal, total_faces);
  const unsigned gy = (unsigned)(njobs < 65535 ? njobs : 65535);
  k_odd_edges<<<dim3(num_sms, gy), 256, 0, st>>>(dj, ds, njobs);
  int px = num_sms * 8 / njobs;
  px = px < 1 ? 1 : (px > 64 ? 64 : px);
  k_prefix_x<<<dim3(px, gy), 256, 0, st>>>(dj, njobs);
}
void exclusive_scan(cudaStream_t st, const uint32_t* in, unsigned long long* out,
                    unsigned long long* sums, uint32_t n, unsigned long long* total) {
  if (!n) {
    cudaMemsetAsync(total, 0, sizeof(unsigned long long), st);
    return;
  }
  const uint32_t nb = (n + 1023) / 1024;
  k_scan_local<<<nb, 1024, 0, st>>>(in, out, sums, n);
  k_scan_sums<<<1, 1024, 0, st>>>(sums, nb, total);
  k_scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, sums, n);
}

void shell_sat(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces,
               const FaceScratch& fs, int num_sms, int grid_mult) {
  if (!total_faces) return;
  const uint32_t nb = (total_faces + 1023) / 1024;
  k_shell_count<<<grid_for(total_faces, 256, 65535), 256, 0, st>>>(dj, njobs, total_faces, fs.pcnt,
                                                                   fs.srec);
  k_scan_local<<<nb, 1024, 0, st>>>(fs.pcnt, fs.pbase, fs.psums, total_faces);
  k_scan_sums<<<1, 1024, 0, st>>>(fs.psums, nb, fs.ptotal);
  k_scan_add<<<(total_faces + 255) / 256, 256, 0, st>>>(fs.pbase, fs.psums, total_faces);
  k_shell_flat<<<num_sms * grid_mult, 256, 0, st>>>(dj, fs.pcnt, fs.pbase, fs.ptotal, total_faces, fs.srec);
}
void combine(cudaStream_t st, const JobDesc* dj, const uint32_t* brick_job,
             uint32_t total_bricks, uint8_t* live, int dual) {
  if (total_bricks)
    k_combine<<<grid_for(total_bricks, 1, 1 << 20), 256, 0, st>>>(dj, brick_job, total_bricks, live, dual);
}
void mark_live(cudaStream_t st, const JobDesc* dj, const uint32_t* brick_job,
               uint32_t total_bricks, uint8_t* live) {
  if (total_bricks)
    k_mark_live<<<grid_for(total_bricks, 1, 1 << 20), 256, 0, st>>>(dj, brick_job, total_bricks, live);
}
void compact_live(cudaStream_t st, const uint8_t* live, uint32_t total_bricks, uint32_t* list,
                  uint32_t* count) {
  cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
  if (total_bricks)
    k_compact<<<grid_for(total_bricks, 256, 4096), 256, 0, st>>>(live, total_bricks, list, count);
}

}  // namespace vfk
