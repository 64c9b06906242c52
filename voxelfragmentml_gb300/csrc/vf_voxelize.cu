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
__device__ bool tri_box(const tv& p0, const tv& p1, const tv& p2, const tv& c, const tv& r) {
  satd d;
  d.r = r;
  d.v0 = {SUB(p0.x, c.x), SUB(p0.y, c.y), SUB(p0.z, c.z)};
  d.v1 = {SUB(p1.x, c.x), SUB(p1.y, c.y), SUB(p1.z, c.z)};
  d.v2 = {SUB(p2.x, c.x), SUB(p2.y, c.y), SUB(p2.z, c.z)};
  tv e0 = {SUB(d.v1.x, d.v0.x), SUB(d.v1.y, d.v0.y), SUB(d.v1.z, d.v0.z)};
  tv e1 = {SUB(d.v2.x, d.v1.x), SUB(d.v2.y, d.v1.y), SUB(d.v2.z, d.v1.z)};
  tv e2 = {SUB(d.v0.x, d.v2.x), SUB(d.v0.y, d.v2.y), SUB(d.v0.z, d.v2.z)};
  float fx = fabsf(e0.x), fy = fabsf(e0.y), fz = fabsf(e0.z);
  if (!x01(d, e0.z, e0.y, fz, fy)) return false;
  if (!y02(d, e0.z, e0.x, fz, fx)) return false;
  if (!z12(d, e0.y, e0.x, fy, fx)) return false;
  fx = fabsf(e1.x); fy = fabsf(e1.y); fz = fabsf(e1.z);
  if (!x01(d, e1.z, e1.y, fz, fy)) return false;
  if (!y02(d, e1.z, e1.x, fz, fx)) return false;
  if (!z0(d, e1.y, e1.x, fy, fx)) return false;
  fx = fabsf(e2.x); fy = fabsf(e2.y); fz = fabsf(e2.z);
  if (!x2(d, e2.z, e2.y, fz, fy)) return false;
  if (!y1(d, e2.z, e2.x, fz, fx)) return false;
  if (!z12(d, e2.y, e2.x, fy, fx)) return false;
  float mn, mx;
  mm3(d.v0.x, d.v1.x, d.v2.x, mn, mx);
  if (mn > d.r.x || mx < -d.r.x) return false;
  mm3(d.v0.y, d.v1.y, d.v2.y, mn, mx);
  if (mn > d.r.y || mx < -d.r.y) return false;
  mm3(d.v0.z, d.v1.z, d.v2.z, mn, mx);
  if (mn > d.r.z || mx < -d.r.z) return false;
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

__device__ __forceinline__ int float_cell(float f, int n) {
  if (!(f > -1.0e9f)) f = -1.0e9f;
  if (f > 1.0e9f) f = 1.0e9f;
  return vf_clampi((int)floorf(f), -2, n + 1);
}

// the exact test of one voxel (reference operation order) and the mark
__device__ __forceinline__ void test_cell(const JobDesc& J, const float* cs, const tv& p0,
                                          const tv& p1, const tv& p2, int i, int jj, int k) {
  tv bmin = {ADD(J.amin[0], MUL(cs[0], (float)i)), ADD(J.amin[1], MUL(cs[1], (float)jj)),
             ADD(J.amin[2], MUL(cs[2], (float)k))};
  tv bmax = {ADD(bmin.x, cs[0]), ADD(bmin.y, cs[1]), ADD(bmin.z, cs[2])};
  tv ce = {__fdiv_rn(ADD(bmax.x, bmin.x), 2.0f), __fdiv_rn(ADD(bmax.y, bmin.y), 2.0f),
           __fdiv_rn(ADD(bmax.z, bmin.z), 2.0f)};
  tv r = {SUB(bmax.x, ce.x), SUB(bmax.y, ce.y), SUB(bmax.z, ce.z)};
  if (tri_box(p0, p1, p2, ce, r))
    atomicOr(J.shell + ((size_t)i * J.Y + jj) * J.Zw + (k >> 5), 1u << (k & 31));
}

// Per-face setup of the shell test.  Candidates: the triangle's cell bbox
// grown by one cell.  Pruning: two of the SAT's own separating axes are
// evaluated early with a margin of a quarter cell -- (1) the triangle's
// projection on the plane orthogonal to its dominant normal axis c against
// each column's square (the edge x c axes and the a, b box axes), (2) the
// plane slab along c (the plane-box test).  A dropped box is separated by at
// least 0.25 cell along a SAT axis, far beyond float rounding, so the exact
// SAT would reject it too: the marked set equals testing the full bbox.
// Work items: columns (a, b) when pruning, else every bbox cell.
struct ShellSetup {
  float cs[3], q0[3], nr[3], Pa[3], Pb[3];
  float ha, hb, w;
  tv p0, p1, p2;
  int lo[3], n[3];
  int c, ax, bx;
  bool prune;
  uint32_t items;
};

__device__ bool shell_setup(const JobDesc& J, uint32_t f, ShellSetup& S) {
  const uint32_t dims[3] = {J.X, J.Y, J.Z};
  for (int a = 0; a < 3; ++a) S.cs[a] = __fdiv_rn(SUB(J.amax[a], J.amin[a]), (float)dims[a]);
  const uint32_t* fi = J.faces + 3 * (size_t)f;
  if (fi[0] >= J.nverts || fi[1] >= J.nverts || fi[2] >= J.nverts) return false;
  const float* q0 = J.verts + 3 * (size_t)fi[0];
  const float* q1 = J.verts + 3 * (size_t)fi[1];
  const float* q2 = J.verts + 3 * (size_t)fi[2];
  for (int a = 0; a < 3; ++a) {
    float mn, mx;
    mm3(q0[a], q1[a], q2[a], mn, mx);
    S.lo[a] = vf_clampi(float_cell(__fdiv_rn(SUB(mn, J.amin[a]), S.cs[a]), dims[a]) - 1, 0, dims[a] - 1);
    const int hi = vf_clampi(float_cell(__fdiv_rn(SUB(mx, J.amin[a]), S.cs[a]), dims[a]) + 1, 0, dims[a] - 1);
    S.n[a] = hi - S.lo[a] + 1;
    S.q0[a] = q0[a];
  }
  S.p0 = {q0[0], q0[1], q0[2]};
  S.p1 = {q1[0], q1[1], q1[2]};
  S.p2 = {q2[0], q2[1], q2[2]};
  const float e1[3] = {q1[0] - q0[0], q1[1] - q0[1], q1[2] - q0[2]};
  const float e2[3] = {q2[0] - q0[0], q2[1] - q0[1], q2[2] - q0[2]};
  S.nr[0] = e1[1] * e2[2] - e1[2] * e2[1];
  S.nr[1] = e1[2] * e2[0] - e1[0] * e2[2];
  S.nr[2] = e1[0] * e2[1] - e1[1] * e2[0];
  int c = 0;
  if (fabsf(S.nr[1]) > fabsf(S.nr[c])) c = 1;
  if (fabsf(S.nr[2]) > fabsf(S.nr[c])) c = 2;
  S.c = c;
  S.ax = (c + 1) % 3;
  S.bx = (c + 2) % 3;
  const float e1n = fabsf(e1[0]) + fabsf(e1[1]) + fabsf(e1[2]);
  const float e2n = fabsf(e2[0]) + fabsf(e2[1]) + fabsf(e2[2]);
  S.prune = fabsf(S.nr[c]) > 1e-3f * e1n * e2n && fabsf(S.nr[c]) > 0.0f;
  if (!S.prune) {
    S.items = (uint32_t)(S.n[0] * S.n[1] * S.n[2]);
    return true;
  }
  // projected triangle (relative to q0), counter-clockwise
  float P1a = e1[S.ax], P1b = e1[S.bx], P2a = e2[S.ax], P2b = e2[S.bx];
  if (S.nr[c] < 0.0f) { float t = P1a; P1a = P2a; P2a = t; t = P1b; P1b = P2b; P2b = t; }
  S.Pa[0] = 0.0f; S.Pa[1] = P1a; S.Pa[2] = P2a;
  S.Pb[0] = 0.0f; S.Pb[1] = P1b; S.Pb[2] = P2b;
  S.ha = 0.75f * S.cs[S.ax];  // half cell + quarter-cell margin
  S.hb = 0.75f * S.cs[S.bx];
  const float hc = 0.75f * S.cs[c];
  S.w = hc + fabsf(S.nr[S.ax]) / fabsf(S.nr[c]) * S.ha + fabsf(S.nr[S.bx]) / fabsf(S.nr[c]) * S.hb;
  S.items = (uint32_t)(S.n[S.ax] * S.n[S.bx]);
  return true;
}

__device__ void shell_item(const JobDesc& J, const ShellSetup& S, uint32_t q) {
  if (!S.prune) {
    const int k = S.lo[2] + (int)(q % S.n[2]);
    const int jj = S.lo[1] + (int)((q / S.n[2]) % S.n[1]);
    const int i = S.lo[0] + (int)(q / (S.n[2] * S.n[1]));
    test_cell(J, S.cs, S.p0, S.p1, S.p2, i, jj, k);
    return;
  }
  const int ax = S.ax, bx = S.bx, c = S.c;
  const int ia = S.lo[ax] + (int)(q / S.n[bx]), ib = S.lo[bx] + (int)(q % S.n[bx]);
  const float ca = (J.amin[ax] + S.cs[ax] * ((float)ia + 0.5f)) - S.q0[ax];
  const float cb = (J.amin[bx] + S.cs[bx] * ((float)ib + 0.5f)) - S.q0[bx];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int f2 = (e + 1) % 3;
    const float dx = S.Pa[f2] - S.Pa[e], dy = S.Pb[f2] - S.Pb[e];
    const float E = dx * (cb - S.Pb[e]) - dy * (ca - S.Pa[e]);
    if (E + fabsf(dx) * S.hb + fabsf(dy) * S.ha < 0.0f) return;
  }
  const float tc = S.q0[c] - (S.nr[ax] * ca + S.nr[bx] * cb) / S.nr[c];
  const int klo = max(S.lo[c], (int)floorf((tc - S.w - J.amin[c]) / S.cs[c] - 0.5f));
  const int khi = min(S.lo[c] + S.n[c] - 1, (int)ceilf((tc + S.w - J.amin[c]) / S.cs[c] - 0.5f));
  for (int k = klo; k <= khi; ++k) {
    int idx[3];
    idx[ax] = ia;
    idx[bx] = ib;
    idx[c] = k;
    test_cell(J, S.cs, S.p0, S.p1, S.p2, idx[0], idx[1], idx[2]);
  }
}

__global__ void k_shell_count(const JobDesc* jobs, int njobs, uint32_t total, uint32_t* scnt) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const JobDesc& J = jobs[job_of_face(jobs, njobs, g)];
    ShellSetup S;
    scnt[g] = shell_setup(J, g - J.face_base, S) ? S.items : 0u;
  }
}

__global__ void __launch_bounds__(256) k_shell_flat(const JobDesc* jobs, int njobs,
                                                    const uint32_t* scnt,
                                                    const unsigned long long* sbase,
                                                    const unsigned long long* stotal,
                                                    uint32_t total_faces) {
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
    const JobDesc* J = nullptr;
    unsigned long long fb = 0;
    for (unsigned long long p = base + lane; p < end; p += 32) {
      while (p >= sbase[g] + scnt[g]) ++g;
      if (g != cached) {
        cached = g;
        J = &jobs[job_of_face(jobs, njobs, g)];
        shell_setup(*J, g - J->face_base, S);
        fb = sbase[g];
      }
      shell_item(*J, S, (uint32_t)(p - fb));
    }
  }
}
#undef MUL
#undef ADD
#undef SUB

// one CTA per brick, one thread per (x,y) row of 32 z voxels = one word
__global__ void __launch_bounds__(256) k_combine(const JobDesc* jobs, const uint32_t* brick_job,
                                                 uint32_t total, uint8_t* live, int dual) {
  for (uint32_t b = blockIdx.x; b < total; b += gridDim.x) {
    const JobDesc& J = jobs[brick_job[b]];
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t x = bx * VF_BX + threadIdx.x / VF_BY, y = by * VF_BY + threadIdx.x % VF_BY;
    const uint32_t z0 = bz * VF_BZ;
    uint32_t word = 0;
    if (x < J.X && y < J.Y) {
      const size_t w = ((size_t)x * J.Y + y) * J.Zw + bz;
      word = J.par[w] | J.shell[w];
      // bits at z >= Z are never set, so the row padding is written as 0
      const uint32_t nz = min((uint32_t)VF_BZ, J.Zp - z0);  // multiple of 8
      uint4* dst = reinterpret_cast<uint4*>(J.grid + vf_gidx(J, x, y, z0));
      uint4* dst2 = reinterpret_cast<uint4*>(J.grid2 + vf_gidx(J, x, y, z0));
      for (uint32_t q = 0; q < nz / 8; ++q) {
        uint32_t bits = word >> (8 * q);
        uint4 v;
        v.x = (bits & 1u) | ((bits >> 1) & 1u) << 16;
        v.y = ((bits >> 2) & 1u) | ((bits >> 3) & 1u) << 16;
        v.z = ((bits >> 4) & 1u) | ((bits >> 5) & 1u) << 16;
        v.w = ((bits >> 6) & 1u) | ((bits >> 7) & 1u) << 16;
        dst[q] = v;
        if (dual) dst2[q] = v;
      }
    }
    const int any = __syncthreads_or(word != 0);
    if (threadIdx.x == 0) live[b] = any ? 1 : 0;
  }
}

// liveness of a brick from the current label grid (after an upload)
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
                   uint32_t total_faces, const FaceScratch& fs, int num_sms) {
  if (!total_faces) return;
  const uint32_t nb = (total_faces + 1023) / 1024;
  k_scan_local<<<nb, 1024, 0, st>>>(fs.pcnt, fs.pbase, fs.psums, total_faces);
  k_scan_sums<<<1, 1024, 0, st>>>(fs.psums, nb, fs.ptotal);
  k_scan_add<<<(total_faces + 255) / 256, 256, 0, st>>>(fs.pbase, fs.psums, total_faces);
  k_parity_flat<<<num_sms * 16, 256, 0, st>>>(dj, njobs, fs.pcnt, fs.pbase, fs.ptotal, total_faces);
  const unsigned gy = (unsigned)(njobs < 65535 ? njobs : 65535);
  k_odd_edges<<<dim3(num_sms, gy), 256, 0, st>>>(dj, ds, njobs);
  int px = num_sms * 8 / njobs;
  px = px < 1 ? 1 : (px > 64 ? 64 : px);
  k_prefix_x<<<dim3(px, gy), 256, 0, st>>>(dj, njobs);
}
void shell_sat(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces,
               const FaceScratch& fs, int num_sms) {
  if (!total_faces) return;
  const uint32_t nb = (total_faces + 1023) / 1024;
  k_shell_count<<<grid_for(total_faces, 256, 65535), 256, 0, st>>>(dj, njobs, total_faces, fs.pcnt);
  k_scan_local<<<nb, 1024, 0, st>>>(fs.pcnt, fs.pbase, fs.psums, total_faces);
  k_scan_sums<<<1, 1024, 0, st>>>(fs.psums, nb, fs.ptotal);
  k_scan_add<<<(total_faces + 255) / 256, 256, 0, st>>>(fs.pbase, fs.psums, total_faces);
  k_shell_flat<<<num_sms * 16, 256, 0, st>>>(dj, njobs, fs.pcnt, fs.pbase, fs.ptotal, total_faces);
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
