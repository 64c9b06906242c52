// vf_voxelize.cu -- solid voxelization of triangle meshes on sm_103a.
//
// Occupancy of a voxel = (some triangle overlaps the voxel box: FP32 SAT in
// the operation order of Intersections3D.h:204-258) OR (the voxel sample
// point is inside the mesh by tetra parity: Tetravoxelizer.cpp:42-92, 198-315).
//
// Stages, all batched over every job of a batch:
//   centroid_and_slices : one 1024-thread block per job; fixed-order
//                         lane sums of the vertices + the slice planes
//   tetra_prep          : one thread per face -> tetrahedron (face + centroid)
//                         in NDC, vertices sorted by y, slice range
//   parity_raster       : (tetrahedron, slice) pairs flattened by a prefix
//                         sum over the faces; each thread rasterises a run
//                         of 64 pairs (cross-section triangles, exact integer
//                         edge functions, XOR into bit planes)
//   shell_sat           : per-face work items (columns of the triangle's
//                         footprint) flattened by a prefix sum; each thread
//                         tests a run of 16 items with the exact SAT
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

__global__ void k_tetra(const JobDesc* jobs, JobState* st, int njobs, uint32_t total,
                        uint32_t* pcnt) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += gridDim.x * blockDim.x) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    const uint32_t f = g - J.face_base;
    const uint32_t* fi = J.faces + 3 * (size_t)f;
    if (fi[0] >= J.nverts || fi[1] >= J.nverts || fi[2] >= J.nverts) {
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
    tv v[4];
    for (int k = 0; k < 3; ++k) v[k] = to_ndc(J.verts + 3 * (size_t)J.faces[3 * (size_t)f + k], ctr, dim);
    v[3] = to_ndc(st[j].centroid, ctr, dim);
    // sort4Vec3ByLowerY (Tetravoxelizer.h:75-81)
    tv t;
#define SW(a, b) if (v[a].y > v[b].y) { t = v[a]; v[a] = v[b]; v[b] = t; }
    SW(0, 1) SW(2, 3) SW(0, 2) SW(1, 3) SW(1, 2)
#undef SW
    float4* o = J.tets + 3 * (size_t)f;
    o[0] = make_float4(v[0].x, v[0].y, v[0].z, v[1].x);
    o[1] = make_float4(v[1].y, v[1].z, v[2].x, v[2].y);
    o[2] = make_float4(v[2].z, v[3].x, v[3].y, v[3].z);
    // slices with A.y < ys[s] <= D.y
    uint32_t s0 = upper_bound_f(J.ys, J.Y, v[0].y);
    uint32_t s1e = upper_bound_f(J.ys, J.Y, v[3].y);
    J.tet_range[f] = (s1e > s0) ? (s0 | ((s1e - 1) << 16)) : 0xFFFFu;  // s0=0xFFFF,s1=0: none
    pcnt[g] = s1e > s0 ? s1e - s0 : 0u;  // (tetrahedron, slice) pairs of this face
  }
}

// ---- exact raster (see the oracle for the rule) ---------------------------
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
__device__ __forceinline__ long long edge_fn(int ax, int az, int bx, int bz, long long px,
                                             long long pz) {
  return (long long)(bx - ax) * (pz - az) - (long long)(bz - az) * (px - ax);
}
__device__ __forceinline__ int owns_edge(int ax, int az, int bx, int bz) {
  int dz = bz - az, dx = bx - ax;
  return (dz < 0) || (dz == 0 && dx > 0);
}

// Narrow [lo, hi] (k' in [0, nk]) to the k' with q + k' * sk > 0.
__device__ __forceinline__ void span_bound(long long q, long long sk, int nk, int& lo, int& hi) {
  if (sk == 0) {
    if (q <= 0) { lo = 1; hi = 0; }
    return;
  }
  if (sk > 0) {  // increasing in k': smallest k' with a positive value
    int k = 0;
    if (q <= 0) {
      const float est = __fdividef((float)(-q), (float)sk) + 1.0f;
      k = (int)fminf(fmaxf(floorf(est), 0.0f), (float)(nk + 1));
    }
    while (k <= nk && q + (long long)k * sk <= 0) ++k;
    while (k > 0 && q + (long long)(k - 1) * sk > 0) --k;
    lo = max(lo, k);
  } else {       // decreasing in k': largest k' with a positive value
    if (q <= 0) { lo = 1; hi = 0; return; }
    const float est = __fdividef((float)q, (float)(-sk));
    int k = (int)fminf(fmaxf(floorf(est), -1.0f), (float)nk);
    while (k >= 0 && q + (long long)k * sk <= 0) --k;
    while (k < nk && q + (long long)(k + 1) * sk > 0) ++k;
    hi = min(hi, k);
  }
}

// Rasterise one cross-section triangle (NDC x,z) into the bit planes of
// `slice` with XOR.  Same rule as the oracle: vertices snapped to 1/256 pixel,
// pixel centres tested with exact integer edge functions, a sample exactly
// on an edge belongs to the triangle for which it is a top-left edge.  With
// integer E, "E > 0 || (E == 0 && owns)" is "E + owns > 0".
__device__ void raster_xor(const JobDesc& J, uint32_t slice, float ax, float az, float bx,
                           float bz, float cx, float cz) {
  const float hw = __fmul_rn(0.5f, (float)J.X), hh = __fmul_rn(0.5f, (float)J.Z);
  int x0 = to_fixed(ax, hw), z0 = to_fixed(az, hh);
  int x1 = to_fixed(bx, hw), z1 = to_fixed(bz, hh);
  int x2 = to_fixed(cx, hw), z2 = to_fixed(cz, hh);
  const int mnx = min(x0, min(x1, x2)), mxx = max(x0, max(x1, x2));
  const int mnz = min(z0, min(z1, z2)), mxz = max(z0, max(z1, z2));
  // pixel centres 256*i + 128 inside [mn, mx] (fixed point)
  const int ilo = max((mnx + 127) >> 8, 0), ihi = min((mxx - 128) >> 8, (int)J.X - 1);
  const int klo = max((mnz + 127) >> 8, 0), khi = min((mxz - 128) >> 8, (int)J.Z - 1);
  if (ilo > ihi || klo > khi) return;
  const long long area = edge_fn(x0, z0, x1, z1, x2, z2);
  if (area == 0) return;
  if (area < 0) { int tx = x1, tz = z1; x1 = x2; z1 = z2; x2 = tx; z2 = tz; }
  const long long b0 = owns_edge(x0, z0, x1, z1), b1 = owns_edge(x1, z1, x2, z2),
                  b2 = owns_edge(x2, z2, x0, z0);
  const long long px0 = (long long)ilo * 256 + 128, pz0 = (long long)klo * 256 + 128;
  // edge values (+ tie bias) at the first pixel centre; steps per k and per i
  const long long r0 = edge_fn(x0, z0, x1, z1, px0, pz0) + b0;
  const long long r1 = edge_fn(x1, z1, x2, z2, px0, pz0) + b1;
  const long long r2 = edge_fn(x2, z2, x0, z0, px0, pz0) + b2;
  const long long sk0 = 256LL * (x1 - x0), sk1 = 256LL * (x2 - x1), sk2 = 256LL * (x0 - x2);
  const long long si0 = -256LL * (z1 - z0), si1 = -256LL * (z2 - z1), si2 = -256LL * (z0 - z2);
  uint32_t* const col = J.par + (size_t)slice * J.Zw;  // + i * Y * Zw per pixel column
  const size_t istride = (size_t)J.Y * J.Zw;
  if (ihi - ilo <= 1 && khi - klo <= 1) {
    // <= 2x2 candidate pixels (almost every cross-section): no loops
#pragma unroll
    for (int di = 0; di < 2; ++di) {
      if (ilo + di > ihi) break;
      const long long e0 = r0 + di * si0, e1 = r1 + di * si1, e2 = r2 + di * si2;
      const bool in0 = (e0 > 0) & (e1 > 0) & (e2 > 0);
      const bool in1 = (klo + 1 <= khi) & (e0 + sk0 > 0) & (e1 + sk1 > 0) & (e2 + sk2 > 0);
      uint32_t* row = col + (size_t)(ilo + di) * istride;
      const uint32_t w0 = (uint32_t)klo >> 5, w1 = (uint32_t)(klo + 1) >> 5;
      const uint32_t m0 = in0 ? 1u << (klo & 31) : 0u, m1 = in1 ? 1u << ((klo + 1) & 31) : 0u;
      if (w0 == w1) {
        if (m0 | m1) atomicXor(row + w0, m0 | m1);
      } else {
        if (m0) atomicXor(row + w0, m0);
        if (m1) atomicXor(row + w1, m1);
      }
    }
    return;
  }
  // span path: for pixel column i the covered k form one interval (the
  // triangle is convex); each edge bounds it from one side.  The bound is
  // estimated with a float division and then fixed with exact integer edge
  // values, so the covered set is exactly the per-pixel test's.
  const int nk = khi - klo;
  long long q0 = r0, q1 = r1, q2 = r2;
  for (int i = ilo; i <= ihi; ++i, q0 += si0, q1 += si1, q2 += si2) {
    int lo = 0, hi = nk;
    span_bound(q0, sk0, nk, lo, hi);
    span_bound(q1, sk1, nk, lo, hi);
    span_bound(q2, sk2, nk, lo, hi);
    if (lo > hi) continue;
    uint32_t* row = col + (size_t)i * istride;
    const int ka = klo + lo, kb = klo + hi;
    for (int w = ka >> 5; w <= (kb >> 5); ++w) {
      const int a = max(ka, w << 5) & 31, b = min(kb, (w << 5) + 31) & 31;
      const uint32_t m = (b == 31 ? 0xFFFFFFFFu : ((2u << b) - 1u)) & ~((1u << a) - 1u);
      atomicXor(row + w, m);
    }
  }
}

// one (tetrahedron, slice) pair: the 1-2 cross-section triangles
// (Tetravoxelizer.cpp:59-89; endpoint choice without divergent branches)
__device__ __forceinline__ void cross_section(const JobDesc& J, const tv& A, const tv& B,
                                              const tv& Cc, const tv& D, uint32_t s) {
  const float sl = J.ys[s];
  float p0x, p0z, v1x, v1z, v2x, v2z;
  interp(A, D, sl, p0x, p0z);
  const bool ab = sl <= B.y, ac = sl <= Cc.y;
  interp(ab ? A : B, ab ? B : D, sl, v1x, v1z);
  interp(ac ? A : Cc, ac ? Cc : D, sl, v2x, v2z);
  raster_xor(J, s, p0x, p0z, v1x, v1z, v2x, v2z);
  if (B.y < sl && sl <= Cc.y) {
    float bx, bz;
    interp(B, Cc, sl, bx, bz);
    raster_xor(J, s, bx, bz, v2x, v2z, v1x, v1z);
  }
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

__global__ void __launch_bounds__(256, 4) k_parity_flat(const JobDesc* jobs, int njobs,
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
    tv A, B, Cc, D;
    const JobDesc* J = nullptr;
    uint32_t s0 = 0;
    unsigned long long fb = 0, fe = 0;
    for (unsigned long long p = base + lane; p < end; p += 32) {
      // advance the face cursor (faces with no item have pbase equal to the next)
      while (p >= pbase[g] + pcnt[g]) ++g;
      if (g != cached) {
        cached = g;
        J = &jobs[job_of_face(jobs, njobs, g)];
        const uint32_t f = g - J->face_base;
        const float4* o = J->tets + 3 * (size_t)f;
        const float4 q0 = o[0], q1 = o[1], q2 = o[2];
        A = {q0.x, q0.y, q0.z};
        B = {q0.w, q1.x, q1.y};
        Cc = {q1.z, q1.w, q2.x};
        D = {q2.y, q2.z, q2.w};
        s0 = J->tet_range[f] & 0xFFFFu;
        fb = pbase[g];
        fe = fb + pcnt[g];
      }
      (void)fe;
      cross_section(*J, A, B, Cc, D, s0 + (uint32_t)(p - fb));
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
void parity_raster(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces,
                   const FaceScratch& fs, int num_sms) {
  if (!total_faces) return;
  const uint32_t nb = (total_faces + 1023) / 1024;
  k_scan_local<<<nb, 1024, 0, st>>>(fs.pcnt, fs.pbase, fs.psums, total_faces);
  k_scan_sums<<<1, 1024, 0, st>>>(fs.psums, nb, fs.ptotal);
  k_scan_add<<<(total_faces + 255) / 256, 256, 0, st>>>(fs.pbase, fs.psums, total_faces);
  k_parity_flat<<<num_sms * 16, 256, 0, st>>>(dj, njobs, fs.pcnt, fs.pbase, fs.ptotal, total_faces);
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
