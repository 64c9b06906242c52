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
//   parity_raster       : one warp per tetrahedron, lanes over its slices;
//                         cross-section triangles rasterised with exact
//                         integer edge functions, XOR into bit planes
//   shell_sat           : one warp per triangle, lanes over candidate voxels
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

__global__ void k_tetra(const JobDesc* jobs, JobState* st, int njobs, uint32_t total) {
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += gridDim.x * blockDim.x) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    const uint32_t f = g - J.face_base;
    const uint32_t* fi = J.faces + 3 * (size_t)f;
    if (fi[0] >= J.nverts || fi[1] >= J.nverts || fi[2] >= J.nverts) {
      atomicOr(&st[j].err, VF_JERR_INVALID);  // bad face: never dereferenced
      J.tet_range[f] = 0xFFFFu;
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
__device__ __forceinline__ long long fdiv_floor(long long a, long long b) {
  long long q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}

__device__ void raster_xor(const JobDesc& J, uint32_t slice, float ax, float az, float bx,
                           float bz, float cx, float cz) {
  const float hw = __fmul_rn(0.5f, (float)J.X), hh = __fmul_rn(0.5f, (float)J.Z);
  int x0 = to_fixed(ax, hw), z0 = to_fixed(az, hh);
  int x1 = to_fixed(bx, hw), z1 = to_fixed(bz, hh);
  int x2 = to_fixed(cx, hw), z2 = to_fixed(cz, hh);
  long long area = edge_fn(x0, z0, x1, z1, x2, z2);
  if (area == 0) return;
  if (area < 0) { int tx = x1, tz = z1; x1 = x2; z1 = z2; x2 = tx; z2 = tz; }
  int mnx = min(x0, min(x1, x2)), mxx = max(x0, max(x1, x2));
  int mnz = min(z0, min(z1, z2)), mxz = max(z0, max(z1, z2));
  long long ilo = fdiv_floor((long long)mnx - 128 + 255, 256), ihi = fdiv_floor((long long)mxx - 128, 256);
  long long klo = fdiv_floor((long long)mnz - 128 + 255, 256), khi = fdiv_floor((long long)mxz - 128, 256);
  if (ilo < 0) ilo = 0;
  if (klo < 0) klo = 0;
  if (ihi > (long long)J.X - 1) ihi = (long long)J.X - 1;
  if (khi > (long long)J.Z - 1) khi = (long long)J.Z - 1;
  const int o01 = owns_edge(x0, z0, x1, z1), o12 = owns_edge(x1, z1, x2, z2),
            o20 = owns_edge(x2, z2, x0, z0);
  for (long long i = ilo; i <= ihi; ++i) {
    const long long px = i * 256 + 128;
    uint32_t* row = J.par + ((size_t)i * J.Y + slice) * J.Zw;
    uint32_t word = 0xFFFFFFFFu, bits = 0;
    for (long long k = klo; k <= khi; ++k) {
      const long long pz = k * 256 + 128;
      long long e0 = edge_fn(x0, z0, x1, z1, px, pz);
      long long e1 = edge_fn(x1, z1, x2, z2, px, pz);
      long long e2 = edge_fn(x2, z2, x0, z0, px, pz);
      bool in = (e0 > 0 || (e0 == 0 && o01)) && (e1 > 0 || (e1 == 0 && o12)) &&
                (e2 > 0 || (e2 == 0 && o20));
      if (!in) continue;
      uint32_t w = (uint32_t)(k >> 5);
      if (w != word) {
        if (bits) atomicXor(row + word, bits);
        word = w;
        bits = 0;
      }
      bits ^= 1u << (k & 31);
    }
    if (bits) atomicXor(row + word, bits);
  }
}

__global__ void k_parity(const JobDesc* jobs, int njobs, uint32_t total) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < total; g += warps) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    const uint32_t f = g - J.face_base;
    const uint32_t rg = J.tet_range[f];
    const uint32_t s0 = rg & 0xFFFFu, s1 = rg >> 16;
    if (s0 > s1) continue;
    const float4* o = J.tets + 3 * (size_t)f;
    float4 q0 = o[0], q1 = o[1], q2 = o[2];
    tv A = {q0.x, q0.y, q0.z}, B = {q0.w, q1.x, q1.y}, Cc = {q1.z, q1.w, q2.x},
       D = {q2.y, q2.z, q2.w};
    for (uint32_t s = s0 + lane; s <= s1; s += 32) {
      const float sl = J.ys[s];
      float p0x, p0z, v1x, v1z, v2x, v2z;
      interp(A, D, sl, p0x, p0z);
      if (sl <= B.y) interp(A, B, sl, v1x, v1z); else interp(B, D, sl, v1x, v1z);
      if (sl <= Cc.y) interp(A, Cc, sl, v2x, v2z); else interp(Cc, D, sl, v2x, v2z);
      raster_xor(J, s, p0x, p0z, v1x, v1z, v2x, v2z);
      if (B.y < sl && sl <= Cc.y) {
        float bx, bz;
        interp(B, Cc, sl, bx, bz);
        raster_xor(J, s, bx, bz, v2x, v2z, v1x, v1z);
      }
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

__global__ void k_shell(const JobDesc* jobs, int njobs, uint32_t total) {
  const int lane = threadIdx.x & 31;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < total; g += warps) {
    const int j = job_of_face(jobs, njobs, g);
    const JobDesc& J = jobs[j];
    const uint32_t f = g - J.face_base;
    const uint32_t dims[3] = {J.X, J.Y, J.Z};
    float cs[3];
    for (int a = 0; a < 3; ++a) cs[a] = __fdiv_rn(SUB(J.amax[a], J.amin[a]), (float)dims[a]);
    const uint32_t* fi = J.faces + 3 * (size_t)f;
    if (fi[0] >= J.nverts || fi[1] >= J.nverts || fi[2] >= J.nverts) continue;  // flagged by k_tetra
    const float* q0 = J.verts + 3 * (size_t)fi[0];
    const float* q1 = J.verts + 3 * (size_t)fi[1];
    const float* q2 = J.verts + 3 * (size_t)fi[2];
    int lo[3], n[3];
    for (int a = 0; a < 3; ++a) {
      float mn, mx;
      mm3(q0[a], q1[a], q2[a], mn, mx);
      lo[a] = vf_clampi(float_cell(__fdiv_rn(SUB(mn, J.amin[a]), cs[a]), dims[a]) - 1, 0, dims[a] - 1);
      int hi = vf_clampi(float_cell(__fdiv_rn(SUB(mx, J.amin[a]), cs[a]), dims[a]) + 1, 0, dims[a] - 1);
      n[a] = hi - lo[a] + 1;
    }
    const tv p0 = {q0[0], q0[1], q0[2]}, p1 = {q1[0], q1[1], q1[2]}, p2 = {q2[0], q2[1], q2[2]};
    const int cnt = n[0] * n[1] * n[2];
    for (int c = lane; c < cnt; c += 32) {
      const int k = lo[2] + c % n[2];
      const int jj = lo[1] + (c / n[2]) % n[1];
      const int i = lo[0] + c / (n[2] * n[1]);
      tv bmin = {ADD(J.amin[0], MUL(cs[0], (float)i)), ADD(J.amin[1], MUL(cs[1], (float)jj)),
                 ADD(J.amin[2], MUL(cs[2], (float)k))};
      tv bmax = {ADD(bmin.x, cs[0]), ADD(bmin.y, cs[1]), ADD(bmin.z, cs[2])};
      tv ce = {__fdiv_rn(ADD(bmax.x, bmin.x), 2.0f), __fdiv_rn(ADD(bmax.y, bmin.y), 2.0f),
               __fdiv_rn(ADD(bmax.z, bmin.z), 2.0f)};
      tv r = {SUB(bmax.x, ce.x), SUB(bmax.y, ce.y), SUB(bmax.z, ce.z)};
      if (tri_box(p0, p1, p2, ce, r))
        atomicOr(J.shell + ((size_t)i * J.Y + jj) * J.Zw + (k >> 5), 1u << (k & 31));
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
                uint32_t total_faces) {
  if (total_faces) k_tetra<<<grid_for(total_faces, 256, 65535), 256, 0, st>>>(dj, ds, njobs, total_faces);
}
void parity_raster(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces) {
  if (total_faces) k_parity<<<grid_for(total_faces, 8, 1 << 20), 256, 0, st>>>(dj, njobs, total_faces);
}
void shell_sat(cudaStream_t st, const JobDesc* dj, int njobs, uint32_t total_faces) {
  if (total_faces) k_shell<<<grid_for(total_faces, 8, 1 << 20), 256, 0, st>>>(dj, njobs, total_faces);
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
