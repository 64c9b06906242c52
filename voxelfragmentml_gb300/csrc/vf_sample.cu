// vf_sample.cu -- CADModel::sampleCPU (CADModel.cpp:264-370) on sm_103a: a
// point cloud of at most S points on each of a set of triangle meshes (the
// fragment meshes of vf_grid_triangulate, or one caller mesh), every mesh at
// once.
//
//   k_pc_area     one thread per face: area |cross(v2-v1, v3-v1)| / 2
//   k_pc_chunks   one thread per 1024-face chunk of a mesh: double sum and max
//   k_pc_mesh     one thread per mesh: sumArea (chunk sums in order, rounded to
//                 float), maxArea, the noise length NB
//   k_pc_select   one CTA per mesh with S <= T: S distinct faces, the first ones
//                 of the draw sequence; 256 draws per round tested in parallel
//                 (already chosen, or drawn earlier in the round), then ranked
//                 in draw order, so the set equals the sequential rejection
//                 sampler's
//   k_pc_count    samples per face: max(ceil(a / sumArea * S), 1) when S > T,
//                 else 1 for a chosen face; an exclusive scan places them
//   k_pc_points   one thread per face: its samples (noise pair, fold, v1 + u r.x
//                 + v r.y); more than S samples keep the systematic sample
//                 floor((i+1) S / P) > floor(i S / P)
// Every float step is rounded as written, as the oracle does.
#include "vf.h"
#include "vf_kernels.h"

namespace {

constexpr uint32_t CHUNK = 1024;

__device__ __forceinline__ int ceil_count(float x) {
  const float c = ceilf(x);
  if (!(c > 1.0f)) return 1;
  if (c >= 2147483647.0f) return 0x7FFFFFFF;
  return (int)c;
}

__device__ __forceinline__ float noise_at(uint64_t seed, uint32_t key, uint64_t j) {
  return vf_u01(vf_hash(seed, VF_STREAM_SAMPLE, ((uint64_t)key << 40) + j));
}

// mesh of global face s: the last m with face_off[m] <= s
__device__ __forceinline__ uint32_t mesh_of(const unsigned long long* face_off, uint32_t F, uint64_t s) {
  uint32_t lo = 0, hi = F;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (face_off[mid] <= s) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void tri(const float4* V, const unsigned long long* vert_off, uint32_t m,
                                    const uint4& f, float v1[3], float u[3], float v[3]) {
  const uint64_t b = vert_off[m];
  const float4 a = V[b + f.x], p = V[b + f.y], q = V[b + f.z];
  v1[0] = a.x; v1[1] = a.y; v1[2] = a.z;
  u[0] = __fsub_rn(p.x, a.x); u[1] = __fsub_rn(p.y, a.y); u[2] = __fsub_rn(p.z, a.z);
  v[0] = __fsub_rn(q.x, a.x); v[1] = __fsub_rn(q.y, a.y); v[2] = __fsub_rn(q.z, a.z);
}

__global__ void __launch_bounds__(256) k_pc_area(const float4* V, const uint4* Fc,
                                                 const unsigned long long* vert_off,
                                                 const unsigned long long* face_off, uint32_t F,
                                                 uint64_t nfaces, float* area) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nfaces;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = mesh_of(face_off, F, s);
    float v1[3], u[3], v[3];
    tri(V, vert_off, m, Fc[s], v1, u, v);
    const float cx = __fsub_rn(__fmul_rn(u[1], v[2]), __fmul_rn(v[1], u[2]));
    const float cy = __fsub_rn(__fmul_rn(u[2], v[0]), __fmul_rn(v[2], u[0]));
    const float cz = __fsub_rn(__fmul_rn(u[0], v[1]), __fmul_rn(v[0], u[1]));
    area[s] = __fdiv_rn(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)),
                                             __fmul_rn(cz, cz))),
                        2.0f);
  }
}

// chunk c covers faces [cstart[c], min(cstart[c] + CHUNK, end of its mesh))
__global__ void __launch_bounds__(256) k_pc_chunks(const float* area, const unsigned long long* cstart,
                                                   const unsigned long long* cend, uint32_t nchunks,
                                                   double* csum, float* cmax) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    float mx = 0.0f;
    for (uint64_t t = cstart[c]; t < cend[c]; ++t) {
      s = __dadd_rn(s, (double)area[t]);
      mx = fmaxf(mx, area[t]);
    }
    csum[c] = s;
    cmax[c] = mx;
  }
}

// per mesh: [0] sumArea, [1] maxArea (floats); nb[m] = noise length
__global__ void k_pc_mesh(const double* csum, const float* cmax, const unsigned long long* mchunk,
                          uint32_t F, uint32_t S, float* msum, uint64_t* nb) {
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < F; m += gridDim.x * blockDim.x) {
    double s = 0.0;
    float mx = 0.0f;
    for (uint64_t c = mchunk[m]; c < mchunk[m + 1]; ++c) {
      s = __dadd_rn(s, csum[c]);
      mx = fmaxf(mx, cmax[c]);
    }
    const float sum = __double2float_rn(s);
    msum[m] = sum;
    nb[m] = 2ull * (uint64_t)ceil_count(__fmul_rn(__fdiv_rn(mx, sum), (float)S));
  }
}

// one CTA per mesh with S <= T (list `sel`): S distinct faces, the first ones
// of the draw sequence, marked in the face bitmap `chosen` (global face bits)
__global__ void __launch_bounds__(256) k_pc_select(const uint32_t* sel, const unsigned long long* face_off,
                                                   const uint32_t* keys, uint32_t S, uint64_t seed,
                                                   uint32_t* chosen, uint32_t* err) {
  __shared__ uint32_t face[256];
  __shared__ uint32_t s_got;
  __shared__ uint32_t wsum[8];
  const uint32_t m = sel[blockIdx.x];
  const uint64_t base = face_off[m];
  const uint32_t T = (uint32_t)(face_off[m + 1] - base);
  const uint32_t key = keys[m];
  const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) s_got = 0;
  __syncthreads();
  const uint64_t limit = 64ull * T + 4096u;
  for (uint64_t j0 = 0; j0 < limit; j0 += 256) {
    const uint64_t j = j0 + t;
    const float uf = vf_u01(vf_hash(seed, VF_STREAM_SAMPLE_FACE, ((uint64_t)key << 40) + j));
    uint32_t f = (uint32_t)__fmul_rn(uf, (float)T);
    if (f > T - 1) f = T - 1;
    face[t] = f;
    __syncthreads();
    const uint64_t g = base + f;
    bool fresh = j < limit && !((chosen[g >> 5] >> (g & 31)) & 1u);
    for (uint32_t k = 0; k < t && fresh; ++k) fresh = face[k] != f;  // drawn earlier this round
    // rank of the fresh draws in draw order
    const unsigned b = __ballot_sync(0xFFFFFFFFu, fresh);
    if (lane == 0) wsum[w] = (uint32_t)__popc(b);
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t k = 0; k < w; ++k) before += wsum[k];
    const uint32_t rank = s_got + before + (uint32_t)__popc(b & ((1u << lane) - 1u));
    if (fresh && rank < S) atomicOr(chosen + (g >> 5), 1u << (g & 31));
    __syncthreads();
    if (t == 0) {
      uint32_t n = 0;
      for (uint32_t k = 0; k < 8; ++k) n += wsum[k];
      s_got = min(S, s_got + n);
    }
    __syncthreads();
    if (s_got >= S) break;
  }
  if (t == 0 && s_got < S) atomicOr(err, 1u);
}

// samples per face; big[m] = 1 when S > T
__global__ void __launch_bounds__(256) k_pc_count(const float* area, const unsigned long long* face_off,
                                                  uint32_t F, uint64_t nfaces, const float* msum,
                                                  const uint8_t* big, uint32_t S, const uint32_t* chosen,
                                                  uint32_t* cnt) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nfaces;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = mesh_of(face_off, F, s);
    cnt[s] = big[m] ? (uint32_t)ceil_count(__fmul_rn(__fdiv_rn(area[s], msum[m]), (float)S))
                    : ((chosen[s >> 5] >> (s & 31)) & 1u);
  }
}

__global__ void __launch_bounds__(256) k_pc_points(const float4* V, const uint4* Fc,
                                                   const unsigned long long* vert_off,
                                                   const unsigned long long* face_off, uint32_t F,
                                                   uint64_t nfaces, const uint32_t* cnt,
                                                   const unsigned long long* soff, const uint64_t* nb,
                                                   const uint8_t* big, const uint32_t* keys,
                                                   const unsigned long long* out_off, uint32_t S,
                                                   uint64_t seed, float4* out) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nfaces;
       s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t n = cnt[s];
    if (!n) continue;
    const uint32_t m = mesh_of(face_off, F, s);
    const uint64_t first = soff[face_off[m]];  // the mesh's first sample
    const uint64_t P = soff[face_off[m + 1]] - first;
    const uint64_t NB = nb[m];
    float v1[3], u[3], v[3];
    tri(V, vert_off, m, Fc[s], v1, u, v);
    const uint64_t tl = s - face_off[m];
    for (uint32_t k = 0; k < n; ++k) {
      const uint64_t i = soff[s] - first + k;
      uint64_t slot = i;
      if (big[m] && P > S) {
        const uint64_t hi = (i + 1) * S / P, lo = i * S / P;
        if (hi == lo) continue;
        slot = hi - 1;
      }
      const uint64_t ni = big[m] ? i : tl;
      float rx = noise_at(seed, keys[m], ni % NB), ry = noise_at(seed, keys[m], (ni + 1) % NB);
      if (__fadd_rn(rx, ry) >= 1.0f) {
        rx = __fsub_rn(1.0f, rx);
        ry = __fsub_rn(1.0f, ry);
      }
      float4 p;
      p.x = __fadd_rn(__fadd_rn(v1[0], __fmul_rn(u[0], rx)), __fmul_rn(v[0], ry));
      p.y = __fadd_rn(__fadd_rn(v1[1], __fmul_rn(u[1], rx)), __fmul_rn(v[1], ry));
      p.z = __fadd_rn(__fadd_rn(v1[2], __fmul_rn(u[2], rx)), __fmul_rn(v[2], ry));
      p.w = 1.0f;
      out[out_off[m] + slot] = p;
    }
  }
}

// P per mesh from the scanned sample offsets
__global__ void k_pc_totals(const unsigned long long* soff, const unsigned long long* face_off, uint32_t F,
                            unsigned long long* P) {
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < F; m += gridDim.x * blockDim.x)
    P[m] = soff[face_off[m + 1]] - soff[face_off[m]];
}

inline int blocks_for(uint64_t n, int num_sms) {
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)num_sms * 8));
}

}  // namespace

namespace vfk {

void pc_areas(cudaStream_t st, const SampleMeshes& M, float* area, const unsigned long long* cstart,
              const unsigned long long* cend, uint32_t nchunks, double* csum, float* cmax,
              const unsigned long long* mchunk, uint32_t S, float* msum, uint64_t* nb, int num_sms) {
  if (M.nfaces) {
    k_pc_area<<<blocks_for(M.nfaces, num_sms), 256, 0, st>>>(M.verts, M.faces, M.vert_off, M.face_off, M.F,
                                                             M.nfaces, area);
    k_pc_chunks<<<blocks_for(nchunks, num_sms), 256, 0, st>>>(area, cstart, cend, nchunks, csum, cmax);
  }
  k_pc_mesh<<<(M.F + 255) / 256, 256, 0, st>>>(csum, cmax, mchunk, M.F, S, msum, nb);
}

void pc_select(cudaStream_t st, const SampleMeshes& M, const uint32_t* sel, uint32_t nsel, uint32_t S,
               uint64_t seed, uint32_t* chosen, uint32_t* err) {
  if (nsel) k_pc_select<<<nsel, 256, 0, st>>>(sel, M.face_off, M.keys, S, seed, chosen, err);
}

void pc_count(cudaStream_t st, const SampleMeshes& M, const float* area, const float* msum,
              const uint8_t* big, uint32_t S, const uint32_t* chosen, uint32_t* cnt,
              unsigned long long* P, unsigned long long* soff, unsigned long long* sums, int num_sms) {
  if (!M.nfaces) return;
  k_pc_count<<<blocks_for(M.nfaces, num_sms), 256, 0, st>>>(area, M.face_off, M.F, M.nfaces, msum, big, S,
                                                            chosen, cnt);
  exclusive_scan(st, cnt, soff, sums, (uint32_t)M.nfaces, soff + M.nfaces);
  k_pc_totals<<<(M.F + 255) / 256, 256, 0, st>>>(soff, M.face_off, M.F, P);
}

void pc_points(cudaStream_t st, const SampleMeshes& M, const uint32_t* cnt, const unsigned long long* soff,
               const uint64_t* nb, const uint8_t* big, const unsigned long long* out_off, uint32_t S,
               uint64_t seed, float4* out, int num_sms) {
  if (!M.nfaces) return;
  k_pc_points<<<blocks_for(M.nfaces, num_sms), 256, 0, st>>>(M.verts, M.faces, M.vert_off, M.face_off, M.F,
                                                             M.nfaces, cnt, soff, nb, big, M.keys, out_off,
                                                             S, seed, out);
}

}  // namespace vfk
