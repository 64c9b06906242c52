/*
 * vf_oracle_sample.c -- CPU oracle of CADModel::sampleCPU (CADModel.cpp:264-370):
 * a point cloud of at most S points on a triangle mesh, as the dataset
 * generator samples every fragment mesh (CADScene.cpp:129-143, 340-372).
 *
 * TEST INFRASTRUCTURE ONLY (see vf_oracle.h).
 *
 * The reference, for a mesh of T faces (areas a_t = |cross(v2-v1, v3-v1)| / 2,
 * Triangle3D.cpp:38-43; sumArea and maxArea, Model3D.cpp:238-261):
 *  - a noise buffer of NB = 2 * max(1, ceil(maxArea / sumArea * S)) floats in
 *    [0, 1) (Seeder::getFloatNoise);
 *  - S > T: face t gets n_t = max(ceil(a_t / sumArea * S), 1) samples; sample
 *    i (its place in the output) takes r = (noise[i % NB], noise[(i+1) % NB]),
 *    r = 1 - r when r.x + r.y >= 1, p = v1 + u*r.x + v*r.y; more than S
 *    samples are cut to S (PointCloud3D::subselect);
 *  - S <= T: S distinct faces drawn uniformly (rejection), one sample each,
 *    with r = (noise[t % NB], noise[(t+1) % NB]) for face t.
 * Fixed here (the reference leaves them to OpenMP, std::random_device and
 * rand()): samples in face order (the reference places them in whatever
 * order its threads take the critical section); sumArea summed in double over
 * chunks of 1024 faces in order, then the chunk sums in order, rounded to
 * float (the reference's float reduction order varies with the threads); the
 * noise and the face draws from the counter-based hash, keyed by the mesh's
 * key (a fragment value); subselect keeps the systematic sample i with
 * floor((i+1) S / P) > floor(i S / P) of the P samples (the reference keeps
 * a shuffled prefix from an unseeded generator, which no run can repeat);
 * a ceil that is NaN or below 1 counts as 1, one above INT_MAX as INT_MAX.
 */
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "vf_oracle.h"

#define VFO_STREAM_SAMPLE 6u       /* noise buffer */
#define VFO_STREAM_SAMPLE_FACE 7u  /* face draws */
#define CHUNK 1024u

static int ceil_count(float x) {
  const float c = ceilf(x);
  if (!(c > 1.0f)) return 1;
  if (c >= 2147483647.0f) return INT_MAX;
  return (int)c;
}

static float noise_at(uint64_t seed, uint32_t key, uint64_t j) {
  return vfo_u01(vfo_hash(seed, VFO_STREAM_SAMPLE, ((uint64_t)key << 40) + j));
}

static void tri(const float* V, const uint32_t* f, float v1[3], float u[3], float v[3]) {
  for (int a = 0; a < 3; ++a) {
    v1[a] = V[4 * (size_t)f[0] + a];
    u[a] = V[4 * (size_t)f[1] + a] - v1[a];
    v[a] = V[4 * (size_t)f[2] + a] - v1[a];
  }
}

static float area_of(const float u[3], const float v[3]) {
  const float cx = u[1] * v[2] - v[1] * u[2];
  const float cy = u[2] * v[0] - v[2] * u[0];
  const float cz = u[0] * v[1] - v[0] * u[1];
  return sqrtf(cx * cx + cy * cy + cz * cz) / 2.0f;
}

static void point(const float v1[3], const float u[3], const float v[3], float rx, float ry,
                  float* out) {
  if (rx + ry >= 1.0f) {
    rx = 1.0f - rx;
    ry = 1.0f - ry;
  }
  for (int a = 0; a < 3; ++a) out[a] = v1[a] + u[a] * rx + v[a] * ry;
  out[3] = 1.0f;
}

int vfo_sample_mesh(const float* verts, const uint32_t* faces, uint32_t nfaces, uint32_t S,
                    uint64_t seed, uint32_t key, float* out, uint64_t* nout) {
  *nout = 0;
  if (!nfaces || !S) return 0;
  const uint32_t T = nfaces;
  float* area = (float*)malloc((size_t)T * sizeof(float));
  if (!area) return VFO_ERR_RANGE;
  float maxArea = 0.0f;
  double total = 0.0;
  for (uint32_t c0 = 0; c0 < T; c0 += CHUNK) {
    double part = 0.0;
    for (uint32_t t = c0; t < T && t < c0 + CHUNK; ++t) {
      float v1[3], u[3], v[3];
      tri(verts, faces + 4 * (size_t)t, v1, u, v);
      area[t] = area_of(u, v);
      part += (double)area[t];
      if (area[t] > maxArea) maxArea = area[t];
    }
    total += part;
  }
  const float sumArea = (float)total;
  const uint64_t NB = 2ull * (uint64_t)ceil_count(maxArea / sumArea * (float)S);
  int st = 0;
  if (S > T) {
    uint64_t P = 0;
    for (uint32_t t = 0; t < T; ++t) P += (uint64_t)ceil_count(area[t] / sumArea * (float)S);
    uint64_t i = 0;
    for (uint32_t t = 0; t < T; ++t) {
      float v1[3], u[3], v[3];
      tri(verts, faces + 4 * (size_t)t, v1, u, v);
      const uint64_t n = (uint64_t)ceil_count(area[t] / sumArea * (float)S);
      for (uint64_t k = 0; k < n; ++k, ++i) {
        uint64_t slot = i;
        if (P > S) {
          const uint64_t hi = (i + 1) * S / P, lo = i * S / P;
          if (hi == lo) continue;
          slot = hi - 1;
        }
        point(v1, u, v, noise_at(seed, key, i % NB), noise_at(seed, key, (i + 1) % NB),
              out + 4 * slot);
      }
    }
    *nout = P > S ? S : P;
  } else {
    uint8_t* active = (uint8_t*)calloc(T, 1);
    if (!active) {
      free(area);
      return VFO_ERR_RANGE;
    }
    const uint64_t limit = 64ull * T + 4096u;
    uint32_t got = 0;
    for (uint64_t j = 0; got < S && j < limit; ++j) {
      const float uf = vfo_u01(vfo_hash(seed, VFO_STREAM_SAMPLE_FACE, ((uint64_t)key << 40) + j));
      uint32_t f = (uint32_t)(uf * (float)T);
      if (f > T - 1) f = T - 1;
      if (!active[f]) {
        active[f] = 1;
        ++got;
      }
    }
    if (got < S) {
      st = VFO_ERR_RANGE;
    } else {
      uint64_t slot = 0;
      for (uint32_t t = 0; t < T; ++t) {
        if (!active[t]) continue;
        float v1[3], u[3], v[3];
        tri(verts, faces + 4 * (size_t)t, v1, u, v);
        point(v1, u, v, noise_at(seed, key, t % NB), noise_at(seed, key, (t + 1) % NB),
              out + 4 * slot);
        ++slot;
      }
      *nout = S;
    }
    free(active);
  }
  free(area);
  return st;
}
