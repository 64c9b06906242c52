// vf_api.cu -- the extern "C" entry points declared in include/vf.h.
//
// vf_grid_* calls map a RegularGrid operation onto the batch machinery with
// one job and a subset of stages; vf_batch_run / vf_plain_run run whole
// jobs; vf_server_* runs the continuous-batching loop on its own thread.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include <sys/mman.h>
#include <sys/syscall.h>
#include <unistd.h>

#include "vf_runtime.h"

namespace vfr {
const char* last_error();
void dims_for_aabb(const float mn[3], const float mx[3], uint32_t maxv, uint32_t out[3]);
}  // namespace vfr

using vfr::fail;

namespace {
std::mutex g_host_mu;
std::map<void*, size_t> g_host_mapped;  // vf_host_alloc buffers placed by mbind
constexpr int kMpolPreferred = 1;       // MPOL_PREFERRED (linux/mempolicy.h)

// host NUMA node closest to the current device, or -1
int device_host_numa() {
  int dev = 0, node = -1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&node, cudaDevAttrHostNumaId, dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return node;
}
}  // namespace

#define VF_CK(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(VF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct vf_ctx {
  vfr::Ctx c;
};

// device state of vf_grid_triangulate, kept for vf_grid_meshes
struct MeshState {
  vfr::DevBuf mask, vbase, rcnt, rbase, trcnt, tbase, sums, tot, present, dense, table, vkey, vown,
      vflag, vperm, tmp, vinv, tkey, tv, tperm, hist, hbase, vert, gface, face, voff, foff, acc, err,
      deg, start, ustart, ent, nbr, meta;
  std::vector<uint16_t> values;
  uint64_t V = 0, T = 0;
  bool ready = false;
  // phase boundaries on the grid's stream: 0 start, 1 counted, 2 sizes read
  // back, 3 records + split + positions + faces, 4 smoothing lists, 5
  // smoothed, 6 end
  cudaEvent_t ev[7] = {};
  float phase_ms[6] = {};
  // [0] vertices [1] faces [2] boundary vertices [3] face incidences summed by
  // the smoothing [4] neighbour entries [5] neighbour entries of boundary vertices
  uint64_t counters[6] = {};
  void release(vfr::Ctx& c) {
    for (cudaEvent_t& e : ev)
      if (e) {
        cudaEventDestroy(e);
        e = nullptr;
      }
    for (vfr::DevBuf* b : {&mask, &vbase, &rcnt, &rbase, &trcnt, &tbase, &sums, &tot, &present,
                           &dense, &table, &vkey, &vown, &vflag, &vperm, &tmp, &vinv, &tkey, &tv,
                           &tperm, &hist, &hbase, &vert, &gface, &face, &voff, &foff, &acc, &err,
                           &deg, &start, &ustart, &ent, &nbr, &meta})
      c.free_buf(*b);
    ready = false;
  }
};

// device scratch of the impact path (rays, nearSeeds)
struct ImpactState {
  vfr::DevBuf rays, hits, frags, out, status, bits;
  void release(vfr::Ctx& c) {
    for (vfr::DevBuf* b : {&rays, &hits, &frags, &out, &status, &bits}) c.free_buf(*b);
  }
};

// device state of point sampling (CADModel::sampleCPU)
struct SampleState {
  vfr::DevBuf area, cstart, cend, csum, cmax, mchunk, msum, nb, big, sel, chosen, err, cnt, P, soff,
      sums, out_off, out, keys, verts, faces, voff, foff;
  uint64_t npoints = 0;
  std::vector<uint64_t> offsets;  // per mesh, F + 1
  bool ready = false;
  void release(vfr::Ctx& c) {
    for (vfr::DevBuf* b : {&area, &cstart, &cend, &csum, &cmax, &mchunk, &msum, &nb, &big, &sel, &chosen,
                           &err, &cnt, &P, &soff, &sums, &out_off, &out, &keys, &verts, &faces, &voff,
                           &foff})
      c.free_buf(*b);
    ready = false;
  }
};

struct vf_grid {
  vf_ctx* ctx = nullptr;
  vfr::Batch b;
  vf_job job;
  std::vector<uint32_t> seeds;  // last seeds used by fracture_model
  MeshState mesh;
  ImpactState impact;
  SampleState sample;
};

extern "C" {

void vf_params_default(vf_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->algorithm = VF_FLOOD;         // _fractureAlgorithm(FLOOD)
  p->distance = VF_CHEBYSHEV;      // _distanceFunction(CHEBYSHEV)
  p->num_seeds = 8;                // _numSeeds(8)
  p->num_extra_seeds = 0;          // dataset mode sets extra seeds explicitly
  p->merge_distance = VF_EUCLIDEAN;
  p->seed_location = VF_OUTER;     // CADScene.cpp:633
  p->seed = 80;                    // _seed(80)
  p->noise_amplitude = 0.0f;
  p->noise_period = 16;
  p->erode = 0;
  p->erosion_type = VF_ELLIPSE;
  p->erosion_size = 3;
  p->erosion_iterations = 3;
  p->erosion_probability = 0.5f;
  p->erosion_threshold = 0.5f;
  p->boundary_size = 1;            // detectBoundaries(1)
  p->num_impacts = 0;    // _numImpacts(0)
  p->bias_seeds = 32;    // _biasSeeds(32)
  p->bias_focus = 5;     // _biasFocus(5)
}

const char* vf_last_error(void) { return vfr::last_error(); }

const char* vf_status_string(vf_status s) {
  switch (s) {
    case VF_OK: return "ok";
    case VF_ERR_INVALID: return "invalid argument";
    case VF_ERR_CUDA: return "CUDA error";
    case VF_ERR_OOM: return "out of device memory / budget";
    case VF_ERR_SEED_SEARCH: return "seed search exceeded the try limit";
    case VF_ERR_RANGE: return "value out of range";
    case VF_ERR_TIMEOUT: return "bounded device wait expired";
    case VF_ERR_NOT_BUILT: return "CUDA path unavailable";
    case VF_ERR_BUSY: return "server queue full";
    default: return "unknown status";
  }
}

const char* vf_version(void) { return "vfgb300 1.0 sm_103a"; }

vf_status vf_ctx_create(int device, size_t hbm_budget, vf_ctx** out) {
  if (!out) return fail(VF_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(VF_ERR_NOT_BUILT, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(VF_ERR_INVALID, "device index out of range");
  VF_CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  VF_CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major * 10 + prop.minor < 100)
    return fail(VF_ERR_NOT_BUILT, "this library is built for sm_103a (GB300)");
  vf_ctx* c = new vf_ctx();
  c->c.device = device;
  c->c.num_sms = prop.multiProcessorCount;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  c->c.budget = hbm_budget ? hbm_budget : (size_t)(0.9 * (double)fr);
  if (cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(VF_ERR_CUDA, "stream creation failed");
  }
  for (int i = 0; i < 16; ++i) cudaEventCreate(&c->c.ev[i]);
  cudaEventCreateWithFlags(&c->c.ev_relax, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->c.ev_compute, cudaEventDisableTiming);
  vf_status s = c->c.batch.init(&c->c, false);
  if (s) {
    delete c;
    return s;
  }
  *out = c;
  return VF_OK;
}

vf_status vf_ctx_destroy(vf_ctx* ctx) {
  if (!ctx) return VF_OK;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  ctx->c.batch.release();
  for (int i = 0; i < 16; ++i) cudaEventDestroy(ctx->c.ev[i]);
  if (ctx->c.ev_relax) cudaEventDestroy(ctx->c.ev_relax);
  if (ctx->c.ev_compute) cudaEventDestroy(ctx->c.ev_compute);
  cudaStreamDestroy(ctx->c.stream);
  delete ctx;
  return VF_OK;
}

vf_status vf_ctx_synchronize(vf_ctx* ctx) {
  if (!ctx) return fail(VF_ERR_INVALID, "ctx is NULL");
  VF_CK(cudaStreamSynchronize(ctx->c.stream));
  return VF_OK;
}

size_t vf_ctx_bytes_in_use(const vf_ctx* ctx) { return ctx ? ctx->c.in_use : 0; }

// Pinned host memory.  Buffers of 1 MiB and more are placed on the host NUMA
// node closest to the current device (cudaDevAttrHostNumaId): anonymous
// pages with a preferred-node policy (mbind), then page-locked and mapped
// with cudaHostRegister.  On a host with several CPU sockets the copy
// engines and the direct-write pack kernels then move labels over the
// GPU's own host link instead of crossing the socket interconnect.  Smaller
// buffers, and hosts that report no NUMA node, use cudaMallocHost.
void* vf_host_alloc(size_t bytes) {
  const int node = device_host_numa();
  if (node >= 0 && node < 64 && bytes >= ((size_t)1 << 20)) {
    const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
    const size_t len = (bytes + pg - 1) / pg * pg;
    void* p = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (p != MAP_FAILED) {
      const unsigned long mask = 1ul << node;
      if (syscall(SYS_mbind, p, len, kMpolPreferred, &mask, 8 * sizeof(mask) + 1, 0) == 0 &&
          cudaHostRegister(p, len, cudaHostRegisterPortable | cudaHostRegisterMapped) ==
              cudaSuccess) {
        std::lock_guard<std::mutex> lk(g_host_mu);
        g_host_mapped[p] = len;
        return p;
      }
      cudaGetLastError();  // a failed registration leaves no sticky error
      munmap(p, len);
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}
void vf_host_free(void* p) {
  if (!p) return;
  size_t len = 0;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_mapped.find(p);
    if (it != g_host_mapped.end()) {
      len = it->second;
      g_host_mapped.erase(it);
    }
  }
  if (len) {
    cudaHostUnregister(p);
    munmap(p, len);
  } else {
    cudaFreeHost(p);
  }
}

int vf_host_numa_node(const void* p) {
  if (!p) return -1;
  const uintptr_t pg = (uintptr_t)sysconf(_SC_PAGESIZE);
  void* pages[1] = {reinterpret_cast<void*>(reinterpret_cast<uintptr_t>(p) & ~(pg - 1))};
  int status[1] = {-1};
  if (syscall(SYS_move_pages, 0, 1ul, pages, nullptr, status, 0) != 0) return -1;
  return status[0] >= 0 ? status[0] : -1;
}

vf_status vf_ctx_host_numa(vf_ctx* ctx, int* node) {
  if (!ctx || !node) return fail(VF_ERR_INVALID, "NULL argument");
  *node = -1;
  int v = -1;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrHostNumaId, ctx->c.device) == cudaSuccess) *node = v;
  cudaGetLastError();
  return VF_OK;
}

vf_status vf_ctx_copy_bandwidth(vf_ctx* ctx, size_t bytes, float* h2d_gbs, float* d2h_gbs) {
  if (!ctx || !h2d_gbs || !d2h_gbs || bytes == 0) return fail(VF_ERR_INVALID, "bad argument");
  VF_CK(cudaSetDevice(ctx->c.device));
  void* h = vf_host_alloc(bytes);
  if (!h) return fail(VF_ERR_OOM, "pinned host allocation failed");
  std::memset(h, 1, bytes);
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    vf_host_free(h);
    return fail(VF_ERR_OOM, "device allocation for the copy probe failed");
  }
  cudaStream_t st = ctx->c.stream;
  cudaEvent_t e[3];
  for (auto& x : e) cudaEventCreate(&x);
  float best_h2d = 0.f, best_d2h = 0.f;
  cudaError_t err = cudaSuccess;
  for (int rep = 0; rep < 3 && err == cudaSuccess; ++rep) {
    cudaEventRecord(e[0], st);
    cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    cudaEventRecord(e[1], st);
    cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(e[2], st);
    err = cudaEventSynchronize(e[2]);
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, e[0], e[1]);
    cudaEventElapsedTime(&b, e[1], e[2]);
    if (a > 0.f) best_h2d = std::max(best_h2d, (float)(bytes / (a * 1e6)));
    if (b > 0.f) best_d2h = std::max(best_d2h, (float)(bytes / (b * 1e6)));
  }
  for (auto& x : e) cudaEventDestroy(x);
  cudaFree(d);
  vf_host_free(h);
  if (err != cudaSuccess) return fail(VF_ERR_CUDA, std::string("copy probe: ") + cudaGetErrorString(err));
  *h2d_gbs = best_h2d;
  *d2h_gbs = best_d2h;
  return VF_OK;
}

vf_status vf_dims_for_aabb(const float aabb_min[3], const float aabb_max[3], uint32_t max_voxels,
                           uint32_t dims_out[3]) {
  if (!aabb_min || !aabb_max || !dims_out) return fail(VF_ERR_INVALID, "NULL argument");
  vfr::dims_for_aabb(aabb_min, aabb_max, max_voxels, dims_out);
  return VF_OK;
}

// ---- grid -----------------------------------------------------------------
static vf_status grid_run(vf_grid* g, uint32_t stages) {
  cudaSetDevice(g->ctx->c.device);
  vfr::Batch& B = g->b;
  const vf_job* jp = &g->job;
  B.stages = stages;
  vf_status s = B.plan(&jp, 1);
  if (s) return s;
  s = B.enqueue_batched();
  if (s) return s;
  s = B.finish(nullptr);
  // keep the current grid in buffer 0
  const vfr::JobPlan& p = B.plans[0];
  if (p.final_cur == 1 && (stages & (vfr::ST_PERTURB | vfr::ST_ERODE))) {
    VF_CK(cudaMemcpyAsync(B.grid0.p, B.grid1.p, (size_t)p.X * p.Y * p.Zp * 2,
                          cudaMemcpyDeviceToDevice, B.stream));
    VF_CK(cudaStreamSynchronize(B.stream));
  }
  return s;
}

vf_status vf_grid_create(vf_ctx* ctx, uint32_t X, uint32_t Y, uint32_t Z, const float aabb_min[3],
                         const float aabb_max[3], vf_grid** out) {
  if (!ctx || !out) return fail(VF_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (X < 2 || Y < 2 || Z < 2 || X > VF_MAX_DIM || Y > VF_MAX_DIM || Z > VF_MAX_DIM)
    return fail(VF_ERR_INVALID, "grid dims must be in [2, 4096]");
  vf_grid* g = new vf_grid();
  g->ctx = ctx;
  std::memset(&g->job, 0, sizeof(g->job));
  g->job.dims[0] = X; g->job.dims[1] = Y; g->job.dims[2] = Z;
  for (int a = 0; a < 3; ++a) {
    g->job.aabb_min[a] = aabb_min ? aabb_min[a] : 0.0f;
    g->job.aabb_max[a] = aabb_max ? aabb_max[a] : (float)(a == 0 ? X : a == 1 ? Y : Z);
  }
  bool ok = false;
  for (int a = 0; a < 3; ++a) ok |= g->job.aabb_min[a] != g->job.aabb_max[a];
  if (!ok) {
    delete g;
    return fail(VF_ERR_INVALID, "degenerate AABB");
  }
  vf_params_default(&g->job.params);
  g->job.params.num_seeds = 0;
  vf_status s = g->b.init(&ctx->c, true);
  if (!s) {
    const vf_job* jp = &g->job;
    s = g->b.plan(&jp, 1);
  }
  if (!s) {
    const vfr::JobPlan& p = g->b.plans[0];
    const size_t bytes = (size_t)p.X * p.Y * p.Zp * 2;
    if (cudaMemsetAsync(g->b.grid0.p, 0, bytes, g->b.stream) != cudaSuccess ||
        cudaMemsetAsync(g->b.grid1.p, 0, bytes, g->b.stream) != cudaSuccess ||
        cudaStreamSynchronize(g->b.stream) != cudaSuccess)
      s = fail(VF_ERR_CUDA, "grid clear failed");
  }
  if (s) {
    g->b.release();
    delete g;
    return s;
  }
  *out = g;
  return VF_OK;
}

vf_status vf_grid_destroy(vf_grid* g) {
  if (!g) return VF_OK;
  cudaSetDevice(g->ctx->c.device);
  if (g->b.stream) cudaStreamSynchronize(g->b.stream);
  g->mesh.release(g->ctx->c);
  g->impact.release(g->ctx->c);
  g->sample.release(g->ctx->c);
  g->b.release();
  delete g;
  return VF_OK;
}

vf_status vf_grid_dims(const vf_grid* g, uint32_t dims[3]) {
  if (!g || !dims) return fail(VF_ERR_INVALID, "NULL argument");
  for (int a = 0; a < 3; ++a) dims[a] = g->job.dims[a];
  return VF_OK;
}

vf_status vf_grid_upload(vf_grid* g, const uint16_t* host) {
  if (!g || !host) return fail(VF_ERR_INVALID, "NULL argument");
  cudaSetDevice(g->ctx->c.device);
  const vfr::JobPlan& p = g->b.plans[0];
  const size_t bytes = (size_t)p.X * p.Y * p.Zp * 2;
  cudaStream_t st = g->b.stream;
  VF_CK(cudaMemsetAsync(g->b.grid0.p, 0, bytes, st));
  VF_CK(cudaMemsetAsync(g->b.grid1.p, 0, bytes, st));
  VF_CK(cudaMemcpy2DAsync(g->b.grid0.p, (size_t)p.Zp * 2, host, (size_t)p.Z * 2, (size_t)p.Z * 2,
                          (size_t)p.X * p.Y, cudaMemcpyHostToDevice, st));
  VF_CK(cudaStreamSynchronize(st));
  return VF_OK;
}

vf_status vf_grid_download(vf_grid* g, uint16_t* host) {
  if (!g || !host) return fail(VF_ERR_INVALID, "NULL argument");
  cudaSetDevice(g->ctx->c.device);
  const vfr::JobPlan& p = g->b.plans[0];
  VF_CK(cudaMemcpy2DAsync(host, (size_t)p.Z * 2, g->b.grid0.p, (size_t)p.Zp * 2, (size_t)p.Z * 2,
                          (size_t)p.X * p.Y, cudaMemcpyDeviceToHost, g->b.stream));
  VF_CK(cudaStreamSynchronize(g->b.stream));
  return VF_OK;
}

vf_status vf_grid_export_rle(vf_grid* g, uint8_t* out, size_t cap, size_t* written) {
  if (!g || !written) return fail(VF_ERR_INVALID, "NULL argument");
  cudaSetDevice(g->ctx->c.device);
  vfr::Batch& B = g->b;
  const vfr::JobPlan& p = B.plans[0];
  const uint64_t rows = (uint64_t)p.X * p.Y, nvox = rows * p.Z;
  if (nvox >= 0xFFFFFFFFull) return fail(VF_ERR_RANGE, "RLE export: grids of 2^32 voxels or more");
  vfr::Ctx& c = g->ctx->c;
  vf_status s;
  if ((s = c.alloc(B.rle_cnt, rows * 4)) || (s = c.alloc(B.rle_base, rows * 8)) ||
      (s = c.alloc(B.rle_sums, ((rows + 1023) / 1024 + 2) * 8)) || (s = c.alloc(B.rle_tot, 64)))
    return s;
  cudaStream_t st = B.stream;
  const uint16_t* grid = static_cast<const uint16_t*>(B.grid0.p);
  vfk::rle_count(st, grid, p.X, p.Y, p.Z, p.Zp, static_cast<uint32_t*>(B.rle_cnt.p), c.num_sms);
  unsigned long long* tot = static_cast<unsigned long long*>(B.rle_tot.p);
  vfk::exclusive_scan(st, static_cast<uint32_t*>(B.rle_cnt.p),
                      static_cast<unsigned long long*>(B.rle_base.p),
                      static_cast<unsigned long long*>(B.rle_sums.p), (uint32_t)rows, tot);
  unsigned long long nruns = 0;
  VF_CK(cudaMemcpyAsync(&nruns, tot, 8, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  const size_t need = 12 + 6 * (size_t)nruns;
  *written = need;
  if (!out) {
    if (cap) return fail(VF_ERR_INVALID, "out is NULL");
    return VF_OK;  // size query
  }
  if (cap < need) return fail(VF_ERR_RANGE, "RLE export: buffer smaller than " + std::to_string(need) + " bytes");
  if ((s = c.alloc(B.rle_starts, std::max<size_t>(nruns, 1) * 8)) ||
      (s = c.alloc(B.rle_rec, std::max<size_t>(nruns, 1) * 6)))
    return s;
  vfk::rle_write(st, grid, p.X, p.Y, p.Z, p.Zp, static_cast<unsigned long long*>(B.rle_base.p), tot,
                 static_cast<unsigned long long*>(B.rle_starts.p), static_cast<uint16_t*>(B.rle_rec.p),
                 c.num_sms);
  const uint32_t d[3] = {p.X, p.Y, p.Z};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 4; ++b) out[4 * a + b] = (uint8_t)(d[a] >> (8 * b));
  if (nruns) VF_CK(cudaMemcpyAsync(out + 12, B.rle_rec.p, 6 * (size_t)nruns, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  return VF_OK;
}

void vf_mc_params_default(uint32_t max_voxels, vf_mc_params* p) {
  if (!p) return;
  // MarchingCubes.cpp:400-401: iterations = maxVoxels * _(non)BoundaryMCIterations,
  // converted to unsigned; FractureParameters.h:93-94, 109-110
  p->nonboundary_iterations = (uint32_t)((float)max_voxels * 0.048f);
  p->nonboundary_weight = 0.9f;
  p->boundary_iterations = (uint32_t)((float)max_voxels * 0.048f);
  p->boundary_weight = 0.2f;
}

vf_status vf_grid_triangulate(vf_grid* g, const vf_mc_params* mp, uint32_t* nmeshes,
                              uint64_t* nverts, uint64_t* nfaces) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  vf_mc_params dp;
  const uint32_t* d = g->job.dims;
  if (!mp) {
    vf_mc_params_default(std::max(d[0], std::max(d[1], d[2])), &dp);
    mp = &dp;
  }
  cudaSetDevice(g->ctx->c.device);
  vfr::Ctx& c = g->ctx->c;
  vfr::Batch& B = g->b;
  MeshState& M = g->mesh;
  M.ready = false;
  const vfr::JobPlan& p = B.plans[0];
  const uint64_t rows = (uint64_t)p.X * p.Y, nvox = rows * p.Z;
  const uint64_t crows = (uint64_t)(p.X + 1) * (p.Y + 1);
  if (nvox >= 0xFFFFFFFFull) return fail(VF_ERR_RANGE, "triangulate: grids of 2^32 voxels or more");
  cudaStream_t st = B.stream;
  const int nsm = c.num_sms;
  const vfk::MeshGrid G{static_cast<const uint16_t*>(B.grid0.p), p.X, p.Y, p.Z, p.Zp};
  vf_status s;
  const uint64_t npad = rows * p.Zp;  // face masks and id bases use the grid's row pitch
  if ((s = c.alloc(M.mask, npad)) || (s = c.alloc(M.vbase, npad * 4)) ||
      (s = c.alloc(M.rcnt, rows * 4)) || (s = c.alloc(M.rbase, rows * 8)) ||
      (s = c.alloc(M.trcnt, crows * 4)) || (s = c.alloc(M.tbase, crows * 8)) ||
      (s = c.alloc(M.tot, 64)) || (s = c.alloc(M.present, 32768)) ||
      (s = c.alloc(M.dense, 32768 * 2)) || (s = c.alloc(M.table, 256 * 9)) ||
      (s = c.alloc(M.err, 64)))
    return s;
  auto scan_scratch = [&](uint64_t n) { return c.alloc(M.sums, ((n + 1023) / 1024 + 2) * 8); };
  if ((s = scan_scratch(std::max(rows, crows)))) return s;
  unsigned long long tri[256];
  uint8_t ntri[256];
  vfk::mc_pack_table(tri, ntri);
  unsigned long long* dtri = static_cast<unsigned long long*>(M.table.p);
  uint8_t* dntri = reinterpret_cast<uint8_t*>(dtri + 256);
  VF_CK(cudaMemcpyAsync(dtri, tri, sizeof(tri), cudaMemcpyHostToDevice, st));
  VF_CK(cudaMemcpyAsync(dntri, ntri, sizeof(ntri), cudaMemcpyHostToDevice, st));
  for (cudaEvent_t& e : M.ev)
    if (!e) VF_CK(cudaEventCreate(&e));
  VF_CK(cudaEventRecord(M.ev[0], st));
  VF_CK(cudaMemsetAsync(M.present.p, 0, 32768, st));
  VF_CK(cudaMemsetAsync(M.err.p, 0, 4, st));
  auto sums = static_cast<unsigned long long*>(M.sums.p);
  auto tot = static_cast<unsigned long long*>(M.tot.p);
  auto mask = static_cast<uint8_t*>(M.mask.p);
  auto rbase = static_cast<unsigned long long*>(M.rbase.p);
  auto tbase = static_cast<unsigned long long*>(M.tbase.p);
  auto err = static_cast<uint32_t*>(M.err.p);
  // counts: vertices (exposed faces of fragment voxels) and triangles; the
  // mask kernel stores non-zero masks only
  VF_CK(cudaMemsetAsync(mask, 0, npad, st));
  vfk::mc_vertex_count(st, G, mask, static_cast<uint32_t*>(M.rcnt.p),
                       static_cast<uint8_t*>(M.present.p), nsm);
  vfk::exclusive_scan(st, static_cast<uint32_t*>(M.rcnt.p), rbase, sums, (uint32_t)rows, tot);
  vfk::mc_tri_count(st, G, dtri, dntri, static_cast<uint32_t*>(M.trcnt.p), nsm);
  vfk::exclusive_scan(st, static_cast<uint32_t*>(M.trcnt.p), tbase, sums, (uint32_t)crows, tot + 1);
  VF_CK(cudaEventRecord(M.ev[1], st));
  unsigned long long tots[2] = {0, 0};
  std::vector<uint8_t> present(32768);
  VF_CK(cudaMemcpyAsync(tots, tot, 16, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaMemcpyAsync(present.data(), M.present.p, 32768, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  const uint64_t V = tots[0], T = tots[1];
  if (V >= (1ull << 28) || T >= 0xFFFFFFFFull)
    return fail(VF_ERR_RANGE, "triangulate: 2^28 vertices or 2^32 triangles or more");
  std::vector<uint16_t> dense(32768, 0xFFFFu);
  M.values.clear();
  for (uint32_t v = 2; v < 32768; ++v)
    if (present[v]) {
      dense[v] = (uint16_t)M.values.size();
      M.values.push_back((uint16_t)v);
    }
  const uint32_t F = (uint32_t)M.values.size();
  VF_CK(cudaMemcpyAsync(M.dense.p, dense.data(), 32768 * 2, cudaMemcpyHostToDevice, st));
  const uint16_t* ddense = static_cast<const uint16_t*>(M.dense.p);
  const uint64_t V1 = std::max<uint64_t>(V, 1), T1 = std::max<uint64_t>(T, 1);
  const uint64_t hw = std::max(vfk::split_hist_words(V), vfk::split_hist_words(T));
  if ((s = c.alloc(M.vkey, V1 * 2)) || (s = c.alloc(M.vown, V1 * 8)) ||
      (s = c.alloc(M.vflag, ((V1 + 31) / 32) * 4)) || (s = c.alloc(M.vperm, V1 * 4)) ||
      (s = c.alloc(M.vinv, V1 * 4)) || (s = c.alloc(M.tmp, std::max(V1, T1) * 4)) ||
      (s = c.alloc(M.tkey, T1 * 2)) || (s = c.alloc(M.tv, T1 * 16)) ||
      (s = c.alloc(M.tperm, T1 * 4)) || (s = c.alloc(M.hist, hw * 4)) ||
      (s = c.alloc(M.hbase, hw * 8)) || (s = scan_scratch(std::max<uint64_t>(hw, std::max(rows, crows)))) ||
      (s = c.alloc(M.vert, V1 * 16)) || (s = c.alloc(M.gface, T1 * 16)) ||
      (s = c.alloc(M.face, T1 * 16)) || (s = c.alloc(M.voff, (F + 1) * 8)) ||
      (s = c.alloc(M.foff, (F + 1) * 8)) || (s = c.alloc(M.acc, V1 * 16)) ||
      (s = c.alloc(M.deg, V1 * 4)) || (s = c.alloc(M.start, (V1 + 1) * 8)) ||
      (s = c.alloc(M.ent, T1 * 3 * 8)) || (s = c.alloc(M.ustart, (V1 + 1) * 8)) ||
      (s = c.alloc(M.nbr, T1 * 3 * 4)) || (s = c.alloc(M.meta, V1 * 8)) ||
      (s = scan_scratch(std::max<uint64_t>(V1, hw))))
    return s;
  sums = static_cast<unsigned long long*>(M.sums.p);
  auto vkey = static_cast<uint16_t*>(M.vkey.p);
  auto vown = static_cast<unsigned long long*>(M.vown.p);
  auto vflag = static_cast<uint32_t*>(M.vflag.p);
  auto vperm = static_cast<uint32_t*>(M.vperm.p);
  auto vinv = static_cast<uint32_t*>(M.vinv.p);
  auto tkey = static_cast<uint16_t*>(M.tkey.p);
  auto tv = static_cast<uint4*>(M.tv.p);
  auto tperm = static_cast<uint32_t*>(M.tperm.p);
  auto vert = static_cast<float4*>(M.vert.p);
  auto gface = static_cast<uint4*>(M.gface.p);
  auto voff = static_cast<unsigned long long*>(M.voff.p);
  auto foff = static_cast<unsigned long long*>(M.foff.p);
  VF_CK(cudaEventRecord(M.ev[2], st));
  VF_CK(cudaMemsetAsync(vflag, 0, ((V1 + 31) / 32) * 4, st));
  vfk::mc_vertex_emit(st, G, mask, rbase, ddense, static_cast<uint32_t*>(M.vbase.p), vkey, vown, nsm);
  vfk::mc_tri_emit(st, G, dtri, dntri, tbase, mask, static_cast<const uint32_t*>(M.vbase.p), ddense,
                   tkey, tv, vflag, err, nsm);
  auto tmp = static_cast<uint32_t*>(M.tmp.p);
  auto hist = static_cast<uint32_t*>(M.hist.p);
  auto hbase = static_cast<unsigned long long*>(M.hbase.p);
  vfk::stable_split16(st, vkey, V, F, tmp, vperm, hist, hbase, sums, tot + 2);
  vfk::stable_split16(st, tkey, T, F, tmp, tperm, hist, hbase, sums, tot + 3);
  // the grid's affine map (RegularGrid.cpp:478-480): s = size / dims, min - s
  float sc[3], c0[3];
  for (int a = 0; a < 3; ++a) {
    const float size = g->job.aabb_max[a] - g->job.aabb_min[a];
    sc[a] = size / (float)d[a];
    c0[a] = g->job.aabb_min[a] - sc[a];
  }
  vfk::mc_outputs(st, G, vperm, vown, vflag, V, sc, c0, vinv, vert, tperm, tv, T, gface, nsm);
  vfk::mc_offsets(st, vkey, vperm, V, F, voff);
  vfk::mc_offsets(st, tkey, tperm, T, F, foff);
  VF_CK(cudaEventRecord(M.ev[3], st));
  auto ustart = static_cast<unsigned long long*>(M.ustart.p);
  auto start = static_cast<unsigned long long*>(M.start.p);
  const bool smooth = (mp->nonboundary_iterations || mp->boundary_iterations) && V && T;
  if (smooth)
    VF_CK(vfk::mc_smooth_lists(st, gface, T, vert, V, static_cast<uint32_t*>(M.deg.p), start, ustart,
                               sums, static_cast<uint2*>(M.ent.p), static_cast<uint32_t*>(M.nbr.p),
                               static_cast<uint2*>(M.meta.p), err, tot + 4, nsm));
  VF_CK(cudaEventRecord(M.ev[4], st));
  if (smooth)
    VF_CK(vfk::mc_smooth_iterate(st, vert, static_cast<float4*>(M.acc.p), V,
                                 static_cast<const uint2*>(M.meta.p),
                                 static_cast<const uint32_t*>(M.nbr.p), mp->nonboundary_iterations,
                                 mp->nonboundary_weight, mp->boundary_iterations,
                                 mp->boundary_weight, nsm));
  VF_CK(cudaEventRecord(M.ev[5], st));
  vfk::mc_local_faces(st, gface, tperm, tkey, voff, T, static_cast<uint4*>(M.face.p), nsm);
  VF_CK(cudaEventRecord(M.ev[6], st));
  uint32_t herr = 0;
  unsigned long long smc[4] = {0, 0, 0, 0};  // incidences, entries, boundary vertices, their entries
  VF_CK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  if (smooth) {
    VF_CK(cudaMemcpyAsync(smc + 0, start + V, 8, cudaMemcpyDeviceToHost, st));
    VF_CK(cudaMemcpyAsync(smc + 1, ustart + V, 8, cudaMemcpyDeviceToHost, st));
    VF_CK(cudaMemcpyAsync(smc + 2, tot + 4, 16, cudaMemcpyDeviceToHost, st));
  }
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  for (int i = 0; i < 6; ++i) cudaEventElapsedTime(&M.phase_ms[i], M.ev[i], M.ev[i + 1]);
  const uint64_t cn[6] = {V, T, smc[2], smc[0], smc[1], smc[3]};
  std::memcpy(M.counters, cn, sizeof(cn));
  if (herr & 1u) return fail(VF_ERR_CUDA, "triangulate: a triangle edge has no vertex (internal check)");
  if (herr & 2u) return fail(VF_ERR_RANGE, "triangulate: a vertex has too many incident faces");
  M.V = V;
  M.T = T;
  M.ready = true;
  if (nmeshes) *nmeshes = F;
  if (nverts) *nverts = V;
  if (nfaces) *nfaces = T;
  return VF_OK;
}

vf_status vf_grid_mesh_phase_ms(const vf_grid* g, float* ms, uint32_t n) {
  if (!g || (n && !ms)) return fail(VF_ERR_INVALID, "NULL argument");
  if (!g->mesh.ready) return fail(VF_ERR_INVALID, "no meshes: call vf_grid_triangulate first");
  for (uint32_t i = 0; i < n && i < 6; ++i) ms[i] = g->mesh.phase_ms[i];
  return VF_OK;
}

vf_status vf_grid_mesh_counters(const vf_grid* g, uint64_t* out, uint32_t n) {
  if (!g || (n && !out)) return fail(VF_ERR_INVALID, "NULL argument");
  if (!g->mesh.ready) return fail(VF_ERR_INVALID, "no meshes: call vf_grid_triangulate first");
  for (uint32_t i = 0; i < n && i < 6; ++i) out[i] = g->mesh.counters[i];
  return VF_OK;
}

// CADModel::sampleCPU for the meshes M (host copy of their face offsets: fo);
// the points stay in P.out at P.offsets
static vf_status sample_meshes(vfr::Ctx& c, cudaStream_t st, SampleState& P, vfk::SampleMeshes M,
                               const std::vector<uint64_t>& fo, uint32_t S, uint64_t seed) {
  P.ready = false;
  const uint32_t F = M.F;
  std::vector<unsigned long long> cs, ce, mc(F + 1);
  std::vector<uint8_t> big(std::max<uint32_t>(F, 1));
  std::vector<uint32_t> sel;
  for (uint32_t m = 0; m < F; ++m) {
    mc[m] = cs.size();
    for (uint64_t t = fo[m]; t < fo[m + 1]; t += 1024) {
      cs.push_back(t);
      ce.push_back(std::min<uint64_t>(t + 1024, fo[m + 1]));
    }
    const uint64_t T = fo[m + 1] - fo[m];
    big[m] = S > T ? 1 : 0;
    if (!big[m] && T) sel.push_back(m);
  }
  mc[F] = cs.size();
  const uint32_t nch = (uint32_t)cs.size();
  const uint64_t nf = M.nfaces, nf1 = std::max<uint64_t>(nf, 1), F1 = std::max<uint32_t>(F, 1);
  vf_status s;
  if ((s = c.alloc(P.area, nf1 * 4)) || (s = c.alloc(P.cstart, std::max<uint32_t>(nch, 1) * 8)) ||
      (s = c.alloc(P.cend, std::max<uint32_t>(nch, 1) * 8)) ||
      (s = c.alloc(P.csum, std::max<uint32_t>(nch, 1) * 8)) ||
      (s = c.alloc(P.cmax, std::max<uint32_t>(nch, 1) * 4)) || (s = c.alloc(P.mchunk, (F1 + 1) * 8)) ||
      (s = c.alloc(P.msum, F1 * 4)) || (s = c.alloc(P.nb, F1 * 8)) || (s = c.alloc(P.big, F1)) ||
      (s = c.alloc(P.sel, F1 * 4)) || (s = c.alloc(P.chosen, ((nf1 + 31) / 32) * 4)) ||
      (s = c.alloc(P.err, 16)) || (s = c.alloc(P.cnt, nf1 * 4)) || (s = c.alloc(P.P, F1 * 8)) ||
      (s = c.alloc(P.soff, (nf1 + 1) * 8)) || (s = c.alloc(P.sums, ((nf1 + 1023) / 1024 + 2) * 8)) ||
      (s = c.alloc(P.out_off, (F1 + 1) * 8)))
    return s;
  if (nch) {
    VF_CK(cudaMemcpyAsync(P.cstart.p, cs.data(), nch * 8, cudaMemcpyHostToDevice, st));
    VF_CK(cudaMemcpyAsync(P.cend.p, ce.data(), nch * 8, cudaMemcpyHostToDevice, st));
  }
  VF_CK(cudaMemcpyAsync(P.mchunk.p, mc.data(), (F + 1) * 8, cudaMemcpyHostToDevice, st));
  VF_CK(cudaMemcpyAsync(P.big.p, big.data(), big.size(), cudaMemcpyHostToDevice, st));
  if (!sel.empty())
    VF_CK(cudaMemcpyAsync(P.sel.p, sel.data(), sel.size() * 4, cudaMemcpyHostToDevice, st));
  VF_CK(cudaMemsetAsync(P.chosen.p, 0, ((nf1 + 31) / 32) * 4, st));
  VF_CK(cudaMemsetAsync(P.err.p, 0, 4, st));
  const int nsm = c.num_sms;
  auto msum = static_cast<float*>(P.msum.p);
  auto nb = static_cast<uint64_t*>(P.nb.p);
  auto bigd = static_cast<const uint8_t*>(P.big.p);
  auto chosen = static_cast<uint32_t*>(P.chosen.p);
  auto cnt = static_cast<uint32_t*>(P.cnt.p);
  auto soff = static_cast<unsigned long long*>(P.soff.p);
  vfk::pc_areas(st, M, static_cast<float*>(P.area.p), static_cast<const unsigned long long*>(P.cstart.p),
                static_cast<const unsigned long long*>(P.cend.p), nch, static_cast<double*>(P.csum.p),
                static_cast<float*>(P.cmax.p), static_cast<const unsigned long long*>(P.mchunk.p), S, msum,
                nb, nsm);
  vfk::pc_select(st, M, static_cast<const uint32_t*>(P.sel.p), (uint32_t)sel.size(), S, seed, chosen,
                 static_cast<uint32_t*>(P.err.p));
  vfk::pc_count(st, M, static_cast<const float*>(P.area.p), msum, bigd, S, chosen, cnt,
                static_cast<unsigned long long*>(P.P.p), soff, static_cast<unsigned long long*>(P.sums.p),
                nsm);
  std::vector<unsigned long long> Pm(F1, 0);
  uint32_t err = 0;
  if (nf) VF_CK(cudaMemcpyAsync(Pm.data(), P.P.p, F * 8, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaMemcpyAsync(&err, P.err.p, 4, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  if (err) return fail(VF_ERR_RANGE, "sample: the face draws ran out before S distinct faces");
  P.offsets.assign(F + 1, 0);
  for (uint32_t m = 0; m < F; ++m) {
    const uint64_t T = fo[m + 1] - fo[m];
    const uint64_t n = !T ? 0 : (big[m] ? std::min<uint64_t>(Pm[m], S) : S);
    P.offsets[m + 1] = P.offsets[m] + n;
  }
  P.npoints = P.offsets[F];
  if ((s = c.alloc(P.out, std::max<uint64_t>(P.npoints, 1) * 16))) return s;
  VF_CK(cudaMemcpyAsync(P.out_off.p, P.offsets.data(), (F + 1) * 8, cudaMemcpyHostToDevice, st));
  vfk::pc_points(st, M, cnt, soff, nb, bigd, static_cast<const unsigned long long*>(P.out_off.p), S, seed,
                 static_cast<float4*>(P.out.p), nsm);
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  P.ready = true;
  return VF_OK;
}

vf_status vf_grid_sample_meshes(vf_grid* g, uint32_t max_samples, uint64_t seed, uint64_t* point_offsets,
                                uint64_t* npoints) {
  if (!g || !npoints) return fail(VF_ERR_INVALID, "NULL argument");
  MeshState& M = g->mesh;
  if (!M.ready) return fail(VF_ERR_INVALID, "no meshes: call vf_grid_triangulate first");
  cudaSetDevice(g->ctx->c.device);
  vfr::Ctx& c = g->ctx->c;
  SampleState& P = g->sample;
  cudaStream_t st = g->b.stream;
  const uint32_t F = (uint32_t)M.values.size();
  std::vector<uint64_t> fo(F + 1, 0);
  std::vector<uint32_t> keys(M.values.begin(), M.values.end());
  vf_status s;
  if ((s = c.alloc(P.keys, std::max<uint32_t>(F, 1) * 4))) return s;
  if (F) {
    VF_CK(cudaMemcpyAsync(fo.data(), M.foff.p, (F + 1) * 8, cudaMemcpyDeviceToHost, st));
    VF_CK(cudaMemcpyAsync(P.keys.p, keys.data(), F * 4, cudaMemcpyHostToDevice, st));
    VF_CK(cudaStreamSynchronize(st));
  }
  vfk::SampleMeshes SM{static_cast<const float4*>(M.vert.p), static_cast<const uint4*>(M.face.p),
                       static_cast<const unsigned long long*>(M.voff.p),
                       static_cast<const unsigned long long*>(M.foff.p),
                       static_cast<const uint32_t*>(P.keys.p), F, M.T};
  if (!F) {
    P.offsets.assign(1, 0);
    P.npoints = 0;
    P.ready = true;
  } else if ((s = sample_meshes(c, st, P, SM, fo, max_samples, seed))) {
    return s;
  }
  *npoints = P.npoints;
  if (point_offsets) std::memcpy(point_offsets, P.offsets.data(), P.offsets.size() * 8);
  return VF_OK;
}

vf_status vf_grid_points(vf_grid* g, float* points) {
  if (!g || !points) return fail(VF_ERR_INVALID, "NULL argument");
  SampleState& P = g->sample;
  if (!P.ready) return fail(VF_ERR_INVALID, "no points: call vf_grid_sample_meshes first");
  cudaSetDevice(g->ctx->c.device);
  if (P.npoints)
    VF_CK(cudaMemcpyAsync(points, P.out.p, P.npoints * 16, cudaMemcpyDeviceToHost, g->b.stream));
  VF_CK(cudaStreamSynchronize(g->b.stream));
  return VF_OK;
}

vf_status vf_sample_mesh(vf_ctx* ctx, const float* verts, uint32_t nverts, const uint32_t* faces,
                         uint32_t nfaces, uint32_t max_samples, uint64_t seed, float* points,
                         uint64_t* npoints) {
  if (!ctx || !npoints || (nfaces && (!verts || !faces)) || (max_samples && !points))
    return fail(VF_ERR_INVALID, "NULL argument");
  for (uint64_t i = 0; i < 3ull * nfaces; ++i)
    if (faces[i] >= nverts) return fail(VF_ERR_INVALID, "face index out of range");
  *npoints = 0;
  if (!nfaces || !max_samples) return VF_OK;
  cudaSetDevice(ctx->c.device);
  vfr::Ctx& c = ctx->c;
  SampleState P;
  std::vector<float> v4(4 * (size_t)nverts);
  std::vector<uint32_t> f4(4 * (size_t)nfaces);
  for (uint32_t i = 0; i < nverts; ++i) {
    v4[4 * (size_t)i] = verts[3 * (size_t)i];
    v4[4 * (size_t)i + 1] = verts[3 * (size_t)i + 1];
    v4[4 * (size_t)i + 2] = verts[3 * (size_t)i + 2];
    v4[4 * (size_t)i + 3] = 0.0f;
  }
  for (uint32_t i = 0; i < nfaces; ++i) {
    f4[4 * (size_t)i] = faces[3 * (size_t)i];
    f4[4 * (size_t)i + 1] = faces[3 * (size_t)i + 1];
    f4[4 * (size_t)i + 2] = faces[3 * (size_t)i + 2];
    f4[4 * (size_t)i + 3] = 0;
  }
  const unsigned long long vo[2] = {0, nverts}, fo2[2] = {0, nfaces};
  const uint32_t key = 0;
  cudaStream_t st = c.stream;
  vf_status s;
  if ((s = c.alloc(P.verts, v4.size() * 4)) || (s = c.alloc(P.faces, f4.size() * 4)) ||
      (s = c.alloc(P.voff, 16)) || (s = c.alloc(P.foff, 16)) || (s = c.alloc(P.keys, 4))) {
    P.release(c);
    return s;
  }
  cudaMemcpyAsync(P.verts.p, v4.data(), v4.size() * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(P.faces.p, f4.data(), f4.size() * 4, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(P.voff.p, vo, 16, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(P.foff.p, fo2, 16, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(P.keys.p, &key, 4, cudaMemcpyHostToDevice, st);
  vfk::SampleMeshes SM{static_cast<const float4*>(P.verts.p), static_cast<const uint4*>(P.faces.p),
                       static_cast<const unsigned long long*>(P.voff.p),
                       static_cast<const unsigned long long*>(P.foff.p),
                       static_cast<const uint32_t*>(P.keys.p), 1, nfaces};
  const std::vector<uint64_t> fo = {0, nfaces};
  s = sample_meshes(c, st, P, SM, fo, max_samples, seed);
  if (!s) {
    if (P.npoints) {
      const cudaError_t e = cudaMemcpy(points, P.out.p, P.npoints * 16, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) s = fail(VF_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    }
    *npoints = P.npoints;
  }
  P.release(c);
  return s;
}

vf_status vf_grid_meshes(vf_grid* g, uint16_t* values, uint64_t* vert_offsets,
                         uint64_t* face_offsets, float* verts, uint32_t* faces) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  MeshState& M = g->mesh;
  if (!M.ready) return fail(VF_ERR_INVALID, "no meshes: call vf_grid_triangulate first");
  cudaSetDevice(g->ctx->c.device);
  cudaStream_t st = g->b.stream;
  const size_t F = M.values.size();
  if (values) std::memcpy(values, M.values.data(), F * 2);
  if (vert_offsets) VF_CK(cudaMemcpyAsync(vert_offsets, M.voff.p, (F + 1) * 8, cudaMemcpyDeviceToHost, st));
  if (face_offsets) VF_CK(cudaMemcpyAsync(face_offsets, M.foff.p, (F + 1) * 8, cudaMemcpyDeviceToHost, st));
  if (verts && M.V) VF_CK(cudaMemcpyAsync(verts, M.vert.p, M.V * 16, cudaMemcpyDeviceToHost, st));
  if (faces && M.T) VF_CK(cudaMemcpyAsync(faces, M.face.p, M.T * 16, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  return VF_OK;
}

static vfk::ImpactGrid impact_grid(const vf_grid* g) {
  const vfr::JobPlan& p = g->b.plans[0];
  vfk::ImpactGrid G;
  G.g = static_cast<const uint16_t*>(g->b.grid0.p);
  G.X = p.X;
  G.Y = p.Y;
  G.Z = p.Z;
  G.Zp = p.Zp;
  const uint32_t d[3] = {p.X, p.Y, p.Z};
  for (int a = 0; a < 3; ++a) {
    G.amin[a] = g->job.aabb_min[a];
    G.amax[a] = g->job.aabb_max[a];
    // RegularGrid::setAABB (RegularGrid.cpp:437): _cellSize = _aabb.size() / _numDivs
    G.cell[a] = (G.amax[a] - G.amin[a]) / (float)d[a];
  }
  return G;
}

vf_status vf_ray_entry_voxels(vf_grid* g, const float* rays, uint32_t n, uint32_t* out) {
  if (!g || (n && (!rays || !out))) return fail(VF_ERR_INVALID, "NULL argument");
  if (!n) return VF_OK;
  for (uint32_t r = 0; r < n; ++r)
    if (rays[6 * r + 3] == 0.0f && rays[6 * r + 4] == 0.0f && rays[6 * r + 5] == 0.0f)
      return fail(VF_ERR_INVALID, "ray " + std::to_string(r) + " has a zero direction");
  cudaSetDevice(g->ctx->c.device);
  vfr::Ctx& c = g->ctx->c;
  ImpactState& I = g->impact;
  vf_status s;
  if ((s = c.alloc(I.rays, (size_t)n * 24)) || (s = c.alloc(I.hits, (size_t)n * 12))) return s;
  // batches of rays walk a packed occupancy bitmap (built once per call);
  // a few rays read the labels directly
  const vfr::JobPlan& p = g->b.plans[0];
  const size_t bitbytes = (size_t)p.X * p.Y * ((p.Z + 31) / 32) * 4;
  uint32_t* bits = nullptr;
  if (n >= 4096) {
    if ((s = c.alloc(I.bits, bitbytes))) return s;
    bits = static_cast<uint32_t*>(I.bits.p);
  }
  cudaStream_t st = g->b.stream;
  VF_CK(cudaMemcpyAsync(I.rays.p, rays, (size_t)n * 24, cudaMemcpyHostToDevice, st));
  vfk::ray_entry(st, impact_grid(g), static_cast<const float*>(I.rays.p), n,
                 static_cast<uint32_t*>(I.hits.p), bits, c.num_sms);
  VF_CK(cudaMemcpyAsync(out, I.hits.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  return VF_OK;
}

vf_status vf_near_seeds(vf_grid* g, const uint32_t* frags_xyzw, uint32_t nfrags,
                        uint32_t num_impacts, uint32_t num_seeds, uint32_t spreading, uint64_t seed,
                        uint32_t* out_xyzw, uint32_t* nout) {
  if (!g || !out_xyzw || !nout || (nfrags && !frags_xyzw)) return fail(VF_ERR_INVALID, "NULL argument");
  const vfr::JobPlan& p = g->b.plans[0];
  const uint32_t mind = std::min(p.X, std::min(p.Y, p.Z));
  if (num_impacts && !nfrags) return fail(VF_ERR_INVALID, "nearSeeds: impacts need at least one seed");
  if (num_impacts && (spreading < 1 || spreading > mind))
    return fail(VF_ERR_INVALID, "nearSeeds: spreading must be in [1, min(dims)]");
  if (num_seeds > VF_MAX_SEEDS) return fail(VF_ERR_INVALID, "nearSeeds: too many seeds");
  if (num_impacts > (1u << 20)) return fail(VF_ERR_INVALID, "nearSeeds: too many impacts");
  for (uint32_t i = 0; i < nfrags; ++i)
    if (frags_xyzw[4 * i] >= p.X + 1 || frags_xyzw[4 * i + 1] >= p.Y + 1 || frags_xyzw[4 * i + 2] >= p.Z + 1)
      return fail(VF_ERR_INVALID, "nearSeeds: seed outside the grid");
  std::memcpy(out_xyzw, frags_xyzw, (size_t)nfrags * 16);
  *nout = nfrags;
  if (!num_impacts || !num_seeds) return VF_OK;
  cudaSetDevice(g->ctx->c.device);
  vfr::Ctx& c = g->ctx->c;
  ImpactState& I = g->impact;
  vf_status s;
  if ((s = c.alloc(I.frags, (size_t)nfrags * 16)) || (s = c.alloc(I.out, (size_t)num_seeds * 16)) ||
      (s = c.alloc(I.status, 16)))
    return s;
  cudaStream_t st = g->b.stream;
  VF_CK(cudaMemcpyAsync(I.frags.p, frags_xyzw, (size_t)nfrags * 16, cudaMemcpyHostToDevice, st));
  const uint32_t label0 = frags_xyzw[4 * (nfrags - 1) + 3];
  vfk::near_seeds(st, impact_grid(g), static_cast<const uint32_t*>(I.frags.p), nfrags, num_impacts,
                  num_seeds, spreading, seed, label0, static_cast<uint32_t*>(I.out.p),
                  static_cast<uint32_t*>(I.status.p));
  uint32_t status[2] = {0, 0};
  VF_CK(cudaMemcpyAsync(status, I.status.p, 8, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaStreamSynchronize(st));
  VF_CK(cudaGetLastError());
  if (status[1]) return fail(VF_ERR_SEED_SEARCH, "nearSeeds: an impact found too few surface voxels");
  if (status[0] > num_seeds) return fail(VF_ERR_CUDA, "nearSeeds: count out of range");
  VF_CK(cudaMemcpy(out_xyzw + 4 * (size_t)nfrags, I.out.p, (size_t)status[0] * 16, cudaMemcpyDeviceToHost));
  *nout = nfrags + status[0];
  return VF_OK;
}

vf_status vf_voxelize(vf_grid* g, const float* verts, uint32_t nverts, const uint32_t* faces,
                      uint32_t nfaces) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  if (nfaces && (!verts || !faces || !nverts)) return fail(VF_ERR_INVALID, "mesh pointers missing");
  for (uint64_t i = 0; i < 3ull * nfaces; ++i)
    if (faces[i] >= nverts) return fail(VF_ERR_INVALID, "face index out of range");
  g->job.verts = verts;
  g->job.nverts = nverts;
  g->job.faces = faces;
  g->job.nfaces = nfaces;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_VOX);
  g->job.verts = nullptr;
  g->job.faces = nullptr;
  g->job.nverts = g->job.nfaces = 0;
  return s;
}

static vf_status seeds_out(vf_grid* g, uint32_t* out, uint32_t* nout) {
  vfr::Batch& B = g->b;
  const uint32_t n = B.h_state[0].nseeds;
  if (out && n)
    VF_CK(cudaMemcpy(out, static_cast<uint32_t*>(B.seeds.p) + B.plans[0].o_seeds,
                     sizeof(uint32_t) * 4 * n, cudaMemcpyDeviceToHost));
  if (nout) *nout = n;
  return VF_OK;
}

vf_status vf_sample_seeds(vf_grid* g, uint32_t n, uint64_t seed, int location, uint32_t* out) {
  if (!g || (n && !out)) return fail(VF_ERR_INVALID, "NULL argument");
  if (n > 254) return fail(VF_ERR_RANGE, "at most 254 seeds (8-bit fragment ids 2..255)");
  if (location < VF_INNER || location > VF_BOTH) return fail(VF_ERR_INVALID, "location out of range");
  vf_params saved = g->job.params;
  g->job.params.num_seeds = (int32_t)n;
  g->job.params.num_extra_seeds = 0;
  g->job.params.num_impacts = 0;
  g->job.params.seed = seed;
  g->job.params.seed_location = location;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_SEED);
  g->job.params = saved;
  if (s) return s;
  return seeds_out(g, out, nullptr);
}

vf_status vf_merge_seeds(const uint32_t* frags, uint32_t nfrags, uint32_t* seeds, uint32_t nseeds,
                         int dfunc) {
  // Seeder::mergeSeeds (Seeder.cpp:115-152) -- host bookkeeping, as in the reference
  if (nseeds == 0) return VF_OK;
  if (!frags || !seeds || nfrags == 0) return fail(VF_ERR_INVALID, "NULL or empty argument");
  if (dfunc < 0 || dfunc > 2) return fail(VF_ERR_INVALID, "distance out of range");
  uint32_t idf[256] = {0};
  for (uint32_t k = 0; k < nseeds; ++k) {
    float best = FLT_MAX;
    int nearest = -1;
    for (uint32_t i = 0; i < nfrags; ++i) {
      const float dx = (float)seeds[4 * k] - (float)frags[4 * i];
      const float dy = (float)seeds[4 * k + 1] - (float)frags[4 * i + 1];
      const float dz = (float)seeds[4 * k + 2] - (float)frags[4 * i + 2];
      float d;
      if (dfunc == VF_EUCLIDEAN) d = std::sqrt(dx * dx + dy * dy + dz * dz);
      else if (dfunc == VF_MANHATTAN) d = std::fabs(dx) + std::fabs(dy) + std::fabs(dz);
      else d = std::max(std::fabs(dx), std::max(std::fabs(dy), std::fabs(dz)));
      if (d < best) { best = d; nearest = (int)i; }
    }
    const uint32_t w = frags[4 * nearest + 3];
    if (w > 255) return fail(VF_ERR_RANGE, "fragment label above 255");
    const uint32_t pre = ++idf[w];
    if (pre > 127) return fail(VF_ERR_RANGE, "sub-seed prefix above 127");
    seeds[4 * k + 3] = w | (pre << 8);
  }
  return VF_OK;
}

vf_status vf_fracture_seeds(vf_grid* g, const vf_params* p, uint32_t* out, uint32_t* nout) {
  if (!g || !p) return fail(VF_ERR_INVALID, "NULL argument");
  vf_params saved = g->job.params;
  g->job.params = *p;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_SEED);
  g->job.params = saved;
  if (s) return s;
  return seeds_out(g, out, nout);
}

vf_status vf_fracture(vf_grid* g, int algorithm, int distance, const uint32_t* seeds,
                      uint32_t nseeds) {
  if (!g || (nseeds && !seeds)) return fail(VF_ERR_INVALID, "NULL argument");
  if (nseeds > VF_MAX_SEEDS) return fail(VF_ERR_RANGE, "at most 4095 seeds");
  vf_params saved = g->job.params;
  g->job.params.algorithm = algorithm;
  g->job.params.distance = distance;
  g->job.params.num_seeds = 0;
  g->job.params.num_extra_seeds = 0;
  g->job.params.noise_amplitude = 0.0f;
  g->job.params.erode = 0;
  g->b.given.assign(1, {seeds, nseeds});
  vf_status s = nseeds ? grid_run(g, vfr::ST_SEED | vfr::ST_FRACTURE) : VF_OK;
  g->b.given.clear();
  g->job.params = saved;
  return s;
}

vf_status vf_fracture_plain(vf_grid* g, int distance, const uint32_t* seeds, uint32_t nseeds,
                            uint32_t* waves_out) {
  if (!g || (nseeds && !seeds)) return fail(VF_ERR_INVALID, "NULL argument");
  if (nseeds > VF_MAX_SEEDS) return fail(VF_ERR_RANGE, "at most 4095 seeds");
  // a plain job on the grid's occupancy: the plain runner voxelizes, so run
  // it on a copy of the job whose mesh is the grid itself: seed + flood
  // stages of the plain path over buffer 0
  cudaSetDevice(g->ctx->c.device);
  vf_params saved = g->job.params;
  g->job.params.algorithm = VF_FLOOD;
  g->job.params.distance = distance;
  g->job.params.num_seeds = 0;
  g->job.params.num_extra_seeds = 0;
  g->job.params.noise_amplitude = 0.0f;
  g->job.params.erode = 0;
  g->b.given.assign(1, {seeds, nseeds});
  vfr::Batch& B = g->b;
  const vf_job* jp = &g->job;
  B.stages = vfr::ST_SEED | vfr::ST_FRACTURE;
  vf_status s = B.plan(&jp, 1);
  vf_job_result r;
  if (!s) s = B.enqueue_plain_and_wait(&r, /*skip_vox=*/true);
  if (!s && waves_out) *waves_out = r.flood_passes;
  g->b.given.clear();
  g->job.params = saved;
  return s;
}

vf_status vf_perturb(vf_grid* g, float amplitude, uint32_t period, uint64_t seed) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  if (!(amplitude >= 0.0f) || amplitude > 64.0f || period == 0)
    return fail(VF_ERR_INVALID, "amplitude must be in [0, 64] and period >= 1");
  if (amplitude == 0.0f) return VF_OK;
  vf_params saved = g->job.params;
  g->job.params.noise_amplitude = amplitude;
  g->job.params.noise_period = period;
  g->job.params.seed = seed;
  g->job.params.erode = 0;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_PERTURB);
  g->job.params = saved;
  return s;
}

vf_status vf_detect_boundaries(vf_grid* g, int boundary_size) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  if (boundary_size < 0 || boundary_size > 3) return fail(VF_ERR_INVALID, "boundary_size must be in [0, 3]");
  vf_params saved = g->job.params;
  g->job.params.boundary_size = boundary_size;
  g->job.params.erode = 0;
  g->job.params.noise_amplitude = 0.0f;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_DETECT);
  g->job.params = saved;
  return s;
}

vf_status vf_erode(vf_grid* g, int type, uint32_t size, uint32_t iterations, float probability,
                   float threshold, uint64_t seed) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  vf_params saved = g->job.params;
  g->job.params.erode = 1;
  g->job.params.erosion_type = type;
  g->job.params.erosion_size = (int32_t)size;
  g->job.params.erosion_iterations = (int32_t)iterations;
  g->job.params.erosion_probability = probability;
  g->job.params.erosion_threshold = threshold;
  g->job.params.seed = seed;
  g->job.params.noise_amplitude = 0.0f;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_ERODE);
  g->job.params = saved;
  return s;
}

vf_status vf_remove_isolated(vf_grid* g) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  vf_params saved = g->job.params;
  g->job.params.erode = 1;
  g->job.params.erosion_iterations = 0;
  g->job.params.noise_amplitude = 0.0f;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_ERODE);
  g->job.params = saved;
  return s;
}

vf_status vf_undo_mask(vf_grid* g) {
  if (!g) return fail(VF_ERR_INVALID, "grid is NULL");
  cudaSetDevice(g->ctx->c.device);
  vfr::Batch& B = g->b;
  const vf_job* jp = &g->job;
  B.stages = 0;
  vf_status s = B.plan(&jp, 1);
  if (s) return s;
  const JobDesc* T = reinterpret_cast<const JobDesc*>(B.h_tables);
  VF_CK(cudaMemcpyAsync(B.tables.p, B.h_tables, sizeof(JobDesc), cudaMemcpyHostToDevice, B.stream));
  vfk::plain_undo_mask(B.stream, B.dtable(0), T[0]);
  VF_CK(cudaStreamSynchronize(B.stream));
  VF_CK(cudaGetLastError());
  return VF_OK;
}

vf_status vf_count_values(vf_grid* g, uint32_t* counts, uint32_t ncounts, uint64_t* occupied) {
  if (!g || (ncounts && !counts)) return fail(VF_ERR_INVALID, "NULL argument");
  g->job.ncounts = ncounts;
  g->job.out_counts = counts;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_COUNT | vfr::ST_DOWNLOAD);
  g->job.ncounts = 0;
  g->job.out_counts = nullptr;
  if (occupied) *occupied = g->b.h_state[0].occupied;
  return s;
}

vf_status vf_fracture_model(vf_grid* g, const vf_params* p, uint32_t* seeds_out_, uint32_t* nseeds_out) {
  if (!g || !p) return fail(VF_ERR_INVALID, "NULL argument");
  vf_params saved = g->job.params;
  g->job.params = *p;
  g->b.given.clear();
  vf_status s = grid_run(g, vfr::ST_SEED | vfr::ST_FRACTURE | vfr::ST_PERTURB | vfr::ST_ERODE |
                                vfr::ST_DETECT);
  g->job.params = saved;
  vf_status s2 = seeds_out(g, seeds_out_, nseeds_out);
  return s ? s : s2;
}

// ---- whole jobs -----------------------------------------------------------
size_t vf_job_footprint(const vf_job* job) { return job ? vfr::job_footprint(*job) : 0; }

vf_status vf_batch_run(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs, vf_job_result* results) {
  if (!ctx || (njobs && !jobs)) return fail(VF_ERR_INVALID, "NULL argument");
  if (njobs == 0) return VF_OK;
  cudaSetDevice(ctx->c.device);
  vfr::Batch& B = ctx->c.batch;
  ctx->c.resident = false;
  std::vector<const vf_job*> ptrs(njobs);
  for (uint32_t i = 0; i < njobs; ++i) ptrs[i] = jobs + i;
  B.stages = vfr::ST_ALL;
  B.given.clear();
  vf_status s = B.plan(ptrs.data(), njobs);
  if (s) return s;
  s = B.enqueue_batched();
  if (s) return s;
  return B.finish(results);
}

vf_status vf_batch_prepare(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs) {
  if (!ctx || (njobs && !jobs)) return fail(VF_ERR_INVALID, "NULL argument");
  cudaSetDevice(ctx->c.device);
  vfr::Batch& B = ctx->c.batch;
  ctx->c.resident = false;
  std::vector<const vf_job*> ptrs(njobs);
  for (uint32_t i = 0; i < njobs; ++i) ptrs[i] = jobs + i;
  B.stages = vfr::ST_ALL;
  B.given.clear();
  vf_status s = B.plan(ptrs.data(), njobs);
  if (s) return s;
  s = B.upload_inputs();
  if (s) return s;
  VF_CK(cudaStreamSynchronize(B.stream));
  ctx->c.resident = true;
  return VF_OK;
}

vf_status vf_batch_execute(vf_ctx* ctx, int download, vf_job_result* results) {
  if (!ctx) return fail(VF_ERR_INVALID, "ctx is NULL");
  if (!ctx->c.resident) return fail(VF_ERR_INVALID, "no prepared batch (call vf_batch_prepare)");
  cudaSetDevice(ctx->c.device);
  vfr::Batch& B = ctx->c.batch;
  vf_status s = B.execute_resident(download != 0);
  if (s) return s;
  return B.finish(results);
}

// ---- tuning ------------------------------------------------------------------
static vf_status set_tuning(vfr::Ctx& c, const int32_t* v, uint32_t n) {
  vfr::Tuning t = c.tune;
  if (n > 0) t.parity_grid = v[0];
  if (n > 1) t.shell_grid = v[1];
  if (n > 2) t.flood_sweeps = v[2];
  if (n > 3) t.flood_ctas = v[3];
  if (t.parity_grid < 1 || t.parity_grid > 64 || t.shell_grid < 1 || t.shell_grid > 64 ||
      t.flood_sweeps < 1 || t.flood_sweeps > 96 || t.flood_ctas < 0 || t.flood_ctas > 8)
    return fail(VF_ERR_RANGE, "tuning: grids in [1, 64] CTAs/SM, sweeps in [1, 96], flood CTAs/SM in [0, 8]");
  c.tune = t;
  c.batch.drop_graphs();  // captured chains hold the old launch settings
  return VF_OK;
}

vf_status vf_ctx_set_tuning(vf_ctx* ctx, const int32_t* values, uint32_t n) {
  if (!ctx || (n && !values)) return fail(VF_ERR_INVALID, "NULL argument");
  return set_tuning(ctx->c, values, n);
}

vf_status vf_ctx_set_flood_wait_limit(vf_ctx* ctx, uint32_t spins) {
  if (!ctx) return fail(VF_ERR_INVALID, "ctx is NULL");
  ctx->c.tune.flood_wait_spins = spins;
  ctx->c.batch.drop_graphs();  // captured chains hold the old limit
  return VF_OK;
}

vf_status vf_ctx_get_tuning(vf_ctx* ctx, int32_t* values, uint32_t n) {
  if (!ctx || (n && !values)) return fail(VF_ERR_INVALID, "NULL argument");
  const int32_t v[4] = {ctx->c.tune.parity_grid, ctx->c.tune.shell_grid, ctx->c.tune.flood_sweeps,
                        ctx->c.tune.flood_ctas};
  for (uint32_t i = 0; i < n; ++i) values[i] = i < 4 ? v[i] : 0;
  return VF_OK;
}

vf_status vf_autotune(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs, int32_t* chosen, uint32_t n) {
  if (!ctx || !jobs || !njobs || (n && !chosen)) return fail(VF_ERR_INVALID, "NULL argument or no jobs");
  vf_status s = vf_batch_prepare(ctx, jobs, njobs);
  if (s) return s;
  vfr::Ctx& c = ctx->c;
  vfr::Batch& B = c.batch;
  // one direct run of the stage chain; returns the device ms of stage `stage`
  auto run = [&](int stage, float* ms) -> vf_status {
    vf_status r = B.enqueue_batched(false, false);
    if (!r) r = B.finish(nullptr);
    if (r) return r;
    *ms = c.last_stage_ms[stage];
    return VF_OK;
  };
  float warm = 0.f;
  if ((s = run(0, &warm))) return s;
  struct Knob { int index, stage; std::vector<int32_t> cand; };
  const Knob knobs[] = {{0, 2, {4, 8, 16, 32}},      // parity grid   (stage: parity)
                        {1, 3, {6, 12, 24}},         // shell grid    (stage: shell)
                        {2, 6, {8, 16, 32, 96}},     // sweeps/visit  (stage: fracture)
                        {3, 6, {2, 3, 0}}};          // flood CTAs/SM (stage: fracture)
  for (const Knob& k : knobs) {
    int32_t best_v = 0;
    float best = 3.0e38f;
    for (int32_t v : k.cand) {
      int32_t cur[4];
      vf_ctx_get_tuning(ctx, cur, 4);
      cur[k.index] = v;
      if ((s = set_tuning(c, cur, 4))) return s;
      float t = 3.0e38f;
      for (int rep = 0; rep < 2; ++rep) {
        float ms = 0.f;
        if ((s = run(k.stage, &ms))) return s;
        t = std::min(t, ms);
      }
      if (t < best) { best = t; best_v = v; }
    }
    int32_t cur[4];
    vf_ctx_get_tuning(ctx, cur, 4);
    cur[k.index] = best_v;
    if ((s = set_tuning(c, cur, 4))) return s;
  }
  return chosen ? vf_ctx_get_tuning(ctx, chosen, n) : VF_OK;
}

vf_status vf_ctx_flood_stats(vf_ctx* ctx, uint64_t* passes, uint64_t* sweeps, uint64_t* maxit_hits) {
  if (!ctx) return fail(VF_ERR_INVALID, "ctx is NULL");
  if (passes) *passes = ctx->c.last_flood_passes;
  if (sweeps) *sweeps = ctx->c.last_flood_sweeps;
  if (maxit_hits) *maxit_hits = ctx->c.last_flood_maxit;
  return VF_OK;
}

vf_status vf_ctx_flood_pass_sizes(vf_ctx* ctx, uint32_t* out, uint32_t n) {
  if (!ctx || (n && !out)) return fail(VF_ERR_INVALID, "NULL argument");
  const uint64_t passes = ctx->c.last_flood_passes;
  for (uint32_t i = 0; i < n; ++i) out[i] = (i < 256 && i < passes) ? ctx->c.last_pass_sizes[i] : 0u;
  return VF_OK;
}

vf_status vf_ctx_last_graph(vf_ctx* ctx, int* replayed) {
  if (!ctx || !replayed) return fail(VF_ERR_INVALID, "NULL argument");
  *replayed = ctx->c.batch.last_run_graph ? 1 : 0;
  return VF_OK;
}

vf_status vf_ctx_flood_counters(vf_ctx* ctx, uint64_t* out, uint32_t n) {
  if (!ctx || (n && !out)) return fail(VF_ERR_INVALID, "NULL argument");
  for (uint32_t i = 0; i < n && i < VF_FLOOD_NCOUNTERS; ++i) out[i] = ctx->c.last_flood_counters[i];
  for (uint32_t i = VF_FLOOD_NCOUNTERS; i < n; ++i) out[i] = 0;
  return VF_OK;
}

vf_status vf_ctx_stage_ms(vf_ctx* ctx, float* ms, uint32_t n) {
  if (!ctx || (n && !ms)) return fail(VF_ERR_INVALID, "NULL argument");
  for (uint32_t i = 0; i < n && i < 11; ++i) ms[i] = ctx->c.last_stage_ms[i];
  return VF_OK;
}

vf_status vf_plain_run(vf_ctx* ctx, const vf_job* jobs, uint32_t njobs, vf_job_result* results) {
  if (!ctx || (njobs && !jobs)) return fail(VF_ERR_INVALID, "NULL argument");
  cudaSetDevice(ctx->c.device);
  vfr::Batch& B = ctx->c.batch;
  ctx->c.resident = false;
  vf_status first = VF_OK;
  uint64_t launches = 0;
  for (uint32_t i = 0; i < njobs; ++i) {
    const vf_job* jp = jobs + i;
    B.stages = vfr::ST_ALL;
    B.given.clear();
    vf_status s = B.plan(&jp, 1);
    if (!s) s = B.enqueue_plain_and_wait(results ? results + i : nullptr, false);
    launches += B.launches;
    if (s && results) results[i].status = s;
    if (s && !first) first = s;
  }
  ctx->c.last_launches = launches;
  return first;
}

// ---- events / stats ---------------------------------------------------------
vf_status vf_ctx_event_record(vf_ctx* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 16) return fail(VF_ERR_INVALID, "bad slot");
  VF_CK(cudaEventRecord(ctx->c.ev[slot], ctx->c.stream));
  return VF_OK;
}
vf_status vf_ctx_event_elapsed(vf_ctx* ctx, int a, int b, float* ms) {
  if (!ctx || !ms || a < 0 || b < 0 || a >= 16 || b >= 16) return fail(VF_ERR_INVALID, "bad slot");
  VF_CK(cudaEventSynchronize(ctx->c.ev[b]));
  VF_CK(cudaEventElapsedTime(ms, ctx->c.ev[a], ctx->c.ev[b]));
  return VF_OK;
}
vf_status vf_ctx_last_stats(vf_ctx* ctx, uint64_t* launches, float* flood_ms, uint64_t* flood_bytes,
                            uint64_t* flood_visits) {
  if (!ctx) return fail(VF_ERR_INVALID, "ctx is NULL");
  if (launches) *launches = ctx->c.last_launches;
  if (flood_ms) *flood_ms = ctx->c.last_flood_ms;
  // algorithmic bytes of a brick visit: every voxel's label read and written
  if (flood_bytes)  // visits that staged the brick (4 B per voxel, label read + write)
    *flood_bytes = (ctx->c.last_flood_visits - ctx->c.last_flood_counters[16]) * (uint64_t)VF_BRICK_VOXELS * 4u;
  if (flood_visits) *flood_visits = ctx->c.last_flood_visits;
  return VF_OK;
}

}  // extern "C"

// ---- server -------------------------------------------------------------------
struct vf_server {
  vf_ctx* ctx = nullptr;
  size_t budget = 0;
  uint32_t max_inflight = 3, max_batch = 128;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv, cv_done;
  struct Pending {
    vf_job job;
    uint64_t ticket;
    double submit_ms;
    size_t footprint;
  };
  struct Slot {
    vfr::Batch b;
    bool busy = false;
    std::vector<Pending> jobs;
    std::vector<vf_job> job_copies;
    size_t footprint = 0;
  };
  std::deque<Pending> pending;
  std::deque<vf_job_result> done;
  std::vector<Slot> slots;
  size_t in_flight_bytes = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  vf_status fatal = VF_OK;
  std::chrono::steady_clock::time_point t0;
  double now_ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  void loop();
};

void vf_server::loop() {
  cudaSetDevice(ctx->c.device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    bool progressed = false;
    // completions
    for (Slot& s : slots) {
      if (!s.busy) continue;
      if (cudaEventQuery(s.b.ev_done) == cudaErrorNotReady) continue;
      lk.unlock();
      std::vector<vf_job_result> res(s.jobs.size());
      vf_status st = s.b.finish(res.data());
      const double t = now_ms();
      lk.lock();
      for (size_t i = 0; i < s.jobs.size(); ++i) {
        if (st && !res[i].status) res[i].status = st == VF_ERR_CUDA ? st : res[i].status;
        res[i].submit_ms = s.jobs[i].submit_ms;
        res[i].done_ms = t;
        res[i].user_tag = s.jobs[i].job.user_tag;
        done.push_back(res[i]);
      }
      in_flight_bytes -= s.footprint;
      s.busy = false;
      s.jobs.clear();
      progressed = true;
    }
    if (!done.empty()) cv_done.notify_all();
    // admission: FIFO jobs that fit the free budget go to a free slot
    for (Slot& s : slots) {
      if (s.busy || pending.empty()) continue;
      std::vector<Pending> take;
      size_t fp = 0;
      while (!pending.empty() && take.size() < max_batch &&
             (take.empty() ? in_flight_bytes + pending.front().footprint <= budget || in_flight_bytes == 0
                           : in_flight_bytes + fp + pending.front().footprint <= budget)) {
        fp += pending.front().footprint;
        take.push_back(pending.front());
        pending.pop_front();
      }
      if (take.empty()) break;
      in_flight_bytes += fp;
      s.footprint = fp;
      s.jobs = take;
      s.busy = true;
      lk.unlock();
      s.job_copies.resize(take.size());
      std::vector<const vf_job*> ptrs(take.size());
      for (size_t i = 0; i < take.size(); ++i) {
        s.job_copies[i] = take[i].job;
        ptrs[i] = &s.job_copies[i];
      }
      s.b.stages = vfr::ST_ALL;
      s.b.given.clear();
      vf_status st = s.b.plan(ptrs.data(), (uint32_t)ptrs.size());
      if (!st) st = s.b.enqueue_batched();
      lk.lock();
      if (st) {
        const double t = now_ms();
        for (const Pending& p : take) {
          vf_job_result r;
          std::memset(&r, 0, sizeof(r));
          r.status = st;
          r.submit_ms = p.submit_ms;
          r.done_ms = t;
          r.user_tag = p.job.user_tag;
          done.push_back(r);
        }
        in_flight_bytes -= fp;
        s.busy = false;
        s.jobs.clear();
        cv_done.notify_all();
      }
      progressed = true;
    }
    bool any_busy = false;
    for (Slot& s : slots) any_busy |= s.busy;
    if (stop && !any_busy && pending.empty()) break;
    if (!progressed) {
      if (any_busy) cv.wait_for(lk, std::chrono::microseconds(50));
      else cv.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

extern "C" {

vf_status vf_server_create(vf_ctx* ctx, size_t hbm_budget, uint32_t max_inflight,
                           uint32_t max_batch_jobs, vf_server** out) {
  if (!ctx || !out) return fail(VF_ERR_INVALID, "NULL argument");
  vf_server* s = new vf_server();
  s->ctx = ctx;
  s->budget = hbm_budget ? hbm_budget : ctx->c.budget / 2;
  s->max_inflight = std::max(1u, std::min(max_inflight ? max_inflight : 3u, 8u));
  s->max_batch = std::max(1u, max_batch_jobs ? max_batch_jobs : 128u);
  s->slots.resize(s->max_inflight);
  for (auto& sl : s->slots) {
    vf_status st = sl.b.init(&ctx->c, true);
    if (st) {
      for (auto& x : s->slots) x.b.release();
      delete s;
      return st;
    }
  }
  s->t0 = std::chrono::steady_clock::now();
  s->th = std::thread([s] { s->loop(); });
  *out = s;
  return VF_OK;
}

vf_status vf_server_submit(vf_server* s, const vf_job* job, uint64_t* ticket) {
  if (!s || !job) return fail(VF_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->pending.size() > 1000000) return fail(VF_ERR_BUSY, "server queue full");
  vf_server::Pending p;
  p.job = *job;
  p.ticket = s->next_ticket++;
  p.submit_ms = s->now_ms();
  p.footprint = vfr::job_footprint(*job);
  s->pending.push_back(p);
  if (ticket) *ticket = p.ticket;
  s->cv.notify_all();
  return VF_OK;
}

vf_status vf_server_poll(vf_server* s, vf_job_result* out, uint32_t max, uint32_t* n, int wait_ms) {
  if (!s || !n || (max && !out)) return fail(VF_ERR_INVALID, "NULL argument");
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && wait_ms > 0)
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [s] { return !s->done.empty(); });
  uint32_t k = 0;
  while (k < max && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *n = k;
  return VF_OK;
}

// ---- pipelined batches ---------------------------------------------------------
struct vf_pipeline {
  vf_ctx* ctx = nullptr;
  std::vector<vfr::Batch> slots;        // fixed size: batches keep raw device pointers
  std::vector<std::vector<vf_job>> jobs;  // the submitted jobs of each slot
  std::deque<int> order;                // slots in flight, oldest first
};

vf_status vf_pipeline_create(vf_ctx* ctx, uint32_t depth, vf_pipeline** out) {
  if (!ctx || !out) return fail(VF_ERR_INVALID, "NULL argument");
  if (depth < 1 || depth > 4) return fail(VF_ERR_RANGE, "pipeline depth must be in [1, 4]");
  cudaSetDevice(ctx->c.device);
  vf_pipeline* p = new vf_pipeline();
  p->ctx = ctx;
  p->slots.resize(depth);
  p->jobs.resize(depth);
  for (auto& b : p->slots) {
    vf_status st = b.init(&ctx->c, true);
    if (st) {
      for (auto& x : p->slots) x.release();
      delete p;
      return st;
    }
    b.dma_download = true;
  }
  *out = p;
  return VF_OK;
}

vf_status vf_pipeline_submit(vf_pipeline* p, const vf_job* jobs, uint32_t njobs) {
  if (!p || (njobs && !jobs)) return fail(VF_ERR_INVALID, "NULL argument");
  if (njobs == 0) return fail(VF_ERR_INVALID, "empty batch");
  if (p->order.size() >= p->slots.size())
    return fail(VF_ERR_BUSY, "pipeline full: collect a batch first");
  cudaSetDevice(p->ctx->c.device);
  int slot = 0;
  while (std::find(p->order.begin(), p->order.end(), slot) != p->order.end()) ++slot;
  vfr::Batch& B = p->slots[slot];
  p->jobs[slot].assign(jobs, jobs + njobs);
  std::vector<const vf_job*> ptrs(njobs);
  for (uint32_t i = 0; i < njobs; ++i) ptrs[i] = &p->jobs[slot][i];
  B.stages = vfr::ST_ALL;
  B.given.clear();
  vf_status s = B.plan(ptrs.data(), njobs);
  if (!s) s = B.enqueue_batched();
  if (s) {
    // nothing of a failed enqueue is left running: wait for what was issued
    cudaStreamSynchronize(B.stream);
    return s;
  }
  p->order.push_back(slot);
  return VF_OK;
}

vf_status vf_pipeline_collect(vf_pipeline* p, vf_job_result* results, uint32_t max,
                              uint32_t* njobs) {
  if (!p || !njobs) return fail(VF_ERR_INVALID, "NULL argument");
  if (p->order.empty()) return fail(VF_ERR_INVALID, "no batch in flight");
  const int slot = p->order.front();
  const uint32_t n = (uint32_t)p->jobs[slot].size();
  if (max < n || (n && !results)) return fail(VF_ERR_INVALID, "results array shorter than the batch");
  cudaSetDevice(p->ctx->c.device);
  p->order.pop_front();
  *njobs = n;
  return p->slots[slot].finish(results);
}

vf_status vf_pipeline_destroy(vf_pipeline* p) {
  if (!p) return VF_OK;
  cudaSetDevice(p->ctx->c.device);
  for (int slot : p->order) cudaStreamSynchronize(p->slots[slot].stream);
  for (auto& b : p->slots) b.release();
  delete p;
  return VF_OK;
}

vf_status vf_server_destroy(vf_server* s) {
  if (!s) return VF_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  for (auto& sl : s->slots) sl.b.release();
  delete s;
  return VF_OK;
}

}  // extern "C"
