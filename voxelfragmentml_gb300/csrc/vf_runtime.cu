// vf_runtime.cu -- batch planning and stage sequencing (host side).
//
// The order of stages per job is CADScene::fractureModel's
// (CADScene.cpp:624-691) after RegularGrid::fill (RegularGrid.cpp:173-212):
//   voxelize -> seeds -> Flood|Naive fracture -> [perturb] ->
//   erode (detectBoundaries + erodeGrid per iteration, removeIsolated) |
//   detectBoundaries -> countValues.
// The batched path runs each stage once over every job of the batch; the
// plain path runs one job at a time with per-voxel kernels and a per-wave
// flood loop (the reference's execution shape).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <functional>

#include "vf_runtime.h"

namespace vfr {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }
vf_status fail(vf_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

#define VF_CK(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail(VF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

enum {
  T_VOX = 0, T_SEED, T_FLOOD, T_NAIVE, T_PERT, T_DET1, T_DET3, T_ISO, T_CNT, T_FIXED
};
static inline uint32_t t_edet(uint32_t i) { return T_FIXED + 2 * i; }
static inline uint32_t t_ero(uint32_t i) { return T_FIXED + 2 * i + 1; }

static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// A buffer that must grow is freed and allocated again with headroom: the
// factor `grow` set by the caller (Batch::plan), else 1/8 more.  Where the
// budget or the device cannot hold that, the exact size is tried.
vf_status Ctx::alloc(DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return VF_OK;
  if (dry) {
    dry_need += bytes;
    dry_freed += b.cap;
    return VF_OK;
  }
  free_buf(b);
  const size_t grown = grow > 0.0 ? (size_t)((double)bytes * grow) : bytes + bytes / 8;
  const size_t tries[2] = {align_up(grown, 1 << 20), align_up(bytes, 1 << 20)};
  std::string why;
  for (size_t want : tries) {
    if (budget && in_use + want > budget) {
      why = "device budget exceeded: need " + std::to_string(want) + " more bytes, " +
            std::to_string(budget - in_use) + " left";
      continue;
    }
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();  // the failed allocation leaves no sticky error
      b.p = nullptr;
      why = std::string("cudaMalloc: ") + cudaGetErrorString(e);
      continue;
    }
    b.cap = want;
    in_use += want;
    return VF_OK;
  }
  return fail(VF_ERR_OOM, why);
}
void Ctx::free_buf(DevBuf& b) {
  if (b.p) {
    cudaFree(b.p);
    in_use -= b.cap;
  }
  b.p = nullptr;
  b.cap = 0;
}

vf_status Batch::init(Ctx* c, bool own) {
  ctx = c;
  own_stream = own;
  if (own) VF_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  else stream = c->stream;
  VF_CK(cudaEventCreate(&ev_flood0));
  VF_CK(cudaEventCreate(&ev_flood1));
  VF_CK(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
  for (int i = 0; i < NSTAGE_EV; ++i) VF_CK(cudaEventCreate(&ev_stage[i]));
  VF_CK(cudaMallocHost(&h_scal, 512 * sizeof(uint32_t)));
  return VF_OK;
}

// events for timing and completion: inside a stream capture they must be
// recorded as external event nodes so that the host can wait on them and
// time them when the graph runs
cudaError_t Batch::record_event(cudaEvent_t e, cudaStream_t st) {
  return capturing ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal) : cudaEventRecord(e, st);
}

void Batch::drop_graphs() {
  for (int i = 0; i < 2; ++i) {
    if (gexec[i]) cudaGraphExecDestroy(gexec[i]);
    gexec[i] = nullptr;
    glaunches[i] = 0;
  }
}

vf_status Batch::execute_resident(bool download) {
  bool host_steps = false;
  for (const JobPlan& p : plans) host_steps |= p.prefix_possible;
  last_run_graph = false;
  if (!graphs_ok || host_steps) return enqueue_batched(false, download);
  const int gi = download ? 1 : 0;
  if (!gexec[gi]) {
    vfk::flood_prepare(ctx->num_sms);  // function attributes outside the capture
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      graphs_ok = false;
      return enqueue_batched(false, download);
    }
    capturing = true;
    vf_status s = enqueue_batched(false, download);
    capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(stream, &g);
    cudaGraphExec_t ex = nullptr;
    const cudaError_t ei = (!s && ec == cudaSuccess && g) ? cudaGraphInstantiate(&ex, g, 0) : cudaErrorUnknown;
    if (g) cudaGraphDestroy(g);
    if (s || ei != cudaSuccess) {
      cudaGetLastError();
      if (ex) cudaGraphExecDestroy(ex);
      graphs_ok = false;  // run this chain with direct launches from now on
      return enqueue_batched(false, download);
    }
    gexec[gi] = ex;
    glaunches[gi] = launches;
  }
  launches = glaunches[gi];
  VF_CK(cudaGraphLaunch(gexec[gi], stream));
  last_run_graph = true;
  return VF_OK;
}

void Batch::release() {
  drop_graphs();
  if (!ctx) return;
  for (DevBuf* b : {&grid0, &grid1, &keys, &par, &tets, &range, &ys, &seeds, &counts, &lat,
                    &verts, &faces, &emask, &etab, &tables, &state, &brick_job, &live, &list, &lcount,
                    &q[0], &q[1], &q[2], &scal, &epoch, &fdir, &front[0], &front[1], &pcnt, &pbase,
                    &psums, &srec, &stage_out, &rle_cnt, &rle_base, &rle_sums, &rle_tot, &rle_starts,
                    &rle_rec, &tmaps})
    ctx->free_buf(*b);
  if (h_tables) cudaFreeHost(h_tables);
  if (h_state) cudaFreeHost(h_state);
  if (h_scal) cudaFreeHost(h_scal);
  h_tables = nullptr;
  h_state = nullptr;
  h_scal = nullptr;
  if (ev_flood0) cudaEventDestroy(ev_flood0);
  if (ev_flood1) cudaEventDestroy(ev_flood1);
  if (ev_done) cudaEventDestroy(ev_done);
  for (int i = 0; i < NSTAGE_EV; ++i)
    if (ev_stage[i]) cudaEventDestroy(ev_stage[i]);
  ev_flood0 = ev_flood1 = ev_done = nullptr;
  if (own_stream && stream) cudaStreamDestroy(stream);
  stream = nullptr;
  ctx = nullptr;
}

size_t Batch::table_off(uint32_t t) const { return (size_t)t * jobs.size(); }
const JobDesc* Batch::dtable(uint32_t t) const {
  return reinterpret_cast<const JobDesc*>(tables.p) + table_off(t);
}

// --------------------------------------------------------------------------
static void mesh_aabb(const vf_job& j, float mn[3], float mx[3]) {
  for (int a = 0; a < 3; ++a) { mn[a] = FLT_MAX; mx[a] = -FLT_MAX; }
  for (uint32_t i = 0; i < j.nverts; ++i)
    for (int a = 0; a < 3; ++a) {
      const float v = j.verts[3 * (size_t)i + a];
      mn[a] = std::min(mn[a], v);
      mx[a] = std::max(mx[a], v);
    }
}

void dims_for_aabb(const float mn[3], const float mx[3], uint32_t maxv, uint32_t out[3]) {
  // CADScene::allocateMeshGrid (CADScene.cpp:545-561)
  float size[3];
  for (int a = 0; a < 3; ++a) size[a] = mx[a] - mn[a];
  const float longest = std::max(size[0], std::max(size[1], size[2]));
  for (int a = 0; a < 3; ++a) {
    const float v = ((float)maxv * size[a]) / longest;
    int d = (int)std::floor(v);
    while (d % 4 != 0) ++d;
    while (d % 4 != 0 || d > (int)maxv) --d;
    out[a] = d < 0 ? 0u : (uint32_t)d;
  }
}

// RegularGrid::erode mask and activation limit (RegularGrid.cpp:84-120)
static void erosion_mask(int type, uint32_t k, float threshold, std::vector<float>& mask,
                         float& limit) {
  const uint32_t msz = k * k * k;
  const int cc = (int)std::floor((float)k / 2.0f);
  mask.assign(msz, 0.0f);
  float activations = 0.0f;
  if (type == VF_SQUARE) {
    std::fill(mask.begin(), mask.end(), 1.0f);
    activations = (float)msz;
  } else if (type == VF_CROSS) {
    for (uint32_t x = 0; x < k; ++x) mask[x * k * k + cc * k + cc] = 1.0f;
    for (uint32_t y = 0; y < k; ++y) mask[cc * k * k + y * k + cc] = 1.0f;
    for (uint32_t z = 0; z < k; ++z) mask[cc * k * k + cc * k + z] = 1.0f;
    activations = 1.0f / 3.0f * (float)msz;
  } else {
    for (uint32_t x = 0; x < k; ++x)
      for (uint32_t y = 0; y < k; ++y)
        for (uint32_t z = 0; z < k; ++z) {
          const float dx = (float)x - (float)cc, dy = (float)y - (float)cc,
                      dz = (float)z - (float)cc;
          const float d = std::sqrt(dx * dx + dy * dy + dz * dz);
          if (d < (float)cc + FLT_EPSILON) {
            mask[x * k * k + y * k + z] = 1.0f;
            activations = activations + 1.0f;
          }
        }
  }
  activations = activations / (float)msz;
  limit = activations * threshold;
}

static vf_status check_params(const vf_params& p, uint32_t& ek) {
  if (p.algorithm != VF_NAIVE && p.algorithm != VF_FLOOD)
    return fail(VF_ERR_INVALID, "algorithm must be VF_NAIVE or VF_FLOOD");
  if (p.distance < 0 || p.distance > 2 || p.merge_distance < 0 || p.merge_distance > 2)
    return fail(VF_ERR_INVALID, "distance function out of range");
  if (p.num_seeds < 0 || p.num_seeds > 254) return fail(VF_ERR_RANGE, "num_seeds must be in [0, 254]");
  if (p.num_impacts < 0 || p.num_impacts > (1 << 20))
    return fail(VF_ERR_INVALID, "num_impacts must be in [0, 2^20]");
  if (p.num_impacts > 0 && (p.bias_seeds < 0 || p.bias_seeds > 254 || p.bias_focus < 1))
    return fail(VF_ERR_INVALID, "bias_seeds must be in [0, 254] and bias_focus >= 1");
  const int bias = p.num_impacts > 0 ? p.bias_seeds : 0;
  if (p.num_extra_seeds < 0 || 2 * (p.num_seeds + bias) + p.num_extra_seeds > (int)VF_MAX_SEEDS)
    return fail(VF_ERR_RANGE, "2*(num_seeds + bias_seeds) + num_extra_seeds must be <= 4095");
  if (p.seed_location < VF_INNER || p.seed_location > VF_BOTH)
    return fail(VF_ERR_INVALID, "seed_location out of range");
  if (!(p.noise_amplitude >= 0.0f) || p.noise_amplitude > 64.0f)
    return fail(VF_ERR_INVALID, "noise_amplitude must be in [0, 64]");
  if (p.noise_amplitude > 0.0f && p.noise_period == 0)
    return fail(VF_ERR_INVALID, "noise_period must be >= 1");
  if (p.boundary_size < 0 || p.boundary_size > 3)
    return fail(VF_ERR_INVALID, "boundary_size must be in [0, 3]");
  ek = 0;
  if (p.erode) {
    if (p.erosion_type < VF_SQUARE || p.erosion_type > VF_CROSS)
      return fail(VF_ERR_INVALID, "erosion_type out of range");
    uint32_t k = (uint32_t)std::max(p.erosion_size, 0);
    if (!(k % 2)) ++k;
    if (k > 7) return fail(VF_ERR_INVALID, "erosion_size must be <= 7");
    if (p.erosion_iterations < 0 || p.erosion_iterations > 64)
      return fail(VF_ERR_INVALID, "erosion_iterations must be in [0, 64]");
    ek = k;
  }
  return VF_OK;
}

// slots of a job's edge parity table: a power of two >= 4 * nfaces (load
// <= 0.75 for a triangle soup, <= 0.375 for a closed mesh)
static uint32_t edge_slots(uint32_t nfaces) {
  uint64_t c = 64;
  while (c < 4ull * nfaces) c <<= 1;
  return (uint32_t)std::min<uint64_t>(c, 1ull << 31);
}

size_t job_footprint(const vf_job& j) {
  uint32_t d[3] = {j.dims[0], j.dims[1], j.dims[2]};
  if (!d[0] && !d[1] && !d[2]) d[0] = d[1] = d[2] = j.max_dim;
  const size_t X = d[0], Y = d[1], Z = d[2];
  const size_t Zp = vf_roundup((uint32_t)Z, 8), Zk = vf_roundup((uint32_t)Z, 4), Zw = (Z + 31) / 32;
  size_t b = X * Y * Zp * 2 * 2 + X * Y * Zw * 4 * 2 + (size_t)j.nfaces * (48 + 4 + 12) +
             (size_t)edge_slots(j.nfaces) * 8 + (size_t)j.nverts * 12 + 65536;
  if (j.params.algorithm == VF_FLOOD) b += X * Y * Zk * 4;
  // per brick: owner, live flag, list, 3 queues, epoch, change record
  b += ((X + VF_BX - 1) / VF_BX) * ((Y + VF_BY - 1) / VF_BY) * ((Z + VF_BZ - 1) / VF_BZ) *
       (4 + 1 + 4 + 12 + 4 + 4 * vfk::FLOOD_FDIR);
  return b;
}

vf_status Batch::plan(const vf_job* const* js, uint32_t n) {
  drop_graphs();  // captured chains refer to the previous plan's tables and buffers
  graphs_ok = true;
  jobs.assign(js, js + n);
  plans.assign(n, JobPlan());
  sz = Sizes();
  for (uint32_t i = 0; i < n; ++i) {
    const vf_job& j = *js[i];
    JobPlan& p = plans[i];
    uint32_t ek = 0;
    vf_status s = check_params(j.params, ek);
    if (s) return fail(s, "job " + std::to_string(i) + ": " + last_error());
    if (j.nfaces && (!j.verts || !j.faces || !j.nverts))
      return fail(VF_ERR_INVALID, "job " + std::to_string(i) + ": mesh pointers missing");
    if (j.nverts >= 0x80000000u || j.nfaces >= 0x20000000u)
      return fail(VF_ERR_RANGE, "job " + std::to_string(i) + ": at most 2^31 - 1 vertices and 2^29 - 1 faces");
    bool aabb_given = false;
    for (int a = 0; a < 3; ++a) aabb_given |= j.aabb_min[a] != j.aabb_max[a];
    if (aabb_given) {
      for (int a = 0; a < 3; ++a) { p.amin[a] = j.aabb_min[a]; p.amax[a] = j.aabb_max[a]; }
    } else {
      if (!j.nverts) return fail(VF_ERR_INVALID, "job " + std::to_string(i) + ": no AABB and no mesh");
      mesh_aabb(j, p.amin, p.amax);
    }
    uint32_t d[3] = {j.dims[0], j.dims[1], j.dims[2]};
    if (!d[0] && !d[1] && !d[2]) {
      if (!j.max_dim) return fail(VF_ERR_INVALID, "job " + std::to_string(i) + ": dims and max_dim are 0");
      dims_for_aabb(p.amin, p.amax, j.max_dim, d);
    }
    for (int a = 0; a < 3; ++a)
      if (d[a] < 2 || d[a] > VF_MAX_DIM)
        return fail(VF_ERR_INVALID, "job " + std::to_string(i) + ": grid dims must be in [2, 4096]");
    p.X = d[0]; p.Y = d[1]; p.Z = d[2];
    p.Zp = vf_roundup(p.Z, 8); p.Zk = vf_roundup(p.Z, 4); p.Zw = (p.Z + 31) / 32;
    p.nbx = (p.X + VF_BX - 1) / VF_BX; p.nby = (p.Y + VF_BY - 1) / VF_BY; p.nbz = (p.Z + VF_BZ - 1) / VF_BZ;
    p.nbricks = p.nbx * p.nby * p.nbz;
    p.ncounts = std::max(j.ncounts, 256u);
    const int32_t bias = j.params.num_impacts > 0 ? j.params.bias_seeds : 0;
    p.seeds_cap = std::max<uint32_t>(2 * (j.params.num_seeds + bias) + j.params.num_extra_seeds, 1);
    const uint32_t ngiven = i < given.size() ? given[i].second : 0u;
    if (ngiven > VF_MAX_SEEDS) return fail(VF_ERR_RANGE, "at most 4095 seeds");
    p.seeds_cap = std::max(p.seeds_cap, ngiven);
    p.ek = ek;
    p.elimit = 0.f;
    if (ek) erosion_mask(j.params.erosion_type, ek, j.params.erosion_threshold, p.emask, p.elimit);
    p.lat_nx = p.lat_ny = p.lat_nz = 0;
    if (j.params.noise_amplitude > 0.0f) {
      p.lat_nx = (p.X - 1) / j.params.noise_period + 2;
      p.lat_ny = (p.Y - 1) / j.params.noise_period + 2;
      p.lat_nz = (p.Z - 1) / j.params.noise_period + 2;
    }
    p.prefix_possible = j.params.algorithm == VF_FLOOD && (j.params.num_extra_seeds > 0 || ngiven > 0);
    const size_t vox = (size_t)p.X * p.Y;
    p.o_grid = sz.grid; sz.grid += align_up(vox * p.Zp, 128);
    p.o_keys = sz.keys; if (j.params.algorithm == VF_FLOOD) sz.keys += align_up(vox * p.Zk, 64);
    p.o_par = sz.par; sz.par += align_up(vox * p.Zw, 64);
    p.o_tets = sz.tets; sz.tets += align_up((size_t)j.nfaces * 3, 16);
    p.o_range = sz.range; sz.range += align_up(j.nfaces, 64);
    p.ecap = j.nfaces ? edge_slots(j.nfaces) : 0u;
    p.o_etab = sz.etab; sz.etab += p.ecap;
    p.o_ys = sz.ys; sz.ys += align_up(p.Y, 64);
    p.o_seeds = sz.seeds; sz.seeds += align_up(4 * (size_t)p.seeds_cap, 64);
    p.o_counts = sz.counts; sz.counts += align_up(p.ncounts, 64);
    p.o_lat = sz.lat; sz.lat += align_up((size_t)p.lat_nx * p.lat_ny * p.lat_nz * 3, 64);
    p.o_verts = sz.verts; sz.verts += align_up((size_t)j.nverts * 3, 64);
    p.o_faces = sz.faces; sz.faces += align_up((size_t)j.nfaces * 3, 64);
    p.o_emask = sz.emask; sz.emask += align_up(p.emask.size(), 64);
    // rows without z padding (Z a multiple of 8) are already the host layout:
    // the copy engine takes them from the label grid itself
    p.dma = dma_download && j.out_labels != nullptr && p.Zp != p.Z;
    p.o_out = sz.out;
    if (p.dma) sz.out += align_up(vox * p.Z, 128);  // 256-byte aligned u16 rows
    sz.bricks += p.nbricks;
    sz.faces_total += j.nfaces;
    if (j.params.erode) sz.max_iters = std::max(sz.max_iters, (uint32_t)j.params.erosion_iterations);
  }
  // arenas (grow-only)
  Ctx& c = *ctx;
  vf_status s;
  auto alloc_all = [&]() -> vf_status {
    vf_status s;
#define ALLOC(buf, bytes) if ((s = c.alloc(buf, (bytes)))) return s
  ALLOC(grid0, std::max<size_t>(sz.grid * 2, 256));
  ALLOC(grid1, std::max<size_t>(sz.grid * 2, 256));
  ALLOC(keys, std::max<size_t>(sz.keys * 4, 256));
  ALLOC(par, std::max<size_t>(sz.par * 8, 256));  // par + shell
  ALLOC(tets, std::max<size_t>(sz.tets * 16, 256));
  ALLOC(range, std::max<size_t>(sz.range * 4, 256));
  ALLOC(etab, std::max<size_t>(sz.etab * 8, 256));
  ALLOC(ys, std::max<size_t>(sz.ys * 4, 256));
  ALLOC(seeds, std::max<size_t>(sz.seeds * 4, 256));
  ALLOC(counts, std::max<size_t>(sz.counts * 4, 256));
  ALLOC(lat, std::max<size_t>(sz.lat * 4, 256));
  ALLOC(verts, std::max<size_t>(sz.verts * 4, 256));
  ALLOC(faces, std::max<size_t>(sz.faces * 4, 256));
  ALLOC(emask, std::max<size_t>(sz.emask * 4, 256));
  ntables = T_FIXED + 2 * sz.max_iters;
  ALLOC(tables, sizeof(JobDesc) * ntables * std::max<size_t>(n, 1));
  ALLOC(state, sizeof(JobState) * std::max<size_t>(n, 1));
  const size_t nb = std::max<uint32_t>(sz.bricks, 1);
  ALLOC(brick_job, nb * 4);
  ALLOC(live, nb);
  ALLOC(list, nb * 4);
  ALLOC(lcount, 256);
  for (int i = 0; i < 3; ++i) ALLOC(q[i], nb * 4);
  ALLOC(epoch, nb * 4);
  ALLOC(fdir, nb * vfk::FLOOD_FDIR * 4);
  ALLOC(scal, 4096);
  const size_t nf = std::max<uint32_t>(sz.faces_total, 1);
  ALLOC(pcnt, nf * 4);
  ALLOC(pbase, nf * 8);
  ALLOC(psums, ((nf + 1023) / 1024 + 1) * 8);
  ALLOC(srec, nf * 96);
  if (sz.out) ALLOC(stage_out, sz.out * 2);
  ALLOC(tmaps, vfk::KEYS_MAP_BYTES * std::max<size_t>(n, 1));
#undef ALLOC
    return VF_OK;
  };
  // The arenas that must grow take twice what this plan needs when that fits
  // the budget (else 1/8 more, else the exact sizes), so that a stream of
  // batches of varying size regrows them rarely: each regrowth frees (a
  // device-wide synchronisation) and allocates again, which stalled a server
  // under load for about 300 ms per event.  The factor is chosen for the
  // plan as a whole (a dry run adds up the growth first), so that early
  // arenas do not take the room later ones need.
  c.dry = true;
  c.dry_need = c.dry_freed = 0;
  (void)alloc_all();
  c.dry = false;
  {
    const size_t base = c.in_use - std::min(c.in_use, c.dry_freed);
    const size_t slack = (size_t)64 << 20;  // 1 MB rounding of each arena
    const size_t need = c.dry_need;
    double f = 2.0;
    if (c.budget && base + 2 * need + slack > c.budget)
      f = base + need + need / 8 + slack <= c.budget ? 1.125 : 1.0;
    c.grow = f;
  }
  s = alloc_all();
  c.grow = 0.0;
  if (s) return s;
  // pinned staging: stage tables, erosion masks, then the keys tensor maps
  // (128-byte aligned, as CUtensorMap requires 64)
  tmap_off = align_up(sizeof(JobDesc) * ntables * std::max<size_t>(n, 1) + sz.emask * 4, 128);
  const size_t tbytes = tmap_off + vfk::KEYS_MAP_BYTES * std::max<size_t>(n, 1) + 256;
  if (tbytes > h_tables_cap) {
    if (h_tables) cudaFreeHost(h_tables);
    h_tables_cap = align_up(tbytes * 2, 1 << 16);
    VF_CK(cudaMallocHost(&h_tables, h_tables_cap));
  }
  const size_t sbytes = sizeof(JobState) * std::max<size_t>(n, 1);
  if (sbytes > h_state_cap) {
    if (h_state) cudaFreeHost(h_state);
    h_state_cap = align_up(sbytes * 2, 1 << 16);
    VF_CK(cudaMallocHost(reinterpret_cast<void**>(&h_state), h_state_cap));
  }
  // stage tables
  const uint32_t nt = ntables;
  JobDesc* T = reinterpret_cast<JobDesc*>(h_tables);
  float* hm = reinterpret_cast<float*>(T + (size_t)nt * n);
  uint32_t brick_base = 0, face_base = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const vf_job& j = *js[i];
    JobPlan& p = plans[i];
    for (size_t m = 0; m < p.emask.size(); ++m) hm[p.o_emask + m] = p.emask[m];
    JobDesc d;
    std::memset(&d, 0, sizeof(d));
    d.X = p.X; d.Y = p.Y; d.Z = p.Z; d.Zp = p.Zp; d.Zk = p.Zk; d.Zw = p.Zw;
    d.nbx = p.nbx; d.nby = p.nby; d.nbz = p.nbz; d.brick_base = brick_base; d.nbricks = p.nbricks;
    uint16_t* g0 = static_cast<uint16_t*>(grid0.p) + p.o_grid;
    uint16_t* g1 = static_cast<uint16_t*>(grid1.p) + p.o_grid;
    d.keys = static_cast<uint32_t*>(keys.p) + p.o_keys;
    {
      void* map = static_cast<char*>(h_tables) + tmap_off + vfk::KEYS_MAP_BYTES * i;
      std::memset(map, 0, vfk::KEYS_MAP_BYTES);
      std::string why;
      if (j.params.algorithm == VF_FLOOD && !vfk::encode_keys_map(map, d.keys, p.X, p.Y, p.Zk, &why))
        return fail(VF_ERR_CUDA, "job " + std::to_string(i) + ": " + why);
    }
    d.par = static_cast<uint32_t*>(par.p) + p.o_par;
    d.shell = static_cast<uint32_t*>(par.p) + sz.par + p.o_par;
    d.verts = static_cast<float*>(verts.p) + p.o_verts;
    d.faces = static_cast<uint32_t*>(faces.p) + p.o_faces;
    d.nverts = j.nverts; d.nfaces = j.nfaces; d.face_base = face_base;
    for (int a = 0; a < 3; ++a) { d.amin[a] = p.amin[a]; d.amax[a] = p.amax[a]; }
    {
      const uint32_t dd[3] = {p.X, p.Y, p.Z};
      for (int a = 0; a < 3; ++a) {
        const float size = p.amax[a] - p.amin[a];  // RegularGrid.cpp:426-441
        d.cs[a] = size / (float)dd[a];
        d.ics[a] = 1.0f / d.cs[a];
      }
    }
    d.tets = static_cast<float4*>(tets.p) + p.o_tets;
    d.tet_range = static_cast<uint32_t*>(range.p) + p.o_range;
    d.etab = static_cast<unsigned long long*>(etab.p) + p.o_etab;
    d.ecap = p.ecap;
    d.ys = static_cast<float*>(ys.p) + p.o_ys;
    d.seeds = static_cast<uint32_t*>(seeds.p) + p.o_seeds;
    d.seeds_cap = p.seeds_cap;
    d.seeds_given = i < given.size() ? given[i].second : 0u;
    d.counts = static_cast<uint32_t*>(counts.p) + p.o_counts;
    d.ncounts = p.ncounts;
    const vf_params& q = j.params;
    d.algorithm = q.algorithm; d.distance = q.distance; d.num_seeds = q.num_seeds;
    d.num_extra = q.num_extra_seeds; d.merge_distance = q.merge_distance;
    d.seed_location = q.seed_location; d.seed = q.seed;
    d.noise_amplitude = q.noise_amplitude; d.noise_period = q.noise_period;
    d.erode = q.erode; d.erosion_type = q.erosion_type; d.erosion_size = q.erosion_size;
    d.erosion_iterations = q.erosion_iterations; d.erosion_probability = q.erosion_probability;
    d.erosion_threshold = q.erosion_threshold; d.boundary_size = q.boundary_size;
    d.num_impacts = q.num_impacts; d.bias_seeds = q.bias_seeds; d.bias_focus = q.bias_focus;
    d.lattice = static_cast<float*>(lat.p) + p.o_lat;
    d.lat_nx = p.lat_nx; d.lat_ny = p.lat_ny; d.lat_nz = p.lat_nz;
    d.emask = static_cast<float*>(emask.p) + p.o_emask;
    d.elimit = p.elimit;
    d.ek = (int32_t)p.ek;
    // labels straight from the kernel into the caller's buffer when the GPU
    // can address it (pinned host memory is mapped under unified addressing)
    p.packed = false;
    d.out = nullptr;
    d.row_base = sz.rows;
    sz.rows += (uint64_t)p.X * p.Y;
    d.out_dma = 0;
    if (p.dma) {
      d.out = static_cast<uint16_t*>(stage_out.p) + p.o_out;
      d.out_dma = 1;
      p.packed = true;
    } else if (!dma_download && j.out_labels && ((uintptr_t)j.out_labels & 1) == 0) {
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, j.out_labels) == cudaSuccess && at.devicePointer &&
          at.type != cudaMemoryTypeUnregistered) {
        d.out = static_cast<uint16_t*>(at.devicePointer);
        p.packed = true;
      } else {
        cudaGetLastError();
      }
    }
    uint16_t* buf[2] = {g0, g1};
    int cur = 0;
    auto put = [&](uint32_t t, bool active, int src, int dst, int bs) {
      JobDesc e = d;
      e.active = active ? 1u : 0u;
      e.grid = buf[src];
      e.grid2 = buf[dst];
      e.boundary_size = bs;
      T[(size_t)t * n + i] = e;
    };
    put(T_VOX, true, 0, 1, q.boundary_size);
    put(T_SEED, true, 0, 1, q.boundary_size);
    put(T_FLOOD, q.algorithm == VF_FLOOD, 0, 1, q.boundary_size);
    put(T_NAIVE, q.algorithm == VF_NAIVE, 0, 1, q.boundary_size);
    const bool pert = q.noise_amplitude > 0.0f;
    put(T_PERT, pert, cur, 1 - cur, q.boundary_size);
    if (pert) cur ^= 1;
    for (uint32_t it = 0; it < sz.max_iters; ++it) {
      const bool on = q.erode && (int)it < q.erosion_iterations;
      put(t_edet(it), on, cur, 1 - cur, 1);  // erode() calls detectBoundaries(1)
      put(t_ero(it), on, cur, 1 - cur, 1);
      if (on) cur ^= 1;
    }
    put(T_ISO, q.erode != 0, cur, 1 - cur, q.boundary_size);
    if (q.erode) cur ^= 1;
    put(T_DET1, !q.erode && q.boundary_size <= 1, cur, 1 - cur, q.boundary_size);
    put(T_DET3, !q.erode && q.boundary_size > 1, cur, 1 - cur, q.boundary_size);
    put(T_CNT, true, cur, 1 - cur, q.boundary_size);
    p.final_cur = cur;
    brick_base += p.nbricks;
    face_base += j.nfaces;
  }
  return VF_OK;
}

// --------------------------------------------------------------------------
static vf_status map_job_status(uint32_t err) {
  if (err & VF_JERR_INVALID) return VF_ERR_INVALID;
  if (err & VF_JERR_SEED_SEARCH) return VF_ERR_SEED_SEARCH;
  if (err & VF_JERR_TIMEOUT) return VF_ERR_TIMEOUT;
  if (err & (VF_JERR_RANGE | VF_JERR_DIST_OVERFLOW)) return VF_ERR_RANGE;
  return VF_OK;
}

namespace {
__global__ void k_brick_job(const JobDesc* jobs, uint32_t* brick_job) {
  const JobDesc& J = jobs[blockIdx.y];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < J.nbricks;
       i += gridDim.x * blockDim.x)
    brick_job[J.brick_base + i] = blockIdx.y;
}
}  // namespace

// inputs: meshes, given seeds, stage tables, erosion masks (host -> device)
static vf_status upload_inputs_impl(Batch& B) {
  const uint32_t n = (uint32_t)B.jobs.size();
  cudaStream_t st = B.stream;
  for (uint32_t i = 0; i < n && (B.stages & ST_VOX); ++i) {
    const vf_job& j = *B.jobs[i];
    const JobPlan& p = B.plans[i];
    if (j.nverts)
      VF_CK(cudaMemcpyAsync(static_cast<float*>(B.verts.p) + p.o_verts, j.verts,
                            sizeof(float) * 3 * (size_t)j.nverts, cudaMemcpyHostToDevice, st));
    if (j.nfaces)
      VF_CK(cudaMemcpyAsync(static_cast<uint32_t*>(B.faces.p) + p.o_faces, j.faces,
                            sizeof(uint32_t) * 3 * (size_t)j.nfaces, cudaMemcpyHostToDevice, st));
  }
  for (uint32_t i = 0; i < n && i < B.given.size(); ++i)
    if (B.given[i].second)
      VF_CK(cudaMemcpyAsync(static_cast<uint32_t*>(B.seeds.p) + B.plans[i].o_seeds, B.given[i].first,
                            sizeof(uint32_t) * 4 * B.given[i].second, cudaMemcpyHostToDevice, st));
  const size_t tb = sizeof(JobDesc) * B.ntables * n;
  VF_CK(cudaMemcpyAsync(B.tables.p, B.h_tables, tb, cudaMemcpyHostToDevice, st));
  if (B.sz.emask)
    VF_CK(cudaMemcpyAsync(B.emask.p, static_cast<char*>(B.h_tables) + tb, B.sz.emask * 4,
                          cudaMemcpyHostToDevice, st));
  VF_CK(cudaMemcpyAsync(B.tmaps.p, static_cast<char*>(B.h_tables) + B.tmap_off,
                        vfk::KEYS_MAP_BYTES * n, cudaMemcpyHostToDevice, st));
  return VF_OK;
}

vf_status Batch::upload_inputs() { return upload_inputs_impl(*this); }

// per-run scratch: job states, bit planes, counts, flood words, brick map
static vf_status reset_scratch(Batch& B) {
  const uint32_t n = (uint32_t)B.jobs.size();
  cudaStream_t st = B.stream;
  VF_CK(cudaMemsetAsync(B.state.p, 0, sizeof(JobState) * n, st));
  if (B.stages & ST_VOX) {
    VF_CK(cudaMemsetAsync(B.par.p, 0, B.sz.par * 8, st));
    VF_CK(cudaMemsetAsync(B.etab.p, 0xFF, B.sz.etab * 8, st));  // every slot empty
  }
  VF_CK(cudaMemsetAsync(B.counts.p, 0, B.sz.counts * 4, st));
  VF_CK(cudaMemsetAsync(B.scal.p, 0, 4096, st));
  uint32_t maxb = 1;
  for (const JobPlan& p : B.plans) maxb = std::max(maxb, p.nbricks);
  k_brick_job<<<dim3(std::min<uint32_t>((maxb + 255) / 256, 1024), n), 256, 0, st>>>(
      B.dtable(T_VOX), static_cast<uint32_t*>(B.brick_job.p));
  B.launches += 1;
  return VF_OK;
}

static vf_status upload_common(Batch& B) {
  vf_status s = upload_inputs_impl(B);
  if (s) return s;
  return reset_scratch(B);
}

static void voxelize_stages(Batch& B, const std::function<void(int)>& mark) {
  const uint32_t n = (uint32_t)B.jobs.size();
  cudaStream_t st = B.stream;
  const JobDesc* tv = B.dtable(T_VOX);
  JobState* ds = static_cast<JobState*>(B.state.p);
  vfk::FaceScratch fsc;
  fsc.pcnt = static_cast<uint32_t*>(B.pcnt.p);
  fsc.pbase = static_cast<unsigned long long*>(B.pbase.p);
  fsc.psums = static_cast<unsigned long long*>(B.psums.p);
  fsc.ptotal = static_cast<unsigned long long*>(B.scal.p) + 256;  // bytes 2048..2055
  fsc.srec = static_cast<float4*>(B.srec.p);
  vfk::centroid_and_slices(st, tv, ds, n);
  vfk::tetra_prep(st, tv, ds, n, B.sz.faces_total, fsc);
  mark(2);
  vfk::parity_raster(st, tv, ds, n, B.sz.faces_total, fsc, B.ctx->num_sms, B.ctx->tune.parity_grid);
  mark(3);
  vfk::shell_sat(st, tv, n, B.sz.faces_total, fsc, B.ctx->num_sms, B.ctx->tune.shell_grid);
  mark(4);
  vfk::combine(st, tv, static_cast<uint32_t*>(B.brick_job.p), B.sz.bricks,
               static_cast<uint8_t*>(B.live.p), 1);
  vfk::compact_live(st, static_cast<uint8_t*>(B.live.p), B.sz.bricks,
                    static_cast<uint32_t*>(B.list.p), static_cast<uint32_t*>(B.lcount.p));
  B.launches += 16;
}

static vfk::FloodScratch flood_scratch(Batch& B) {
  vfk::FloodScratch fs;
  for (int i = 0; i < 3; ++i) fs.queue[i] = static_cast<uint32_t*>(B.q[i].p);
  uint32_t* sc = static_cast<uint32_t*>(B.scal.p);
  fs.qcount = sc + 0;    // [3]
  fs.qhead = sc + 4;     // [3]
  fs.barrier = sc + 8;   // [2]
  fs.err = sc + 12;      // [1]
  fs.stats = sc + 16;    // [VF_FLOOD_NCOUNTERS]: visits, passes, busy warp-sweeps, timeouts, sweeps,
                         // sweep-cap hits, active row-sweeps, changed voxels, the
                         // first out-of-range access (code, two values), the SM
                         // cycles / 256 of five phases of the relaxation CTAs and
                         // the visits that found nothing new
  fs.epoch = static_cast<uint32_t*>(B.epoch.p);
  fs.fdir = static_cast<uint32_t*>(B.fdir.p);
  fs.max_passes = 1u << 20;
  fs.total_bricks = B.sz.bricks;
  fs.njobs = (uint32_t)B.jobs.size();
  fs.max_sweeps = B.ctx->tune.flood_sweeps;
  fs.ctas_per_sm = B.ctx->tune.flood_ctas;
  fs.wait_spins = B.ctx->tune.flood_wait_spins;
  fs.tmaps = B.tmaps.p;
  fs.pass_sizes = sc + 128;  // [256]
  return fs;
}

// the flood relaxation, after the last one issued on the context (any stream)
cudaError_t Batch::relax_serialized(cudaStream_t st, const JobDesc* tf, JobState* ds,
                                    const uint32_t* bj, const uint8_t* lv, const vfk::FloodScratch& fs) {
  const bool chain = !capturing && ctx->ev_relax;
  std::unique_lock<std::mutex> lk(ctx->relax_mu, std::defer_lock);
  if (chain) lk.lock();
  if (chain && ctx->ev_relax_used) {
    cudaError_t e = cudaStreamWaitEvent(st, ctx->ev_relax, 0);
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = vfk::flood_relax(st, tf, ds, bj, lv, fs, ctx->num_sms, &relax_blocks);
  if (e == cudaSuccess && chain) {
    e = cudaEventRecord(ctx->ev_relax, st);
    ctx->ev_relax_used = e == cudaSuccess;
  }
  return e;
}

vf_status Batch::enqueue_batched(bool do_upload, bool do_download) {
  const uint32_t n = (uint32_t)jobs.size();
  cudaStream_t st = stream;
  launches = 0;
  flood_timed = false;
  for (int i = 0; i < NSTAGE_EV; ++i) stage_rec[i] = false;
  std::function<void(int)> mark = [&](int i) {
    if (record_event(ev_stage[i], st) == cudaSuccess) stage_rec[i] = true;
  };
  mark(0);
  vf_status s = do_upload ? upload_inputs_impl(*this) : VF_OK;
  if (s) return s;
  mark(1);
  const bool chain = !capturing && ctx->ev_compute;
  if (chain) {
    std::lock_guard<std::mutex> lk(ctx->relax_mu);
    if (ctx->ev_compute_used) VF_CK(cudaStreamWaitEvent(st, ctx->ev_compute, 0));
  }
  s = reset_scratch(*this);
  if (s) return s;
  JobState* ds = static_cast<JobState*>(state.p);
  const uint32_t* bj = static_cast<uint32_t*>(brick_job.p);
  uint32_t* lst = static_cast<uint32_t*>(list.p);
  uint32_t* lc = static_cast<uint32_t*>(lcount.p);
  uint8_t* lv = static_cast<uint8_t*>(live.p);
  const uint32_t maxc = sz.bricks;
  if (stages & ST_VOX) {
    voxelize_stages(*this, mark);
  } else {
    // live bricks of an existing grid
    vfk::mark_live(st, dtable(T_VOX), bj, sz.bricks, lv);
    vfk::compact_live(st, lv, sz.bricks, lst, lc);
    launches += 2;
  }
  mark(5);
  if (stages & (ST_SEED | ST_FRACTURE)) {
    vfk::sample_seeds(st, dtable(T_SEED), ds, n);
    launches += 1;
  }
  mark(6);
  bool any_flood = false, any_naive = false, any_pert = false, any_erode = false,
       any_det1 = false, any_det3 = false, any_prefix = false;
  for (uint32_t i = 0; i < n; ++i) {
    const vf_params& q = jobs[i]->params;
    any_flood |= q.algorithm == VF_FLOOD;
    any_naive |= q.algorithm == VF_NAIVE;
    any_pert |= q.noise_amplitude > 0.0f;
    any_erode |= q.erode != 0;
    any_det1 |= !q.erode && q.boundary_size <= 1;
    any_det3 |= !q.erode && q.boundary_size > 1;
    any_prefix |= plans[i].prefix_possible;
  }
  if (!(stages & ST_FRACTURE)) any_flood = any_naive = false;
  if (!(stages & ST_PERTURB)) any_pert = false;
  if (!(stages & ST_ERODE)) any_erode = false;
  if (!(stages & ST_DETECT)) any_det1 = any_det3 = false;
  const uint32_t erode_iters = (stages & ST_ERODE) ? sz.max_iters : 0u;
  vfk::FloodScratch fs = flood_scratch(*this);
  if (any_flood) {
    const JobDesc* tf = dtable(T_FLOOD);
    vfk::flood_seed_bricks(st, tf, ds, n, lv, lst, lc);
    vfk::flood_init_keys(st, tf, lst, lc, maxc, bj, lv);
    vfk::flood_seed(st, tf, ds, n, fs, lv);
    VF_CK(record_event(ev_flood0, st));
    cudaError_t e = relax_serialized(st, tf, ds, bj, lv, fs);
    if (e != cudaSuccess) return fail(VF_ERR_CUDA, std::string("flood relax launch: ") + cudaGetErrorString(e));
    VF_CK(record_event(ev_flood1, st));
    flood_timed = true;
    vfk::flood_finalize(st, tf, ds, lst, lc, maxc, bj, 0);
    launches += 5;
    if (any_prefix) {
      // competition to a fixed point (host loop), disjoint cleanup, re-flood
      for (int it = 0; it < 1 << 20; ++it) {
        for (uint32_t i = 0; i < n; ++i)
          VF_CK(cudaMemsetAsync(&ds[i].changed, 0, sizeof(uint32_t), st));
        vfk::flood_competition(st, tf, ds, lst, lc, maxc, bj);
        VF_CK(cudaMemcpyAsync(h_state, ds, sizeof(JobState) * n, cudaMemcpyDeviceToHost, st));
        VF_CK(cudaStreamSynchronize(st));
        launches += 1;
        bool any = false;
        for (uint32_t i = 0; i < n; ++i) any |= h_state[i].changed != 0;
        if (!any) break;
      }
      vfk::flood_disjoint(st, tf, ds, n, lst, lc, maxc, bj, fs, lv);
      e = relax_serialized(st, tf, ds, bj, lv, fs);
      if (e != cudaSuccess) return fail(VF_ERR_CUDA, std::string("flood relax launch: ") + cudaGetErrorString(e));
      vfk::flood_finalize(st, tf, ds, lst, lc, maxc, bj, 1);
      launches += 6;
    }
  }
  if (any_naive) { vfk::naive(st, dtable(T_NAIVE), ds, lst, lc, maxc, bj); launches += 1; }
  mark(7);
  if (any_pert) {
    vfk::lattice(st, dtable(T_PERT), n);
    vfk::perturb(st, dtable(T_PERT), lst, lc, maxc, bj);
    launches += 2;
  }
  mark(8);
  for (uint32_t it = 0; it < erode_iters; ++it) {
    vfk::detect_boundaries(st, dtable(t_edet(it)), lst, lc, maxc, bj);
    vfk::erode(st, dtable(t_ero(it)), lst, lc, maxc, bj);
    launches += 2;
  }
  if (any_erode) { vfk::remove_isolated(st, dtable(T_ISO), lst, lc, maxc, bj); launches += 1; }
  if (any_det1) { vfk::detect_boundaries(st, dtable(T_DET1), lst, lc, maxc, bj); launches += 1; }
  if (any_det3) { vfk::detect_boundaries_wide(st, dtable(T_DET3), lst, lc, maxc, bj); launches += 1; }
  mark(9);
  if (stages & ST_COUNT) {
    vfk::count_values(st, dtable(T_CNT), ds, lst, lc, maxc, bj);
    launches += 1;
  }
  mark(10);
  if (chain) {
    std::lock_guard<std::mutex> lk(ctx->relax_mu);
    VF_CK(cudaEventRecord(ctx->ev_compute, st));
    ctx->ev_compute_used = true;
  }
  VF_CK(cudaGetLastError());
  // downloads
  if ((stages & ST_DOWNLOAD) && do_download) {
    bool any_packed = false;
    for (uint32_t i = 0; i < n; ++i) any_packed |= plans[i].packed;
    if (any_packed) {
      vfk::pack_labels(st, dtable(T_CNT), (int)n, sz.rows, ctx->num_sms);
      launches += 1;
    }
  }
  for (uint32_t i = 0; i < n && (stages & ST_DOWNLOAD) && do_download; ++i) {
    const vf_job& j = *jobs[i];
    const JobPlan& p = plans[i];
    const uint16_t* src = static_cast<uint16_t*>(p.final_cur ? grid1.p : grid0.p) + p.o_grid;
    if (p.dma)
      VF_CK(cudaMemcpyAsync(j.out_labels, static_cast<uint16_t*>(stage_out.p) + p.o_out,
                            (size_t)p.X * p.Y * p.Z * 2, cudaMemcpyDeviceToHost, st));
    if (j.out_labels && !p.packed) {
      if (p.Zp == p.Z)
        VF_CK(cudaMemcpyAsync(j.out_labels, src, (size_t)p.X * p.Y * p.Z * 2, cudaMemcpyDeviceToHost, st));
      else
        VF_CK(cudaMemcpy2DAsync(j.out_labels, (size_t)p.Z * 2, src, (size_t)p.Zp * 2, (size_t)p.Z * 2,
                                (size_t)p.X * p.Y, cudaMemcpyDeviceToHost, st));
    }
    if (j.out_counts && j.ncounts)
      VF_CK(cudaMemcpyAsync(j.out_counts, static_cast<uint32_t*>(counts.p) + p.o_counts,
                            sizeof(uint32_t) * j.ncounts, cudaMemcpyDeviceToHost, st));
  }
  VF_CK(cudaMemcpyAsync(h_state, ds, sizeof(JobState) * n, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaMemcpyAsync(h_scal, scal.p, 384 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  mark(11);
  VF_CK(record_event(ev_done, st));
  return VF_OK;
}

vf_status Batch::finish(vf_job_result* res) {
  VF_CK(cudaEventSynchronize(ev_done));
  VF_CK(cudaGetLastError());
  const uint32_t n = (uint32_t)jobs.size();
  const uint32_t ferr = h_scal[12];
  vf_status first = VF_OK;
  for (uint32_t i = 0; i < n; ++i) {
    const vf_job& j = *jobs[i];
    const JobPlan& p = plans[i];
    const JobState& s = h_state[i];
    uint32_t err = s.err;
    if (j.params.algorithm == VF_FLOOD && ferr) err |= VF_JERR_TIMEOUT;
    vf_status st = map_job_status(err);
    if (st && !first) {
      first = st;
      set_error("job " + std::to_string(i) + ": " +
                (st == VF_ERR_SEED_SEARCH ? "seed search exceeded 1e6 tries"
                 : st == VF_ERR_TIMEOUT   ? ((ferr & 8u) ? "flood relaxation skipped an out-of-range brick or key access"
                                                        : "flood did not converge (bounded wait expired)")
                 : st == VF_ERR_RANGE     ? "value out of range (prefix, distance or count)"
                                          : "invalid seeds or parameters"));
    }
    if (res) {
      vf_job_result& r = res[i];
      std::memset(&r, 0, sizeof(r));
      r.status = st;
      r.dims[0] = p.X; r.dims[1] = p.Y; r.dims[2] = p.Z;
      r.nseeds = s.nseeds;
      r.voxels = (uint64_t)p.X * p.Y * p.Z;
      r.occupied = s.occupied;
      r.flood_passes = s.passes;
      r.user_tag = j.user_tag;
      if (j.out_counts)
        for (uint32_t v = 0; v < j.ncounts; ++v) r.fragments += j.out_counts[v] != 0;
    }
  }
  if (flood_timed) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev_flood0, ev_flood1) == cudaSuccess) ctx->last_flood_ms = ms;
    ctx->last_flood_visits = h_scal[16];
    ctx->last_flood_passes = h_scal[17];
    ctx->last_flood_sweeps = h_scal[20];
    ctx->last_flood_maxit = h_scal[21];
    for (int i = 0; i < VF_FLOOD_NCOUNTERS; ++i) ctx->last_flood_counters[i] = h_scal[16 + i];
    for (int i = 0; i < 256; ++i) ctx->last_pass_sizes[i] = h_scal[128 + i];
  } else {
    for (int i = 0; i < VF_FLOOD_NCOUNTERS; ++i) ctx->last_flood_counters[i] = 0;
    ctx->last_flood_ms = 0.f;
    ctx->last_flood_visits = 0;
    ctx->last_flood_passes = 0;
  }
  ctx->last_launches = launches;
  for (int i = 0; i < NSTAGE_EV - 1; ++i) {
    float ms = 0.f;
    if (stage_rec[i] && stage_rec[i + 1] &&
        cudaEventElapsedTime(&ms, ev_stage[i], ev_stage[i + 1]) == cudaSuccess)
      ctx->last_stage_ms[i] = ms;
    else
      ctx->last_stage_ms[i] = 0.f;
  }
  return first;
}

// --------------------------------------------------------------------------
// plain path: one job, per-voxel kernels, one launch + host read per wave
vf_status Batch::enqueue_plain_and_wait(vf_job_result* res, bool skip_vox) {
  cudaStream_t st = stream;
  launches = 0;
  flood_timed = false;
  for (int i = 0; i < NSTAGE_EV; ++i) stage_rec[i] = false;
  const vf_job& j = *jobs[0];
  const JobPlan& p = plans[0];
  const uint64_t N = (uint64_t)p.X * p.Y * p.Z;
  if (N >= (1ull << 32)) return fail(VF_ERR_RANGE, "plain path needs X*Y*Z < 2^32");
  vf_status s = upload_common(*this);
  if (s) return s;
  std::function<void(int)> nomark = [](int) {};
  if (!skip_vox) voxelize_stages(*this, nomark);
  JobState* ds = static_cast<JobState*>(state.p);
  vfk::sample_seeds(st, dtable(T_SEED), ds, 1);
  launches += 1;
  JobDesc hj = reinterpret_cast<JobDesc*>(h_tables)[T_FLOOD];
  const vf_params& q = j.params;
  uint32_t waves = 0;
  if (q.algorithm == VF_FLOOD) {
    // a frontier holds each voxel once, the first one each seed once
    if ((s = ctx->alloc(front[0], (N + VF_MAX_SEEDS) * 4 + 256))) return s;
    if ((s = ctx->alloc(front[1], (N + VF_MAX_SEEDS) * 4 + 256))) return s;
    uint32_t* f0 = static_cast<uint32_t*>(front[0].p);
    uint32_t* f1 = static_cast<uint32_t*>(front[1].p);
    uint32_t* cnt = static_cast<uint32_t*>(scal.p) + 48;  // after the flood counters (16 .. 32)
    const JobDesc* tf = dtable(T_FLOOD);
    vfk::plain_init_keys(st, tf, hj);
    vfk::plain_seed(st, tf, ds, f0, cnt);
    launches += 2;
    for (int pass = 0; pass < 2; ++pass) {
      VF_CK(cudaMemcpyAsync(h_scal + 8, cnt, 4, cudaMemcpyDeviceToHost, st));
      VF_CK(cudaMemcpyAsync(h_state, ds, sizeof(JobState), cudaMemcpyDeviceToHost, st));
      VF_CK(cudaStreamSynchronize(st));
      uint32_t ncur = h_scal[8];
      // while (numDisjointVoxels != 0) (FloodFracturer.cpp:135): no
      // re-flood when the cleanup reset nothing
      if (pass == 1 && h_state[0].disjoint == 0) ncur = 0;
      while (ncur > 0) {  // FloodFracturer.cpp:143-158
        VF_CK(cudaMemsetAsync(cnt, 0, 4, st));
        vfk::plain_wave(st, tf, ds, hj, f0, ncur, f1, cnt);
        VF_CK(cudaMemcpyAsync(h_scal + 8, cnt, 4, cudaMemcpyDeviceToHost, st));
        VF_CK(cudaStreamSynchronize(st));
        launches += 1;
        ncur = h_scal[8];
        std::swap(f0, f1);
        ++waves;
      }
      if (pass == 0) {
        vfk::plain_finalize(st, tf, ds, hj, 0);
        launches += 1;
        if (!p.prefix_possible) break;
        for (int it = 0; it < 1 << 20; ++it) {
          VF_CK(cudaMemsetAsync(&ds[0].changed, 0, sizeof(uint32_t), st));
          vfk::plain_competition(st, tf, ds, hj);
          VF_CK(cudaMemcpyAsync(h_state, ds, sizeof(JobState), cudaMemcpyDeviceToHost, st));
          VF_CK(cudaStreamSynchronize(st));
          launches += 1;
          if (!h_state[0].changed) break;
        }
        vfk::plain_disjoint(st, tf, ds, hj, f0, cnt);
        launches += 3;
      } else {
        vfk::plain_finalize(st, tf, ds, hj, 1);
        launches += 1;
      }
    }
  } else {
    vfk::plain_naive(st, dtable(T_NAIVE), ds, hj);
    launches += 1;
  }
  const JobDesc* T = reinterpret_cast<const JobDesc*>(h_tables);
  if (q.noise_amplitude > 0.0f && (stages & ST_PERTURB)) {
    vfk::lattice(st, dtable(T_PERT), 1);
    vfk::plain_perturb(st, dtable(T_PERT), T[T_PERT]);
    launches += 2;
  }
  for (uint32_t it = 0; it < sz.max_iters && (stages & ST_ERODE); ++it) {
    if (!T[t_ero(it)].active) continue;
    vfk::plain_detect(st, dtable(t_edet(it)), T[t_edet(it)]);
    vfk::plain_erode(st, dtable(t_ero(it)), T[t_ero(it)]);
    launches += 2;
  }
  if (q.erode && (stages & ST_ERODE)) {
    vfk::plain_remove_isolated(st, dtable(T_ISO), T[T_ISO]);
    launches += 1;
  } else if (!q.erode && (stages & ST_DETECT)) {
    if (T[T_DET1].active) vfk::plain_detect(st, dtable(T_DET1), T[T_DET1]);
    else vfk::plain_detect(st, dtable(T_DET3), T[T_DET3]);
    launches += 1;
  }
  if (stages & ST_COUNT) {
    vfk::plain_counts(st, dtable(T_CNT), ds, T[T_CNT]);
    launches += 1;
  }
  VF_CK(cudaGetLastError());
  const uint16_t* src = static_cast<uint16_t*>(p.final_cur ? grid1.p : grid0.p) + p.o_grid;
  if (j.out_labels && (stages & ST_DOWNLOAD))
    VF_CK(cudaMemcpy2DAsync(j.out_labels, (size_t)p.Z * 2, src, (size_t)p.Zp * 2, (size_t)p.Z * 2,
                            (size_t)p.X * p.Y, cudaMemcpyDeviceToHost, st));
  if (j.out_counts && j.ncounts)
    VF_CK(cudaMemcpyAsync(j.out_counts, static_cast<uint32_t*>(counts.p) + p.o_counts,
                          sizeof(uint32_t) * j.ncounts, cudaMemcpyDeviceToHost, st));
  VF_CK(cudaMemcpyAsync(h_state, ds, sizeof(JobState), cudaMemcpyDeviceToHost, st));
  VF_CK(cudaMemcpyAsync(h_scal, scal.p, 64 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  VF_CK(cudaEventRecord(ev_done, st));
  s = finish(res);
  if (res) res[0].flood_passes = waves;
  return s;
}

}  // namespace vfr
