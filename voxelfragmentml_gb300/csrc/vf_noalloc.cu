// vf_noalloc.cu -- flood fracture without any device allocation.
//
// Some callers cannot allocate device memory while they run this step: a
// renderer or simulation that owns every allocation through its own pool,
// code that must not grow its footprint after start-up, or an embedding
// whose allocator is not the CUDA runtime's.  vf_flood_noalloc serves them:
// the caller passes its own device buffers for the input grid, the seeds and
// the output labels, and every intermediate (a padded copy of the grid, the
// flood keys, brick lists and queues, the job descriptor) lives in one
// file-scope device array, g_scratch, of VF_NOALLOC_SCRATCH_BYTES.
//
// Properties of the scratch array:
//   - it is part of the library image: every GPU that loads the library
//     holds it until the process exits;
//   - every call on a device shares it and it keeps the contents of the last
//     call; each call clears what must start at zero before using it;
//   - calls whose work overlaps on the GPU (two host threads, or two streams
//     without ordering between them) race on it and give wrong results;
//   - its flood relaxation is a cooperative launch with a grid-wide barrier
//     that expects the whole GPU: a call must not overlap a vf_ctx's batched
//     flood (vf_batch_run, vf_pipeline_*, a vf_server) on another stream
//     either, or the barrier wait may run out (VF_ERR_TIMEOUT).
// When the call returns an error the contents of d_labels are unspecified.
//
// Host code cannot use the name g_scratch as a device address (on the host
// it is only a stand-in symbol).  The first call on each device, with that
// device current, resolves the address with cudaGetSymbolAddress and caches
// it; make that first call before any stream capture begins.
#include <cstring>
#include <mutex>
#include <string>

#include "vf_runtime.h"

#define VF_NOALLOC_SCRATCH_BYTES (32u << 20)

static __device__ __align__(256) unsigned char g_scratch[VF_NOALLOC_SCRATCH_BYTES];

namespace {

// the keys tensor map, passed by value into the scratch array
struct KeysMap {
  alignas(64) unsigned char b[vfk::KEYS_MAP_BYTES];
};

__global__ void k_noalloc_init(JobDesc d, JobDesc* dst, JobState* st, uint32_t* scal, KeysMap m,
                               KeysMap* mdst) {
  if (threadIdx.x == 0) *dst = d;
  if (threadIdx.x < vfk::KEYS_MAP_BYTES / 4)
    reinterpret_cast<uint32_t*>(mdst->b)[threadIdx.x] = reinterpret_cast<const uint32_t*>(m.b)[threadIdx.x];
  unsigned char* s = reinterpret_cast<unsigned char*>(st);
  for (uint32_t i = threadIdx.x; i < sizeof(JobState); i += blockDim.x) s[i] = 0;
  for (uint32_t i = threadIdx.x; i < 1024; i += blockDim.x) scal[i] = 0;
}

std::mutex g_mu;
void* g_addr[64] = {};  // resolved scratch address per device
int g_sms[64] = {};     // multiprocessor count per device

size_t up(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

extern "C" vf_status vf_flood_noalloc(const uint16_t* d_grid, uint16_t* d_labels, uint32_t X,
                                      uint32_t Y, uint32_t Z, const uint32_t* d_seeds_xyzw,
                                      uint32_t nseeds, int distance, void* stream) {
  using vfr::fail;
  if (!d_grid || !d_labels || (nseeds && !d_seeds_xyzw))
    return fail(VF_ERR_INVALID, "vf_flood_noalloc: NULL buffer");
  if (X < 1 || Y < 1 || Z < 1 || X > VF_MAX_DIM || Y > VF_MAX_DIM || Z > VF_MAX_DIM)
    return fail(VF_ERR_INVALID, "vf_flood_noalloc: dims must be in [1, 4096]");
  if (distance < VF_EUCLIDEAN || distance > VF_CHEBYSHEV)
    return fail(VF_ERR_INVALID, "vf_flood_noalloc: distance out of range");
  if (nseeds > VF_MAX_SEEDS) return fail(VF_ERR_RANGE, "vf_flood_noalloc: at most 4095 seeds");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(VF_ERR_NOT_BUILT, "vf_flood_noalloc: no current CUDA device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      cudaError_t e = cudaGetSymbolAddress(&g_addr[dev], g_scratch);
      if (e != cudaSuccess) {
        g_addr[dev] = nullptr;
        return fail(VF_ERR_CUDA, std::string("vf_flood_noalloc: cudaGetSymbolAddress: ") +
                                     cudaGetErrorString(e));
      }
    }
    base = g_addr[dev];
    if (!g_sms[dev] &&
        cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      g_sms[dev] = 0;
      return fail(VF_ERR_CUDA, "vf_flood_noalloc: device query failed");
    }
  }
  const int num_sms = g_sms[dev];
  // layout of the scratch array
  const uint32_t Zp = vf_roundup(Z, 8), Zk = vf_roundup(Z, 4);
  const uint32_t nbx = (X + VF_BX - 1) / VF_BX, nby = (Y + VF_BY - 1) / VF_BY,
                 nbz = (Z + VF_BZ - 1) / VF_BZ;
  const size_t nb = (size_t)nbx * nby * nbz;
  size_t off = 0;
  const size_t o_desc = off; off += up(sizeof(JobDesc));
  const size_t o_state = off; off += up(sizeof(JobState));
  const size_t o_scal = off; off += up(4096);
  const size_t o_map = off; off += up(sizeof(KeysMap));
  const size_t o_bj = off; off += up(nb * 4);
  const size_t o_live = off; off += up(nb);
  const size_t o_list = off; off += up(nb * 4);
  const size_t o_q0 = off; off += up(nb * 4);
  const size_t o_q1 = off; off += up(nb * 4);
  const size_t o_q2 = off; off += up(nb * 4);
  const size_t o_epoch = off; off += up(nb * 4);
  const size_t o_fdir = off; off += up(nb * 4 * vfk::FLOOD_FDIR);
  const size_t o_grid = off; off += up((size_t)X * Y * Zp * 2);
  const size_t o_keys = off; off += up((size_t)X * Y * Zk * 4);
  if (off > VF_NOALLOC_SCRATCH_BYTES)
    return fail(VF_ERR_RANGE, "vf_flood_noalloc: the grid needs " + std::to_string(off) +
                                  " bytes of scratch; the no-allocation flood holds " +
                                  std::to_string(VF_NOALLOC_SCRATCH_BYTES) +
                                  " bytes (about 5 million voxels)");
  unsigned char* S = static_cast<unsigned char*>(base);
  JobDesc* ddesc = reinterpret_cast<JobDesc*>(S + o_desc);
  JobState* dstate = reinterpret_cast<JobState*>(S + o_state);
  uint32_t* scal = reinterpret_cast<uint32_t*>(S + o_scal);
  uint32_t* bj = reinterpret_cast<uint32_t*>(S + o_bj);
  uint8_t* live = S + o_live;
  uint32_t* list = reinterpret_cast<uint32_t*>(S + o_list);
  uint32_t* lcount = scal + 64;
  uint16_t* grid = reinterpret_cast<uint16_t*>(S + o_grid);
  uint32_t* keys = reinterpret_cast<uint32_t*>(S + o_keys);

  JobDesc d;
  std::memset(&d, 0, sizeof(d));
  d.X = X; d.Y = Y; d.Z = Z; d.Zp = Zp; d.Zk = Zk; d.Zw = (Z + 31) / 32;
  d.nbx = nbx; d.nby = nby; d.nbz = nbz; d.brick_base = 0; d.nbricks = (uint32_t)nb;
  d.grid = grid;
  d.grid2 = grid;
  d.keys = keys;
  d.seeds = const_cast<uint32_t*>(d_seeds_xyzw);  // read only
  d.seeds_cap = nseeds;
  d.seeds_given = nseeds;
  d.algorithm = VF_FLOOD;
  d.distance = distance;
  d.active = 1;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
#define NA_CK(call)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(VF_ERR_CUDA, std::string("vf_flood_noalloc: ") + cudaGetErrorString(e_)); \
  } while (0)
  KeysMap km;
  std::memset(&km, 0, sizeof(km));
  {
    std::string why;
    if (!vfk::encode_keys_map(km.b, keys, X, Y, Zk, &why))
      return fail(VF_ERR_CUDA, "vf_flood_noalloc: " + why);
  }
  KeysMap* dmap = reinterpret_cast<KeysMap*>(S + o_map);
  k_noalloc_init<<<1, 256, 0, st>>>(d, ddesc, dstate, scal, km, dmap);
  // padded copy of the caller's grid (padding z >= Z is zero)
  NA_CK(cudaMemsetAsync(grid, 0, (size_t)X * Y * Zp * 2, st));
  NA_CK(cudaMemcpy2DAsync(grid, (size_t)Zp * 2, d_grid, (size_t)Z * 2, (size_t)Z * 2,
                          (size_t)X * Y, cudaMemcpyDeviceToDevice, st));
  NA_CK(cudaMemsetAsync(bj, 0, nb * 4, st));  // every brick belongs to job 0
  vfk::mark_live(st, ddesc, bj, (uint32_t)nb, live);
  vfk::compact_live(st, live, (uint32_t)nb, list, lcount);
  // Without seeds nothing is claimed: occupied voxels come out FREE (1), as
  // FloodFracturer::build leaves them after homogenize (keys 1 -> label 1).
  if (nseeds) vfk::sample_seeds(st, ddesc, dstate, 1);  // seeds given: count + prefix flag
  vfk::FloodScratch fs;
  fs.queue[0] = reinterpret_cast<uint32_t*>(S + o_q0);
  fs.queue[1] = reinterpret_cast<uint32_t*>(S + o_q1);
  fs.queue[2] = reinterpret_cast<uint32_t*>(S + o_q2);
  fs.qcount = scal + 0;
  fs.qhead = scal + 4;
  fs.barrier = scal + 8;
  fs.err = scal + 12;
  fs.stats = scal + 16;
  fs.epoch = reinterpret_cast<uint32_t*>(S + o_epoch);
  fs.fdir = reinterpret_cast<uint32_t*>(S + o_fdir);
  fs.max_passes = 1u << 20;
  fs.total_bricks = (uint32_t)nb;
  fs.njobs = 1;
  fs.tmaps = dmap;
  if (nseeds) vfk::flood_seed_bricks(st, ddesc, dstate, 1, live, list, lcount);
  vfk::flood_init_keys(st, ddesc, list, lcount, (uint32_t)nb, bj, live);
  if (nseeds) {
    vfk::flood_seed(st, ddesc, dstate, 1, fs, live);
    int blocks = 0;
    NA_CK(vfk::flood_relax(st, ddesc, dstate, bj, live, fs, num_sms, &blocks));
  }
  vfk::flood_finalize(st, ddesc, dstate, list, lcount, (uint32_t)nb, bj, 0);
  NA_CK(cudaMemcpy2DAsync(d_labels, (size_t)Z * 2, grid, (size_t)Zp * 2, (size_t)Z * 2,
                          (size_t)X * Y, cudaMemcpyDeviceToDevice, st));
  NA_CK(cudaGetLastError());
  uint32_t err = 0, ferr = 0, has_prefix = 0;
  NA_CK(cudaMemcpyAsync(&err, &dstate->err, 4, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(&has_prefix, &dstate->has_prefix, 4, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(&ferr, fs.err, 4, cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
  if (err & VF_JERR_INVALID) return fail(VF_ERR_INVALID, "vf_flood_noalloc: seed outside the grid or label not a valid fragment label (<= 0x7FFF, low byte >= 2)");
  if (has_prefix)
    return fail(VF_ERR_INVALID, "vf_flood_noalloc: seed labels with sub-seed prefixes (> 255) need vf_fracture");
  if (ferr) return fail(VF_ERR_TIMEOUT, "vf_flood_noalloc: flood did not converge (bounded wait expired)");
  if (err & VF_JERR_DIST_OVERFLOW) return fail(VF_ERR_RANGE, "vf_flood_noalloc: geodesic distance overflow");
  return VF_OK;
}
