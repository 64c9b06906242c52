// vf_runtime.h -- host runtime of the pipeline (internal).
//
// A Batch owns the device memory of a set of jobs (grow-only arenas), the
// per-stage job tables and a CUDA stream.  enqueue() issues every upload,
// stage and download of the batch asynchronously; finish() waits and fills
// the results.  The context owns one Batch for vf_batch_run / vf_plain_run;
// the server owns one per in-flight micro-batch.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vf.h"
#include "vf_kernels.h"

namespace vfr {

void set_error(const std::string& msg);
vf_status fail(vf_status s, const std::string& msg);

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

struct JobPlan {
  uint32_t X, Y, Z, Zp, Zk, Zw, nbx, nby, nbz, nbricks;
  float amin[3], amax[3];
  size_t o_grid, o_keys, o_par, o_tets, o_range, o_ys, o_seeds, o_counts, o_lat, o_verts,
      o_faces, o_emask, o_etab;
  uint32_t ecap, ncounts, seeds_cap, lat_nx, lat_ny, lat_nz, ek;
  float elimit;
  std::vector<float> emask;
  int final_cur;
  bool prefix_possible;
  bool packed;  // labels written to out_labels by the pack kernel
  bool dma;     // packed into the staging buffer, then copied to out_labels by DMA
  size_t o_out; // the job's labels in the staging buffer (u16)
};

struct Sizes {
  size_t grid = 0, keys = 0, par = 0, tets = 0, range = 0, ys = 0, seeds = 0, counts = 0,
         lat = 0, verts = 0, faces = 0, emask = 0, etab = 0;
  uint32_t bricks = 0, faces_total = 0, max_iters = 0;
  uint64_t rows = 0;  // sum of X * Y over the jobs
  size_t out = 0;     // staging buffer of the DMA download (u16)
};

struct Ctx;

// stage selection for Batch::enqueue_batched (the grid API runs subsets)
enum : uint32_t {
  ST_VOX = 1, ST_SEED = 2, ST_FRACTURE = 4, ST_PERTURB = 8, ST_ERODE = 16, ST_DETECT = 32,
  ST_COUNT = 64, ST_DOWNLOAD = 128, ST_ALL = 255
};

struct Batch {
  Ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf grid0, grid1, keys, par, tets, range, ys, seeds, counts, lat, verts, faces, emask;
  DevBuf etab;  // mesh edge parity tables (voxelizer)
  DevBuf rle_cnt, rle_base, rle_sums, rle_tot, rle_starts, rle_rec;  // RLE export scratch
  DevBuf tables, state, brick_job, live, list, lcount, q[3], scal, epoch, fdir, front[2];
  DevBuf pcnt, pbase, psums, srec;  // flattened per-face work lists, shell setup
  DevBuf stage_out;  // packed labels of the DMA download
  DevBuf tmaps;      // [jobs] TMA descriptors of the flood keys (vfk::KEYS_MAP_BYTES each)
  size_t tmap_off = 0;  // their host copy inside h_tables
  // download by DMA: labels are copied to out_labels by the copy engine, from
  // the label grid when its rows have no padding, else packed first into a
  // device staging buffer (no kernel writes host memory, so the download of
  // one batch overlaps the kernels of the next)
  bool dma_download = false;
  void* h_tables = nullptr;  // pinned staging
  size_t h_tables_cap = 0;
  JobState* h_state = nullptr;  // pinned
  size_t h_state_cap = 0;
  uint32_t* h_scal = nullptr;   // pinned: [0..3] flood stats, [4] err, [8] fcount
  cudaEvent_t ev_flood0 = nullptr, ev_flood1 = nullptr, ev_done = nullptr;
  // stage boundaries: 0 start, 1 inputs uploaded, 2 tetrahedra built,
  // 3 parity rasterised, 4 shell tested, 5 voxelized (combine + live list),
  // 6 seeded, 7 fractured, 8 perturbed, 9 eroded/boundaries, 10 counted,
  // 11 downloaded
  static constexpr int NSTAGE_EV = 12;
  cudaEvent_t ev_stage[NSTAGE_EV] = {};
  bool stage_rec[NSTAGE_EV] = {};
  std::vector<JobPlan> plans;
  std::vector<const vf_job*> jobs;
  Sizes sz;
  size_t bytes = 0;
  uint32_t ntables = 0;
  uint32_t stages = ST_ALL;
  // caller-provided seeds per job (vf_fracture): host xyzw, count
  std::vector<std::pair<const uint32_t*, uint32_t>> given;
  // per-launch bookkeeping
  uint64_t launches = 0;
  bool flood_timed = false;
  int relax_blocks = 0;

  vf_status init(Ctx* c, bool own);
  void release();
  vf_status plan(const vf_job* const* js, uint32_t n);
  vf_status enqueue_batched(bool upload_inputs = true, bool download = true);
  cudaError_t relax_serialized(cudaStream_t st, const JobDesc* tf, JobState* ds, const uint32_t* bj,
                               const uint8_t* lv, const vfk::FloodScratch& fs);
  // the resident stage chain (no uploads) as a CUDA graph: captured on the
  // first execute after plan(), replayed afterwards; falls back to direct
  // launches when the chain has host steps (sub-seed prefix competition) or
  // cannot be captured
  vf_status execute_resident(bool download);
  void drop_graphs();
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // [download]
  uint64_t glaunches[2] = {0, 0};
  bool graphs_ok = true;
  bool last_run_graph = false;
  bool capturing = false;
  cudaError_t record_event(cudaEvent_t e, cudaStream_t st);
  vf_status upload_inputs();
  vf_status enqueue_plain_and_wait(vf_job_result* res, bool skip_vox);
  vf_status finish(vf_job_result* res);
  size_t table_off(uint32_t t) const;
  const JobDesc* dtable(uint32_t t) const;
};

// launch settings chosen by vf_autotune (results never depend on them)
struct Tuning {
  int32_t parity_grid = 16;   // k_parity_flat CTAs per SM
  int32_t shell_grid = 12;    // k_shell_flat CTAs per SM
  int32_t flood_sweeps = 96;  // relaxation sweeps per brick visit (waves per pass)
  int32_t flood_ctas = 0;     // k_relax resident CTAs per SM (0: as many as fit)
  uint32_t flood_wait_spins = 0;  // grid-barrier spin limit of k_relax (0: the default)
};

struct Ctx {
  int device = 0;
  int num_sms = 0;
  Tuning tune;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  size_t in_use = 0;
  // growth of the next alloc calls (0: 1/8 more); Batch::plan sets it for
  // its arenas
  double grow = 0.0;
  // dry run of alloc calls: add up what they would allocate (dry_need) and
  // free (dry_freed) instead
  bool dry = false;
  size_t dry_need = 0, dry_freed = 0;
  cudaEvent_t ev[16] = {};
  // the last flood relaxation issued on any of the context's streams: the
  // next one waits for it, so two cooperative (grid-barrier) launches of
  // batches in flight never share the GPU
  cudaEvent_t ev_relax = nullptr;
  bool ev_relax_used = false;
  std::mutex relax_mu;  // wait + launch + record as one step (server thread, callers)
  // the end of the stage chain of the last batch issued on any stream: the
  // next batch's stages start after it (its upload may run earlier), so the
  // batches in flight compute one after another while each one's download
  // overlaps the next one's kernels
  cudaEvent_t ev_compute = nullptr;
  bool ev_compute_used = false;
  Batch batch;
  // stats of the last batch
  uint64_t last_launches = 0;
  float last_flood_ms = 0.f;
  float last_stage_ms[11] = {};
  bool resident = false;  // batch inputs uploaded by vf_batch_prepare
  uint64_t last_flood_visits = 0;
  uint64_t last_flood_passes = 0;
  uint64_t last_flood_sweeps = 0;
  uint64_t last_flood_counters[VF_FLOOD_NCOUNTERS] = {};  // raw flood counters of the last batched run
  uint32_t last_pass_sizes[256] = {};    // bricks queued per flood pass (first 256)
  uint64_t last_flood_maxit = 0;
  vf_status alloc(DevBuf& b, size_t bytes);
  void free_buf(DevBuf& b);
};

size_t job_footprint(const vf_job& j);

}  // namespace vfr
