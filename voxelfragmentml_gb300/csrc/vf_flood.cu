// vf_flood.cu -- FloodFracturer (FloodFracturer.cpp:98-191) on sm_103a.
//
// The reference runs a breadth-first flood, one compute dispatch and one
// host read-back per wave, and lets the last writer win a tie.  With the
// rule "a voxel claimed in wave t takes the claim of the lowest seed index
// among its wave-(t-1) neighbours", the label of every voxel is the label of
// the seed nearest to it in grid-graph distance through occupied voxels
// (6-neighbourhood for Manhattan, 26 for Euclidean and Chebyshev), ties to
// the lowest seed index.  That fixed point does not depend on the order in
// which voxels are relaxed, so the GPU computes it by relaxation:
//
//   key(v) = ~((dist << 12) | seed_slot)      (0 = EMPTY, 1 = unreached)
//   key(v) <- max(key(v), max_{u in N(v)} key(u) - 4096)
//
// Bricks of 16x16x32 voxels are relaxed to local convergence in shared
// memory (many BFS waves per visit).  A sweep runs only the rows next to new
// halo data (sweep 0, from the brick's change record) or to a row that
// changed in the previous sweep, compacted onto the lowest warps; a row
// update is one forward and one backward pass along its 32-voxel z row.  A
// brick whose boundary voxels changed records what changed in its
// neighbours' change records and puts them on the next pass's queue
// (deduplicated by a pass epoch, appended with warp ballot/popc).  All passes
// of all jobs of a batch run in ONE cooperative persistent kernel; passes are
// separated by a software grid barrier whose spin is bounded (it sets an
// error word and the kernel returns instead of hanging).
//
// Sub-seed prefixes (extra seeds merged into fragments, Seeder.cpp:115-152)
// then go through the reference's competition and disjoint cleanup
// (floodFracturer-comp.glsl:49-62, disjointSet*-comp.glsl): within a
// connected component of one fragment the lowest prefix wins; per fragment
// only voxels with the fragment's minimum prefix survive; the rest is
// re-flooded from all survivors (ties to the lowest label value).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "vf_kernels.h"

namespace {

using vfk::FLOOD_FDIR;

constexpr int KP = 36;                 // smem row pitch (u32): conflict-free 16 B loads
constexpr int KNX = VF_BX + 2, KNY = VF_BY + 2;
constexpr int KROWS = KNX * KNY;
constexpr int TILE_BYTES = KROWS * KP * 4;
constexpr int TILE_SMEM = TILE_BYTES + 128;  // dynamic shared memory: the tile, aligned to 128
constexpr int MAXIT = 96;              // default cap of relaxation sweeps per brick visit

struct FloodArgs {
  const JobDesc* jobs;
  JobState* st;
  const uint32_t* brick_job;
  const uint8_t* live;
  uint32_t* queue[3];
  uint32_t* qcount;  // [3]
  uint32_t* qhead;   // [3]
  uint32_t* epoch;
  uint32_t* bar;     // [2]
  uint32_t* err;
  uint32_t* stats;   // [0] visits, [1] passes, [2] busy warp-sweeps, [3] timeout, [4] sweeps,
                     // [5] visits at the sweep cap, [6] active row-sweeps, [7] key changes,
                     // [8..10] first out-of-range access (code, two values),
                     // [11..15] SM cycles / 256 per phase of the CTAs' work,
                     // [16] visits that found nothing new and staged nothing,
                     // [17] visits that staged their brick but changed no key
  uint32_t max_passes;
  int max_sweeps;    // sweeps per brick visit before the brick re-queues itself
  uint32_t* pass_sizes;  // bricks queued for each of the first 256 passes (or null)
  uint32_t* fdir;        // [nbricks][FLOOD_FDIR] change record (read and cleared by each visit)
  uint32_t nbricks;      // bricks of the batch (queue entries and brick ids are below)
  uint32_t njobs;        // jobs of the batch
  uint32_t wait_spins;   // spins of the pass barrier before it gives up
  const unsigned char* tmaps;  // [njobs] keys tensor maps (KEYS_MAP_BYTES each)
};

// ---- TMA tile loads (cp.async.bulk.tensor) with mbarrier completion -------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok) : "r"(mbar), "r"(phase) : "memory");
  return ok != 0;
}
// bounded wait for the phase `phase` of the mbarrier to complete
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (uint32_t i = 0; i < (1u << 22); ++i)
    if (mbar_try_wait(mbar, phase)) return true;
  return false;
}
// box of the 3-D tensor `map` at (c0 innermost, c1, c2) into shared memory,
// completion counted in bytes on the mbarrier
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void* map, int c0, int c1, int c2,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(mbar) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// A brick id, job id or key address outside its buffer: the access is
// skipped, the flood's error word gets bit 3 (the batch reports the job as
// failed) and the first case is kept in stats[8..10] (code, two values).
__device__ __noinline__ void flood_anomaly(const FloodArgs& a, uint32_t code, uint32_t v0,
                                           uint32_t v1) {
  atomicOr(a.err, 8u);
  if (atomicCAS(a.stats + 8, 0u, code) == 0u) {
    a.stats[9] = v0;
    a.stats[10] = v1;
  }
}

// software grid barrier with a bounded spin (wait_spins polls, 2^26 or about
// 4 s by default); false on timeout
__device__ bool grid_sync(uint32_t* bar, uint32_t nblocks, uint32_t* err, uint32_t* stats,
                          uint32_t wait_spins) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const uint32_t gen = ld_acquire(bar + 1);
    __threadfence();
    const uint32_t arrived = atomicAdd(bar, 1u) + 1u;
    if (arrived == nblocks) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint32_t spins = 0;
      while (ld_acquire(bar + 1) == gen) {
        if (++spins > wait_spins || ld_acquire(err) != 0) {
          atomicOr(err, 2u);
          atomicAdd(stats + 3, 1u);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ uint32_t brick_id(const JobDesc& J, int bx, int by, int bz) {
  return J.brick_base + ((uint32_t)bx * J.nby + (uint32_t)by) * J.nbz + (uint32_t)bz;
}

__device__ __forceinline__ void enqueue(const FloodArgs& a, uint32_t b, uint32_t next_pass,
                                        bool want) {
  // warp-aggregated append of the bricks this warp wants on the next queue
  const int lane = threadIdx.x & 31;
  bool push = false;
  if (want && b >= a.nbricks) {
    flood_anomaly(a, 4u, b, next_pass);
    want = false;
  }
  if (want) push = atomicMax(&a.epoch[b], next_pass + 1u) < next_pass + 1u;
  const unsigned m = __ballot_sync(0xFFFFFFFFu, push);
  if (!m) return;
  const uint32_t q = next_pass % 3u;
  uint32_t base = 0;
  const int leader = __ffs(m) - 1;
  if (lane == leader) base = atomicAdd(&a.qcount[q], (uint32_t)__popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  if (push) a.queue[q][base + __popc(m & ((1u << lane) - 1u))] = b;
}

// relaxation candidate from a neighbour key: one step further (0 when the
// neighbour is EMPTY or unreached)
__device__ __forceinline__ uint32_t step_from(uint32_t m) {
  return m >= 2u * VF_KEY_STEP ? m - VF_KEY_STEP : 0u;
}
// key of a voxel (kk) relaxed by the best neighbour key m; EMPTY stays EMPTY.
// step_from is monotone, so relaxing by max(m1, m2) equals relaxing by m1
// and then by m2.
__device__ __forceinline__ uint32_t relax(uint32_t kk, uint32_t m) {
  return kk ? max(kk, step_from(m)) : 0u;
}
// One step of an in-row chain: relax(kk, max(w, prev)) with the part that
// does not depend on prev, a = relax(kk, w), computed ahead of the chain.
// step_from is monotone, so relax(kk, max(w, prev)) = kk ? max(a, step_from(
// prev)) : 0, and a = 0 when kk = 0: on the chain there is one select (the
// step, taken only for occupied voxels) and one max.
__device__ __forceinline__ uint32_t chain_step(uint32_t a, bool occ, uint32_t prev) {
  const uint32_t s = (occ && prev >= 2u * VF_KEY_STEP) ? prev - VF_KEY_STEP : 0u;
  return max(a, s);
}
// a key at the largest distance the key format holds (its neighbours would
// overflow the distance field)
__device__ __forceinline__ bool at_limit(uint32_t m) {
  return m - VF_KEY_MIN_REACHED < VF_KEY_STEP;
}
__device__ __forceinline__ uint4 max4(uint4 a, uint4 b) {
  return make_uint4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w));
}
__device__ __forceinline__ uint4 lds4(const uint32_t* p) {
  return *reinterpret_cast<const uint4*>(p);
}

// Shared state of the sweeps of one brick visit.
struct SweepShared {
  uint32_t rfw[16];      // [2][8] rows that changed in the previous sweep (bit per row)
  uint32_t wmask[8];     // active rows of each warp in this sweep (bit per lane)
  uint32_t hl[256];      // per row: z halo candidate below the brick (z0-1)
  uint32_t hh[256];      //          z halo candidate above the brick (z0+32)
  uint32_t rowchg[256];  // per row: z positions changed during the visit
  uint8_t occ8[256];     // per row: bit q set when its keys 4q .. 4q+3 hold an occupied voxel
};

// position of the k-th (from 0) set bit of m; k < popc(m)
__device__ __forceinline__ int nth_set_bit(uint32_t m, uint32_t k) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1) {
    const uint32_t lo = (uint32_t)__popc(m & ((1u << w) - 1u));
    if (k >= lo) {
      k -= lo;
      m >>= w;
      pos += w;
    }
  }
  return pos;
}

// Column maximum of the 3 x 3 rows around own_row at row slot s (one z).
__device__ __forceinline__ uint32_t colmax1(const uint32_t* own_row, int s) {
  uint32_t m = 0;
#pragma unroll
  for (int r = 0; r < 9; ++r) m = max(m, own_row[((r / 3 - 1) * KNY + (r % 3 - 1)) * KP + s]);
  return m;
}
// Column maxima of the 3 x 3 rows around own_row at row slots s .. s+3.
__device__ __forceinline__ uint4 colmax4(const uint32_t* own_row, int s) {
  uint4 C = make_uint4(0, 0, 0, 0);
#pragma unroll
  for (int r = 0; r < 9; ++r) C = max4(C, lds4(own_row + ((r / 3 - 1) * KNY + (r % 3 - 1)) * KP + s));
  return C;
}

// Relaxes one row of the staged tile (own_row) in place, on a pair of
// adjacent lanes: lane h = 0 takes the chunks 0..3 (z 0..15), h = 1 the
// chunks 4..7 (z 16..31).  A row update is a forward pass (cross-row
// candidates fused with the increasing-z in-row chain) and a backward pass
// (the decreasing-z chain), both starting from the row's z halo candidates
// hlo / hhi.  occ8 has bit q set when the row's 4-key chunk q holds an
// occupied voxel: empty chunks keep their zero keys and break the in-row
// chain, so both passes skip them (a thin wall crosses a row in a few
// chunks).
// Each lane runs both chains over its half from a lower bound of the chain
// value at the boundary (a key as read: keys only grow), then takes the
// exact boundary value from the other lane by a shuffle.  Along an occupied
// run the chain is max-plus linear: the value a chain carries in from the
// boundary adds step^d(P) at distance d, so the lane raises its keys from
// the boundary while step^d(P) exceeds them (past the first key it does not
// exceed, none it reaches can be exceeded; an empty voxel ends the run).
// The result equals one lane's sequential pass over the whole row for the
// same reads.  All lanes of pair_mask call this (two shuffles each).
// Returns the lane's changed z positions.
template <int CONN>
__device__ __forceinline__ uint32_t relax_half(uint32_t* own_row, int h, uint32_t hlo,
                                               uint32_t hhi, uint32_t occ8, bool full_backward,
                                               unsigned pair_mask) {
  const int q0 = 4 * h, q1 = q0 + 4;
  const uint32_t om = (occ8 >> q0) & 0xFu;
  uint32_t chg = 0;
  // forward: lane 0 from the halo candidate hlo, lane 1 from the key at z 15
  uint32_t prev = h == 0 ? hlo : own_row[4 + 15];
  int last = q0 - 2;  // the chunk relaxed last
  if (CONN == 26) {
    uint4 C = make_uint4(0, 0, 0, 0);
    uint32_t cp = hlo;
#pragma unroll 1
    for (uint32_t m = om; m; m &= m - 1u) {
      const int q = q0 + __ffs(m) - 1;
      if (q != last + 1) {
        C = colmax4(own_row, 4 + 4 * q);
        if (q > 0) {
          cp = colmax1(own_row, 3 + 4 * q);
          if (q != q0) prev = 0u;  // after an empty chunk
        }
      }
      uint4 Cn = make_uint4(hhi, 0, 0, 0);
      if (q + 1 < 8) {
        if (q + 1 < q1 && ((om >> (q + 1 - q0)) & 1u)) Cn = colmax4(own_row, 8 + 4 * q);
        else Cn.x = colmax1(own_row, 8 + 4 * q);
      }
      const uint4 kv = lds4(own_row + 4 + 4 * q);
      const uint32_t w[4] = {max(cp, max(C.x, C.y)), max(C.x, max(C.y, C.z)),
                             max(C.y, max(C.z, C.w)), max(C.z, max(C.w, Cn.x))};
      const uint32_t kk[4] = {kv.x, kv.y, kv.z, kv.w};
      uint32_t f[4], av[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) av[j] = relax(kk[j], w[j]);  // off the chain
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        f[j] = chain_step(av[j], kk[j] != 0u, prev);
        prev = f[j];
        if (f[j] != kk[j]) chg |= 1u << (4 * q + j);
      }
      if ((chg >> (4 * q)) & 0xFu)
        *reinterpret_cast<uint4*>(own_row + 4 + 4 * q) = make_uint4(f[0], f[1], f[2], f[3]);
      cp = C.w; C = Cn; last = q;
    }
  } else {
#pragma unroll 1
    for (uint32_t m = om; m; m &= m - 1u) {
      const int q = q0 + __ffs(m) - 1;
      if (q != last + 1 && q != q0) prev = 0u;  // after an empty chunk
      const uint4 M = max4(max4(lds4(own_row - KNY * KP + 4 + 4 * q), lds4(own_row + KNY * KP + 4 + 4 * q)),
                           max4(lds4(own_row - KP + 4 + 4 * q), lds4(own_row + KP + 4 + 4 * q)));
      const uint4 kv = lds4(own_row + 4 + 4 * q);
      const uint32_t w[4] = {M.x, M.y, M.z, M.w};
      const uint32_t kk[4] = {kv.x, kv.y, kv.z, kv.w};
      uint32_t f[4], av[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) av[j] = relax(kk[j], w[j]);  // off the chain
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        f[j] = chain_step(av[j], kk[j] != 0u, prev);
        prev = f[j];
        if (f[j] != kk[j]) chg |= 1u << (4 * q + j);
      }
      if ((chg >> (4 * q)) & 0xFu)
        *reinterpret_cast<uint4*>(own_row + 4 + 4 * q) = make_uint4(f[0], f[1], f[2], f[3]);
      last = q;
    }
  }
  // lane 1 takes lane 0's exact chain value at z 15 (zero when chunk 3 is empty)
  const uint32_t P = __shfl_xor_sync(pair_mask, last == 3 ? prev : 0u, 1);
  if (h == 1) {
    uint32_t v = P;
#pragma unroll 1
    for (int z = 16; z < 32; ++z) {
      const uint32_t k = own_row[4 + z];
      v = (k != 0u && v >= 2u * VF_KEY_STEP) ? v - VF_KEY_STEP : 0u;
      if (v <= k) break;  // also ends the run at an empty voxel (v = 0)
      own_row[4 + z] = v;
      chg |= 1u << z;
    }
  }
  // Backward over the lane's half: from its top chunk (full_backward; lane 1
  // from the halo candidate hhi, lane 0 from the key at z 16) or from its
  // highest chunk the forward pass changed, down to where nothing changes and
  // no forward change lies below.  The row was consistent along z before
  // this pass, so nothing above the highest changed chunk needs it.
  int q = q1 - 1;
  bool run = full_backward;
  if (!run && chg) {
    run = true;
    q = (31 - __clz(chg)) >> 2;
  }
  if (run) {
    prev = q == 7 ? hhi : own_row[4 + 4 * q + 4];
#pragma unroll 1
    for (; q >= q0; --q) {
      if (!((om >> (q - q0)) & 1u)) {
        if ((chg & (0xFFFFFFFFu >> (28 - 4 * q))) == 0u) break;
        prev = 0u;
        continue;
      }
      const uint4 kv = lds4(own_row + 4 + 4 * q);
      const uint32_t kk[4] = {kv.x, kv.y, kv.z, kv.w};
      uint32_t f[4];
      uint32_t cq = 0;
#pragma unroll
      for (int j = 3; j >= 0; --j) {
        f[j] = chain_step(kk[j], kk[j] != 0u, prev);
        prev = f[j];
        if (f[j] != kk[j]) cq |= 1u << j;
      }
      if (cq) {
        *reinterpret_cast<uint4*>(own_row + 4 + 4 * q) = make_uint4(f[0], f[1], f[2], f[3]);
        chg |= cq << (4 * q);
      } else if ((chg & (0xFFFFFFFFu >> (28 - 4 * q))) == 0u) {
        break;  // this chunk and everything below it unchanged: consistent
      }
    }
  }
  // lane 0 takes lane 1's final key at z 16
  const uint32_t P2 = __shfl_xor_sync(pair_mask, h == 1 ? own_row[4 + 16] : 0u, 1);
  if (h == 0) {
    uint32_t v = P2;
#pragma unroll 1
    for (int z = 15; z >= 0; --z) {
      const uint32_t k = own_row[4 + z];
      v = (k != 0u && v >= 2u * VF_KEY_STEP) ? v - VF_KEY_STEP : 0u;
      if (v <= k) break;
      own_row[4 + z] = v;
      chg |= 1u << z;
    }
  }
  return chg;
}

// The values of a visit that the code after the sweeps needs.  Thread 0
// keeps them in shared memory, and the code after the sweeps reads them back
// there: held in registers across the sweeps they cost spills at 64
// registers per thread (4 CTAs per SM).
struct VisitInfo {
  const JobDesc* J;
  uint32_t b, jid, pass;
  int bx, by, bz;
  int sweeps;  // sweeps run (the loop counter at its end)
};

template <int CONN>
__device__ bool visit_tail(const FloodArgs& a, uint32_t* tile, uint32_t* live27, uint32_t* dirs,
                           int* reenq, SweepShared& sw, unsigned long long* ph, uint32_t* scnt,
                           const VisitInfo* vi);

// One visit of brick b.  False when its tile load did not complete in
// time (the error word is set; the kernel stops).
template <int CONN>
__device__ bool relax_brick(const FloodArgs& a, const JobDesc& J, uint32_t jid, uint32_t b,
                            uint32_t pass, uint32_t* tile, uint32_t* live27, uint32_t* dirs,
                            int* reenq, SweepShared& sw, uint32_t* fbits,
                            unsigned long long* ph, uint32_t i, uint32_t qn, uint32_t* pre,
                            uint32_t mbar, uint32_t& phase, uint32_t* scnt, VisitInfo* vi) {
  // ph (thread 0): SM cycles of [1] live map + staging, [2] sweeps, [3] write-back + enqueue
  // phase timing (thread 0): ph[k] += cycles since the last mark, kept in
  // shared memory so no 64-bit clock lives in registers across the sweeps
  if (threadIdx.x == 0) ph[5] = clock64();
  const uint32_t lb = b - J.brick_base;
  const int bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
  const int x0 = bx * VF_BX, y0 = by * VF_BY, z0 = bz * VF_BZ;
  const int t = threadIdx.x;
  // What changed next to the brick since its last visit (read and cleared).
  // A flag set after the keys it covers were written (writer: fence, then
  // flag) makes the staging loads below see those keys (reader: flag, fence,
  // barrier, loads); a flag this visit does not see stays for the next visit,
  // which the same writer queued.
  uint32_t fv = 0;
  if (t < (int)FLOOD_FDIR) {  // exchange with acquire semantics
    asm volatile("atom.acquire.gpu.global.exch.b32 %0, [%1], %2;"
                 : "=r"(fv) : "l"(a.fdir + (size_t)b * FLOOD_FDIR + t), "r"(0u) : "memory");
    fbits[t] = fv;
  }
  if (t >= 32 && t < 32 + 27) {  // live map of the 27 bricks around (warp 1)
    const int n = t - 32;
    const int dx = n / 9 - 1, dy = (n / 3) % 3 - 1, dz = n % 3 - 1;
    const int nx = bx + dx, ny = by + dy, nz = bz + dz;
    uint32_t l = 0;
    if (nx >= 0 && ny >= 0 && nz >= 0 && nx < (int)J.nbx && ny < (int)J.nby && nz < (int)J.nbz)
      l = a.live[brick_id(J, nx, ny, nz)];
    live27[n] = l;
  }
  if (t == 0) {
    atomicMax(&a.st[jid].passes, pass + 1);
    *dirs = 0; *reenq = 0; scnt[0] = 0; scnt[1] = 0; scnt[2] = 0;
    vi->J = &J; vi->b = b; vi->jid = jid; vi->pass = pass;
    vi->bx = bx; vi->by = by; vi->bz = bz;
  }
  if (!__syncthreads_or(fv != 0)) {  // nothing new around the brick
    if (t == 0) atomicAdd(a.stats + 16, 1u);
    return true;
  }
  // Stage the keys of the brick and its one-voxel halo.  One TMA load (a
  // 3-D box of 36 x 18 x 18 keys at z0-4, y0-1, x0-1 of the job's keys
  // tensor) fills the 18 x 18 rows [x0-1, x0+17) x [y0-1, y0+17) with the
  // keys z0-4 .. z0+31: [3] holds z0-1 and [4 + z] the key z0 + z; keys
  // outside the grid arrive as zero (EMPTY).  The keys z0+32 (slot [0]) are
  // loaded by the threads meanwhile.  Keys of neighbour bricks without
  // occupied voxels are never initialised, so their parts of the tile are
  // cleared once the load has landed.  Thread 224 also claims this CTA's
  // next brick of the pass (while much of the pass is left), so the next
  // visit starts without a claim round trip.
  if (t == 0) {
    // the neighbours' key writes acquired with the change record, and this
    // CTA's own accesses to the tile, ordered before the async-proxy copy
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(mbar, (uint32_t)TILE_BYTES);
    tma_load_3d(smem_u32(tile), a.tmaps + (size_t)jid * vfk::KEYS_MAP_BYTES, z0 - 4, y0 - 1,
                x0 - 1, mbar);
  }
  uint32_t htop[2];
  bool bad = false;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int q = t + u * 256;
    htop[u] = 0;
    if (q < KROWS) {
      const int lx = q / KNY - 1, ly = q % KNY - 1;
      const int x = x0 + lx, y = y0 + ly, z = z0 + VF_BZ;
      if (x >= 0 && y >= 0 && x < (int)J.X && y < (int)J.Y && z < (int)J.Zk) {
        const int dx = lx < 0 ? 0 : (lx >= VF_BX ? 2 : 1);
        const int dy = ly < 0 ? 0 : (ly >= VF_BY ? 2 : 1);
        if (live27[dx * 9 + dy * 3 + 2]) {
          const size_t ki = vf_kidx(J, x, y, z);
          if (ki < (size_t)J.X * J.Y * J.Zk) htop[u] = __ldcg(J.keys + ki);
          else bad = true;
        }
      }
    }
  }
  if (t == 224 && i + 2u * gridDim.x < qn) {
    const uint32_t c = atomicAdd(&a.qhead[pass % 3u], 1u);
    if (c < qn) *pre = c;
  }
  if (bad) flood_anomaly(a, 3u, b, (uint32_t)t);
  const bool landed = mbar_wait(mbar, phase);
  if (__syncthreads_or(!landed)) {
    // the copy did not complete in time: report it, give it one more bounded
    // wait so that nothing is in flight into this CTA's tile, and stop
    if (t == 0) atomicOr(a.err, 16u);
    mbar_wait(mbar, phase);
    return false;
  }
  phase ^= 1u;
  // clear the parts of bricks without occupied voxels, place the keys z0+32
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int q = t + u * 256;
    if (q < KROWS) {
      uint32_t* row = tile + q * KP;
      const int lx = q / KNY, ly = q % KNY;
      const int dx = lx == 0 ? 0 : (lx == KNX - 1 ? 2 : 1);
      const int dy = ly == 0 ? 0 : (ly == KNY - 1 ? 2 : 1);
      if (!live27[dx * 9 + dy * 3 + 1]) {
#pragma unroll
        for (int c = 0; c < VF_BZ / 4; ++c)
          *reinterpret_cast<uint4*>(row + 4 + 4 * c) = make_uint4(0, 0, 0, 0);
      }
      if (!live27[dx * 9 + dy * 3 + 0]) row[3] = 0u;
      row[0] = htop[u];
    }
  }
  __syncthreads();
  if (t == 0) { const unsigned long long now = clock64(); ph[1] += now - ph[5]; ph[5] = now; }
  const int tx = t / VF_BY, ty = t % VF_BY;
  uint32_t* own_row = tile + ((tx + 1) * KNY + (ty + 1)) * KP;
  // Row layout (KP u32): [0] key z0+32, [3] key z0-1, [4 + z] key z0 + z.  The
  // z halo candidates are fixed for the visit (other bricks' keys).
  uint32_t hlo, hhi;
  if (CONN == 26) {
    hlo = 0; hhi = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      const uint32_t* rp = own_row + ((r / 3 - 1) * KNY + (r % 3 - 1)) * KP;
      hlo = max(hlo, rp[3]);
      hhi = max(hhi, rp[0]);
    }
  } else {
    hlo = own_row[3];
    hhi = own_row[0];
  }
  // scnt: [0] active row-sweeps, [2] busy warp-sweeps (thread 0), [1] key changes
  sw.hl[t] = hlo;
  sw.hh[t] = hhi;
  sw.rowchg[t] = 0;
  uint32_t occ8 = 0;
#pragma unroll
  for (int q = 0; q < VF_BZ / 4; ++q) {
    const uint4 kv = lds4(own_row + 4 + 4 * q);
    if ((kv.x | kv.y | kv.z | kv.w) != 0u) occ8 |= 1u << q;
  }
  sw.occ8[t] = (uint8_t)occ8;
  // Sweep 0 runs the rows that read a changed key: x/y face, edge and corner
  // neighbours mark whole faces and edges, the z neighbours the changed rows
  // (26: widened by one row in x and y); bit 13 marks every row.
  bool act0;
  {
    const uint32_t d = fbits[0];
    const uint32_t dxm = 2u | (tx == 0 ? 1u : 0u) | (tx == VF_BX - 1 ? 4u : 0u);
    const uint32_t dym = 2u | (ty == 0 ? 1u : 0u) | (ty == VF_BY - 1 ? 4u : 0u);
    uint32_t hit = 0;
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
      for (int dy = 0; dy < 3; ++dy)
        if ((dxm >> dx) & (dym >> dy) & 1u) hit |= (d >> (dx * 9 + dy * 3)) & 7u;
    // the z neighbours name exactly the rows whose end voxel they improve
    const uint32_t zc = (((fbits[1 + (tx >> 1)] | fbits[9 + (tx >> 1)]) >> ((tx & 1) * 16)) & 0xFFFFu);
    hit |= (zc >> ty) & 1u;
    act0 = hit != 0 && occ8 != 0u;  // a row without occupied voxels never changes
  }
  // Sweeps.  The rows to run are compacted onto the lowest threads (one list
  // per sweep), so a sweep with n active rows keeps ceil(n / 32) warps busy.
  // A row runs when a neighbour row changed in the previous sweep (its own
  // changes are already final along z against the neighbour values it read);
  // sweep 0 runs the rows next to new halo data (act0).  sw.rfw[s & 1] holds
  // the rows that changed in sweep s - 1 (bit row & 31 of word row >> 5, row
  // t = x * 16 + y, so word w holds x-rows 2w and 2w + 1).
  const int lane = t & 31, wid = t >> 5;
  int it = 0, cur = 0;
  for (; it < a.max_sweeps; ++it) {
    const uint32_t* pw = sw.rfw + cur * 8;
    bool active;
    if (it == 0) {
      active = act0;
    } else {
      const uint32_t m0 = tx > 0 ? (pw[(tx - 1) >> 1] >> (((tx - 1) & 1) * 16)) & 0xFFFFu : 0u;
      const uint32_t m1 = (pw[tx >> 1] >> ((tx & 1) * 16)) & 0xFFFFu;
      const uint32_t m2 = tx < VF_BX - 1 ? (pw[(tx + 1) >> 1] >> (((tx + 1) & 1) * 16)) & 0xFFFFu : 0u;
      if (CONN == 26)
        active = ((((m0 | m2) << 1) & (7u << ty)) | ((m1 << 1) & (5u << ty))) != 0;
      else
        active = ((((m0 | m2) >> ty) & 1u) | ((m1 << 1) & (5u << ty))) != 0;
      active = active && sw.occ8[t] != 0;
    }
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, active);
    if (lane == 0) sw.wmask[wid] = bal;
    if (t < 8) sw.rfw[(cur ^ 1) * 8 + t] = 0u;  // filled by this sweep's changes
    __syncthreads();
    // The lane pair (t, t ^ 1) takes the idx-th active row, idx = t / 2 (and
    // 128 more per round when more than 128 rows are active): the k-th
    // active lane of warp ws.
    uint32_t n = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) n += (uint32_t)__popc(sw.wmask[i]);
    uint32_t chg = 0;
    for (uint32_t base = 0; base < n; base += 128u) {
      const uint32_t idx = base + ((uint32_t)t >> 1);
      const unsigned pm = __ballot_sync(0xFFFFFFFFu, idx < n);
      if (idx < n) {
        uint32_t acc = 0, k = 0;
        int ws = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const uint32_t c = (uint32_t)__popc(sw.wmask[i]);
          if (idx >= acc && idx < acc + c) {
            ws = i;
            k = idx - acc;
          }
          acc += c;
        }
        const int row = 32 * ws + nth_set_bit(sw.wmask[ws], k);
        uint32_t* rr = tile + (((row >> 4) + 1) * KNY + ((row & 15) + 1)) * KP;
        const uint32_t c = relax_half<CONN>(rr, t & 1, sw.hl[row], sw.hh[row], sw.occ8[row],
                                            it == 0, pm);
        if (c) {
          atomicOr(&sw.rfw[(cur ^ 1) * 8 + (row >> 5)], 1u << (row & 31));
          atomicOr(&sw.rowchg[row], c);
          chg |= c;
        }
      }
    }
    cur ^= 1;
    if (t == 0) { scnt[0] += n; scnt[2] += (2u * n + 31u) / 32u; }
    if (chg) atomicAdd(&scnt[1], (uint32_t)__popc(chg));
    if (!__syncthreads_or(chg != 0)) break;
  }
  if (t == 0) vi->sweeps = it;
  return visit_tail<CONN>(a, tile, live27, dirs, reenq, sw, ph, scnt, vi);
}

// The rest of a visit, after the sweeps: the distance limit, write-back,
// notifications and statistics.
template <int CONN>
__device__ bool visit_tail(const FloodArgs& a, uint32_t* tile, uint32_t* live27, uint32_t* dirs,
                           int* reenq, SweepShared& sw, unsigned long long* ph, uint32_t* scnt,
                           const VisitInfo* vi) {
  const int t = threadIdx.x;
  const JobDesc& J = *vi->J;
  const uint32_t b = vi->b, jid = vi->jid, pass = vi->pass;
  const int bx = vi->bx, by = vi->by, bz = vi->bz;
  const int x0 = bx * VF_BX, y0 = by * VF_BY, z0 = bz * VF_BZ;
  const int tx = t / VF_BY, ty = t % VF_BY;
  uint32_t* own_row = tile + ((tx + 1) * KNY + (ty + 1)) * KP;
  uint32_t overflow = 0;
  const uint32_t changed = sw.rowchg[t];
  // Distance limit: an unreached voxel next to a key at the largest distance
  // the key format holds.  Checked on the converged tile, and only when some
  // key of the tile (row or halo) is at that distance.
  {
    bool lim = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint4 v = lds4(own_row + 4 + 4 * q);
      lim |= at_limit(v.x) | at_limit(v.y) | at_limit(v.z) | at_limit(v.w);
    }
    lim |= at_limit(own_row[0]) | at_limit(own_row[3]);
    if (t < 2 * KNY + 2 * VF_BX) {  // the 68 halo rows of the 18 x 18 tile
      const int lx = t < KNY ? 0 : t < 2 * KNY ? KNX - 1 : 1 + (t - 2 * KNY) % VF_BX;
      const int ly = t < KNY ? t : t < 2 * KNY ? t - KNY : (t < 2 * KNY + VF_BX ? 0 : KNY - 1);
      const uint32_t* hr = tile + (lx * KNY + ly) * KP;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const uint4 v = lds4(hr + 4 + 4 * q);
        lim |= at_limit(v.x) | at_limit(v.y) | at_limit(v.z) | at_limit(v.w);
      }
      lim |= at_limit(hr[0]) | at_limit(hr[3]);
    }
    if (__syncthreads_or(lim)) {
      // key at z (-1 .. 32) of a row: [3] z0-1, [4 + z], [0] z0+32
      auto at = [](const uint32_t* r, int z) { return r[z < 0 ? 3 : (z >= VF_BZ ? 0 : 4 + z)]; };
      for (int z = 0; z < VF_BZ; ++z) {
        if (own_row[4 + z] != VF_KEY_UNREACHED) continue;
        uint32_t m = max(at(own_row, z - 1), at(own_row, z + 1));
        if (CONN == 26) {
          for (int r = 0; r < 9; ++r) {
            const uint32_t* rp = own_row + ((r / 3 - 1) * KNY + (r % 3 - 1)) * KP;
            m = max(m, max(at(rp, z - 1), max(at(rp, z), at(rp, z + 1))));
          }
        } else {
          m = max(m, max(max(own_row[-KNY * KP + 4 + z], own_row[KNY * KP + 4 + z]),
                         max(own_row[-KP + 4 + z], own_row[KP + 4 + z])));
        }
        if (at_limit(m)) overflow = 1;
      }
    }
  }
  if (t == 0) { const unsigned long long now = clock64(); ph[2] += now - ph[5]; ph[5] = now; }
  const int x = x0 + tx, y = y0 + ty;
  if (changed && x < (int)J.X && y < (int)J.Y) {
    // write back the changed 32-byte sectors of the row
    const int nq = min(VF_BZ, (int)J.Zk - z0) / 4;
    const size_t ki = vf_kidx(J, x, y, z0);
    uint4* dst = reinterpret_cast<uint4*>(J.keys + ki);
    if (ki + 4 * (size_t)nq <= (size_t)J.X * J.Y * J.Zk && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nq && ((changed >> (8 * (q >> 1))) & 0xFFu)) __stcg(dst + q, lds4(own_row + 4 + 4 * q));
    } else {
      flood_anomaly(a, 5u, b, (uint32_t)ki);
    }
  }
  if (overflow) atomicOr(&a.st[jid].err, VF_JERR_DIST_OVERFLOW);
  // Notifications.  A neighbour brick is queued (and its change record set)
  // only when a voxel this visit changed can improve one of its voxels,
  // judged against the neighbour's keys staged in the halo.  Staged keys can
  // only be lower than the neighbour's current ones (keys never decrease),
  // so a halo voxel that no changed voxel improves here cannot be improved
  // in the neighbour either: skipping it loses nothing.  This drops the
  // visits a front would otherwise send back to the brick it came from.
  // changed key of interior row r (brick coordinates) at z, or 0
  auto chg_key = [&](int rx, int ry, int z) -> uint32_t {
    const uint32_t c = sw.rowchg[rx * VF_BY + ry];
    return ((c >> z) & 1u) ? tile[((rx + 1) * KNY + (ry + 1)) * KP + 4 + z] : 0u;
  };
  // (a) the z faces, per interior row: the halo voxels below (z0-1) and
  //     above (z0+32) the row, against the changed keys of the window rows
  //     at z0 and z0+31 (26: the interior rows of the 3x3 around; 6: the row)
  bool lo_imp = false, hi_imp = false;
  {
    const uint32_t klo = own_row[3], khi = own_row[0];
    if (klo | khi) {
      uint32_t mlo = 0, mhi = 0;
      if (CONN == 26) {
#pragma unroll
        for (int r = 0; r < 9; ++r) {
          const int rx = tx + r / 3 - 1, ry = ty + r % 3 - 1;
          if (rx < 0 || ry < 0 || rx >= VF_BX || ry >= VF_BY) continue;
          mlo = max(mlo, chg_key(rx, ry, 0));
          mhi = max(mhi, chg_key(rx, ry, VF_BZ - 1));
        }
      } else {
        mlo = chg_key(tx, ty, 0);
        mhi = chg_key(tx, ty, VF_BZ - 1);
      }
      lo_imp = klo != 0u && step_from(mlo) > klo;
      hi_imp = khi != 0u && step_from(mhi) > khi;
    }
  }
  // (b) the x/y faces, edges and corners: one thread per halo row of the
  //     tile's perimeter.  C(z) = the largest changed key at z among the
  //     interior rows next to the halo row; a halo voxel at z is improvable
  //     when step(max of C over its z window) beats its key.  Chunks of four
  //     keys with one chunk of look-ahead, as in relax_half.
  if (t < 2 * KNY + 2 * VF_BX) {
    const int lx = t < KNY ? 0 : t < 2 * KNY ? KNX - 1 : 1 + (t - 2 * KNY) % VF_BX;
    const int ly = t < KNY ? t : t < 2 * KNY ? t - KNY : (t < 2 * KNY + VF_BX ? 0 : KNY - 1);
    const uint32_t* hr = tile + (lx * KNY + ly) * KP;
    // Interior rows next to this halo row, as a line of up to three rows
    // (brick coordinates): the halo row's inward neighbour (ix, iy) and, for
    // 26, its two neighbours along the halo edge (dx, dy) when inside.  A
    // corner halo row has one (26) or none (6).  Rows outside get a zero mask.
    const bool xs = lx == 0 || lx == KNX - 1, ys = ly == 0 || ly == KNY - 1;
    const int ix = lx == 0 ? 0 : (lx == KNX - 1 ? VF_BX - 1 : lx - 1);
    const int iy = ly == 0 ? 0 : (ly == KNY - 1 ? VF_BY - 1 : ly - 1);
    const int ex = xs ? 0 : 1, ey = xs ? 1 : 0;  // direction along the edge
    uint32_t cm[3] = {0u, 0u, 0u};
    int base_row = (ix + 1) * KNY + (iy + 1);    // tile row of the middle row
    const int stride_row = ex * KNY + ey;        // tile rows between the three
    if (CONN == 26 || xs != ys) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int rx = ix + (k - 1) * ex, ry = iy + (k - 1) * ey;
        const bool in = (CONN == 26 || k == 1) && rx >= 0 && ry >= 0 && rx < VF_BX && ry < VF_BY &&
                        !(xs && ys && k != 1);
        cm[k] = in ? sw.rowchg[rx * VF_BY + ry] : 0u;
      }
    }
    const uint32_t u = cm[0] | cm[1] | cm[2];
    if (u) {
      // changed keys of the adjacent rows at chunk q, column maximum
      auto chunkC = [&](int q) -> uint4 {
        uint4 c = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const uint32_t m = cm[k] >> (4 * q);
          if (!(m & 0xFu)) continue;
          const uint4 v = lds4(tile + (base_row + (k - 1) * stride_row) * KP + 4 + 4 * q);
          c.x = max(c.x, (m & 1u) ? v.x : 0u);
          c.y = max(c.y, (m & 2u) ? v.y : 0u);
          c.z = max(c.z, (m & 4u) ? v.z : 0u);
          c.w = max(c.w, (m & 8u) ? v.w : 0u);
        }
        return c;
      };
      auto imp = [](uint32_t w, uint32_t kh) { return kh != 0u && step_from(w) > kh; };
      bool face = false, below = false, above = false;
      uint4 Cc = chunkC(0);
      uint32_t cprev = 0;
      if (CONN == 26) below = imp(Cc.x, hr[3]);  // z0-1 reads C(z0)
#pragma unroll 1
      for (int q = 0; q < 8; ++q) {
        // changed keys at z = 4q-1 .. 4q+4 reach this chunk's halo voxels
        const uint32_t win = q == 0 ? (u & 0x1Fu) : ((u >> (4 * q - 1)) & 0x3Fu);
        if (win) {
          const uint4 Cn = (CONN == 26 && q < 7) ? chunkC(q + 1) : make_uint4(0, 0, 0, 0);
          const uint4 kh = lds4(hr + 4 + 4 * q);
          uint32_t w0, w1, w2, w3;
          if (CONN == 26) {
            w0 = max(cprev, max(Cc.x, Cc.y));
            w1 = max(Cc.x, max(Cc.y, Cc.z));
            w2 = max(Cc.y, max(Cc.z, Cc.w));
            w3 = max(Cc.z, max(Cc.w, Cn.x));
          } else {
            w0 = Cc.x; w1 = Cc.y; w2 = Cc.z; w3 = Cc.w;
          }
          face |= imp(w0, kh.x) | imp(w1, kh.y) | imp(w2, kh.z) | imp(w3, kh.w);
          cprev = Cc.w;
          Cc = CONN == 26 ? Cn : (q < 7 ? chunkC(q + 1) : Cc);
        } else {
          cprev = 0u;
          Cc = q < 7 ? chunkC(q + 1) : Cc;
        }
      }
      if (CONN == 26) above = imp(cprev, hr[0]);  // z0+32 reads C(z0+31)
      const int sx = lx == 0 ? 0 : (lx == KNX - 1 ? 2 : 1);
      const int sy = ly == 0 ? 0 : (ly == KNY - 1 ? 2 : 1);
      const uint32_t dmh = (below ? 1u << (sx * 9 + sy * 3 + 0) : 0u) |
                           (face ? 1u << (sx * 9 + sy * 3 + 1) : 0u) |
                           (above ? 1u << (sx * 9 + sy * 3 + 2) : 0u);
      if (dmh) atomicOr(dirs, dmh);
    }
  }
  // rows of the z neighbours that read an improvable key (exact row masks)
  const unsigned zlo = __ballot_sync(0xFFFFFFFFu, lo_imp);
  const unsigned zhi = __ballot_sync(0xFFFFFFFFu, hi_imp);
  if ((t & 31) == 0 && (zlo | zhi))
    atomicOr(dirs, (zlo ? 1u << (1 * 9 + 1 * 3 + 0) : 0u) | (zhi ? 1u << (1 * 9 + 1 * 3 + 2) : 0u));
  // statistics: active row-sweeps and key changes (block sums in shared memory)
  if (t == 0) {
    const int it = vi->sweeps;
    if (it == a.max_sweeps) *reenq = 1;
    atomicAdd(a.stats + 4, (uint32_t)it + 1u);  // sweeps (statistics)
    if (it == a.max_sweeps) atomicAdd(a.stats + 5, 1u);
  }
  __syncthreads();
  if (t == 0) {
    atomicAdd(a.stats + 6, scnt[0]);
    atomicAdd(a.stats + 7, scnt[1]);
    atomicAdd(a.stats + 2, scnt[2]);
    if (scnt[1] == 0) atomicAdd(a.stats + 17, 1u);  // staged, but no key changed
  }
  // change records of the neighbours, after the key writes above (fence), then
  // the neighbours go on the next pass's queue
  if (t < 32 || (t & 31) == 0) asm volatile("fence.acq_rel.gpu;" ::: "memory");
  if ((t & 31) == 0) {
    const int w = t >> 5;
    if (zlo && live27[1 * 9 + 1 * 3 + 0]) {  // below: its keys at z0'+32 are our bottom layer
      const uint32_t nb = brick_id(J, bx, by, bz - 1);
      if (nb < a.nbricks) atomicOr(&a.fdir[(size_t)nb * FLOOD_FDIR + 9 + w], zlo);
    }
    if (zhi && live27[1 * 9 + 1 * 3 + 2]) {  // above: its keys at z0'-1 are our top layer
      const uint32_t nb = brick_id(J, bx, by, bz + 1);
      if (nb < a.nbricks) atomicOr(&a.fdir[(size_t)nb * FLOOD_FDIR + 1 + w], zhi);
    }
  }
  if (t < 32) {
    const uint32_t dm = *dirs;
    bool want = false;
    uint32_t nb = 0;
    if (t < 27 && ((dm >> t) & 1u) && live27[t]) {
      want = true;
      nb = brick_id(J, bx + t / 9 - 1, by + (t / 3) % 3 - 1, bz + t % 3 - 1);
      // seen from nb this brick is in direction 26 - t; z faces use the row masks
      if (t != 1 * 9 + 1 * 3 + 0 && t != 1 * 9 + 1 * 3 + 2 && nb < a.nbricks)
        atomicOr(&a.fdir[(size_t)nb * FLOOD_FDIR], 1u << (26 - t));
    }
    if (t == 27 && *reenq) {  // sweep cap: the brick comes back with every row
      want = true;
      nb = b;
      atomicOr(&a.fdir[(size_t)b * FLOOD_FDIR], 1u << 13);
    }
    enqueue(a, nb, pass + 1, want);
  }
  if (t == 0) ph[3] += clock64() - ph[5];
  return true;
}

__global__ void __launch_bounds__(256, 4) k_relax(FloodArgs args) {
  // The arguments are read from a shared copy: the kernel and the functions
  // it calls take them by reference, and a shared-memory struct is an
  // ordinary addressable object (no address of the parameter space is taken).
  __shared__ FloodArgs a;
  if (threadIdx.x == 0) a = args;
  __syncthreads();
  // the tile, a TMA destination: 128-byte aligned inside the dynamic shared
  // memory (TILE_SMEM = TILE_BYTES + 128)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* tile = reinterpret_cast<uint32_t*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  __shared__ uint32_t live27[27];
  __shared__ uint32_t dirs;
  __shared__ int reenq;
  __shared__ uint32_t item;
  __shared__ uint32_t pre;  // queue index of the next brick, claimed ahead (~0: none)
  __shared__ SweepShared sw;
  __shared__ uint32_t fbits[FLOOD_FDIR];
  // thread 0: SM cycles per phase (see flush below); [5] the phase mark of a
  // visit, [6] the clock at the last claim
  __shared__ unsigned long long ph[7];
  __shared__ uint32_t scnt[3];   // per visit: active row-sweeps, key changes, busy warp-sweeps
  __shared__ VisitInfo vinfo;
  // the pass, its queue length and its visits: read back from shared memory
  // around each visit (registers held across a visit cost spills)
  __shared__ uint32_t pass_p, pass_qn, pass_visits;
  __shared__ __align__(8) unsigned long long tile_bar;  // completion of the tile loads
  const uint32_t mbar = smem_u32(&tile_bar);
  uint32_t phase = 0;  // parity of the tile load in flight (uniform across the CTA)
  if (threadIdx.x < 5) ph[threadIdx.x] = 0;
  if (threadIdx.x == 0) {
    pre = 0xFFFFFFFFu;
    pass_p = 0;
    mbar_init(mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  for (;;) {
    const uint32_t p0 = pass_p;
    if (p0 >= a.max_passes) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.qcount[(p0 + 2) % 3] = 0;
      a.qhead[(p0 + 2) % 3] = 0;
    }
    if (threadIdx.x == 0) {
      pass_qn = ld_acquire(&a.qcount[p0 % 3u]);
      pass_visits = 0;
      if (a.pass_sizes && blockIdx.x == 0 && p0 < 256) a.pass_sizes[p0] = pass_qn;
    }
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) {
        ph[6] = clock64();
        item = pre != 0xFFFFFFFFu ? pre : atomicAdd(&a.qhead[pass_p % 3u], 1u);
        pre = 0xFFFFFFFFu;
      }
      __syncthreads();
      const uint32_t i = item, p = pass_p, qn = pass_qn, cur = p % 3u;
      if (i >= qn) break;
      const uint32_t b = a.queue[cur][i];
      if (b >= a.nbricks) {
        if (threadIdx.x == 0) flood_anomaly(a, 1u, b, i);
        continue;
      }
      const uint32_t jid = a.brick_job[b];
      if (jid >= a.njobs) {
        if (threadIdx.x == 0) flood_anomaly(a, 2u, b, jid);
        continue;
      }
      const JobDesc& J = a.jobs[jid];
      const int conn6 = J.distance == 1;
      if (threadIdx.x == 0) ph[0] += clock64() - ph[6];
      const bool ok =
          conn6 ? relax_brick<6>(a, J, jid, b, p, tile, live27, &dirs, &reenq, sw, fbits, ph, i,
                                 qn, &pre, mbar, phase, scnt, &vinfo)
                : relax_brick<26>(a, J, jid, b, p, tile, live27, &dirs, &reenq, sw, fbits, ph, i,
                                  qn, &pre, mbar, phase, scnt, &vinfo);
      if (!ok) return;  // tile load timed out (error word set; the others stop at the barrier)
      if (threadIdx.x == 0) ++pass_visits;
    }
    const uint32_t p = pass_p;
    if (threadIdx.x == 0 && pass_visits) atomicAdd(&a.stats[0], pass_visits);
    const bool synced = grid_sync(a.bar, gridDim.x, a.err, a.stats, a.wait_spins);
    if (threadIdx.x == 0) {
      // phase cycles: [0] claim, [1] staging, [2] sweeps, [3] write-back +
      // enqueue, [4] from the failed claim through the pass barrier; added to
      // stats[11..15] in units of 256 cycles
      ph[4] += clock64() - ph[6];
      for (int i = 0; i < 5; ++i) {
        const uint32_t c = (uint32_t)(ph[i] >> 8);
        if (c) atomicAdd(a.stats + 11 + i, c);
        ph[i] &= 255u;
      }
    }
    if (!synced) return;
    const uint32_t nn = ld_acquire(&a.qcount[(p + 1) % 3]);
    if (nn == 0 || ld_acquire(a.err) != 0) {
      if (blockIdx.x == 0 && threadIdx.x == 0) a.stats[1] = p + 1;
      return;
    }
    if (threadIdx.x == 0) pass_p = p + 1;
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.stats[1] = a.max_passes;
    atomicOr(a.err, 4u);  // did not converge
  }
}

// ---------------------------------------------------------------------------
// keys from the label grid: EMPTY -> 0, occupied -> 1 (unreached)
//
// Row kernels over live bricks (k_init_keys, k_finalize): one brick per CTA
// iteration, eight lanes per (x, y) row with the lanes along z.  A lane
// handles 4 voxels (8 bytes of labels, 16 bytes of keys), so one warp
// instruction covers 4 rows of the brick with contiguous bytes per row.  A
// thread takes rows r, r + 32, ... r + 224 and issues all 8 loads before
// its stores.
constexpr int ROW_UNITS = VF_BX * VF_BY * (VF_BZ / 4) / 256;

__global__ void __launch_bounds__(256) k_init_keys(const JobDesc* jobs, const uint32_t* list,
                                                   const uint32_t* count, const uint32_t* brick_job) {
  const uint32_t n = *count;
  const uint32_t q = threadIdx.x & 7, r0 = threadIdx.x >> 3;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const JobDesc& J = jobs[brick_job[b]];
    if (!J.active) continue;
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t z = bz * VF_BZ + 4 * q;
    // Zk is a multiple of 4 and Zp >= Zk: the lane's 4 keys and 4 labels
    // are inside the row when z < Zk
    if (z >= J.Zk) continue;
    uint2 a[ROW_UNITS];
    bool ok[ROW_UNITS];
#pragma unroll
    for (int i = 0; i < ROW_UNITS; ++i) {
      const uint32_t r = r0 + 32u * i;
      const uint32_t x = bx * VF_BX + r / VF_BY, y = by * VF_BY + r % VF_BY;
      ok[i] = x < J.X && y < J.Y;
      a[i] = ok[i] ? *reinterpret_cast<const uint2*>(J.grid + vf_gidx(J, x, y, z)) : make_uint2(0, 0);
    }
#pragma unroll
    for (int i = 0; i < ROW_UNITS; ++i) {
      if (!ok[i]) continue;
      const uint32_t r = r0 + 32u * i;
      const uint32_t x = bx * VF_BX + r / VF_BY, y = by * VF_BY + r % VF_BY;
      __stcg(reinterpret_cast<uint4*>(J.keys + vf_kidx(J, x, y, z)),
             make_uint4((a[i].x & 0xFFFFu) ? 1u : 0u, (a[i].x >> 16) ? 1u : 0u,
                        (a[i].y & 0xFFFFu) ? 1u : 0u, (a[i].y >> 16) ? 1u : 0u));
    }
  }
}

// seed bricks must be live (a caller may seed an EMPTY voxel)
__global__ void k_seed_bricks(const JobDesc* jobs, JobState* st, int njobs, uint8_t* live,
                              uint32_t* list, uint32_t* count) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  const JobDesc& J = jobs[j];
  if (!J.active) return;
  JobState& s = st[j];
  for (int f = 0; f < 256; ++f) s.minprefix[f] = 0xFFFFFFFFu;
  s.passes = 0;
  s.disjoint = 0;
  const uint32_t ns = s.nseeds;
  for (uint32_t i = 0; i < ns; ++i) {
    const uint32_t x = J.seeds[4 * i], y = J.seeds[4 * i + 1], z = J.seeds[4 * i + 2],
                   w = J.seeds[4 * i + 3];
    // label = frag | prefix << 8 (Seeder.cpp:150), fragment id >= 2
    if (x >= J.X || y >= J.Y || z >= J.Z || w > 0x7FFFu || (w & 0xFFu) <= VOXEL_FREE) {
      s.err |= VF_JERR_INVALID;
      continue;
    }
    const uint32_t b = J.brick_base + ((x / VF_BX) * J.nby + y / VF_BY) * J.nbz + z / VF_BZ;
    if (!live[b]) {
      live[b] = 1;
      list[atomicAdd(count, 1u)] = b;
    }
  }
}

// seeds into the keys (later seeds win a shared voxel, as grid.set in list
// order does, FloodFracturer.cpp:101-103) and their bricks onto queue 0
__global__ void k_seed_keys(const JobDesc* jobs, JobState* st, int njobs, uint32_t* epoch,
                            uint32_t* queue0, uint32_t* qcount, uint32_t* fdir) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  const JobDesc& J = jobs[j];
  if (!J.active) return;
  JobState& s = st[j];
  if (s.err) return;
  const uint32_t ns = s.nseeds;
  for (uint32_t i = 0; i < ns; ++i) {
    const uint32_t x = J.seeds[4 * i], y = J.seeds[4 * i + 1], z = J.seeds[4 * i + 2];
    J.keys[vf_kidx(J, x, y, z)] = ~i;
    const uint32_t b = J.brick_base + ((x / VF_BX) * J.nby + y / VF_BY) * J.nbz + z / VF_BZ;
    atomicOr(&fdir[(size_t)b * FLOOD_FDIR], 1u << 13);  // first visit: every row
    if (atomicMax(&epoch[b], 1u) < 1u) queue0[atomicAdd(qcount, 1u)] = b;
  }
}

// keys -> labels (undoMask fused: & 0xFF unless prefixes must survive)
__global__ void __launch_bounds__(256) k_finalize(const JobDesc* jobs, const JobState* st,
                                                  const uint32_t* list, const uint32_t* count,
                                                  const uint32_t* brick_job, int pass2) {
  // label of each seed slot for the job of the current brick (reloaded when
  // the job changes): the seed's label (pass 1) or the pass-2 rank value,
  // reduced to the fragment byte unless the sub-seed prefixes are kept
  __shared__ uint16_t lab[4096];
  __shared__ int cached;
  if (threadIdx.x == 0) cached = -1;
  __syncthreads();
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active) continue;  // uniform across the CTA
    const JobState& s = st[j];
    if (pass2 && !s.has_prefix) continue;  // keys of every prefix job are final here
    if ((int)j != cached) {  // uniform: cached changes only between barriers
      __syncthreads();
      const bool keep_prefix = !pass2 && s.has_prefix;
      const uint32_t nl = pass2 ? 256u : min(s.nseeds, 4096u);
      for (uint32_t k = threadIdx.x; k < nl; k += blockDim.x) {
        uint32_t v = pass2 ? s.rank_value[k] : J.seeds[4 * k + 3];
        if (!keep_prefix) v &= 0xFFu;
        lab[k] = (uint16_t)v;
      }
      if (threadIdx.x == 0) cached = (int)j;
      __syncthreads();
    }
    // rows as in k_init_keys: 8 lanes per row along z, 4 keys per lane
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t z = bz * VF_BZ + 4 * (threadIdx.x & 7), r0 = threadIdx.x >> 3;
    if (z >= J.Zk) continue;
    uint4 k4[ROW_UNITS];
    bool ok[ROW_UNITS];
#pragma unroll
    for (int i = 0; i < ROW_UNITS; ++i) {
      const uint32_t r = r0 + 32u * i;
      const uint32_t x = bx * VF_BX + r / VF_BY, y = by * VF_BY + r % VF_BY;
      ok[i] = x < J.X && y < J.Y;
      k4[i] = ok[i] ? __ldcg(reinterpret_cast<const uint4*>(J.keys + vf_kidx(J, x, y, z)))
                    : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int i = 0; i < ROW_UNITS; ++i) {
      if (!ok[i]) continue;
      const uint32_t r = r0 + 32u * i;
      const uint32_t x = bx * VF_BX + r / VF_BY, y = by * VF_BY + r % VF_BY;
      const uint32_t ks[4] = {k4[i].x, k4[i].y, k4[i].z, k4[i].w};
      uint32_t lv[4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const uint32_t key = ks[h];
        // reached: the slot's label; else 0 EMPTY, 1 FREE
        lv[h] = key >= VF_KEY_MIN_REACHED ? (uint32_t)lab[(~key) & 0xFFFu] : key;
      }
      *reinterpret_cast<uint2*>(J.grid + vf_gidx(J, x, y, z)) =
          make_uint2(lv[0] | (lv[1] << 16), lv[2] | (lv[3] << 16));
    }
  }
}
__global__ void __launch_bounds__(256) k_competition(const JobDesc* jobs, JobState* st,
                                                     const uint32_t* list, const uint32_t* count,
                                                     const uint32_t* brick_job) {
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active || !st[j].has_prefix) continue;
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const int x = bx * VF_BX + threadIdx.x / VF_BY, y = by * VF_BY + threadIdx.x % VF_BY;
    const int z0 = bz * VF_BZ;
    if (x >= (int)J.X || y >= (int)J.Y) continue;
    const bool six = J.distance == 1;
    bool any = false;
    for (int z = z0; z < min(z0 + VF_BZ, (int)J.Z); ++z) {
      volatile uint16_t* gv = J.grid + vf_gidx(J, x, y, z);
      const uint32_t g = *gv;
      if (g <= VOXEL_FREE) continue;
      const uint32_t f = g & 0xFFu;
      uint32_t p = g >> 8;
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dz = -1; dz <= 1; ++dz) {
            const int nz = (dx != 0) + (dy != 0) + (dz != 0);
            if (nz == 0 || (six && nz != 1)) continue;
            const int ux = x + dx, uy = y + dy, uz = z + dz;
            if (ux < 0 || uy < 0 || uz < 0 || ux >= (int)J.X || uy >= (int)J.Y || uz >= (int)J.Z) continue;
            const uint32_t u = *(volatile uint16_t*)(J.grid + vf_gidx(J, ux, uy, uz));
            if (u > VOXEL_FREE && (u & 0xFFu) == f && (u >> 8) < p) p = u >> 8;
          }
      if (p != (g >> 8)) { *gv = (uint16_t)(f | (p << 8)); any = true; }
    }
    if (any) atomicOr(&st[j].changed, 1u);
  }
}

__global__ void __launch_bounds__(256) k_minprefix(const JobDesc* jobs, JobState* st,
                                                   const uint32_t* list, const uint32_t* count,
                                                   const uint32_t* brick_job) {
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active || !st[j].has_prefix) continue;
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t x = bx * VF_BX + threadIdx.x / VF_BY, y = by * VF_BY + threadIdx.x % VF_BY;
    const uint32_t z0 = bz * VF_BZ;
    if (x >= J.X || y >= J.Y) continue;
    for (uint32_t z = z0; z < min(z0 + VF_BZ, J.Z); ++z) {
      const uint32_t g = J.grid[vf_gidx(J, x, y, z)];
      if (g > VOXEL_FREE) atomicMin(&st[j].minprefix[g & 0xFFu], g >> 8);
    }
  }
}

// per job: surviving values sorted -> re-flood slots (ties to lowest value)
__global__ void k_ranks(const JobDesc* jobs, JobState* st, int njobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs || !jobs[j].active || !st[j].has_prefix) return;
  JobState& s = st[j];
  uint32_t nr = 0;
  for (uint32_t f = 0; f < 256; ++f)
    if (s.minprefix[f] != 0xFFFFFFFFu) s.rank_value[nr++] = f | (s.minprefix[f] << 8);
  for (uint32_t a = 1; a < nr; ++a) {  // insertion sort, <= 254 entries
    const uint32_t v = s.rank_value[a];
    uint32_t b = a;
    while (b > 0 && s.rank_value[b - 1] > v) { s.rank_value[b] = s.rank_value[b - 1]; --b; }
    s.rank_value[b] = v;
  }
  for (uint32_t r = 0; r < nr; ++r) s.value_rank[s.rank_value[r] & 0xFFu] = r;
  s.nranks = nr;
}

// disjointSetStack: non-minimal prefixes -> FREE; survivors keyed by slot
__global__ void __launch_bounds__(256) k_disjoint_reset(const JobDesc* jobs, JobState* st,
                                                        const uint32_t* list, const uint32_t* count,
                                                        const uint32_t* brick_job) {
  const uint32_t n = *count;
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const uint32_t b = list[it];
    const uint32_t j = brick_job[b];
    const JobDesc& J = jobs[j];
    if (!J.active || !st[j].has_prefix) continue;
    JobState& s = st[j];
    const uint32_t lb = b - J.brick_base;
    const uint32_t bz = lb % J.nbz, by = (lb / J.nbz) % J.nby, bx = lb / (J.nbz * J.nby);
    const uint32_t x = bx * VF_BX + threadIdx.x / VF_BY, y = by * VF_BY + threadIdx.x % VF_BY;
    const uint32_t z0 = bz * VF_BZ;
    uint32_t reset = 0;
    if (x < J.X && y < J.Y) {
      for (uint32_t z = z0; z < min(z0 + VF_BZ, J.Zk); ++z) {
        uint32_t key = 0;
        if (z < J.Z) {
          uint16_t* gp = J.grid + vf_gidx(J, x, y, z);
          const uint32_t g = *gp;
          if (g == VOXEL_FREE) key = VF_KEY_UNREACHED;
          else if (g > VOXEL_FREE) {
            if ((g >> 8) != s.minprefix[g & 0xFFu]) {
              *gp = VOXEL_FREE;
              key = VF_KEY_UNREACHED;
              ++reset;
            } else {
              key = ~s.value_rank[g & 0xFFu];
            }
          }
        }
        J.keys[vf_kidx(J, x, y, z)] = key;
      }
    }
    if (reset) atomicAdd(&s.disjoint, reset);
  }
}

__global__ void k_enqueue_pass2(const JobDesc* jobs, const JobState* st, const uint32_t* list,
                                const uint32_t* count, const uint32_t* brick_job,
                                uint32_t* epoch, uint32_t* queue0, uint32_t* qcount,
                                uint32_t* fdir) {
  const uint32_t n = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t b = list[i];
    const uint32_t j = brick_job[b];
    if (!jobs[j].active || !st[j].has_prefix || !st[j].disjoint) continue;
    fdir[(size_t)b * FLOOD_FDIR] = 1u << 13;  // keys were reset: every row
    if (atomicMax(&epoch[b], 1u) < 1u) queue0[atomicAdd(qcount, 1u)] = b;
  }
}

}  // namespace

namespace vfk {

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
std::once_flag g_encode_once;
}  // namespace

bool encode_keys_map(void* map128, const uint32_t* keys, uint32_t X, uint32_t Y, uint32_t Zk,
                     std::string* err) {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    cudaGetLastError();
  });
  if (!g_encode_tiled) {
    if (err) *err = "cuTensorMapEncodeTiled is not available from the CUDA driver";
    return false;
  }
  // dims innermost first: z (Zk, a multiple of 4: 16-byte row strides), y, x
  const cuuint64_t dims[3] = {Zk, Y, X};
  const cuuint64_t strides[2] = {(cuuint64_t)Zk * 4u, (cuuint64_t)Zk * 4u * Y};
  const cuuint32_t box[3] = {(cuuint32_t)KP, (cuuint32_t)KNY, (cuuint32_t)KNX};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = g_encode_tiled(
      static_cast<CUtensorMap*>(map128), CU_TENSOR_MAP_DATA_TYPE_UINT32, 3,
      const_cast<uint32_t*>(keys), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (err) *err = "cuTensorMapEncodeTiled failed (CUresult " + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

static inline int brick_grid(uint32_t max_count) {
  uint32_t g = max_count ? max_count : 1;
  return (int)(g > (1u << 20) ? (1u << 20) : g);
}

void flood_init_keys(cudaStream_t st, const JobDesc* dj, const uint32_t* list,
                     const uint32_t* count, uint32_t max_count, const uint32_t* brick_job,
                     const uint8_t*) {
  if (max_count) k_init_keys<<<brick_grid(max_count), 256, 0, st>>>(dj, list, count, brick_job);
}

void flood_seed_bricks(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs, uint8_t* live,
                       uint32_t* list, uint32_t* count) {
  if (njobs > 0) k_seed_bricks<<<(njobs + 127) / 128, 128, 0, st>>>(dj, ds, njobs, live, list, count);
}

void flood_seed(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                const FloodScratch& fs, const uint8_t*) {
  cudaMemsetAsync(fs.epoch, 0, sizeof(uint32_t) * fs.total_bricks, st);
  cudaMemsetAsync(fs.qcount, 0, sizeof(uint32_t) * 3, st);
  cudaMemsetAsync(fs.qhead, 0, sizeof(uint32_t) * 3, st);
  cudaMemsetAsync(fs.barrier, 0, sizeof(uint32_t) * 2, st);
  cudaMemsetAsync(fs.fdir, 0, sizeof(uint32_t) * FLOOD_FDIR * fs.total_bricks, st);
  if (njobs > 0)
    k_seed_keys<<<(njobs + 127) / 128, 128, 0, st>>>(dj, ds, njobs, fs.epoch, fs.queue[0], fs.qcount,
                                                      fs.fdir);
}

static int relax_blocks(int num_sms) {
  static int per_sm[64] = {};  // per device: the attribute is set on each device
  const int dv = cur_dev();
  if (per_sm[dv] < 1) {
    int n = 0;
    cudaFuncSetAttribute(k_relax, cudaFuncAttributeMaxDynamicSharedMemorySize, TILE_SMEM);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_relax, 256, TILE_SMEM) != cudaSuccess)
      n = 1;
    per_sm[dv] = n < 1 ? 1 : n;
  }
  return per_sm[dv] * num_sms;
}

void flood_prepare(int num_sms) { (void)relax_blocks(num_sms); }

cudaError_t flood_relax(cudaStream_t st, const JobDesc* dj, JobState* ds,
                        const uint32_t* brick_job, const uint8_t* live,
                        const FloodScratch& fs, int num_sms, int* blocks_used) {
  FloodArgs a;
  a.jobs = dj;
  a.st = ds;
  a.brick_job = brick_job;
  a.live = live;
  a.queue[0] = fs.queue[0];
  a.queue[1] = fs.queue[1];
  a.queue[2] = fs.queue[2];
  a.qcount = fs.qcount;
  a.qhead = fs.qhead;
  a.epoch = fs.epoch;
  a.bar = fs.barrier;
  a.err = fs.err;
  a.stats = fs.stats;
  a.max_passes = fs.max_passes;
  a.max_sweeps = (fs.max_sweeps > 0 && fs.max_sweeps <= MAXIT) ? fs.max_sweeps : MAXIT;
  a.pass_sizes = fs.pass_sizes;
  a.fdir = fs.fdir;
  a.nbricks = fs.total_bricks;
  a.njobs = fs.njobs;
  a.wait_spins = fs.wait_spins ? fs.wait_spins : (1u << 26);
  a.tmaps = static_cast<const unsigned char*>(fs.tmaps);
  if (!a.tmaps) return cudaErrorInvalidValue;
  int blocks = relax_blocks(num_sms);
  if (fs.ctas_per_sm > 0 && fs.ctas_per_sm * num_sms < blocks) blocks = fs.ctas_per_sm * num_sms;
  if (blocks_used) *blocks_used = blocks;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)k_relax, dim3(blocks), dim3(256), args,
                                     TILE_SMEM, st);
}

void flood_finalize(cudaStream_t st, const JobDesc* dj, const JobState* ds, const uint32_t* list,
                    const uint32_t* count, uint32_t max_count, const uint32_t* brick_job,
                    int pass2) {
  if (max_count) k_finalize<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job, pass2);
}

void flood_competition(cudaStream_t st, const JobDesc* dj, JobState* ds, const uint32_t* list,
                       const uint32_t* count, uint32_t max_count, const uint32_t* brick_job) {
  if (max_count) k_competition<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job);
}

void flood_disjoint(cudaStream_t st, const JobDesc* dj, JobState* ds, int njobs,
                    const uint32_t* list, const uint32_t* count, uint32_t max_count,
                    const uint32_t* brick_job, const FloodScratch& fs, const uint8_t*) {
  if (!max_count) return;
  k_minprefix<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job);
  k_ranks<<<(njobs + 127) / 128, 128, 0, st>>>(dj, ds, njobs);
  k_disjoint_reset<<<brick_grid(max_count), 256, 0, st>>>(dj, ds, list, count, brick_job);
  cudaMemsetAsync(fs.epoch, 0, sizeof(uint32_t) * fs.total_bricks, st);
  cudaMemsetAsync(fs.qcount, 0, sizeof(uint32_t) * 3, st);
  cudaMemsetAsync(fs.qhead, 0, sizeof(uint32_t) * 3, st);
  cudaMemsetAsync(fs.barrier, 0, sizeof(uint32_t) * 2, st);
  cudaMemsetAsync(fs.fdir, 0, sizeof(uint32_t) * FLOOD_FDIR * fs.total_bricks, st);
  k_enqueue_pass2<<<brick_grid((max_count + 255) / 256), 256, 0, st>>>(
      dj, ds, list, count, brick_job, fs.epoch, fs.queue[0], fs.qcount, fs.fdir);
}

}  // namespace vfk
