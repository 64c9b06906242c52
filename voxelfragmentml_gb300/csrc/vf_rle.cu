// vf_rle.cu -- RegularGrid::exportRLE (RegularGrid.cpp:672-714) on sm_103a.
//
// Format: u32 X, Y, Z, then one {u16 value, u32 repetitions} record per run of
// equal values along the x-major voxel order (index (x*Y + y)*Z + z), packed,
// little endian.  The grid lives in HBM as rows of Zp >= Z voxels.
//
//   k_rle_rows    one warp per (x, y) row: run starts in the row (a voxel
//                 starts a run when it differs from the voxel before it in
//                 x-major order; voxel 0 always does), counted with ballots
//   scan          exclusive prefix sum of the row counts -> first run of a row
//   k_rle_starts  one warp per row: run r's (value << 32 | start index)
//   k_rle_records one thread per run: repetitions = next start - start,
//                 record written as three u16 (every record starts at an even
//                 byte offset, so 2-byte stores are aligned)
//
// Grids of 2^32 voxels or more are rejected by the caller: below that no run
// reaches the u32 repetition limit, so runs never split.
#include "vf_kernels.h"

namespace {

__global__ void __launch_bounds__(256) k_rle_rows(const uint16_t* g, uint32_t Y, uint32_t Z,
                                                  uint32_t Zp, uint64_t rows, uint32_t* cnt) {
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const uint16_t* row = g + r * Zp;
    // the voxel before z = 0 is the last voxel of the previous row
    uint32_t prev_last = r ? (uint32_t)g[(r - 1) * Zp + (Z - 1)] : 0x10000u;
    uint32_t n = 0;
    for (uint32_t z0 = 0; z0 < Z; z0 += 32) {
      const uint32_t z = z0 + lane;
      const uint32_t v = z < Z ? (uint32_t)row[z] : 0u;
      uint32_t before = __shfl_up_sync(0xFFFFFFFFu, v, 1);
      if (lane == 0) before = prev_last;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, z < Z && v != before);
      n += __popc(m);
      prev_last = __shfl_sync(0xFFFFFFFFu, v, 31);
    }
    if (lane == 0) cnt[r] = n;
  }
}

__global__ void __launch_bounds__(256) k_rle_starts(const uint16_t* g, uint32_t Y, uint32_t Z,
                                                    uint32_t Zp, uint64_t rows,
                                                    const unsigned long long* base,
                                                    unsigned long long* starts) {
  const int lane = threadIdx.x & 31;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nw) {
    const uint16_t* row = g + r * Zp;
    uint32_t prev_last = r ? (uint32_t)g[(r - 1) * Zp + (Z - 1)] : 0x10000u;
    unsigned long long out = base[r];
    for (uint32_t z0 = 0; z0 < Z; z0 += 32) {
      const uint32_t z = z0 + lane;
      const uint32_t v = z < Z ? (uint32_t)row[z] : 0u;
      uint32_t before = __shfl_up_sync(0xFFFFFFFFu, v, 1);
      if (lane == 0) before = prev_last;
      const bool st = z < Z && v != before;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, st);
      if (st)
        starts[out + __popc(m & ((1u << lane) - 1u))] =
            ((unsigned long long)v << 32) | (unsigned long long)(r * Z + z);
      out += __popc(m);
      prev_last = __shfl_sync(0xFFFFFFFFu, v, 31);
    }
  }
}

__global__ void __launch_bounds__(256) k_rle_records(const unsigned long long* starts,
                                                     const unsigned long long* nruns,
                                                     uint64_t nvox, uint16_t* rec) {
  const uint64_t R = *nruns;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < R;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long s = starts[i];
    const uint64_t a = s & 0xFFFFFFFFull;
    const uint64_t b = i + 1 < R ? (starts[i + 1] & 0xFFFFFFFFull) : nvox;
    const uint32_t rep = (uint32_t)(b - a);
    uint16_t* o = rec + 3 * i;
    o[0] = (uint16_t)(s >> 32);
    o[1] = (uint16_t)(rep & 0xFFFFu);
    o[2] = (uint16_t)(rep >> 16);
  }
}

}  // namespace

namespace vfk {

void rle_count(cudaStream_t st, const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, uint32_t Zp,
               uint32_t* row_cnt, int num_sms) {
  const uint64_t rows = (uint64_t)X * Y;
  if (rows) k_rle_rows<<<num_sms * 8, 256, 0, st>>>(g, Y, Z, Zp, rows, row_cnt);
}

void rle_write(cudaStream_t st, const uint16_t* g, uint32_t X, uint32_t Y, uint32_t Z, uint32_t Zp,
               const unsigned long long* row_base, const unsigned long long* nruns,
               unsigned long long* starts, uint16_t* records, int num_sms) {
  const uint64_t rows = (uint64_t)X * Y;
  if (!rows) return;
  k_rle_starts<<<num_sms * 8, 256, 0, st>>>(g, Y, Z, Zp, rows, row_base, starts);
  k_rle_records<<<num_sms * 8, 256, 0, st>>>(starts, nruns, rows * Z, records);
}

}  // namespace vfk
