/*
 * vf.hpp -- header-only C++17 facade over the C ABI in vf.h, shaped like the
 * reference's fracture classes so that their callers keep their call shape:
 *
 *   vf::Grid                     RegularGrid (MeshFragments/Source/
 *                                DataStructures/RegularGrid.h:142-367)
 *   vf::Seeder::uniform /        Seeder::uniform, Seeder::mergeSeeds
 *   vf::Seeder::mergeSeeds       (MeshFragments/Source/Fracturer/Seeder.h:59-76)
 *   vf::Fracturer                fracturer::Fracturer (Fracturer.h:28-57):
 *                                build(grid, seeds, params), init, destroy,
 *                                prepareSSBOs, setDistanceFunction
 *   vf::FloodFracturer,          the singleton fracturers (FloodFracturer.h:13,
 *   vf::NaiveFracturer           NaiveFracturer.h:13)
 *   vf::DistanceFunction         fracturer::DistanceFunction (Fracturer.h:10-14)
 *
 * Seeds are vf::Seed {x, y, z, w}, the layout of glm::uvec4.  Errors become
 * exceptions on this side of the ABI only: vf::SeederSearchError for
 * VF_ERR_SEED_SEARCH (Seeder::SeederSearchError, Seeder.h:19-22), vf::Error
 * for the rest; the C ABI itself never throws.  The GPU work of a grid runs
 * on its context's stream, as the C calls do.
 */
#ifndef VF_HPP
#define VF_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "vf.h"

namespace vf {

class Error : public std::runtime_error {
 public:
  Error(vf_status s, const std::string& what) : std::runtime_error(what), status_(s) {}
  vf_status status() const { return status_; }

 private:
  vf_status status_;
};

class SeederSearchError : public Error {
 public:
  explicit SeederSearchError(const std::string& what) : Error(VF_ERR_SEED_SEARCH, what) {}
};

inline void check(vf_status s) {
  if (s == VF_OK) return;
  const std::string msg = std::string(vf_status_string(s)) + ": " + vf_last_error();
  if (s == VF_ERR_SEED_SEARCH) throw SeederSearchError(msg);
  throw Error(s, msg);
}

enum DistanceFunction : int {
  EUCLIDEAN_DISTANCE = VF_EUCLIDEAN,
  MANHATTAN_DISTANCE = VF_MANHATTAN,
  CHEBYSHEV_DISTANCE = VF_CHEBYSHEV
};

enum Location : int { INNER = VF_INNER, OUTER = VF_OUTER, BOTH = VF_BOTH };

struct Seed {  // glm::uvec4: x, y, z, label
  uint32_t x, y, z, w;
};

// A device context (one per device; replaces the GL context).
class Context {
 public:
  explicit Context(int device = 0, size_t hbm_budget = 0) { check(vf_ctx_create(device, hbm_budget, &h_)); }
  ~Context() { vf_ctx_destroy(h_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  vf_ctx* handle() const { return h_; }

 private:
  vf_ctx* h_ = nullptr;
};

// RegularGrid: a uint16 label grid on the device, x-major.
class Grid {
 public:
  Grid(Context& ctx, uint32_t X, uint32_t Y, uint32_t Z, const float aabb_min[3],
       const float aabb_max[3])
      : dims_{X, Y, Z} {
    check(vf_grid_create(ctx.handle(), X, Y, Z, aabb_min, aabb_max, &h_));
  }
  ~Grid() { vf_grid_destroy(h_); }
  Grid(const Grid&) = delete;
  Grid& operator=(const Grid&) = delete;
  vf_grid* handle() const { return h_; }

  // RegularGrid::getNumSubdivisions
  const uint32_t* getNumSubdivisions() const { return dims_; }
  size_t size() const { return (size_t)dims_[0] * dims_[1] * dims_[2]; }
  // RegularGrid::fill(Model3D*): tri-box shell + tetra-parity interior
  void fill(const std::vector<float>& xyz, const std::vector<uint32_t>& tri) {
    check(vf_voxelize(h_, xyz.data(), (uint32_t)(xyz.size() / 3), tri.data(),
                      (uint32_t)(tri.size() / 3)));
  }
  // RegularGrid::updateSSBO / updateGrid
  void upload(const std::vector<uint16_t>& host) {
    if (host.size() != size()) throw Error(VF_ERR_INVALID, "grid size mismatch");
    check(vf_grid_upload(h_, host.data()));
  }
  std::vector<uint16_t> data() const {
    std::vector<uint16_t> out(size());
    check(vf_grid_download(h_, out.data()));
    return out;
  }
  void detectBoundaries(int boundary_size = 1) { check(vf_detect_boundaries(h_, boundary_size)); }
  void erode(int type, uint32_t size, uint32_t iterations, float probability, float threshold,
             uint64_t seed) {
    check(vf_erode(h_, type, size, iterations, probability, threshold, seed));
  }
  void undoMask() { check(vf_undo_mask(h_)); }
  // RegularGrid::countValues: counts[v] for every value v > 1
  std::vector<uint32_t> countValues(uint32_t ncounts = 256, uint64_t* occupied = nullptr) {
    std::vector<uint32_t> c(ncounts);
    uint64_t occ = 0;
    check(vf_count_values(h_, c.data(), ncounts, &occ));
    if (occupied) *occupied = occ;
    return c;
  }
  // RegularGrid::exportRLE, to memory
  std::vector<uint8_t> exportRLE() {
    size_t n = 0;
    check(vf_grid_export_rle(h_, nullptr, 0, &n));
    std::vector<uint8_t> out(n);
    check(vf_grid_export_rle(h_, out.data(), out.size(), &n));
    return out;
  }

 private:
  vf_grid* h_ = nullptr;
  uint32_t dims_[3];
};

struct Seeder {
  // Seeder::uniform(grid, n, seed, location): labels 2..n+1 in (x, y, z) order
  static std::vector<Seed> uniform(Grid& grid, uint32_t n, uint64_t seed, Location loc = OUTER) {
    std::vector<Seed> s(n);
    check(vf_sample_seeds(grid.handle(), n, seed, loc, n ? &s[0].x : nullptr));
    return s;
  }
  // Seeder::mergeSeeds(frags, seeds, dfunc): seeds take frag | (k << 8)
  static void mergeSeeds(const std::vector<Seed>& frags, std::vector<Seed>& seeds,
                         DistanceFunction dfunc) {
    check(vf_merge_seeds(frags.empty() ? nullptr : &frags[0].x, (uint32_t)frags.size(),
                         seeds.empty() ? nullptr : &seeds[0].x, (uint32_t)seeds.size(), dfunc));
  }
};

// fracturer::Fracturer: the interface every fracturer implements
class Fracturer {
 public:
  virtual ~Fracturer() = default;
  // Split the occupied voxels of `grid` into fragments, in place.
  // params may be null (the distance function set here is used).
  virtual void build(Grid& grid, const std::vector<Seed>& seeds, const vf_params* params) = 0;
  // GPU resources are owned by the grid's context: nothing to set up or free
  virtual void init(const vf_params*) {}
  virtual void prepareSSBOs(const vf_params*) {}
  virtual void destroy() {}
  virtual bool setDistanceFunction(DistanceFunction dfunc) {
    if (dfunc != EUCLIDEAN_DISTANCE && dfunc != MANHATTAN_DISTANCE && dfunc != CHEBYSHEV_DISTANCE)
      return false;
    dfunc_ = dfunc;
    return true;
  }

 protected:
  void run(int algorithm, Grid& grid, const std::vector<Seed>& seeds, const vf_params* params) {
    const int d = params ? params->distance : dfunc_;
    check(vf_fracture(grid.handle(), algorithm, d, seeds.empty() ? nullptr : &seeds[0].x,
                      (uint32_t)seeds.size()));
  }
  DistanceFunction dfunc_ = CHEBYSHEV_DISTANCE;  // FractureParameters default
};

// FloodFracturer::build (FloodFracturer.cpp:98-191): multi-source BFS over
// the occupied voxels, same-wave ties to the lowest seed index
class FloodFracturer : public Fracturer {
 public:
  static FloodFracturer* getInstance() {
    static FloodFracturer f;
    return &f;
  }
  void build(Grid& grid, const std::vector<Seed>& seeds, const vf_params* params) override {
    run(VF_FLOOD, grid, seeds, params);
  }
};

// NaiveFracturer::build (NaiveFracturer.cpp:26-68): nearest seed by the metric
class NaiveFracturer : public Fracturer {
 public:
  static NaiveFracturer* getInstance() {
    static NaiveFracturer f;
    return &f;
  }
  void build(Grid& grid, const std::vector<Seed>& seeds, const vf_params* params) override {
    run(VF_NAIVE, grid, seeds, params);
  }
};

}  // namespace vf

#endif
