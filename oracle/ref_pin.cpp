// ref_pin.cpp -- C entry points over the reference's own code, compiled from
// the reference tree by oracle/Makefile (target `ref`, into oracle/_ref/).
// TEST INFRASTRUCTURE ONLY: tests compare the oracle's restatements with
// these on random inputs.  Nothing here is product code.
//
//   vfr_tri_box   Intersections3D::intersect(Triangle3D&, AABB&)
//                 (MeshFragments/Source/Geometry/3D/Intersections3D.h:204-258,
//                 helpers :260-420) on the reference's Triangle3D and AABB
//                 (Triangle3D.cpp, AABB.cpp), unchanged.
#include <cstdint>

#include "Geometry/3D/Intersections3D.h"

extern "C" int vfr_tri_box(const float p0[3], const float p1[3], const float p2[3],
                           const float box_min[3], const float box_max[3]) {
  Triangle3D t(vec3(p0[0], p0[1], p0[2]), vec3(p1[0], p1[1], p1[2]), vec3(p2[0], p2[1], p2[2]));
  AABB box(vec3(box_min[0], box_min[1], box_min[2]), vec3(box_max[0], box_max[1], box_max[2]));
  return Intersections3D::intersect(t, box) ? 1 : 0;
}

// n triangles (9 floats each) against n boxes (min xyz, max xyz): out[i] 0/1
extern "C" void vfr_tri_box_batch(const float* tris, const float* boxes, uint32_t n, uint8_t* out) {
  for (uint32_t i = 0; i < n; ++i)
    out[i] = (uint8_t)vfr_tri_box(tris + 9 * (size_t)i, tris + 9 * (size_t)i + 3,
                                  tris + 9 * (size_t)i + 6, boxes + 6 * (size_t)i,
                                  boxes + 6 * (size_t)i + 3);
}

//   vfr_naive     fracturer::NaiveFracturer::build with _launchGPU = false,
//                 i.e. NaiveFracturer::buildCPU (MeshFragments/Source/
//                 Fracturer/NaiveFracturer.cpp:26-68), unchanged, on a grid
//                 of X*Y*Z uint16 labels (x-major) and n seeds (x, y, z, label)
#include "Fracturer/NaiveFracturer.h"

extern "C" int vfr_naive(uint16_t* grid, uint32_t X, uint32_t Y, uint32_t Z, const uint32_t* seeds,
                         uint32_t nseeds, int dfunc) {
  if (dfunc < 0 || dfunc > 2) return 1;
  RegularGrid g(uvec3(X, Y, Z));
  const size_t n = (size_t)X * Y * Z;
  RegularGrid::CellGrid* cells = g.data();
  for (size_t i = 0; i < n; ++i) cells[i]._value = grid[i];
  std::vector<glm::uvec4> s(nseeds);
  for (uint32_t i = 0; i < nseeds; ++i)
    s[i] = glm::uvec4(seeds[4 * i], seeds[4 * i + 1], seeds[4 * i + 2], seeds[4 * i + 3]);
  FractureParameters fp;
  fp._distanceFunction = dfunc;
  fp._launchGPU = false;
  fracturer::NaiveFracturer* f = fracturer::NaiveFracturer::getInstance();
  f->setDistanceFunction(static_cast<fracturer::DistanceFunction>(dfunc));
  f->build(g, s, &fp);
  for (size_t i = 0; i < n; ++i) grid[i] = cells[i]._value;
  return 0;
}

//   vfr_merge_seeds   fracturer::Seeder::mergeSeeds (MeshFragments/Source/
//                     Fracturer/Seeder.cpp:115-152), unchanged: every seed
//                     joins its nearest fragment, label frag | (k << 8)
#include "Fracturer/Seeder.h"

extern "C" int vfr_merge_seeds(const uint32_t* frags, uint32_t nfrags, uint32_t* seeds,
                               uint32_t nseeds, int dfunc) {
  if (dfunc < 0 || dfunc > 2 || nfrags == 0) return 1;
  std::vector<glm::uvec4> f(nfrags), s(nseeds);
  for (uint32_t i = 0; i < nfrags; ++i)
    f[i] = glm::uvec4(frags[4 * i], frags[4 * i + 1], frags[4 * i + 2], frags[4 * i + 3]);
  for (uint32_t i = 0; i < nseeds; ++i)
    s[i] = glm::uvec4(seeds[4 * i], seeds[4 * i + 1], seeds[4 * i + 2], seeds[4 * i + 3]);
  fracturer::Seeder::mergeSeeds(f, s, static_cast<fracturer::DistanceFunction>(dfunc));
  for (uint32_t i = 0; i < nseeds; ++i) seeds[4 * i + 3] = s[i].w;
  return 0;
}
