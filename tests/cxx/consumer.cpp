// A C++ consumer of the library, written the way the reference's callers
// use RegularGrid, Seeder and the fracturers (CADScene::fractureModel,
// CADScene.cpp:624-691), through include/vf.hpp over include/vf.h.
//
// usage: consumer <grid.bin> <out.bin> X Y Z nseeds seed distance
//   grid.bin: X*Y*Z uint16 occupancy (x-major); out.bin gets, in order:
//   uint32 nseeds, 4*nseeds uint32 seeds, X*Y*Z uint16 labels after the
//   flood and detectBoundaries(1), 256 uint32 counts, uint64 occupied.
// Exit codes: 0 ok, 3 no CUDA device (vf::Error with VF_ERR_NOT_BUILT),
// 2 usage or I/O, 1 any other library error.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "vf.hpp"

int main(int argc, char** argv) {
  if (argc != 9) {
    std::cerr << "usage: consumer grid.bin out.bin X Y Z nseeds seed distance\n";
    return 2;
  }
  const uint32_t X = std::atoi(argv[3]), Y = std::atoi(argv[4]), Z = std::atoi(argv[5]);
  const uint32_t n = std::atoi(argv[6]);
  const uint64_t seed = std::strtoull(argv[7], nullptr, 10);
  const int dist = std::atoi(argv[8]);
  std::vector<uint16_t> occ((size_t)X * Y * Z);
  {
    std::ifstream in(argv[1], std::ios::binary);
    if (!in.read(reinterpret_cast<char*>(occ.data()), occ.size() * 2)) return 2;
  }
  try {
    vf::Context ctx(0);
    const float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {1.f, 1.f, 1.f};
    vf::Grid grid(ctx, X, Y, Z, lo, hi);
    grid.upload(occ);
    std::vector<vf::Seed> seeds = vf::Seeder::uniform(grid, n, seed, vf::BOTH);
    vf::Fracturer* fr = vf::FloodFracturer::getInstance();
    if (!fr->setDistanceFunction(static_cast<vf::DistanceFunction>(dist))) return 2;
    fr->build(grid, seeds, nullptr);
    grid.detectBoundaries(1);
    std::vector<uint16_t> labels = grid.data();
    uint64_t occupied = 0;
    std::vector<uint32_t> counts = grid.countValues(256, &occupied);
    std::ofstream out(argv[2], std::ios::binary);
    const uint32_t ns = (uint32_t)seeds.size();
    out.write(reinterpret_cast<const char*>(&ns), 4);
    out.write(reinterpret_cast<const char*>(seeds.data()), seeds.size() * sizeof(vf::Seed));
    out.write(reinterpret_cast<const char*>(labels.data()), labels.size() * 2);
    out.write(reinterpret_cast<const char*>(counts.data()), counts.size() * 4);
    out.write(reinterpret_cast<const char*>(&occupied), 8);
    return out ? 0 : 2;
  } catch (const vf::SeederSearchError& e) {
    std::cerr << "seeder search error: " << e.what() << "\n";
    return 1;
  } catch (const vf::Error& e) {
    std::cerr << e.what() << "\n";
    return e.status() == VF_ERR_NOT_BUILT ? 3 : 1;
  }
}
