// RegularGrid.h stand-in for the reference pin (oracle/_ref, test
// infrastructure only).  The reference's RegularGrid owns an OpenGL buffer;
// NaiveFracturer::buildCPU only reads the subdivisions and the cell array,
// so this stand-in holds exactly those, with the reference's constants
// (RegularGrid.h:12-13), cell record (RegularGrid.h:21-27) and x-major index
// (RegularGrid.cpp:1031-1034).
#pragma once
#include "stdafx.h"
#include "Geometry/3D/AABB.h"
#include "Utilities/RandomUtilities.h"

#define VOXEL_EMPTY 0
#define VOXEL_FREE 1

class RegularGrid {
 public:
  struct CellGrid {
    uint16_t _value;
    CellGrid() : _value(VOXEL_EMPTY) {}
    CellGrid(uint16_t value) : _value(value) {}
  };

 protected:
  std::vector<CellGrid> _grid;
  uvec3 _numDivs;

 public:
  explicit RegularGrid(const uvec3& numDivs)
      : _grid((size_t)numDivs.x * numDivs.y * numDivs.z), _numDivs(numDivs) {}
  static unsigned getPositionIndex(int x, int y, int z, const uvec3& numDivs) {
    return x * numDivs.y * numDivs.z + y * numDivs.z + z;
  }
  CellGrid* data() { return _grid.data(); }
  glm::uvec3 getNumSubdivisions() const { return _numDivs; }
  GLuint ssbo() { return 0; }
  void swap(CellGrid* newGrid, unsigned size) { std::copy(newGrid, newGrid + size, _grid.begin()); }
  void set(int x, int y, int z, uint16_t i) { _grid[getPositionIndex(x, y, z, _numDivs)]._value = i; }
  // named by Seeder.cpp's seed placement, which the pin does not call
  bool isOccupied(int x, int y, int z) const {
    return _grid[getPositionIndex(x, y, z, _numDivs)]._value != VOXEL_EMPTY;
  }
  bool isBoundary(int x, int y, int z, int n = 1) const {
    for (int i = std::max(0, x - n); i <= std::min((int)_numDivs.x - 1, x + n); ++i)
      for (int j = std::max(0, y - n); j <= std::min((int)_numDivs.y - 1, y + n); ++j)
        for (int k = std::max(0, z - n); k <= std::min((int)_numDivs.z - 1, z + n); ++k)
          if (!isOccupied(i, j, k)) return true;
    return false;
  }
};
