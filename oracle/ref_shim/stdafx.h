// stdafx.h stand-in for the reference pin (oracle/_ref, test infrastructure
// only).  The reference's precompiled header pulls in windows.h, GLEW, GLFW,
// glm, lodepng and CGAL; the pinned functions need only the standard library
// and the vector types, which glm_shim.h provides.
#pragma once
#include <algorithm>
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <functional>
#include <iostream>
#include <list>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>
#include <math.h>

namespace std {
using ::fabsf;  // std::fabsf (C++17 <cmath>), missing from some libstdc++ releases
}

#include "glm_shim.h"
#include "Geometry/General/Adapter.h"

typedef unsigned int GLuint;
namespace glm {
typedef unsigned int uint;
}

// Seeder.h (included by the fracturers) names boost.random types for its
// normal-distribution seeding; the pinned code draws nothing from them.
#include "boost/random.hpp"
