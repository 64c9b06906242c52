// boost/random.hpp stand-in for the reference pin (oracle/_ref, test
// infrastructure only).  Seeder.cpp defines boost.random members for its
// normal-distribution seeding (FractureParameters::BOOST_NORMAL_DISTRIBUTION);
// the pinned function (Seeder::mergeSeeds) draws nothing, so these types only
// need to exist.  Calling operator() reports the misuse.
#pragma once
#include <stdexcept>

namespace boost {
struct mt19937 {};
template <typename T = double> struct normal_distribution {
  normal_distribution(T = T(0), T = T(1)) {}
};
template <typename E, typename D> struct variate_generator {
  variate_generator(E, D) {}
  double operator()() { throw std::logic_error("boost.random stand-in: not for drawing"); }
};
}  // namespace boost
