// Test infrastructure: boost::random::mt19937 stand-in.  The C++ standard's
// std::mt19937 is the same engine (same recurrence, tempering and 32-bit
// seeding), from an independent implementation (libstdc++).
#pragma once
#include <cmath>
#include <random>

namespace boost {
namespace random {
typedef std::mt19937 mt19937;
}
}  // namespace boost
