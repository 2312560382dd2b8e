// Test infrastructure: boost::random::uniform_01 stand-in for a 32-bit engine
// with the full range (mt19937): the draw times 2^-32 (Boost's published
// method: draw / (max - min + 1), redrawn while the result is not below 1,
// which never happens for this engine).
#pragma once
#include <cmath>

namespace boost {
namespace random {
template <class RealType = double>
class uniform_01 {
 public:
  template <class Engine>
  RealType operator()(Engine &eng) const {
    static_assert(Engine::min() == 0 && Engine::max() == 0xFFFFFFFFu, "32-bit engines only");
    return RealType(eng()) * (RealType(1) / RealType(4294967296.0));
  }
};
}  // namespace random
}  // namespace boost
