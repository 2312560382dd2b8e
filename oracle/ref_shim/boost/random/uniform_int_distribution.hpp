// Test infrastructure: boost::random::uniform_int_distribution stand-in for a
// 32-bit engine with the full range [0, 2^32-1] (mt19937).  Boost's published
// method: a range of 0 returns the lower bound without drawing; otherwise the
// draw is divided by the bucket size floor(2^32 / (range+1)) and redrawn while
// the quotient is above the range.
#pragma once
#include <cmath>
#include <cstdint>

namespace boost {
namespace random {
template <class IntType = int>
class uniform_int_distribution {
  IntType lo_, hi_;

 public:
  uniform_int_distribution(IntType lo, IntType hi) : lo_(lo), hi_(hi) {}
  template <class Engine>
  IntType operator()(Engine &eng) const {
    static_assert(Engine::min() == 0 && Engine::max() == 0xFFFFFFFFu, "32-bit engines only");
    const std::uint32_t range = (std::uint32_t)hi_ - (std::uint32_t)lo_;
    if (range == 0) return lo_;
    if (range == 0xFFFFFFFFu) return (IntType)((std::uint32_t)eng() + (std::uint32_t)lo_);
    const std::uint32_t bucket = (std::uint32_t)((std::uint64_t(1) << 32) / (std::uint64_t(range) + 1));
    for (;;) {
      const std::uint32_t q = (std::uint32_t)eng() / bucket;
      if (q <= range) return (IntType)(q + (std::uint32_t)lo_);
    }
  }
};
}  // namespace random
}  // namespace boost
