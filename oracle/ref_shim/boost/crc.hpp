// Test infrastructure: a stand-in for the one Boost.CRC type the reference's
// samplers use (boost::crc_32_type: process_bytes, checksum), computed by zlib's
// crc32, so that the reference's sampler sources compile here without Boost.
#pragma once
#include <zlib.h>

#include <cstddef>
#include <cstdint>

namespace boost {
class crc_32_type {
  uLong crc_ = crc32(0L, Z_NULL, 0);

 public:
  void process_bytes(const void *p, std::size_t n) {
    const Bytef *b = static_cast<const Bytef *>(p);
    while (n) {
      const uInt k = n > (1u << 30) ? (1u << 30) : (uInt)n;
      crc_ = crc32(crc_, b, k);
      b += k;
      n -= k;
    }
  }
  std::uint32_t checksum() const { return (std::uint32_t)crc_; }
};
}  // namespace boost
