// Candidate generation of Padenti: the MD5 counter RNG and the feature /
// threshold draws.  The same source compiles for host and device, so the host
// can rebuild a winning candidate bit-identically to the device table, as the
// reference does on its host (cl_tree_trainer_impl_learn_best_featthr.hpp:183-222).
#pragma once

#include "pd_common.cuh"

namespace pd {

PD_HD uint32_t rotl(uint32_t x, int s) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(x, x, s);
#else
  return (x << s) | (x >> (32 - s));
#endif
}

// MD5 (RFC 1321) of the 16-byte little-endian block (s0,s1,s2,s3), padded as
// one 64-byte block: word 4 holds the 0x80 pad byte and word 14 the bit length
// 128.  Returns the four state words, which the reference uses as its random
// numbers (kernels/hist_update.cl:278-369, prng.hpp:107-195).
PD_HD void md5_block(const uint32_t in[4], uint32_t out[4]) {
  constexpr uint32_t K[64] = {
      0xd76aa478u, 0xe8c7b756u, 0x242070dbu, 0xc1bdceeeu, 0xf57c0fafu, 0x4787c62au, 0xa8304613u,
      0xfd469501u, 0x698098d8u, 0x8b44f7afu, 0xffff5bb1u, 0x895cd7beu, 0x6b901122u, 0xfd987193u,
      0xa679438eu, 0x49b40821u, 0xf61e2562u, 0xc040b340u, 0x265e5a51u, 0xe9b6c7aau, 0xd62f105du,
      0x02441453u, 0xd8a1e681u, 0xe7d3fbc8u, 0x21e1cde6u, 0xc33707d6u, 0xf4d50d87u, 0x455a14edu,
      0xa9e3e905u, 0xfcefa3f8u, 0x676f02d9u, 0x8d2a4c8au, 0xfffa3942u, 0x8771f681u, 0x6d9d6122u,
      0xfde5380cu, 0xa4beea44u, 0x4bdecfa9u, 0xf6bb4b60u, 0xbebfbc70u, 0x289b7ec6u, 0xeaa127fau,
      0xd4ef3085u, 0x04881d05u, 0xd9d4d039u, 0xe6db99e5u, 0x1fa27cf8u, 0xc4ac5665u, 0xf4292244u,
      0x432aff97u, 0xab9423a7u, 0xfc93a039u, 0x655b59c3u, 0x8f0ccc92u, 0xffeff47du, 0x85845dd1u,
      0x6fa87e4fu, 0xfe2ce6e0u, 0xa3014314u, 0x4e0811a1u, 0xf7537e82u, 0xbd3af235u, 0x2ad7d2bbu,
      0xeb86d391u};
  constexpr int R[16] = {7, 12, 17, 22, 5, 9, 14, 20, 4, 11, 16, 23, 6, 10, 15, 21};
  const uint32_t m[16] = {in[0], in[1], in[2], in[3], 0x80u, 0u, 0u, 0u,
                          0u,    0u,    0u,    0u,    0u,    0u, 128u, 0u};
  uint32_t a = 0x67452301u, b = 0xefcdab89u, c = 0x98badcfeu, d = 0x10325476u;
#pragma unroll
  for (int i = 0; i < 64; i++) {
    uint32_t fn;
    int g;
    if (i < 16) {
      fn = (b & c) | (~b & d);
      g = i;
    } else if (i < 32) {
      fn = (d & b) | (~d & c);
      g = (5 * i + 1) & 15;
    } else if (i < 48) {
      fn = b ^ c ^ d;
      g = (3 * i + 5) & 15;
    } else {
      fn = c ^ (b | ~d);
      g = (7 * i) & 15;
    }
    const uint32_t tmp = d;
    d = c;
    c = b;
    b = b + rotl(a + fn + K[i] + m[g], R[(i >> 4) * 4 + (i & 3)]);
    a = tmp;
  }
  out[0] = a + 0x67452301u;
  out[1] = b + 0xefcdab89u;
  out[2] = c + 0x98badcfeu;
  out[3] = d + 0x10325476u;
}

// low + (feat_t)((float)r / (float)0xFFFFFFFF * (float)(up - low)), with the
// narrowing of feat_t (kernels/hist_update.cl:94-111,150-151).  (float)0xFFFFFFFF
// is 2^32, and dividing a normal float by a power of two is exact, so the
// quotient is computed as the (identical) product with 2^-32.
template <typename FeatT>
PD_HD FeatT draw(uint32_t r, int32_t lo, int32_t hi) {
  const float range = (float)(int32_t)((uint32_t)hi - (uint32_t)lo);
  const float x = fmul(fmul(u2f(r), 0x1p-32f), range);
  const FeatT delta = (FeatT)(int32_t)x;  // conversion toward zero
  return (FeatT)((int32_t)(FeatT)lo + (int32_t)delta);
}

// Feature vector of candidate f of node `node` (seed (tree,node,f,0), one MD5
// per four entries, chained).
template <typename FeatT>
PD_HD void candidate_feature(uint32_t tree, uint32_t node, uint32_t f, int D, const int32_t *low,
                             const int32_t *up, FeatT *out) {
  uint32_t seed[4] = {tree, node, f, 0u}, st[4];
  for (int i = 0; i < D; i += 4) {
    md5_block(seed, st);
    for (int j = 0; j < 4 && i + j < D; j++) out[i + j] = draw<FeatT>(st[j], low[i + j], up[i + j]);
    seed[0] = st[0];
    seed[1] = st[1];
    seed[2] = st[2];
    seed[3] = st[3];
  }
}

// Threshold t of candidate f of node `node` (seed (tree,node,f,1); threshold t
// is word t%4 of the (t/4+1)-th chained MD5).
template <typename FeatT>
PD_HD FeatT candidate_threshold(uint32_t tree, uint32_t node, uint32_t f, uint32_t t, int32_t lo,
                                int32_t hi) {
  uint32_t seed[4] = {tree, node, f, 1u}, st[4] = {0u, 0u, 0u, 0u};
  for (uint32_t j = 0; j <= t / 4; j++) {
    md5_block(seed, st);
    seed[0] = st[0];
    seed[1] = st[1];
    seed[2] = st[2];
    seed[3] = st[3];
  }
  return draw<FeatT>(st[t & 3u], lo, hi);
}

}  // namespace pd
