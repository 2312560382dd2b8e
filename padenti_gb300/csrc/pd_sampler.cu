// Pixel samplers on the GPU: the reference's UniformImageSampler
// (uniform_image_sampler_impl.hpp:34-63) and ClassWeightedImageSampler
// (classweighted_image_sampler_impl.hpp:25-120) over batches of images, with
// the samples the reference's code returns.
//
// Both seed an MT19937 with the CRC-32 of the image bytes XOR the sampler seed,
// so every image is sampled on its own:
//  1. k_sample_scan, over all images at once (HBM-bound): the CRC-32 of each
//     image as the XOR of per-thread checksums of its bytes, each moved to its
//     place by a multiplication modulo the CRC polynomial, and the number of
//     labelled pixels.
//  2. one CTA per image: MT19937 blocks of 624 words, each twisted in three
//     parallel phases, then
//     - k_sample_uniform: Boost's bucket method on every draw (accepted draws
//       keep their order by a block scan), a bitonic sort of the drawn ranks,
//       one pass over the labels that maps ranks to pixel indices;
//     - k_sample_class_weighted: the per-class reservoir in scan order, 1024
//       pixels per step: a pixel's count within its class and its draw index
//       come from warp matches and block scans; a write lands by atomicMax on
//       its slot (pixel order is scan order, so the last writer of the
//       sequential loop wins); the buckets are then gathered and sorted.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "pd_ctx.cuh"

namespace pd {
namespace {

constexpr uint32_t kSmThreads = 256;
constexpr uint32_t kSmWarps = kSmThreads / 32;
constexpr uint32_t kCrcPoly = 0xEDB88320u;  // CRC-32, reflected
constexpr uint32_t kGfOne = 0x80000000u;    // x^0 in the reflected representation
constexpr uint32_t kGfX8 = 0x00800000u;     // x^8
// Checksum layout: a work item is a 256 KiB slice of an image's bytes, counted
// from the image's end; warp w streams the slice's 32 KiB region w as 16
// blocks of 2 KiB; lane l takes the 64 bytes at 64 l of every block, in two
// chains (even and odd blocks) for instruction-level parallelism.
constexpr uint32_t kPiece = 64;                              // bytes per lane per block
constexpr uint32_t kBlock = 32 * kPiece;                     // 2 KiB
constexpr uint32_t kRegionBlocks = 16;
constexpr uint32_t kRegion = kBlock * kRegionBlocks;         // 32 KiB per warp
constexpr uint32_t kSliceBytes = kRegion * kSmWarps;         // 256 KiB per checksum work item
constexpr uint32_t kGap = 2 * kBlock - kPiece;               // from one piece of a chain to its next
constexpr uint32_t kLabVecsPerItem = 16 * kSmThreads;        // 64 KiB of labels per count work item
constexpr uint32_t kMtN = 624;
constexpr uint32_t kWindow = 4 * kSmThreads;                  // pixels per reservoir step
constexpr uint32_t kNoError = 0xFFFFFFFFu;

// One image of a sampled batch.  Offsets are into the batch's data, label and
// output arrays.
struct SampImage {
  uint64_t data_lo;   // 16-aligned; bytes between data_lo and the image's first byte are zero
  uint64_t data_end;  // 16-aligned end of the image bytes
  uint64_t lab_off;   // 16-aligned; labels padded with zeros to lab_vecs * 16 bytes
  uint64_t out_off;
  uint32_t n_pix;
  uint32_t lab_vecs;
  uint32_t n_slices;  // checksum work items (kSliceBytes each, counted from data_end)
  uint32_t crc0;      // its first checksum work item (checksum items come first)
  uint32_t lab0;      // its first label work item
  uint32_t pad;
};

// ---- arithmetic modulo the CRC-32 polynomial (reflected: bit 31 is x^0) ----
PD_HD uint32_t gf_mul(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 31; i >= 0; i--) {
    p ^= b & (0u - ((a >> i) & 1u));
    b = (b >> 1) ^ (kCrcPoly & (0u - (b & 1u)));
  }
  return p;
}
// x^(8n): the effect of n zero bytes on a CRC register
PD_HD uint32_t gf_x8n(uint64_t n) {
  uint32_t acc = kGfOne, p = kGfX8;
  while (n) {
    if (n & 1) acc = gf_mul(acc, p);
    p = gf_mul(p, p);
    n >>= 1;
  }
  return acc;
}

// ---- MT19937 (Matsumoto and Nishimura 1998) ----
PD_D uint32_t mt_mix(uint32_t a, uint32_t b) {
  const uint32_t y = (a & 0x80000000u) | (b & 0x7FFFFFFFu);
  return (y >> 1) ^ (0x9908B0DFu & (0u - (y & 1u)));
}
PD_D uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9D2C5680u;
  y ^= (y << 15) & 0xEFC60000u;
  return y ^ (y >> 18);
}
// The seeded state (one thread).
PD_D void mt_seed(uint32_t *x, uint32_t s) {
  x[0] = s;
  for (uint32_t i = 1; i < kMtN; i++) x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + i;
}
// The next block d from the state s (all threads of the CTA; ends with a
// barrier).  Word i needs s[i], s[i+1] and s[i+397] for i < 227, the new word
// i-227 after that, and the new word 0 as its successor for i = 623.
PD_D void mt_twist(const uint32_t *s, uint32_t *d) {
  const uint32_t t = threadIdx.x;
  if (t < 227) d[t] = s[t + 397] ^ mt_mix(s[t], s[t + 1]);
  __syncthreads();
  if (t < 227) d[t + 227] = d[t] ^ mt_mix(s[t + 227], s[t + 228]);
  __syncthreads();
  if (t < 170) {
    const uint32_t i = t + 454;
    d[i] = d[i - 227] ^ mt_mix(s[i], i == kMtN - 1 ? d[0] : s[i + 1]);
  }
  __syncthreads();
}

// Exclusive scan of one value per thread over the CTA; *total gets the sum.
// All threads call it (two barriers).
PD_D uint32_t block_scan(uint32_t v, uint32_t *warp_tot, uint32_t *total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  uint32_t before = 0, tot = 0;
#pragma unroll
  for (uint32_t w = 0; w < kSmWarps; w++) {
    const uint32_t c = warp_tot[w];
    before += w < warp ? c : 0;
    tot += c;
  }
  __syncthreads();
  *total = tot;
  return before + x - v;
}

// Ascending bitonic sort of n (a power of two) words in shared memory; the
// caller has synchronised; ends with a barrier.
PD_D void bitonic_sort(uint32_t *a, uint32_t n) {
  for (uint32_t k = 2; k <= n; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += kSmThreads) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const uint32_t x = a[i], y = a[l];
          if ((x > y) == ((i & k) == 0)) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncthreads();
    }
}

PD_D uint32_t nonzero_bytes(uint4 x) {
  return (__popc(__vcmpne4(x.x, 0)) + __popc(__vcmpne4(x.y, 0)) + __popc(__vcmpne4(x.z, 0)) +
          __popc(__vcmpne4(x.w, 0))) >> 3;
}
// Index of the r-th (from 0) nonzero byte of x.
PD_D uint32_t nth_nonzero(uint4 x, uint32_t r) {
  const uint32_t w[4] = {x.x, x.y, x.z, x.w};
  for (uint32_t i = 0; i < 16; i++) {
    if ((w[i >> 2] >> (8 * (i & 3))) & 0xFFu) {
      if (r == 0) return i;
      r--;
    }
  }
  return 15;
}

// x rounded to `bits` significant bits, to nearest, ties to even.
PD_D uint64_t round_sig(uint64_t x, int bits) {
  const int n = 64 - __clzll((long long)x);
  if (n <= bits) return x;
  const int s = n - bits;
  uint64_t q = x >> s;
  const uint64_t rem = x & ((1ull << s) - 1), half = 1ull << (s - 1);
  if (rem > half || (rem == half && (q & 1))) q++;
  return q << s;
}
// roundf((float)(u * c)) with u = v * 2^-32 in double (uniform_01 on MT19937),
// in integers: the exact product v*c rounded to double's 53 bits, then to
// float's 24, then halves away from zero (classweighted_image_sampler_impl.hpp:91).
PD_D uint32_t reservoir_slot(uint32_t v, uint32_t c) {
  const uint64_t p = (uint64_t)v * c;
  if (p < (1ull << 53)) {
    // the double product is exact: one rounding to float, then an exact scaling
    return (uint32_t)roundf(__fmul_rn(__ull2float_rn(p), 0x1p-32f));
  }
  const uint64_t r = round_sig(round_sig(p, 53), 24);
  return (uint32_t)((r + 0x80000000ull) >> 32);
}

// ------------------------------------------------------------------ kernels --
// Shift constants of the checksum, computed once on the host (x^(8n) is the
// effect of n zero bytes): multiplication tables [4][256] for x^(8 kGap) and
// x^(8 kBlock) (a*X is the XOR of the entries of a's four bytes), x^(8 * bytes
// after lane l's piece in its region) for l < 32, x^(8 * bytes after region
// w in its slice) for w < 8, x^(8 kSliceBytes 2^k) for k < 32.
constexpr uint32_t kShiftGap = 0, kShiftBlock = 1024, kShiftLane = 2048, kShiftWarp = 2080, kShiftSlice = 2088,
                   kShiftWords = 2120;

PD_D uint32_t mul_tab(uint32_t a, const uint32_t *M) {
  return M[a & 0xFFu] ^ M[256 + ((a >> 8) & 0xFFu)] ^ M[512 + ((a >> 16) & 0xFFu)] ^ M[768 + (a >> 24)];
}

PD_D void prefetch_l2(const uint8_t *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// 64 bytes into the CRC register r, one table step per byte.
PD_D uint32_t crc_piece(uint32_t r, const uint4 (&q)[4], const uint32_t *T) {
#pragma unroll
  for (uint32_t i = 0; i < 16; i++) {
    const uint4 &x = q[i >> 2];
    r ^= (i & 3) == 0 ? x.x : (i & 3) == 1 ? x.y : (i & 3) == 2 ? x.z : x.w;
#pragma unroll
    for (uint32_t s = 0; s < 4; s++) r = T[(r & 0xFFu) << 5] ^ (r >> 8);
  }
  return r;
}

// Work items: the checksum slices of all images (counted from each image's
// end), then the label chunks of all images; CTAs take the next item from a
// counter.  crc[] starts at each image's initial-value term, count[] and
// *next at zero.
__global__ void __launch_bounds__(kSmThreads, 4) k_sample_scan(const uint8_t *__restrict__ data,
                                                            const uint8_t *__restrict__ labels,
                                                            const SampImage *__restrict__ imgs,
                                                            const uint32_t *__restrict__ item_img, uint32_t n_items,
                                                            uint32_t n_crc_items, const uint32_t *__restrict__ shifts,
                                                            uint32_t *__restrict__ crc, uint32_t *__restrict__ count,
                                                            uint32_t *__restrict__ next) {
  // byte table, one copy per bank: entry e of lane l at [e * 32 + l]
  __shared__ uint32_t tab[256 * 32];
  __shared__ uint32_t mgap[1024], mblock[1024];
  __shared__ uint32_t xs[32];
  __shared__ uint32_t red[kSmWarps];
  __shared__ uint32_t s_item;
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  {
    uint32_t r = t;
    for (int k = 0; k < 8; k++) r = (r >> 1) ^ (kCrcPoly & (0u - (r & 1u)));
    for (uint32_t i = 0; i < 32; i++) tab[t * 32 + ((i + lane) & 31)] = r;
  }
  if (t == 0) s_item = atomicAdd(next, 1u);
  for (uint32_t i = t; i < 1024; i += kSmThreads) {
    mgap[i] = shifts[kShiftGap + i];
    mblock[i] = shifts[kShiftBlock + i];
  }
  if (t < 32) xs[t] = shifts[kShiftSlice + t];
  const uint32_t x_lane = shifts[kShiftLane + lane], x_warp = shifts[kShiftWarp + warp];
  __syncthreads();
  const uint32_t *T = tab + lane;
  for (;;) {
    const uint32_t item = s_item;
    if (item >= n_items) break;
    const uint32_t im = item_img[item];
    const SampImage g = imgs[im];
    if (item < n_crc_items) {
      const uint32_t local = item - g.crc0;
      const int64_t r_end = (int64_t)g.data_end - (int64_t)local * kSliceBytes - (int64_t)(kSmWarps - 1 - warp) * kRegion;
      const int64_t r_beg = r_end - kRegion, lo = (int64_t)g.data_lo;
      uint32_t acc = 0;
      if (r_end > lo) {  // warp-uniform: this warp's region holds image bytes
        const uint8_t *rb = data + r_beg;  // only dereferenced at or after data + lo
        // the first blocks into L2 (lanes 0-15: the 16 lines of one block)
        if (lane < 16)
#pragma unroll
          for (uint32_t j = 0; j < 4; j++)
            if (r_beg + (int64_t)(j * kBlock) >= lo) prefetch_l2(rb + j * kBlock + lane * 128);
        uint32_t s0 = 0, s1 = 0;
#pragma unroll 1
        for (uint32_t j = 0; j < kRegionBlocks; j += 2) {
          if (j + 4 < kRegionBlocks) {
            const uint32_t pj = j + 4 + (lane >> 4);
            if (r_beg + (int64_t)(pj * kBlock) >= lo) prefetch_l2(rb + pj * kBlock + (lane & 15) * 128);
          }
          uint4 q0[4], q1[4];
#pragma unroll
          for (uint32_t i = 0; i < 4; i++) {
            const int64_t a0 = r_beg + (int64_t)(j * kBlock + lane * kPiece + i * 16);
            const int64_t a1 = a0 + kBlock;
            q0[i] = a0 >= lo ? __ldg(reinterpret_cast<const uint4 *>(data + a0)) : make_uint4(0, 0, 0, 0);
            q1[i] = a1 >= lo ? __ldg(reinterpret_cast<const uint4 *>(data + a1)) : make_uint4(0, 0, 0, 0);
          }
          s0 = crc_piece(mul_tab(s0, mgap), q0, T);
          s1 = crc_piece(mul_tab(s1, mgap), q1, T);
        }
        // chain 0 ends one block before chain 1; then to the end of the region
        acc = mul_tab(s0, mblock) ^ s1;
        if (acc) acc = gf_mul(acc, x_lane);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc ^= __shfl_xor_sync(0xFFFFFFFFu, acc, o);
      if (lane == 0) red[warp] = acc ? gf_mul(acc, x_warp) : 0u;
      __syncthreads();
      if (t == 0) {
        uint32_t tot = 0;
        for (uint32_t w = 0; w < kSmWarps; w++) tot ^= red[w];
        if (tot) {
          for (uint32_t k = 0; k < 32; k++)
            if ((local >> k) & 1u) tot = gf_mul(tot, xs[k]);
          atomicXor(&crc[im], tot);
        }
      }
    } else {
      const uint32_t v0 = (item - g.lab0) * kLabVecsPerItem;
      const uint4 *L = reinterpret_cast<const uint4 *>(labels + g.lab_off);
      uint32_t n = 0;
#pragma unroll 4
      for (uint32_t i = 0; i < kLabVecsPerItem / kSmThreads; i++) {
        const uint32_t vi = v0 + i * kSmThreads + t;
        if (vi < g.lab_vecs) n += nonzero_bytes(__ldg(L + vi));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xFFFFFFFFu, n, o);
      if (lane == 0) red[warp] = n;
      __syncthreads();
      if (t == 0) {
        uint32_t tot = 0;
        for (uint32_t w = 0; w < kSmWarps; w++) tot += red[w];
        if (tot) atomicAdd(&count[im], tot);
      }
    }
    __syncthreads();  // everyone has read s_item and red[]
    if (t == 0) s_item = atomicAdd(next, 1u);
    __syncthreads();
  }
}

constexpr uint32_t kWalkVecs = 4;  // label vectors (64 pixels) per thread per step of the rank walk

PD_D void walk_load(uint4 (&x)[kWalkVecs], const uint4 *L, uint32_t v, uint32_t n_vecs) {
#pragma unroll
  for (uint32_t i = 0; i < kWalkVecs; i++) x[i] = v + i < n_vecs ? __ldg(L + v + i) : make_uint4(0, 0, 0, 0);
}

// UniformImageSampler::sample, one CTA per image.  Dynamic shared memory:
// sort_n words (a power of two >= n_samples).
__global__ void __launch_bounds__(kSmThreads) k_sample_uniform(const uint8_t *__restrict__ labels,
                                                               const SampImage *__restrict__ imgs,
                                                               const uint32_t *__restrict__ crc,
                                                               const uint32_t *__restrict__ count, uint32_t n_samples,
                                                               uint32_t seed, uint32_t sort_n,
                                                               uint32_t *__restrict__ out,
                                                               uint32_t *__restrict__ out_count,
                                                               uint32_t *__restrict__ err) {
  extern __shared__ uint32_t keys[];
  __shared__ uint32_t mt[2][kMtN];
  __shared__ uint32_t wtot[kSmWarps];
  const uint32_t im = blockIdx.x, t = threadIdx.x;
  const SampImage g = imgs[im];
  const uint32_t n = count[im];
  if (n == 0) {  // no labelled pixel (the reference draws from an empty buffer)
    if (t == 0) out_count[im] = 0;
    return;
  }
  if (n == 1) {  // range 0: Boost returns the lower bound without drawing
    for (uint32_t i = t; i < n_samples; i += kSmThreads) keys[i] = 0;
  } else {
    if (t == 0) mt_seed(mt[0], crc[im] ^ seed);
    __syncthreads();
    const uint32_t bucket = (uint32_t)(0x100000000ull / n);
    // a draw is accepted with probability above 1/2: twice the blocks that
    // takes on average, and 64 more, end the loop in any case
    const uint32_t max_blocks = 4 * n_samples / kMtN + 64;
    uint32_t got = 0, cur = 0, blocks = 0;
    while (got < n_samples) {
      if (blocks++ == max_blocks) {
        if (t == 0) atomicMin(err + 1, im);
        break;
      }
      mt_twist(mt[cur], mt[cur ^ 1]);
      cur ^= 1;
      uint32_t q[3] = {n, n, n}, ok = 0;
      if (t < kMtN / 3) {
#pragma unroll
        for (uint32_t k = 0; k < 3; k++) {
          q[k] = mt_temper(mt[cur][3 * t + k]) / bucket;
          ok += q[k] < n;
        }
      }
      uint32_t total;
      uint32_t pos = got + block_scan(ok, wtot, &total);
#pragma unroll
      for (uint32_t k = 0; k < 3; k++)
        if (q[k] < n) {
          if (pos < n_samples) keys[pos] = q[k];
          pos++;
        }
      got += total;
    }
  }
  for (uint32_t i = n_samples + t; i < sort_n; i += kSmThreads) keys[i] = 0xFFFFFFFFu;
  __syncthreads();
  bitonic_sort(keys, sort_n);
  // ranks among the labelled pixels -> pixel indices, in one pass over the
  // labels: kWalkVecs label vectors per thread per step, the next step's loaded
  // ahead
  const uint4 *L = reinterpret_cast<const uint4 *>(labels + g.lab_off);
  const uint32_t last = keys[n_samples - 1];
  uint32_t *o = out + g.out_off;
  uint32_t run = 0;
  uint4 xa[kWalkVecs], xb[kWalkVecs];
  walk_load(xa, L, t * kWalkVecs, g.lab_vecs);
  for (uint32_t v0 = 0; v0 < g.lab_vecs && run <= last; v0 += kSmThreads * kWalkVecs) {
    walk_load(xb, L, v0 + kSmThreads * kWalkVecs + t * kWalkVecs, g.lab_vecs);
    uint32_t c[kWalkVecs], ct = 0;
#pragma unroll
    for (uint32_t i = 0; i < kWalkVecs; i++) {
      c[i] = nonzero_bytes(xa[i]);
      ct += c[i];
    }
    uint32_t total;
    const uint32_t base = run + block_scan(ct, wtot, &total);
    if (ct) {
      uint32_t lo = 0, hi = n_samples;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (keys[mid] < base) lo = mid + 1;
        else hi = mid;
      }
      for (uint32_t i = lo; i < n_samples && keys[i] < base + ct; i++) {
        uint32_t r = keys[i] - base, k = 0;
#pragma unroll
        for (uint32_t j = 0; j + 1 < kWalkVecs; j++)
          if (k == j && r >= c[j]) {
            r -= c[j];
            k = j + 1;
          }
        uint4 x = xa[0];
#pragma unroll
        for (uint32_t j = 1; j < kWalkVecs; j++)
          if (k == j) x = xa[j];
        o[i] = (v0 + t * kWalkVecs + k) * 16 + nth_nonzero(x, r);
      }
    }
    run += total;
#pragma unroll
    for (uint32_t i = 0; i < kWalkVecs; i++) xa[i] = xb[i];
  }
  if (t == 0) out_count[im] = n_samples;
}

// ClassWeightedImageSampler::sample, one CTA per image.  Dynamic shared
// memory: n_slots bucket slots (pixel + 1, 0 = empty) then sort_n words.
// Step layout: warp w, round j, lane l holds pixel win + 128 w + 32 j + l, so
// (w, j, l) order is scan order.
__global__ void __launch_bounds__(kSmThreads) k_sample_class_weighted(
    const uint8_t *__restrict__ labels, const SampImage *__restrict__ imgs, const uint32_t *__restrict__ crc,
    const uint32_t *__restrict__ bucket_size, uint32_t n_classes, uint32_t n_slots, uint32_t seed, uint32_t sort_n,
    uint32_t *__restrict__ out, uint32_t *__restrict__ out_count, uint32_t *__restrict__ err) {
  extern __shared__ uint32_t dyn[];
  uint32_t *slots = dyn, *keys = dyn + n_slots;
  __shared__ uint32_t ring[3][kMtN];  // MT block b in ring[b % 3]; the seeded state is block -1
  __shared__ uint32_t bsz[256], boff[256], seen[256];
  __shared__ uint32_t wcnt[kSmWarps][256];
  __shared__ uint32_t wd[kSmWarps];
  __shared__ uint32_t bad;
  const uint32_t im = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t lt = (1u << lane) - 1;
  const SampImage g = imgs[im];
  for (uint32_t k = t; k < n_classes; k += kSmThreads) {
    bsz[k] = bucket_size[k];
    seen[k] = 0;
  }
  for (uint32_t k = t; k < kSmWarps * 256; k += kSmThreads) (&wcnt[0][0])[k] = 0;
  for (uint32_t i = t; i < n_slots; i += kSmThreads) slots[i] = 0;
  if (t == 0) {
    uint32_t o = 0;
    for (uint32_t k = 0; k < n_classes; k++) {
      boff[k] = o;
      o += bucket_size[k];
    }
    bad = 0;
    mt_seed(ring[2], crc[im] ^ seed);
  }
  __syncthreads();
  const uint8_t *lab = labels + g.lab_off;
  uint32_t gen = 0, d_base = 0;
  uint32_t nxt[4];  // the labels of the next step, loaded ahead
#pragma unroll
  for (uint32_t j = 0; j < 4; j++) {
    const uint32_t p = warp * 128 + j * 32 + lane;
    nxt[j] = p < g.n_pix ? lab[p] : 0u;
  }
  for (uint32_t win = 0; win < g.n_pix; win += kWindow) {
    uint32_t cls[4], rank[4];
    bool valid[4];
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
      cls[j] = nxt[j];
      const uint32_t p = win + kWindow + warp * 128 + j * 32 + lane;
      nxt[j] = p < g.n_pix ? lab[p] : 0u;
    }
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
      const uint32_t k = cls[j] - 1u;
      valid[j] = cls[j] != 0 && k < n_classes;
      if (cls[j] != 0 && k >= n_classes) atomicOr(&bad, 1u);
      cls[j] = valid[j] ? k : 0xFFFFFFFFu;
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, cls[j]);
      rank[j] = valid[j] ? wcnt[warp][cls[j]] + __popc(peers & lt) : 0u;
      __syncwarp();
      if (valid[j] && lane == (uint32_t)(__ffs(peers) - 1)) wcnt[warp][cls[j]] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // per class: the count before each warp's pixels (in place), and the running count
    for (uint32_t k = t; k < n_classes; k += kSmThreads) {
      uint32_t acc = seen[k];
#pragma unroll
      for (uint32_t w = 0; w < kSmWarps; w++) {
        const uint32_t c = wcnt[w][k];
        wcnt[w][k] = acc;
        acc += c;
      }
      seen[k] = acc;
    }
    __syncthreads();
    uint32_t didx[4], dcount = 0;
    bool draw[4];
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
      const uint32_t p = win + warp * 128 + j * 32 + lane;
      draw[j] = false;
      if (valid[j]) {
        rank[j] += wcnt[warp][cls[j]];  // pixels of this class before p
        if (rank[j] < bsz[cls[j]]) atomicMax(&slots[boff[cls[j]] + rank[j]], p + 1);
        else draw[j] = true;
      }
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, draw[j]);
      didx[j] = dcount + __popc(m & lt);
      dcount += __popc(m);
    }
    if (lane == 0) wd[warp] = dcount;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (uint32_t w = 0; w < kSmWarps; w++) {
      before += w < warp ? wd[w] : 0;
      total += wd[w];
    }
    if (total) {
      const uint32_t need = (d_base + total - 1) / kMtN;  // last block this step reads
      while (gen <= need) {
        mt_twist(ring[(gen + 2) % 3], ring[gen % 3]);
        gen++;
      }
#pragma unroll
      for (uint32_t j = 0; j < 4; j++)
        if (draw[j]) {
          const uint32_t d = d_base + before + didx[j];
          const uint32_t v = mt_temper(ring[(d / kMtN) % 3][d % kMtN]);
          const uint32_t s = reservoir_slot(v, rank[j]);
          if (s < bsz[cls[j]]) atomicMax(&slots[boff[cls[j]] + s], win + warp * 128 + j * 32 + lane + 1);
        }
      d_base += total;
    }
    __syncwarp();
    for (uint32_t k = lane; k < n_classes; k += 32) wcnt[warp][k] = 0;
    __syncthreads();
  }
  // gather the buckets in class order, sort, write
  uint32_t pos = 0;
  for (uint32_t k = 0; k < n_classes; k++) {
    const uint32_t f = min(seen[k], bsz[k]);
    for (uint32_t s = t; s < f; s += kSmThreads) keys[pos + s] = slots[boff[k] + s] - 1;
    pos += f;
  }
  for (uint32_t i = pos + t; i < sort_n; i += kSmThreads) keys[i] = 0xFFFFFFFFu;
  __syncthreads();
  bitonic_sort(keys, sort_n);
  uint32_t *o = out + g.out_off;
  for (uint32_t i = t; i < pos; i += kSmThreads) o[i] = keys[i];
  if (t == 0) {
    out_count[im] = pos;
    if (bad) atomicMin(err, im);
  }
}

// ------------------------------------------------------------------- host ----
struct SamplerPlan {
  std::vector<uint32_t> bucket;  // class-weighted bucket sizes
  uint32_t stride = 0, sort_n = 1;
};

int plan_sampler(const pd_sampler *s, SamplerPlan *pl) {
  PD_CHECK(s, PD_ERR_INVALID, "null sampler");
  PD_CHECK(s->kind == PD_SAMPLER_UNIFORM || s->kind == PD_SAMPLER_CLASS_WEIGHTED, PD_ERR_INVALID,
           "unknown sampler kind %d", s->kind);
  PD_CHECK(s->n_samples >= 1, PD_ERR_INVALID, "nSamples must be at least 1");
  PD_CHECK(s->pixel_bytes >= 1, PD_ERR_INVALID, "pixel_bytes must be at least 1");
  uint64_t stride = s->n_samples;
  if (s->kind == PD_SAMPLER_CLASS_WEIGHTED) {
    PD_CHECK(s->n_classes >= 1 && s->n_classes <= 255, PD_ERR_INVALID, "nClasses %u outside [1,255]", s->n_classes);
    // m_perClassBucketSize (classweighted_image_sampler_impl.hpp:33,43): float product, then ceil
    const float p = 1.f / (float)s->n_classes;
    pl->bucket.resize(s->n_classes);
    stride = 0;
    for (uint32_t k = 0; k < s->n_classes; k++) {
      const float w = s->weights ? s->weights[k] : p;
      PD_CHECK(std::isfinite(w) && w >= 0.f, PD_ERR_INVALID, "weight %u is %g (weights must be finite and >= 0)", k,
               (double)w);
      const float b = std::ceil(w * (float)s->n_samples);
      PD_CHECK(b <= (float)PD_SAMPLER_MAX_STRIDE, PD_ERR_UNSUPPORTED, "bucket %u holds %g samples (max %d)", k,
               (double)b, PD_SAMPLER_MAX_STRIDE);
      pl->bucket[k] = (uint32_t)b;
      stride += pl->bucket[k];
    }
  }
  PD_CHECK(stride <= PD_SAMPLER_MAX_STRIDE, PD_ERR_UNSUPPORTED, "%llu samples per image (max %d)",
           (unsigned long long)stride, PD_SAMPLER_MAX_STRIDE);
  pl->stride = (uint32_t)stride;
  pl->sort_n = 1;
  while (pl->sort_n < pl->stride) pl->sort_n <<= 1;
  return PD_OK;
}


// Descriptors, item map, initial checksum terms, zero counts, the error word
// and the class-weighted bucket sizes, in one pinned block uploaded with one
// copy.
struct DescLayout {
  size_t shifts = 0, imgs = 0, items = 0, crc = 0, count = 0, err = 0, bucket = 0, bytes = 0;
  uint32_t n_items = 0, n_crc_items = 0;
  DescLayout() = default;
  DescLayout(uint32_t n, uint32_t n_items, uint32_t n_classes) {
    imgs = shifts + ((4ull * kShiftWords + 15) / 16 * 16);
    items = imgs + sizeof(SampImage) * n;
    crc = items + 4ull * n_items;
    count = crc + 4ull * n;
    err = count + 4ull * n;
    bucket = err + 16;  // err[0], err[1]: errors; err[2]: the scan's work counter
    bytes = bucket + 4ull * n_classes;
    this->n_items = n_items;
  }
};

// The checksum's shift constants (kShift*), computed once.
const uint32_t *shift_constants() {
  static const std::vector<uint32_t> tab = [] {
    std::vector<uint32_t> v(kShiftWords);
    const uint32_t xg = gf_x8n(kGap), xb = gf_x8n(kBlock);
    for (uint32_t i = 0; i < 4; i++)
      for (uint32_t e = 0; e < 256; e++) {
        v[kShiftGap + i * 256 + e] = gf_mul(e << (8 * i), xg);
        v[kShiftBlock + i * 256 + e] = gf_mul(e << (8 * i), xb);
      }
    for (uint32_t l = 0; l < 32; l++) v[kShiftLane + l] = gf_x8n((uint64_t)kPiece * (31 - l));
    for (uint32_t w = 0; w < kSmWarps; w++) v[kShiftWarp + w] = gf_x8n((uint64_t)kRegion * (kSmWarps - 1 - w));
    uint32_t p = gf_x8n(kSliceBytes);
    for (uint32_t k = 0; k < 32; k++) {
      v[kShiftSlice + k] = p;
      p = gf_mul(p, p);
    }
    return v;
  }();
  return tab.data();
}

// Uploads the descriptor block and launches the two kernels on a batch that is
// in device memory.  counts/err stay on the device.
int launch_batch(pd_ctx *ctx, const pd_sampler *s, const SamplerPlan &pl, uint32_t n, const uint8_t *data, const uint8_t *labels, uint32_t *out, uint32_t *counts, const DescLayout &lay,
                 uint8_t *dev_desc, const void *host_desc, cudaEvent_t *ev) {
  cudaStream_t st = ctx->stream;
  PD_CUDA(h2d(ctx, dev_desc, host_desc, lay.bytes));
  const SampImage *imgs = reinterpret_cast<const SampImage *>(dev_desc + lay.imgs);
  const uint32_t *item_img = reinterpret_cast<const uint32_t *>(dev_desc + lay.items);
  uint32_t *crc = reinterpret_cast<uint32_t *>(dev_desc + lay.crc);
  uint32_t *cnt = reinterpret_cast<uint32_t *>(dev_desc + lay.count);
  uint32_t *err = reinterpret_cast<uint32_t *>(dev_desc + lay.err);
  int sms = 0, per_sm = 0;
  PD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  PD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sample_scan, kSmThreads, 0));
  const uint32_t grid = std::max(1u, std::min<uint32_t>(lay.n_items, (uint32_t)(sms * std::max(per_sm, 1))));
  PD_CUDA(cudaEventRecord(ev[0], st));
  k_sample_scan<<<grid, kSmThreads, 0, st>>>(data, labels, imgs, item_img, lay.n_items, lay.n_crc_items,
                                             reinterpret_cast<const uint32_t *>(dev_desc + lay.shifts), crc, cnt,
                                             err + 2);
  PD_CUDA(cudaGetLastError());
  PD_CUDA(cudaEventRecord(ev[1], st));
  if (s->kind == PD_SAMPLER_UNIFORM) {
    const size_t smem = (size_t)pl.sort_n * 4;
    PD_CUDA(cudaFuncSetAttribute(k_sample_uniform, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_sample_uniform<<<n, kSmThreads, smem, st>>>(labels, imgs, crc, cnt, s->n_samples, s->seed, pl.sort_n, out,
                                                  counts, err);
  } else {
    const size_t smem = ((size_t)pl.stride + pl.sort_n) * 4;
    PD_CUDA(cudaFuncSetAttribute(k_sample_class_weighted, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_sample_class_weighted<<<n, kSmThreads, smem, st>>>(labels, imgs, crc,
                                                         reinterpret_cast<const uint32_t *>(dev_desc + lay.bucket),
                                                         s->n_classes, pl.stride, s->seed, pl.sort_n, out, counts, err);
  }
  PD_CUDA(cudaGetLastError());
  PD_CUDA(cudaEventRecord(ev[2], st));
  ctx->launches += 2;
  ctx->sample_stats.kernel_launches += 2;
  return PD_OK;
}

// Fills the pinned descriptor block for images described by (data_lo, data
// bytes, lab_off, n_pix, out_off) and returns the item count.
struct ImagePlace {
  uint64_t data_lo, data_end, lab_off, out_off;
  uint64_t data_bytes;
  uint32_t n_pix;
};

int fill_desc(HostBuf &hb, const SamplerPlan &pl, const std::vector<ImagePlace> &place, DescLayout *lay_out) {
  const uint32_t n = (uint32_t)place.size();
  uint64_t n_crc = 0, n_lab = 0;
  std::vector<uint32_t> slices(n), chunks(n);
  for (uint32_t i = 0; i < n; i++) {
    slices[i] = (uint32_t)((place[i].data_end - place[i].data_lo + kSliceBytes - 1) / kSliceBytes);
    chunks[i] = ((place[i].n_pix + 15) / 16 + kLabVecsPerItem - 1) / kLabVecsPerItem;
    n_crc += slices[i];
    n_lab += chunks[i];
  }
  PD_CHECK(n_crc + n_lab < (1ull << 31), PD_ERR_UNSUPPORTED, "batch too large");
  DescLayout lay(n, (uint32_t)(n_crc + n_lab), (uint32_t)pl.bucket.size());
  lay.n_crc_items = (uint32_t)n_crc;
  PD_TRY(hb.ensure(lay.bytes));
  uint8_t *h = hb.as<uint8_t>();
  SampImage *im = reinterpret_cast<SampImage *>(h + lay.imgs);
  uint32_t *item_img = reinterpret_cast<uint32_t *>(h + lay.items);
  uint32_t *crc = reinterpret_cast<uint32_t *>(h + lay.crc);
  uint32_t *cnt = reinterpret_cast<uint32_t *>(h + lay.count);
  uint32_t ic = 0, il = (uint32_t)n_crc;
  for (uint32_t i = 0; i < n; i++) {
    const ImagePlace &p = place[i];
    im[i] = SampImage{p.data_lo, p.data_end, p.lab_off, p.out_off, p.n_pix, (p.n_pix + 15) / 16, slices[i], ic, il, 0};
    for (uint32_t k = 0; k < slices[i]; k++) item_img[ic++] = i;
    for (uint32_t k = 0; k < chunks[i]; k++) item_img[il++] = i;
    // the initial value 0xFFFFFFFF carried past the image bytes, and the final XOR
    // (images of a batch mostly share their size)
    if (i == 0 || p.data_bytes != place[i - 1].data_bytes)
      crc[i] = gf_mul(0xFFFFFFFFu, gf_x8n(p.data_bytes)) ^ 0xFFFFFFFFu;
    else
      crc[i] = crc[i - 1];
    cnt[i] = 0;
  }
  std::memcpy(h + lay.shifts, shift_constants(), 4ull * kShiftWords);
  reinterpret_cast<uint32_t *>(h + lay.err)[0] = kNoError;  // first image with a label above nClasses
  reinterpret_cast<uint32_t *>(h + lay.err)[1] = kNoError;  // first image whose draws hit the block limit
  reinterpret_cast<uint32_t *>(h + lay.err)[2] = 0;         // next work item of the scan
  if (!pl.bucket.empty()) std::memcpy(h + lay.bucket, pl.bucket.data(), pl.bucket.size() * 4);
  *lay_out = lay;
  return PD_OK;
}

int check_errors(const uint32_t *err, uint32_t first, const pd_sampler *s) {
  PD_CHECK(err[0] == kNoError, PD_ERR_INVALID, "image %u has a label above nClasses %u", first + err[0],
           s->n_classes);
  PD_CHECK(err[1] == kNoError, PD_ERR_CUDA, "image %u: the uniform draws hit their block limit", first + err[1]);
  return PD_OK;
}

double event_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace
}  // namespace pd

using namespace pd;

extern "C" int pd_sampler_stride(const pd_sampler *s, uint32_t *stride) {
  PD_CHECK(stride, PD_ERR_INVALID, "null output");
  SamplerPlan pl;
  PD_TRY(plan_sampler(s, &pl));
  *stride = pl.stride;
  return PD_OK;
}

extern "C" int pd_sample_get_stats(pd_ctx *ctx, pd_sample_stats *out) {
  PD_CHECK(ctx && out, PD_ERR_INVALID, "null argument");
  *out = ctx->sample_stats;
  return PD_OK;
}

extern "C" int pd_sample(pd_ctx *ctx, const pd_sampler *s, uint32_t n_images, const void *const *images,
                         const uint8_t *const *labels, const uint32_t *widths, const uint32_t *heights,
                         uint32_t stride, uint32_t *samples, uint32_t *counts) {
  const auto t0 = std::chrono::steady_clock::now();
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  SamplerPlan pl;
  PD_TRY(plan_sampler(s, &pl));
  PD_CHECK(stride >= pl.stride, PD_ERR_INVALID, "stride %u below the %u samples per image this sampler needs", stride,
           pl.stride);
  ctx->sample_stats = pd_sample_stats{};
  if (n_images == 0) return PD_OK;
  PD_CHECK(images && labels && widths && heights && samples && counts, PD_ERR_INVALID, "null argument");
  PD_CUDA(cudaSetDevice(ctx->device));
  const uint64_t h2d0 = ctx->bytes_h2d, d2h0 = ctx->bytes_d2h;
  // groups of images whose staged bytes stay below a bound
  struct Group {
    uint32_t first, n;
    uint64_t data_cur, lab_cur;
    std::vector<ImagePlace> place;
  };
  std::vector<Group> groups;
  const uint64_t kGroupBytes = ctx->sample_group;
  for (uint32_t first = 0; first < n_images;) {
    Group g;
    g.first = first;
    g.data_cur = g.lab_cur = 0;
    uint32_t last = first;
    for (; last < n_images; last++) {
      PD_CHECK(images[last] && labels[last], PD_ERR_INVALID, "image %u has a null buffer", last);
      const uint64_t np = (uint64_t)widths[last] * heights[last];
      PD_CHECK(widths[last] >= 1 && heights[last] >= 1 && np < (1ull << 31), PD_ERR_UNSUPPORTED,
               "image %u is %ux%u (1 to 2^31-1 pixels)", last, widths[last], heights[last]);
      const uint64_t db = np * s->pixel_bytes;
      PD_CHECK(db < (1ull << 40), PD_ERR_UNSUPPORTED, "image %u too large", last);
      // zeros before the bytes so that the image ends on a 256-byte block (the
      // checksum reads 256-byte blocks counted from the end)
      const uint64_t pad = (256 - db % 256) % 256;
      const uint64_t dsz = pad + db, lsz = (np + 15) / 16 * 16;
      if (last > first && g.data_cur + dsz + g.lab_cur + lsz > kGroupBytes) break;
      g.place.push_back(
          ImagePlace{g.data_cur, g.data_cur + dsz, g.lab_cur, (uint64_t)(last - first) * stride, db, (uint32_t)np});
      g.data_cur += dsz;
      g.lab_cur += lsz;
    }
    g.n = last - first;
    groups.push_back(std::move(g));
    first = last;
  }
  // Two slots: the host stages group k into one while the device copies, scans
  // and draws group k - 1 from the other; a slot's results come back to its
  // pinned buffer and reach the caller when the slot is reused or at the end.
  PD_CUDA(cudaStreamSynchronize(ctx->stream));  // no earlier call still reads a slot
  for (auto &sl : ctx->samp)
    for (cudaEvent_t &e : sl.ev)
      if (!e) PD_CUDA(cudaEventCreate(&e));
  int busy[2] = {-1, -1};
  DescLayout lays[2];
  auto finish = [&](int si) -> int {
    pd_ctx::SampSlot &sl = ctx->samp[si];
    const Group &g = groups[busy[si]];
    busy[si] = -1;
    PD_CUDA(cudaEventSynchronize(sl.ev[3]));
    const uint32_t *ho = sl.h_out.as<uint32_t>();
    const uint32_t *err = ho + (uint64_t)g.n * stride + g.n;
    PD_TRY(check_errors(err, g.first, s));
    std::memcpy(samples + (uint64_t)g.first * stride, ho, (uint64_t)g.n * stride * 4);
    std::memcpy(counts + g.first, ho + (uint64_t)g.n * stride, (uint64_t)g.n * 4);
    ctx->sample_stats.ms_scan += event_ms(sl.ev[0], sl.ev[1]);
    ctx->sample_stats.ms_draw += event_ms(sl.ev[1], sl.ev[2]);
    for (const ImagePlace &p : g.place) {
      ctx->sample_stats.data_bytes += p.data_bytes;
      ctx->sample_stats.label_bytes += p.n_pix;
    }
    return PD_OK;
  };
  auto fail = [&](int rc) {  // nothing of a failed call stays in flight
    cudaStreamSynchronize(ctx->stream);
    return rc;
  };
  for (size_t k = 0; k < groups.size(); k++) {
    const int si = (int)(k % 2);
    pd_ctx::SampSlot &sl = ctx->samp[si];
    if (busy[si] >= 0) {
      const int rc = finish(si);
      if (rc != PD_OK) return fail(rc);
    }
    const Group &g = groups[k];
    const uint32_t n = g.n, first = g.first;
    // staging: data then labels, each image's zero padding included
    PD_TRY(sl.h_data.ensure(g.data_cur + g.lab_cur + 16));
    uint8_t *hd = sl.h_data.as<uint8_t>(), *hl = hd + g.data_cur;
    const unsigned nt = std::max(1u, std::min({16u, std::thread::hardware_concurrency(), n}));
    auto work = [&](unsigned th) {
      for (uint32_t i = th; i < n; i += nt) {
        const ImagePlace &p = g.place[i];
        const uint64_t pad = p.data_end - p.data_lo - p.data_bytes;
        std::memset(hd + p.data_lo, 0, pad);
        std::memcpy(hd + p.data_lo + pad, images[first + i], p.data_bytes);
        std::memcpy(hl + p.lab_off, labels[first + i], p.n_pix);
        std::memset(hl + p.lab_off + p.n_pix, 0, (p.n_pix + 15) / 16 * 16 - p.n_pix);
      }
    };
    {
      std::vector<std::thread> th;
      for (unsigned q = 1; q < nt; q++) th.emplace_back(work, q);
      work(0);
      for (auto &x : th) x.join();
    }
    DescLayout &lay = lays[si];
    PD_TRY(fill_desc(sl.h_desc, pl, g.place, &lay));
    PD_TRY(sl.d_data.ensure(g.data_cur + g.lab_cur + 16));
    PD_TRY(sl.d_desc.ensure(lay.bytes));
    const uint64_t out_words = (uint64_t)n * stride + n;
    PD_TRY(sl.d_out.ensure(out_words * 4 + 16));
    PD_TRY(sl.h_out.ensure(out_words * 4 + 16));
    uint8_t *dd = sl.d_data.as<uint8_t>(), *dl = dd + g.data_cur;
    int rc = upload_bytes(ctx, dd, hd, g.data_cur + g.lab_cur);
    uint32_t *dout = sl.d_out.as<uint32_t>(), *dcnt = dout + (uint64_t)n * stride;
    if (rc == PD_OK) rc = launch_batch(ctx, s, pl, n, dd, dl, dout, dcnt, lay, sl.d_desc.as<uint8_t>(),
                                       sl.h_desc.ptr, sl.ev);
    if (rc != PD_OK) return fail(rc);
    // samples, counts and the two error words into the slot's pinned buffer
    uint32_t *ho = sl.h_out.as<uint32_t>();
    PD_CUDA(d2h(ctx, ho, dout, out_words * 4));
    PD_CUDA(d2h(ctx, ho + out_words, sl.d_desc.as<uint8_t>() + lay.err, 8));
    PD_CUDA(cudaEventRecord(sl.ev[3], ctx->stream));
    busy[si] = (int)k;
  }
  // the last two groups, in order
  for (size_t k = groups.size() >= 2 ? groups.size() - 2 : 0; k < groups.size(); k++) {
    const int si = (int)(k % 2);
    if (busy[si] == (int)k) {
      const int rc = finish(si);
      if (rc != PD_OK) return fail(rc);
    }
  }
  ctx->sample_stats.images = n_images;
  ctx->sample_stats.h2d_bytes = ctx->bytes_h2d - h2d0;
  ctx->sample_stats.d2h_bytes = ctx->bytes_d2h - d2h0;
  ctx->sample_stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return PD_OK;
}

extern "C" int pd_sample_device(pd_ctx *ctx, const pd_sampler *s, uint32_t n_images, const void *images_device,
                                const uint8_t *labels_device, uint32_t width, uint32_t height, uint32_t stride,
                                uint32_t *samples_device, uint32_t *counts_device) {
  const auto t0 = std::chrono::steady_clock::now();
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  SamplerPlan pl;
  PD_TRY(plan_sampler(s, &pl));
  PD_CHECK(stride >= pl.stride, PD_ERR_INVALID, "stride %u below the %u samples per image this sampler needs", stride,
           pl.stride);
  ctx->sample_stats = pd_sample_stats{};
  if (n_images == 0) return PD_OK;
  PD_CHECK(images_device && labels_device && samples_device && counts_device, PD_ERR_INVALID, "null argument");
  const uint64_t np = (uint64_t)width * height, db = np * s->pixel_bytes;
  PD_CHECK(width >= 1 && height >= 1 && np < (1ull << 31), PD_ERR_UNSUPPORTED, "images are %ux%u", width, height);
  PD_CHECK(db % 16 == 0 && np % 16 == 0 && ((uintptr_t)images_device % 16) == 0 &&
               ((uintptr_t)labels_device % 16) == 0,
           PD_ERR_UNSUPPORTED,
           "device images need 16-byte aligned buffers and W*H and W*H*pixel_bytes multiples of 16 (pd_sample "
           "takes any size)");
  PD_CUDA(cudaSetDevice(ctx->device));
  const uint64_t h2d0 = ctx->bytes_h2d, d2h0 = ctx->bytes_d2h;
  std::vector<ImagePlace> place(n_images);
  for (uint32_t i = 0; i < n_images; i++)
    place[i] = ImagePlace{i * db, (i + 1) * db, i * np, (uint64_t)i * stride, db, (uint32_t)np};
  DescLayout lay;
  PD_TRY(fill_desc(ctx->h_sm_desc, pl, place, &lay));
  PD_TRY(ctx->sm_desc.ensure(lay.bytes));
  PD_TRY(launch_batch(ctx, s, pl, n_images, static_cast<const uint8_t *>(images_device), labels_device,
                      samples_device, counts_device, lay, ctx->sm_desc.as<uint8_t>(), ctx->h_sm_desc.ptr, ctx->ev));
  uint32_t err[2];
  PD_CUDA(d2h(ctx, err, ctx->sm_desc.as<uint8_t>() + lay.err, 8));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  PD_TRY(check_errors(err, 0, s));
  ctx->sample_stats.images = n_images;
  ctx->sample_stats.data_bytes = db * n_images;
  ctx->sample_stats.label_bytes = np * n_images;
  ctx->sample_stats.ms_scan = event_ms(ctx->ev[0], ctx->ev[1]);
  ctx->sample_stats.ms_draw = event_ms(ctx->ev[1], ctx->ev[2]);
  ctx->sample_stats.h2d_bytes = ctx->bytes_h2d - h2d0;
  ctx->sample_stats.d2h_bytes = ctx->bytes_d2h - d2h0;
  ctx->sample_stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return PD_OK;
}
