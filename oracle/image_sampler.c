/*
 * image_sampler.c -- TEST INFRASTRUCTURE ONLY (part of libpadenti_oracle.so).
 *
 * CPU restatement of Padenti's two pixel samplers, the checker for the CUDA
 * samplers of libpadenti_gb300:
 *   UniformImageSampler::sample        (src/padenti/uniform_image_sampler_impl.hpp:34-63)
 *   ClassWeightedImageSampler          (src/padenti/classweighted_image_sampler_impl.hpp:25-120)
 *
 * The reference draws its randomness from Boost (not vendored; the version is
 * not pinned by its CMakeLists.txt:35).  Restated here from the published
 * algorithms:
 *   - boost::crc_32_type: CRC-32 (reflected polynomial 0xEDB88320, initial
 *     value and final XOR 0xFFFFFFFF).
 *   - boost::random::mt19937: MT19937 (Matsumoto and Nishimura 1998) with the
 *     standard 32-bit seeding.
 *   - boost::random::uniform_int_distribution<> on a 32-bit engine (Boost >=
 *     1.47): range 0 returns the lower bound without a draw; otherwise the
 *     draw v is divided by the bucket size floor(2^32 / (range+1)) and
 *     rejected while the quotient exceeds the range.
 *   - boost::random::uniform_01<double> on a 32-bit engine: v * 2^-32.
 * Parity status: CRC-32 is pinned against zlib (tests), MT19937 against the
 * C++ standard's known answer and numpy; the samplers' own control flow is
 * pinned against the reference's sampler sources compiled in place
 * (oracle/ref_shim/ref_sampler.cpp) over libstdc++'s mt19937 and zlib's CRC.
 * Boost's two distributions are restated, not pinned (Boost is absent).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "padenti_oracle.h"

/* Byte-at-a-time table CRC (the cost of boost::crc_optimal); the table is the
 * bitwise CRC of each byte value. */
static uint32_t crc_table[256];

__attribute__((constructor)) static void crc_table_init(void) {
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t r = i;
    for (int k = 0; k < 8; k++) r = (r & 1u) ? (r >> 1) ^ 0xEDB88320u : r >> 1;
    crc_table[i] = r;
  }
}

uint32_t or_crc32(const uint8_t *p, uint64_t n) {
  uint32_t r = 0xFFFFFFFFu;
  for (uint64_t i = 0; i < n; i++) r = crc_table[(r ^ p[i]) & 0xFFu] ^ (r >> 8);
  return r ^ 0xFFFFFFFFu;
}

void or_mt_seed(or_mt *m, uint32_t s) {
  m->x[0] = s;
  for (int i = 1; i < 624; i++) m->x[i] = 1812433253u * (m->x[i - 1] ^ (m->x[i - 1] >> 30)) + (uint32_t)i;
  m->i = 624;
}

uint32_t or_mt_next(or_mt *m) {
  if (m->i >= 624) {
    for (int k = 0; k < 624; k++) {
      const uint32_t y = (m->x[k] & 0x80000000u) | (m->x[(k + 1) % 624] & 0x7FFFFFFFu);
      m->x[k] = m->x[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
    }
    m->i = 0;
  }
  uint32_t y = m->x[m->i++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9D2C5680u;
  y ^= (y << 15) & 0xEFC60000u;
  y ^= y >> 18;
  return y;
}

/* uniform_int_distribution<>(0, range) (uniform_image_sampler_impl.hpp:47). */
uint32_t or_uniform_int(or_mt *m, uint32_t range) {
  if (range == 0) return 0;
  if (range == 0xFFFFFFFFu) return or_mt_next(m);
  const uint32_t bucket = (uint32_t)((1ull << 32) / ((uint64_t)range + 1));
  for (;;) {
    const uint32_t q = or_mt_next(m) / bucket;
    if (q <= range) return q;
  }
}

double or_uniform01(or_mt *m) { return (double)or_mt_next(m) * (1.0 / 4294967296.0); }

/* m_perClassBucketSize (classweighted_image_sampler_impl.hpp:25-43): float
 * product, then ceil; weights NULL = 1.f/nClasses each. */
uint32_t or_bucket_sizes(uint32_t n_samples, uint32_t n_classes, const float *weights, uint32_t *sizes) {
  uint32_t total = 0;
  const float p = 1.f / (float)n_classes;
  for (uint32_t k = 0; k < n_classes; k++) {
    const float w = weights ? weights[k] : p;
    sizes[k] = (uint32_t)ceilf(w * (float)n_samples);
    total += sizes[k];
  }
  return total;
}

static int cmp_u32(const void *a, const void *b) {
  const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : x > y;
}

/* UniformImageSampler::sample (uniform_image_sampler_impl.hpp:34-63).  An
 * image without labelled pixels returns 0 samples (the reference then draws
 * from an empty buffer). */
uint32_t or_sample_uniform(const void *data, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                           uint32_t n_samples, uint32_t seed, uint32_t *out) {
  uint32_t *nz = (uint32_t *)malloc((size_t)n_pix * sizeof(uint32_t) + 4);
  uint32_t n = 0;
  for (uint32_t i = 0; i < n_pix; i++)
    if (labels[i]) nz[n++] = i;
  if (n == 0) {
    free(nz);
    return 0;
  }
  or_mt m;
  or_mt_seed(&m, or_crc32((const uint8_t *)data, data_bytes) ^ seed);
  for (uint32_t i = 0; i < n_samples; i++) out[i] = nz[or_uniform_int(&m, n - 1)];
  qsort(out, n_samples, sizeof(uint32_t), cmp_u32);
  free(nz);
  return n_samples;
}

/* ClassWeightedImageSampler::sample (classweighted_image_sampler_impl.hpp:52-120):
 * per-class reservoir over the pixels in scan order; a pixel of class k that
 * finds its bucket full draws u and replaces slot roundf(u * seen_k) if it is
 * in the bucket.  Returns the number of samples, or -1 for a label above
 * n_classes (the reference indexes past its buckets then). */
int64_t or_sample_class_weighted(const void *data, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                                 uint32_t n_classes, const uint32_t *sizes, uint32_t seed, uint32_t *out) {
  uint32_t total = 0, off[256], filled[256], seen[256];
  if (n_classes > 256) return -1;
  for (uint32_t k = 0; k < n_classes; k++) {
    off[k] = total;
    total += sizes[k];
    filled[k] = seen[k] = 0;
  }
  uint32_t *bucket = (uint32_t *)malloc((size_t)total * sizeof(uint32_t) + 4);
  or_mt m;
  or_mt_seed(&m, or_crc32((const uint8_t *)data, data_bytes) ^ seed);
  for (uint32_t i = 0; i < n_pix; i++) {
    if (!labels[i]) continue;
    const uint32_t k = labels[i] - 1u;
    if (k >= n_classes) {
      free(bucket);
      return -1;
    }
    if (filled[k] < sizes[k]) {
      bucket[off[k] + filled[k]++] = i;
    } else {
      const uint32_t j = (uint32_t)roundf((float)(or_uniform01(&m) * (double)seen[k]));
      if (j < sizes[k]) bucket[off[k] + j] = i;
    }
    seen[k]++;
  }
  uint32_t n = 0;
  for (uint32_t k = 0; k < n_classes; k++)
    for (uint32_t s = 0; s < filled[k]; s++) out[n++] = bucket[off[k] + s];
  qsort(out, n, sizeof(uint32_t), cmp_u32);
  free(bucket);
  return n;
}

/* A batch of same-size images (images n*data_bytes, labels n*n_pix), over all
 * host threads: the CPU baseline of the samplers.  kind 1 = uniform, 2 =
 * class-weighted (sizes from or_bucket_sizes); out has stride samples per
 * image; counts[i] as the single-image functions return. */
void or_sample_batch(int kind, const void *images, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                     uint32_t n_images, uint32_t n_samples, uint32_t n_classes, const uint32_t *sizes, uint32_t seed,
                     uint32_t stride, uint32_t *out, int64_t *counts) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < (int64_t)n_images; i++) {
    const uint8_t *d = (const uint8_t *)images + (uint64_t)i * data_bytes;
    const uint8_t *l = labels + (uint64_t)i * n_pix;
    counts[i] = kind == 1 ? (int64_t)or_sample_uniform(d, data_bytes, l, n_pix, n_samples, seed, out + (uint64_t)i * stride)
                          : or_sample_class_weighted(d, data_bytes, l, n_pix, n_classes, sizes, seed,
                                                     out + (uint64_t)i * stride);
  }
}
