/*
 * TEST INFRASTRUCTURE ONLY: the seeded synthetic depth maps of the benchmark
 * (the library's pd_synth_depth, padenti_gb300/csrc/pd_synth.cpp) restated in
 * C for the reference arm of bench.py, which must build its inputs without
 * loading the CUDA library.  Same integer arithmetic (splitmix64 counter hash,
 * Irwin-Hall noise, modulo-reduced ranges), so the bytes are identical; a CPU
 * test checks them against pd_synth_depth.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "padenti_oracle.h"

static uint64_t sy_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static uint64_t sy_next(uint64_t *s) { return sy_mix64((*s)++ * 0xD1B54A32D192ED03ull); }
static int64_t sy_range(uint64_t *s, int64_t lo, int64_t hi) {
  return lo + (int64_t)(sy_next(s) % (uint64_t)(hi - lo + 1));
}
static uint64_t sy_stream(uint64_t seed, uint64_t image, uint64_t stream) {
  return sy_mix64(seed ^ sy_mix64(image * 0x100000001ull + stream));
}
static int sy_octant(int64_t dx, int64_t dy) {
  if (dx == 0 && dy == 0) return 0;
  if (dy >= 0 && dx > 0) return dy < dx ? 0 : 1;
  if (dx <= 0 && dy > 0) return -dx < dy ? 2 : 3;
  if (dy <= 0 && dx < 0) return -dy < -dx ? 4 : 5;
  return dx < -dy ? 6 : 7;
}
static int32_t sy_noise(uint64_t base, uint64_t pix, int32_t sigma) {
  int64_t s = 0;
  for (int k = 0; k < 3; k++) {
    const uint64_t h = sy_mix64(base + pix * 3 + (uint64_t)k);
    s += (int64_t)(h & 0xffff) + (int64_t)((h >> 16) & 0xffff) + (int64_t)((h >> 32) & 0xffff) +
         (int64_t)((h >> 48) & 0xffff);
  }
  const int64_t z = 2 * s - 2 * 393210;
  const int64_t num = (int64_t)sigma * z;
  return (int32_t)(num >= 0 ? (num + 65536) >> 17 : -((-num + 65536) >> 17));
}
static int sy_cmp_u32(const void *a, const void *b) {
  const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : (x > y);
}

int or_synth_depth(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t W, uint32_t H,
                   uint32_t min_ell, uint32_t max_ell, uint32_t parts, uint32_t samples_per_image,
                   uint32_t bg_permille, uint16_t *pixels, uint8_t *labels, uint32_t *samples) {
  if (!pixels || !labels || !samples || !W || !H || min_ell > max_ell || bg_permille > 1000) return -1;
  const size_t P = (size_t)W * H;
  int rc = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(min : rc)
  for (int64_t ii = 0; ii < (int64_t)n_images; ii++) {
    const uint64_t id = (uint64_t)first_image + (uint64_t)ii;
    uint64_t rng = sy_stream(seed, id, 0);
    const int64_t bg = sy_range(&rng, 3000, 4000);
    const int64_t n_e = sy_range(&rng, min_ell, max_ell);
    int64_t ell[64][5];
    if (n_e > 64) { rc = -1; continue; }
    for (int64_t e = 0; e < n_e; e++) {
      ell[e][0] = sy_range(&rng, 0, (int64_t)W - 1);
      ell[e][1] = sy_range(&rng, 0, (int64_t)H - 1);
      ell[e][2] = sy_range(&rng, 10, 40);
      ell[e][3] = sy_range(&rng, 10, 40);
      ell[e][4] = sy_range(&rng, 800, 2500);
    }
    const uint64_t nb = sy_stream(seed, id, 1);
    uint16_t *px = pixels + (size_t)ii * P;
    uint8_t *lb = labels + (size_t)ii * P;
    uint32_t *fg = (uint32_t *)malloc(sizeof(uint32_t) * P), *bgp = (uint32_t *)malloc(sizeof(uint32_t) * P);
    size_t nfg = 0, nbg = 0;
    for (uint32_t y = 0; y < H; y++)
      for (uint32_t x = 0; x < W; x++) {
        int64_t best = bg;
        int cls = 0;
        for (int64_t e = 0; e < n_e; e++) {
          const int64_t dx = (int64_t)x - ell[e][0], dy = (int64_t)y - ell[e][1];
          const int64_t ax = ell[e][2], ay = ell[e][3];
          if (dx * dx * ay * ay + dy * dy * ax * ax <= ax * ax * ay * ay && ell[e][4] < best) {
            best = ell[e][4];
            cls = parts ? 1 + sy_octant(dx, dy) : (dx < 0 ? 1 : 2);
          }
        }
        const size_t p = (size_t)y * W + x;
        int64_t v = best + sy_noise(nb, p, 5);
        v = v < 1 ? 1 : (v > 65535 ? 65535 : v);
        px[p] = (uint16_t)v;
        lb[p] = (uint8_t)(cls + 1);
        if (cls) fg[nfg++] = (uint32_t)p;
        else bgp[nbg++] = (uint32_t)p;
      }
    uint64_t srng = sy_stream(seed, id, 2);
    uint32_t n = samples_per_image;
    uint32_t n_bg = (uint32_t)(((uint64_t)n * bg_permille + 500) / 1000);
    if (!nfg) n_bg = n;
    if (!nbg) n_bg = 0;
    const uint32_t n_fg = n - n_bg;
    uint32_t *out = samples + (size_t)ii * samples_per_image;
    for (uint32_t k = 0; k < n_fg; k++) out[k] = fg[(size_t)sy_range(&srng, 0, (int64_t)nfg - 1)];
    for (uint32_t k = 0; k < n_bg; k++) out[n_fg + k] = bgp[(size_t)sy_range(&srng, 0, (int64_t)nbg - 1)];
    qsort(out, n, sizeof(uint32_t), sy_cmp_u32);
    free(fg);
    free(bgp);
  }
  return rc;
}
