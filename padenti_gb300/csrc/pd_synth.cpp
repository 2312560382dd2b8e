// Seeded synthetic training sets (depth maps with ellipse bodies, RGB Voronoi
// images).  Integer-only arithmetic with a counter-based splitmix64 hash, so
// every host produces the same bytes; images are generated in parallel.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "padenti_gb300.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() { return mix64(s++ * 0xD1B54A32D192ED03ull); }
  // uniform integer in [lo, hi] (modulo reduction of 64 random bits)
  int64_t range(int64_t lo, int64_t hi) { return lo + (int64_t)(next() % (uint64_t)(hi - lo + 1)); }
};

inline uint64_t stream_seed(uint64_t seed, uint64_t image, uint64_t stream) {
  return mix64(seed ^ mix64(image * 0x100000001ull + stream));
}

// 8 angular sectors of (dx,dy) by sign and |dx| vs |dy| comparisons.
inline int octant(int64_t dx, int64_t dy) {
  if (dx == 0 && dy == 0) return 0;
  if (dy >= 0 && dx > 0) return dy < dx ? 0 : 1;
  if (dx <= 0 && dy > 0) return -dx < dy ? 2 : 3;
  if (dy <= 0 && dx < 0) return -dy < -dx ? 4 : 5;
  return dx < -dy ? 6 : 7;
}

// Rounded N(0, sigma^2) from an Irwin-Hall sum of twelve 16-bit uniforms.
inline int32_t gauss_noise(uint64_t base, uint64_t pix, int32_t sigma) {
  int64_t s = 0;
  for (int k = 0; k < 3; k++) {
    const uint64_t h = mix64(base + pix * 3 + k);
    s += (int64_t)(h & 0xffff) + (int64_t)((h >> 16) & 0xffff) + (int64_t)((h >> 32) & 0xffff) +
         (int64_t)((h >> 48) & 0xffff);
  }
  const int64_t z = 2 * s - 2 * 393210;  // twice the centred sum (mean 12*32767.5)
  const int64_t num = (int64_t)sigma * z;  // noise = num / 131072, rounded half away from zero
  return (int32_t)(num >= 0 ? (num + 65536) >> 17 : -((-num + 65536) >> 17));
}

template <typename Fn>
void parallel_images(uint32_t n, Fn fn) {
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  nt = std::min<unsigned>(nt, n ? n : 1);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&, t] {
      for (uint32_t i = t; i < n; i += nt) fn(i);
    });
  for (auto &x : th) x.join();
}

void draw_samples(Rng &rng, const std::vector<uint32_t> &fg, const std::vector<uint32_t> &bg, uint32_t n,
                  uint32_t bg_permille, uint32_t *out) {
  uint32_t n_bg = (uint32_t)(((uint64_t)n * bg_permille + 500) / 1000);
  if (fg.empty()) n_bg = n;
  if (bg.empty()) n_bg = 0;
  const uint32_t n_fg = n - n_bg;
  for (uint32_t k = 0; k < n_fg; k++) out[k] = fg[(size_t)rng.range(0, (int64_t)fg.size() - 1)];
  for (uint32_t k = 0; k < n_bg; k++) out[n_fg + k] = bg[(size_t)rng.range(0, (int64_t)bg.size() - 1)];
  std::sort(out, out + n);
}

}  // namespace

extern "C" int pd_synth_depth(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t W, uint32_t H,
                              uint32_t min_ell, uint32_t max_ell, uint32_t parts, uint32_t samples_per_image,
                              uint32_t bg_permille, uint16_t *pixels, uint8_t *labels, uint32_t *samples) {
  if (!pixels || !labels || !samples || !W || !H || min_ell > max_ell || bg_permille > 1000) return PD_ERR_INVALID;
  const size_t P = (size_t)W * H;
  parallel_images(n_images, [&](uint32_t i) {
    const uint64_t id = (uint64_t)first_image + i;
    Rng rng(stream_seed(seed, id, 0));
    const int64_t bg = rng.range(3000, 4000);
    const int64_t n_e = rng.range(min_ell, max_ell);
    struct Ell {
      int64_t cx, cy, ax, ay, d;
    };
    std::vector<Ell> es((size_t)n_e);
    for (auto &e : es) {
      e.cx = rng.range(0, W - 1);
      e.cy = rng.range(0, H - 1);
      e.ax = rng.range(10, 40);
      e.ay = rng.range(10, 40);
      e.d = rng.range(800, 2500);
    }
    const uint64_t nb = stream_seed(seed, id, 1);
    uint16_t *px = pixels + (size_t)i * P;
    uint8_t *lb = labels + (size_t)i * P;
    std::vector<uint32_t> fg, bgp;
    for (uint32_t y = 0; y < H; y++)
      for (uint32_t x = 0; x < W; x++) {
        int64_t best = bg;
        int cls = 0;
        for (const auto &e : es) {
          const int64_t dx = (int64_t)x - e.cx, dy = (int64_t)y - e.cy;
          if (dx * dx * e.ay * e.ay + dy * dy * e.ax * e.ax <= e.ax * e.ax * e.ay * e.ay && e.d < best) {
            best = e.d;
            cls = parts ? 1 + octant(dx, dy) : (dx < 0 ? 1 : 2);
          }
        }
        const size_t p = (size_t)y * W + x;
        int64_t v = best + gauss_noise(nb, p, 5);
        v = std::min<int64_t>(65535, std::max<int64_t>(1, v));
        px[p] = (uint16_t)v;
        lb[p] = (uint8_t)(cls + 1);
        (cls ? fg : bgp).push_back((uint32_t)p);
      }
    Rng srng(stream_seed(seed, id, 2));
    draw_samples(srng, fg, bgp, samples_per_image, bg_permille, samples + (size_t)i * samples_per_image);
  });
  return PD_OK;
}

extern "C" int pd_synth_rgb(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t W, uint32_t H,
                            uint32_t n_classes, uint32_t samples_per_image, uint8_t *pixels, uint8_t *labels,
                            uint32_t *samples) {
  if (!pixels || !labels || !samples || !W || !H || n_classes < 1 || n_classes > 255) return PD_ERR_INVALID;
  const size_t P = (size_t)W * H;
  std::vector<uint8_t> pal((size_t)n_classes * 3);
  Rng prng(stream_seed(seed, 0xFFFFFFFFull, 7));
  for (auto &c : pal) c = (uint8_t)prng.range(0, 255);
  parallel_images(n_images, [&](uint32_t i) {
    const uint64_t id = (uint64_t)first_image + i;
    Rng rng(stream_seed(seed, id, 0));
    const int64_t n_c = rng.range(8, 20);
    struct Cell {
      int64_t x, y, c;
    };
    std::vector<Cell> cs((size_t)n_c);
    for (auto &c : cs) {
      c.x = rng.range(0, W - 1);
      c.y = rng.range(0, H - 1);
      c.c = rng.range(0, n_classes - 1);
    }
    const uint64_t nb = stream_seed(seed, id, 1);
    uint8_t *px = pixels + (size_t)i * P * 3;
    uint8_t *lb = labels + (size_t)i * P;
    for (uint32_t y = 0; y < H; y++)
      for (uint32_t x = 0; x < W; x++) {
        int64_t bd = -1;
        size_t bi = 0;
        for (size_t k = 0; k < cs.size(); k++) {
          const int64_t dx = (int64_t)x - cs[k].x, dy = (int64_t)y - cs[k].y;
          const int64_t d = dx * dx + dy * dy;
          if (bd < 0 || d < bd) {
            bd = d;
            bi = k;
          }
        }
        const size_t p = (size_t)y * W + x;
        const int64_t cls = cs[bi].c;
        const uint64_t h = mix64(nb + p);
        for (int ch = 0; ch < 3; ch++) {
          const int64_t noise = (int64_t)((h >> (16 * ch)) % 41) - 20;
          const int64_t v = (int64_t)pal[(size_t)cls * 3 + ch] + noise;
          px[p * 3 + ch] = (uint8_t)std::min<int64_t>(255, std::max<int64_t>(0, v));
        }
        lb[p] = (uint8_t)(cls + 1);
      }
    Rng srng(stream_seed(seed, id, 2));
    uint32_t *out = samples + (size_t)i * samples_per_image;
    for (uint32_t k = 0; k < samples_per_image; k++) out[k] = (uint32_t)srng.range(0, (int64_t)P - 1);
    std::sort(out, out + samples_per_image);
  });
  return PD_OK;
}
