/*
 * padenti_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of Padenti's training and prediction hot path.  Each
 * function names the reference file:line it follows (paths relative to the
 * Padenti source tree).  Parity is pinned for the MD5 counter RNG (hashlib
 * known answers and the reference prng.hpp compiled from source), for the
 * split rule (the reference learnBestFeature kernel compiled from source) and
 * for the single-offset depth plugin (the reference test/feature.cl compiled
 * from source); the remaining steps are "parity unpinned" (the reference
 * cannot be built here: no OpenCL, Boost or OpenCV) and follow the reference
 * line by line.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (no -ffast-math):
 * every float and double operation below is one IEEE operation in source order.
 */
#include "padenti_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <omp.h>

#define NT(n) num_threads((n) > 0 ? (n) : omp_get_max_threads())

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------ */
/* a1: MD5 (RFC 1321) of one 16-byte block, padded as a single 64-byte block. */
/* Follows kernels/hist_update.cl:278-369 and prng.hpp:107-195: the message   */
/* words are (s0,s1,s2,s3, 0x80, 0..., bit length 128, 0).                    */
/* ------------------------------------------------------------------------ */
static const uint32_t MD5_K[64] = {
  0xd76aa478u, 0xe8c7b756u, 0x242070dbu, 0xc1bdceeeu, 0xf57c0fafu, 0x4787c62au, 0xa8304613u, 0xfd469501u,
  0x698098d8u, 0x8b44f7afu, 0xffff5bb1u, 0x895cd7beu, 0x6b901122u, 0xfd987193u, 0xa679438eu, 0x49b40821u,
  0xf61e2562u, 0xc040b340u, 0x265e5a51u, 0xe9b6c7aau, 0xd62f105du, 0x02441453u, 0xd8a1e681u, 0xe7d3fbc8u,
  0x21e1cde6u, 0xc33707d6u, 0xf4d50d87u, 0x455a14edu, 0xa9e3e905u, 0xfcefa3f8u, 0x676f02d9u, 0x8d2a4c8au,
  0xfffa3942u, 0x8771f681u, 0x6d9d6122u, 0xfde5380cu, 0xa4beea44u, 0x4bdecfa9u, 0xf6bb4b60u, 0xbebfbc70u,
  0x289b7ec6u, 0xeaa127fau, 0xd4ef3085u, 0x04881d05u, 0xd9d4d039u, 0xe6db99e5u, 0x1fa27cf8u, 0xc4ac5665u,
  0xf4292244u, 0x432aff97u, 0xab9423a7u, 0xfc93a039u, 0x655b59c3u, 0x8f0ccc92u, 0xffeff47du, 0x85845dd1u,
  0x6fa87e4fu, 0xfe2ce6e0u, 0xa3014314u, 0x4e0811a1u, 0xf7537e82u, 0xbd3af235u, 0x2ad7d2bbu, 0xeb86d391u};
static const int MD5_R[4][4] = {{7, 12, 17, 22}, {5, 9, 14, 20}, {4, 11, 16, 23}, {6, 10, 15, 21}};

static inline uint32_t rotl32(uint32_t x, int s) { return (x << s) | (x >> (32 - s)); }

void or_md5(const uint32_t in[4], uint32_t out[4]) {
  uint32_t m[16] = {0};
  m[0] = in[0]; m[1] = in[1]; m[2] = in[2]; m[3] = in[3];
  m[4] = 0x80u;      /* padding byte after the 16 message bytes */
  m[14] = 128u;      /* message length in bits */
  uint32_t a = 0x67452301u, b = 0xefcdab89u, c = 0x98badcfeu, d = 0x10325476u;
  for (int i = 0; i < 64; i++) {
    uint32_t fn;
    int g, round = i >> 4;
    if (round == 0) { fn = (b & c) | (~b & d); g = i; }
    else if (round == 1) { fn = (d & b) | (~d & c); g = (5 * i + 1) & 15; }
    else if (round == 2) { fn = b ^ c ^ d; g = (3 * i + 5) & 15; }
    else { fn = c ^ (b | ~d); g = (7 * i) & 15; }
    uint32_t tmp = d;
    d = c;
    c = b;
    b = b + rotl32(a + fn + MD5_K[i] + m[g], MD5_R[round][i & 3]);
    a = tmp;
  }
  out[0] = a + 0x67452301u;
  out[1] = b + 0xefcdab89u;
  out[2] = c + 0x98badcfeu;
  out[3] = d + 0x10325476u;
}

/* ------------------------------------------------------------------------ */
/* a2 + a3: candidate generation.                                           */
/* Features: kernels/hist_update.cl:62-114 (host twin learn_best_featthr:183-208). */
/* Thresholds: kernels/hist_update.cl:127-184 (host twin learn_best_featthr:210-222). */
/* value = low + (feat_t)((float)rand / (float)0xFFFFFFFF * (float)(up - low)) */
/* ------------------------------------------------------------------------ */
static inline int32_t to_feat(float x, int32_t ft) {
  int32_t v = (int32_t)x; /* conversion toward zero */
  return ft == OR_FEAT_I16 ? (int32_t)(int16_t)v : v;
}
static inline int32_t feat_add(int32_t a, int32_t b, int32_t ft) {
  int32_t s = (int32_t)((uint32_t)a + (uint32_t)b);
  return ft == OR_FEAT_I16 ? (int32_t)(int16_t)s : s;
}
static inline int32_t draw(uint32_t r, int32_t lo, int32_t hi, int32_t ft) {
  float range = (float)(int32_t)((uint32_t)hi - (uint32_t)lo);
  float x = (float)r / (float)0xFFFFFFFFu * range;
  return feat_add(lo, to_feat(x, ft), ft);
}

void or_candidate(const or_params *p, uint32_t tree_id, uint32_t node, uint32_t f,
                  int32_t *feat_out, int32_t *thr_out) {
  uint32_t seed[4] = {tree_id, node, f, 0u}, st[4];
  const int D = p->feat_dim;
  for (int i = 0; i < D; i += 4) {
    or_md5(seed, st);
    for (int j = 0; j < 4 && i + j < D; j++)
      feat_out[i + j] = draw(st[j], p->feat_low[i + j], p->feat_up[i + j], p->feat_type);
    memcpy(seed, st, sizeof(st));
  }
  if (!thr_out) return;
  seed[0] = tree_id; seed[1] = node; seed[2] = f; seed[3] = 1u;
  for (uint32_t t = 0; t < p->n_thresholds; t++) {
    if ((t & 3u) == 0) {
      or_md5(seed, st);
      memcpy(seed, st, sizeof(st));
    }
    thr_out[t] = draw(st[t & 3u], p->thr_low, p->thr_up, p->feat_type);
  }
}

/* ------------------------------------------------------------------------ */
/* a4: built-in plugins.                                                    */
/* ------------------------------------------------------------------------ */
#define BG_DEPTH 10000

static inline int32_t depth_at(const uint16_t *img, uint32_t w, uint32_t h, int32_t x, int32_t y) {
  if (x < 0 || y < 0 || (uint32_t)x >= w || (uint32_t)y >= h) return BG_DEPTH;
  uint16_t v = img[(size_t)y * w + (size_t)x];
  return v ? (int32_t)v : BG_DEPTH;
}

int32_t or_feature(int32_t plugin, int32_t feat_type, const void *img, uint32_t w, uint32_t h,
                   uint32_t n_channels, int32_t x, int32_t y, const int32_t *feat) {
  (void)feat_type;
  if (plugin == OR_PLUGIN_DEPTH_DIFF2) {
    /* Two-offset depth difference I(x+u/d(x)) - I(x+v/d(x)); out-of-image and
     * zero-depth probes read 10000; a zero centre depth scales as 10000. */
    const uint16_t *im = (const uint16_t *)img;
    uint16_t c = im[(size_t)y * w + (size_t)x];
    float d = (float)(c ? (int32_t)c : BG_DEPTH);
    int32_t x1 = x + (int32_t)roundf((float)feat[0] / d);
    int32_t y1 = y + (int32_t)roundf((float)feat[1] / d);
    int32_t x2 = x + (int32_t)roundf((float)feat[2] / d);
    int32_t y2 = y + (int32_t)roundf((float)feat[3] / d);
    return depth_at(im, w, h, x1, y1) - depth_at(im, w, h, x2, y2);
  }
  if (plugin == OR_PLUGIN_DEPTH_DIFF1) {
    /* test/feature.cl:29-64 with feat_t = short. */
    const uint16_t *im = (const uint16_t *)img;
    int16_t depth = (int16_t)im[(size_t)y * w + (size_t)x];
    int32_t response = depth;
    int32_t probe;
    if (depth == 0) {
      probe = BG_DEPTH; /* undefined in the reference (division by zero): read as background */
    } else {
      int32_t ox = x + (int32_t)roundf((float)feat[0] * 500.0f / (float)depth);
      int32_t oy = y + (int32_t)roundf((float)feat[1] * 500.0f / (float)depth);
      int out = ox < 0 || oy < 0 || (uint32_t)ox >= w || (uint32_t)oy >= h;
      int16_t dd = out ? (int16_t)BG_DEPTH : (int16_t)im[(size_t)oy * w + (size_t)ox];
      probe = dd ? dd : BG_DEPTH;
    }
    return (int32_t)(int16_t)(response - probe);
  }
  if (plugin == OR_PLUGIN_CHANNEL_DIFF) {
    const uint8_t *im = (const uint8_t *)img;
    int32_t c1 = feat[0] < 0 ? 0 : (feat[0] > 2 ? 2 : feat[0]);
    int32_t c2 = feat[1] < 0 ? 0 : (feat[1] > 2 ? 2 : feat[1]);
    int32_t x1 = x + feat[2], y1 = y + feat[3], x2 = x + feat[4], y2 = y + feat[5];
    int32_t a = 0, b = 0;
    if (x1 >= 0 && y1 >= 0 && (uint32_t)x1 < w && (uint32_t)y1 < h)
      a = im[((size_t)y1 * w + (size_t)x1) * n_channels + (size_t)c1];
    if (x2 >= 0 && y2 >= 0 && (uint32_t)x2 < w && (uint32_t)y2 < h)
      b = im[((size_t)y2 * w + (size_t)x2) * n_channels + (size_t)c2];
    return a - b;
  }
  return 0;
}

/* The tree a feature that reads it sees: this image's node map (NULL: none),
 * the tree's left children and posteriors, the class count, the map's level
 * (root 0) and the tree's node count.  The feature reads the splits of nodes
 * above the level (-1 at and below it) and the posteriors of nodes down to it
 * (0 below): the part of the tree that is the same in training and prediction. */
typedef struct {
  const int32_t *nodes;
  const int32_t *lc;
  const float *post;
  uint32_t K;
  int32_t level, n_nodes;
} tree_view;

static inline int32_t node_level(int32_t n) {
  int32_t l = 0;
  for (uint32_t v = (uint32_t)n + 1u; v > 1u; v >>= 1) l++;
  return l;
}
static inline int32_t view_left_child(const tree_view *tv, int32_t n) {
  if (!tv || !tv->lc || n < 0 || n >= tv->n_nodes || node_level(n) >= tv->level) return -1;
  return tv->lc[n];
}
static inline float view_posterior(const tree_view *tv, int32_t n, int32_t k) {
  if (!tv || !tv->post || n < 0 || n >= tv->n_nodes || node_level(n) > tv->level || k < 0 || (uint32_t)k >= tv->K)
    return 0.0f;
  return tv->post[(size_t)n * tv->K + (uint32_t)k];
}

static int32_t feature_at(int32_t plugin, int32_t feat_type, const void *img, uint32_t w, uint32_t h,
                          uint32_t n_channels, int32_t x, int32_t y, const int32_t *feat, const tree_view *tv) {
  if (plugin != OR_PLUGIN_AUTO_CONTEXT) return or_feature(plugin, feat_type, img, w, h, n_channels, x, y, feat);
  const uint16_t *im = (const uint16_t *)img;
  const int32_t x1 = x + feat[0], y1 = y + feat[1];
  int32_t n1 = 0;
  if (tv && tv->nodes && x1 >= 0 && y1 >= 0 && (uint32_t)x1 < w && (uint32_t)y1 < h)
    n1 = tv->nodes[(size_t)y1 * w + (size_t)x1];
  const int32_t K = tv && tv->K ? (int32_t)tv->K : 1;
  const int32_t k = ((feat[2] % K) + K) % K;
  const float pv = view_posterior(tv, n1, k);
  const int32_t inner = view_left_child(tv, n1) >= 0 ? 2000 : 0;
  const int32_t x3 = x + feat[3];
  const int32_t a = x3 >= 0 && (uint32_t)x3 < w ? (int32_t)im[(size_t)y * w + (size_t)x3] : 0;
  const int32_t b = (int32_t)im[(size_t)y * w + (size_t)x];
  return (int32_t)(pv * 1000.0f) + inner + (a - b) / 16 + n1 % 5;
}

/* ------------------------------------------------------------------------ */
/* Exact log2 of integers in double-double arithmetic (Dekker 1971 products,  */
/* Knuth two-sum, Hida-Li-Bailey double-double add/mul/div), evaluated with   */
/* the series ln(m) = 2 atanh((m-1)/(m+1)).  Only IEEE +,-,*,/ in a fixed     */
/* order, so the table is identical on every IEEE machine.                    */
/* ------------------------------------------------------------------------ */
typedef struct { double hi, lo; } dd_t;

static inline dd_t two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  dd_t r = {s, e};
  return r;
}
static inline dd_t quick_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  dd_t r = {s, e};
  return r;
}
static inline void split27(double a, double *hi, double *lo) {
  double t = 134217729.0 * a;
  *hi = t - (t - a);
  *lo = a - *hi;
}
static inline dd_t two_prod(double a, double b) {
  double p = a * b, ah, al, bh, bl;
  split27(a, &ah, &al);
  split27(b, &bh, &bl);
  double e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
  dd_t r = {p, e};
  return r;
}
static inline dd_t dd_add(dd_t a, dd_t b) {
  dd_t s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
static inline dd_t dd_mul(dd_t a, dd_t b) {
  dd_t p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
static inline dd_t dd_mul_d(dd_t a, double b) {
  dd_t p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
static inline dd_t dd_div(dd_t a, dd_t b) {
  double q1 = a.hi / b.hi;
  dd_t r = dd_add(a, dd_mul_d(b, -q1));
  double q2 = r.hi / b.hi;
  r = dd_add(r, dd_mul_d(b, -q2));
  double q3 = r.hi / b.hi;
  dd_t q = quick_two_sum(q1, q2);
  dd_t q3d = {q3, 0.0};
  return dd_add(q, q3d);
}
/* 2*atanh(z) = 2*(z + z^3/3 + z^5/5 + ...) with a fixed number of terms. */
static dd_t dd_2atanh(dd_t z, int terms) {
  dd_t z2 = dd_mul(z, z), term = z, sum = z;
  for (int k = 1; k <= terms; k++) {
    term = dd_mul(term, z2);
    dd_t den = {(double)(2 * k + 1), 0.0};
    sum = dd_add(sum, dd_div(term, den));
  }
  return dd_mul_d(sum, 2.0);
}
static double dd_log2_u32(uint32_t n, dd_t inv_ln2) {
  if (n <= 1) return 0.0;
  int e = 31;
  while (!((n >> e) & 1u)) e--;
  double m = (double)n / (double)(1u << e); /* exact, in [1,2) */
  if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
  dd_t num = {m - 1.0, 0.0};                 /* exact (Sterbenz) */
  dd_t den = two_sum(m, 1.0);                /* exact pair */
  dd_t z = dd_div(num, den);
  dd_t ln_m = dd_2atanh(z, 24);
  dd_t ed = {(double)e, 0.0};
  dd_t r = dd_add(ed, dd_mul(ln_m, inv_ln2));
  return r.hi;
}

void or_log2_table(uint32_t n, double *out) {
  dd_t one = {1.0, 0.0}, three = {3.0, 0.0};
  dd_t ln2 = dd_2atanh(dd_div(one, three), 40); /* ln 2 = 2 atanh(1/3) */
  dd_t inv_ln2 = dd_div(one, ln2);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) out[i] = dd_log2_u32((uint32_t)i, inv_ln2);
}

/* ------------------------------------------------------------------------ */
/* Dataset helpers                                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint32_t img;
  int32_t x, y;
  uint32_t label; /* class 0..K-1 */
} sample_t;

static sample_t *flatten_samples(const or_dataset *ds, uint64_t *n_out) {
  uint64_t S = ds->samp_off[ds->n_images];
  sample_t *s = (sample_t *)malloc(sizeof(sample_t) * (S ? S : 1));
  for (uint32_t i = 0; i < ds->n_images; i++) {
    for (uint64_t k = ds->samp_off[i]; k < ds->samp_off[i + 1]; k++) {
      uint32_t pix = ds->samples[k];
      s[k].img = i;
      s[k].x = (int32_t)(pix % ds->width[i]);
      s[k].y = (int32_t)(pix / ds->width[i]);
      s[k].label = (uint32_t)ds->labels[ds->lab_off[i] + pix] - 1u;
    }
  }
  *n_out = S;
  return s;
}

static inline const void *image_ptr(const or_dataset *ds, uint32_t i) {
  return ds->pixels + ds->pix_off[i];
}

/* ------------------------------------------------------------------------ */
/* a5 + a6: per-node histograms.                                            */
/* kernels/hist_update.cl:116-186 (indicator feat <= thr per threshold) and  */
/* cl_tree_trainer_impl_traverse_ts.hpp:518-617 (hist[node][label-1][t][f]   */
/* accumulation, samples outside the trained nodes skipped).                 */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t node; uint32_t slot; } node_slot_t;
static int cmp_node_slot(const void *a, const void *b) {
  int32_t x = ((const node_slot_t *)a)->node, y = ((const node_slot_t *)b)->node;
  return (x > y) - (x < y);
}
static int64_t find_slot(const node_slot_t *m, uint32_t n, int32_t node) {
  int64_t lo = 0, hi = (int64_t)n - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) >> 1;
    if (m[mid].node == node) return m[mid].slot;
    if (m[mid].node < node) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

/* Node maps of a training set for features that read the tree: map of image i
 * from moff[i], the tree as the histograms of a depth see it. */
typedef struct {
  const int32_t *map;
  const uint64_t *moff;
  const int32_t *lc;
  const float *post;
  uint32_t K;
  int32_t level, n_nodes;
} set_view;

static int hist_impl(const or_params *p, const or_dataset *ds, uint32_t tree_id, const int32_t *sample_node,
                     const int32_t *nodes, uint32_t n_nodes, uint32_t *hist, int reference_cost, int n_threads,
                     const set_view *sv);

int or_hist(const or_params *p, const or_dataset *ds, uint32_t tree_id,
            const int32_t *sample_node, const int32_t *nodes, uint32_t n_nodes,
            uint32_t *hist, int reference_cost, int n_threads) {
  return hist_impl(p, ds, tree_id, sample_node, nodes, n_nodes, hist, reference_cost, n_threads, NULL);
}

int or_hist_tree(const or_params *p, const or_dataset *ds, uint32_t tree_id, const int32_t *sample_node,
                 const int32_t *nodes, uint32_t n_nodes, uint32_t *hist, const int32_t *maps, const int32_t *lc,
                 const float *post, int32_t level, int32_t tree_nodes, int n_threads) {
  uint64_t *moff = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)ds->n_images + 1));
  moff[0] = 0;
  for (uint32_t i = 0; i < ds->n_images; i++) moff[i + 1] = moff[i] + (uint64_t)ds->width[i] * ds->height[i];
  set_view sv = {maps, moff, lc, post, (uint32_t)p->n_classes, level, tree_nodes};
  const int rc = hist_impl(p, ds, tree_id, sample_node, nodes, n_nodes, hist, 0, n_threads, &sv);
  free(moff);
  return rc;
}

static int hist_impl(const or_params *p, const or_dataset *ds, uint32_t tree_id, const int32_t *sample_node,
                     const int32_t *nodes, uint32_t n_nodes, uint32_t *hist, int reference_cost, int n_threads,
                     const set_view *sv) {
  const uint32_t F = p->n_features, T = p->n_thresholds, K = (uint32_t)p->n_classes;
  const int D = p->feat_dim;
  uint64_t S;
  sample_t *smp = flatten_samples(ds, &S);

  /* node -> slot map */
  node_slot_t *map = (node_slot_t *)malloc(sizeof(node_slot_t) * (n_nodes ? n_nodes : 1));
  for (uint32_t i = 0; i < n_nodes; i++) { map[i].node = nodes[i]; map[i].slot = i; }
  qsort(map, n_nodes, sizeof(node_slot_t), cmp_node_slot);

  /* active samples and their slots */
  uint64_t *act = (uint64_t *)malloc(sizeof(uint64_t) * (S ? S : 1));
  uint32_t *act_slot = (uint32_t *)malloc(sizeof(uint32_t) * (S ? S : 1));
  uint64_t n_act = 0;
  for (uint64_t s = 0; s < S; s++) {
    int64_t sl = find_slot(map, n_nodes, sample_node[s]);
    if (sl >= 0) { act[n_act] = s; act_slot[n_act] = (uint32_t)sl; n_act++; }
  }

  memset(hist, 0, sizeof(uint32_t) * (size_t)n_nodes * K * T * F);

  int32_t *cf = NULL, *ct = NULL;
  if (!reference_cost) {
    cf = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_nodes * F * D);
    ct = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_nodes * F * T);
#pragma omp parallel for schedule(static) NT(n_threads)
    for (int64_t q = 0; q < (int64_t)n_nodes * F; q++)
      or_candidate(p, tree_id, (uint32_t)nodes[q / F], (uint32_t)(q % F), cf + (size_t)q * D, ct + (size_t)q * T);
  }

  /* the active samples grouped by slot (stable counting sort): one (slot, f)
   * work item then counts its samples into a private K x T block and writes
   * the column once (no writes shared between threads) */
  uint64_t *slot_off = (uint64_t *)calloc((size_t)n_nodes + 1, sizeof(uint64_t));
  uint64_t *by_slot = (uint64_t *)malloc(sizeof(uint64_t) * (n_act ? n_act : 1));
  for (uint64_t a = 0; a < n_act; a++) slot_off[act_slot[a] + 1]++;
  for (uint32_t i = 0; i < n_nodes; i++) slot_off[i + 1] += slot_off[i];
  {
    uint64_t *pos = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n_nodes + 1));
    memcpy(pos, slot_off, sizeof(uint64_t) * ((size_t)n_nodes + 1));
    for (uint64_t a = 0; a < n_act; a++) by_slot[pos[act_slot[a]]++] = act[a];
    free(pos);
  }
#pragma omp parallel NT(n_threads)
  {
    int32_t feat[OR_MAX_FEAT_DIM];
    int32_t *thr = (int32_t *)malloc(sizeof(int32_t) * (T ? T : 1));
    uint32_t *loc = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)K * T + 1));
#pragma omp for schedule(dynamic, 16)
    for (int64_t q = 0; q < (int64_t)n_nodes * F; q++) {
      const uint32_t slot = (uint32_t)(q / F), f = (uint32_t)(q % F);
      if (slot_off[slot] == slot_off[slot + 1]) continue;
      memset(loc, 0, sizeof(uint32_t) * (size_t)K * T);
      const int32_t *fv = NULL, *tv = NULL;
      if (!reference_cost) {
        fv = cf + ((size_t)slot * F + (size_t)f) * D;
        tv = ct + ((size_t)slot * F + (size_t)f) * T;
      }
      for (uint64_t a = slot_off[slot]; a < slot_off[slot + 1]; a++) {
        const sample_t *sm = &smp[by_slot[a]];
        if (reference_cost) {
          /* the reference kernel regenerates both MD5 chains per (sample, f) */
          or_candidate(p, tree_id, (uint32_t)nodes[slot], f, feat, thr);
          fv = feat; tv = thr;
        }
        tree_view view = {sv ? sv->map + sv->moff[sm->img] : NULL, sv ? sv->lc : NULL, sv ? sv->post : NULL,
                          sv ? sv->K : 0, sv ? sv->level : 0, sv ? sv->n_nodes : 0};
        int32_t r = feature_at(p->plugin, p->feat_type, image_ptr(ds, sm->img), ds->width[sm->img],
                               ds->height[sm->img], ds->n_channels, sm->x, sm->y, fv, &view);
        uint32_t *lp = loc + (size_t)sm->label * T;
        for (uint32_t t = 0; t < T; t++) lp[t] += (uint32_t)(r <= tv[t]);
      }
      uint32_t *hp = hist + ((size_t)slot * K * T) * F + (size_t)f;
      for (size_t i = 0; i < (size_t)K * T; i++) hp[i * F] = loc[i];
    }
    free(thr);
    free(loc);
  }
  free(slot_off); free(by_slot);
  free(cf); free(ct);
  free(act); free(act_slot); free(map); free(smp);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* a7: best split.                                                          */
/* kernels/learn_best_feature.cl:22-111 + learn_best_featthr.hpp:101-112.    */
/* The reference gain H(parent) - (nL/N H(L) + nR/N H(R)), Shannon entropies  */
/* in log2 with probabilities <= 1e-6 dropped, evaluated exactly from the     */
/* integer counts: n H(c, n) = S(c, n) = sum over classes of                  */
/* c (log2 n - log2 c) in IEEE double with a shared log2 table (the cutoff    */
/* p <= 1e-6 is the integer test 1e6*c <= n), so                              */
/*     gain = S(tot, N)/N - (S(cL, nL) + S(cR, nR)) / N.                      */
/* The first (t-major, f-minor) candidate with the largest gain wins.         */
/* ------------------------------------------------------------------------ */
static inline double sum64(const uint32_t *c, uint32_t K, uint64_t n, const double *L) {
  double s = 0.0;
  for (uint32_t l = 0; l < K; l++) {
    uint64_t cl = c[l];
    if (cl != 0 && cl * 1000000ull > n) {
      double d = L[n] - L[cl];
      double t = (double)cl * d;
      s = s + t;
    }
  }
  return s;
}
static inline double gain64(const uint32_t *cl, const uint32_t *cr, uint32_t K, uint64_t N, uint64_t nL,
                            uint64_t nR, double hp, const double *L) {
  double sl = sum64(cl, K, nL, L);
  double sr = sum64(cr, K, nR, L);
  double w = sl + sr;
  double q = w / (double)N;
  return hp - q;
}
/* The reference formula in FP32 (learn_best_feature.cl:75-93) with the integer
 * cutoff; used only to report the FP32/FP64 disagreement. */
static inline float ent32(const uint32_t *c, uint32_t K, uint64_t n) {
  float s = 0.0f;
  for (uint32_t l = 0; l < K; l++) {
    uint64_t cl = c[l];
    if (cl != 0 && cl * 1000000ull > n) {
      float pr = (float)cl / (float)n;
      s -= pr * log2f(pr);
    }
  }
  return s;
}

int or_split(const or_params *p, const uint32_t *hist, const uint32_t *class_tot,
             uint32_t n_nodes, const double *L, uint64_t table_len,
             int32_t *out_t, int32_t *out_f, double *out_gain,
             float *out_gain32_max, double *out_max_abs_err) {
  const uint32_t F = p->n_features, T = p->n_thresholds, K = (uint32_t)p->n_classes;
  /* the FP32 reference formula only when its maximum or error is asked for */
  const int fp32 = out_gain32_max != NULL || out_max_abs_err != NULL;
  int rc = 0;
  double maxerr_all = 0.0;
  /* nodes are independent; the per-node results do not depend on the schedule */
#pragma omp parallel for schedule(dynamic, 1) reduction(min : rc) reduction(max : maxerr_all)
  for (int64_t ii = 0; ii < (int64_t)n_nodes; ii++) {
    const uint32_t i = (uint32_t)ii;
    const uint32_t *tot = class_tot + (size_t)i * K;
    uint64_t N = 0;
    for (uint32_t l = 0; l < K; l++) N += tot[l];
    out_t[i] = -1; out_f[i] = -1; out_gain[i] = 0.0;
    if (out_gain32_max) out_gain32_max[i] = 0.0f;
    if (N == 0) continue;
    if (N >= table_len) { rc = -1; continue; }
    double hp = sum64(tot, K, N, L) / (double)N;
    float hp32 = fp32 ? ent32(tot, K, N) : 0.0f;
    double best = 0.0;
    float best32 = 0.0f;
    double maxerr = 0.0;
    int have = 0;
    uint32_t cl[64], cr[64];
    for (uint32_t t = 0; t < T; t++) {
      for (uint32_t f = 0; f < F; f++) {
        uint64_t nL = 0, nR = 0;
        for (uint32_t l = 0; l < K; l++) {
          cl[l] = hist[(((size_t)i * K + l) * T + t) * F + f];
          cr[l] = tot[l] - cl[l];
          nL += cl[l]; nR += cr[l];
        }
        double g = gain64(cl, cr, K, N, nL, nR, hp, L);
        if (fp32) {
          float hl32 = ent32(cl, K, nL), hr32 = ent32(cr, K, nR);
          float g32 = hp32 - ((float)nL / (float)N * hl32 + (float)nR / (float)N * hr32);
          double err = fabs((double)g32 - g);
          if (err > maxerr) maxerr = err;
          if ((t == 0 && f == 0) || g32 > best32) best32 = g32;
        }
        if (!have || g > best) { best = g; out_t[i] = (int32_t)t; out_f[i] = (int32_t)f; have = 1; }
      }
    }
    out_gain[i] = best;
    if (out_gain32_max) out_gain32_max[i] = best32;
    if (maxerr > maxerr_all) maxerr_all = maxerr;
  }
  if (out_max_abs_err && maxerr_all > *out_max_abs_err) *out_max_abs_err = maxerr_all;
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Training-set priors: training_set_image_impl.hpp:38-52 (per image, over   */
/* labelled samples) and training_set_impl.hpp:116-133 (mean over images).   */
/* ------------------------------------------------------------------------ */
void or_priors(const or_dataset *ds, uint32_t K, float *out) {
  double *acc = (double *)calloc(K, sizeof(double));
  uint32_t *cnt = (uint32_t *)calloc(K, sizeof(uint32_t));
  for (uint32_t i = 0; i < ds->n_images; i++) {
    memset(cnt, 0, sizeof(uint32_t) * K);
    uint32_t tot = 0;
    for (uint64_t k = ds->samp_off[i]; k < ds->samp_off[i + 1]; k++) {
      uint8_t lab = ds->labels[ds->lab_off[i] + ds->samples[k]];
      if (lab) { cnt[lab - 1]++; tot++; }
    }
    for (uint32_t c = 0; c < K; c++) {
      float pr = (float)cnt[c] / (float)tot;
      acc[c] += (double)pr;
    }
  }
  for (uint32_t c = 0; c < K; c++) out[c] = (float)(acc[c] / (double)ds->n_images);
  free(acc); free(cnt);
}

/* ------------------------------------------------------------------------ */
/* One tree: cl_tree_trainer_impl.hpp:203-255 (depth loop),                  */
/* cl_tree_trainer_impl_init.hpp:333-365 (frontier), learn_best_featthr.hpp: */
/* 117-243 (finalize) and kernels/predict.cl:36-85 (reassignment).           */
/* ------------------------------------------------------------------------ */
/* A rank of candidate-sharded training: it splits on candidates [f0, f1) only
 * and `exchange` turns the ranks' best splits into the global ones (the
 * library's pd_train_tree_sharded protocol). */
typedef struct {
  uint32_t f0, f1;
  or_exchange_fn exchange;
  void *user;
} or_shard;

static int64_t gain_key64(double g) {
  int64_t b;
  memcpy(&b, &g, 8);
  return b < 0 ? (INT64_MIN - b - 1) : b;
}

static int train_tree_impl(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                           const float *root_prior, int32_t *lc, int32_t *feats, int32_t *thrs, float *posts,
                           int32_t *sample_leaf, int reference_cost, int n_threads, or_stats *stats,
                           const or_shard *sh);

int or_train_tree(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                  const float *root_prior, int32_t *lc, int32_t *feats, int32_t *thrs,
                  float *posts, int32_t *sample_leaf, int reference_cost, int n_threads,
                  or_stats *stats) {
  return train_tree_impl(p, ds, tree_id, end_depth, root_prior, lc, feats, thrs, posts, sample_leaf, reference_cost,
                         n_threads, stats, NULL);
}

int or_train_tree_sharded(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                          const float *root_prior, uint32_t f0, uint32_t f1, or_exchange_fn exchange, void *user,
                          int32_t *lc, int32_t *feats, int32_t *thrs, float *posts, int32_t *sample_leaf,
                          int n_threads) {
  if (f0 >= f1 || f1 > p->n_features || !exchange) return -1;
  or_shard sh = {f0, f1, exchange, user};
  return train_tree_impl(p, ds, tree_id, end_depth, root_prior, lc, feats, thrs, posts, sample_leaf, 0, n_threads,
                         NULL, &sh);
}

static int train_tree_impl(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                           const float *root_prior, int32_t *lc, int32_t *feats, int32_t *thrs, float *posts,
                           int32_t *sample_leaf, int reference_cost, int n_threads, or_stats *stats,
                           const or_shard *sh) {
  const uint32_t F = p->n_features, T = p->n_thresholds, K = (uint32_t)p->n_classes;
  const int D = p->feat_dim;
  if (end_depth < 1 || end_depth > 24 || K > 64 || D > OR_MAX_FEAT_DIM || T > 256) return -1;
  const uint64_t n_nodes = (1ull << end_depth) - 1ull;
  uint64_t S;
  sample_t *smp = flatten_samples(ds, &S);
  int32_t *snode = (int32_t *)calloc(S ? S : 1, sizeof(int32_t));
  uint32_t *node_tot = (uint32_t *)calloc(n_nodes, sizeof(uint32_t));
  uint32_t *class_tot = (uint32_t *)calloc(n_nodes * K, sizeof(uint32_t));
  double *L = (double *)malloc(sizeof(double) * (S + 2));
  or_log2_table((uint32_t)(S + 2), L);
  node_tot[0] = (uint32_t)S;
  memcpy(posts, root_prior, sizeof(float) * K);
  or_stats st;
  memset(&st, 0, sizeof(st));

  /* Histogram memory per slice is capped (the reference caps it at 20 GiB). */
  const uint64_t per_node = (uint64_t)K * T * F;
  uint64_t max_slice = (256ull << 20) / (per_node * 4ull);
  if (max_slice < 1) max_slice = 1;

  int32_t *frontier = (int32_t *)malloc(sizeof(int32_t) * ((n_nodes + 1) / 2 + 1));
  uint8_t *split_now = (uint8_t *)calloc(n_nodes, 1);
  /* a feature that reads the tree: every pixel's node (traverse_ts.hpp:140-244),
   * starting at the root, and the tree as a depth's histograms see it */
  const int actx = p->plugin == OR_PLUGIN_AUTO_CONTEXT;
  uint64_t *moff = NULL;
  int32_t *map = NULL, *map2 = NULL;
  if (actx) {
    moff = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)ds->n_images + 1));
    moff[0] = 0;
    for (uint32_t i = 0; i < ds->n_images; i++) moff[i + 1] = moff[i] + (uint64_t)ds->width[i] * ds->height[i];
    map = (int32_t *)calloc(moff[ds->n_images] + 1, sizeof(int32_t));
    map2 = (int32_t *)calloc(moff[ds->n_images] + 1, sizeof(int32_t));
  }
  set_view sv = {map, moff, lc, posts, K, 0, (int32_t)n_nodes};
  for (uint32_t depth = 1; depth < end_depth; depth++) {
    uint32_t nf = 0;
    sv.map = map;
    sv.level = (int32_t)depth - 1; /* the node map's level: the frontier's */
    if (depth == 1) {
      frontier[nf++] = 0;
      for (uint64_t s = 0; s < S; s++) class_tot[smp[s].label]++;
    } else {
      uint64_t first = (1ull << (depth - 1)) - 1ull, cnt = 1ull << (depth - 1);
      for (uint64_t i = 0; i < cnt; i++) {
        uint64_t n = first + i;
        if (lc[n] == -1 && node_tot[n] > p->per_leaf_samples_thr) frontier[nf++] = (int32_t)n;
      }
    }
    for (uint32_t s0 = 0; s0 < nf; s0 += (uint32_t)max_slice) {
      uint32_t ns = nf - s0 < max_slice ? nf - s0 : (uint32_t)max_slice;
      const int32_t *sl = frontier + s0;
      uint32_t *hist = (uint32_t *)malloc(sizeof(uint32_t) * per_node * ns);
      double t0 = now_s();
      hist_impl(p, ds, tree_id, snode, sl, ns, hist, reference_cost, n_threads, actx ? &sv : NULL);
      double t1 = now_s();
      uint32_t *ctot = (uint32_t *)malloc(sizeof(uint32_t) * K * ns);
      for (uint32_t i = 0; i < ns; i++) memcpy(ctot + (size_t)i * K, class_tot + (size_t)sl[i] * K, sizeof(uint32_t) * K);
      int32_t *bt = (int32_t *)malloc(sizeof(int32_t) * ns), *bf = (int32_t *)malloc(sizeof(int32_t) * ns);
      double *bg = (double *)malloc(sizeof(double) * ns);
      uint32_t *xcl = NULL; /* sharded: the global winners' left class counts */
      if (sh) {
        /* this rank's candidates only: the split over columns [f0, f1) */
        const uint32_t Fl = sh->f1 - sh->f0;
        uint32_t *sub = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)ns * K * T * Fl);
        for (size_t r = 0; r < (size_t)ns * K * T; r++)
          memcpy(sub + r * Fl, hist + r * F + sh->f0, sizeof(uint32_t) * Fl);
        or_params pl = *p;
        pl.n_features = Fl;
        or_split(&pl, sub, ctot, ns, L, S + 2, bt, bf, bg, NULL, NULL);
        int64_t *key = (int64_t *)malloc(sizeof(int64_t) * ns), *idx = (int64_t *)malloc(sizeof(int64_t) * ns);
        xcl = (uint32_t *)calloc((size_t)ns * K, sizeof(uint32_t));
        for (uint32_t i = 0; i < ns; i++) {
          key[i] = bt[i] < 0 ? INT64_MIN : gain_key64(bg[i]);
          idx[i] = bt[i] < 0 ? -1 : (int64_t)bt[i] * F + sh->f0 + (uint32_t)bf[i];
          for (uint32_t l = 0; bt[i] >= 0 && l < K; l++)
            xcl[(size_t)i * K + l] = sub[(((size_t)i * K + l) * T + (uint32_t)bt[i]) * Fl + (uint32_t)bf[i]];
        }
        const int xr = sh->exchange(sh->user, ns, K, key, idx, xcl);
        for (uint32_t i = 0; i < ns; i++) {
          bt[i] = idx[i] < 0 ? -1 : (int32_t)(idx[i] / F);
          bf[i] = idx[i] < 0 ? -1 : (int32_t)(idx[i] % F);
        }
        free(key); free(idx); free(sub);
        if (xr != 0) {
          free(xcl); free(hist); free(ctot); free(bt); free(bf); free(bg);
          free(frontier); free(split_now); free(L); free(class_tot); free(node_tot); free(snode); free(smp);
          free(moff); free(map); free(map2);
          return -2;
        }
      } else {
        or_split(p, hist, ctot, ns, L, S + 2, bt, bf, bg, NULL, NULL);
      }
      st.seconds_hist += t1 - t0;
      st.seconds_split += now_s() - t1;
      for (uint32_t i = 0; i < ns; i++) st.evals += (uint64_t)node_tot[sl[i]] * F;
      st.nodes_trained += ns;
      /* finalize: learn_best_featthr.hpp:117-243 */
      for (uint32_t i = 0; i < ns; i++) {
        uint32_t n = (uint32_t)sl[i];
        if (bt[i] < 0) continue;
        uint32_t cl[64], cr[64], lsum = 0, rsum = 0;
        for (uint32_t l = 0; l < K; l++) {
          cl[l] = xcl ? xcl[(size_t)i * K + l] : hist[(((size_t)i * K + l) * T + (uint32_t)bt[i]) * F + (uint32_t)bf[i]];
          cr[l] = class_tot[(size_t)n * K + l] - cl[l];
          lsum += cl[l]; rsum += cr[l];
        }
        if (!lsum || !rsum) continue;
        uint32_t L_ = 2 * n + 1, R_ = 2 * n + 2;
        node_tot[L_] = lsum; node_tot[R_] = rsum;
        for (uint32_t l = 0; l < K; l++) {
          class_tot[(size_t)L_ * K + l] = cl[l];
          class_tot[(size_t)R_ * K + l] = cr[l];
          posts[(size_t)L_ * K + l] = (float)cl[l] / (float)lsum;
          posts[(size_t)R_ * K + l] = (float)cr[l] / (float)rsum;
        }
        lc[L_] = -1; lc[R_] = -1;
        int32_t thr_all[256];
        or_candidate(p, tree_id, n, (uint32_t)bf[i], feats + (size_t)n * D, thr_all);
        thrs[n] = thr_all[bt[i]];
        lc[n] = (int32_t)L_;
        split_now[n] = 1;
        st.nodes_split++;
      }
      free(xcl); free(hist); free(ctot); free(bt); free(bf); free(bg);
    }
    /* reassignment of every sample that sits on a node split at this depth */
#pragma omp parallel for schedule(static) NT(n_threads)
    for (int64_t s = 0; s < (int64_t)S; s++) {
      int32_t n = snode[s];
      if (!split_now[n]) continue;
      const sample_t *sm = &smp[s];
      tree_view tv = {actx ? map + moff[sm->img] : NULL, lc, posts, K, (int32_t)depth - 1, (int32_t)n_nodes};
      int32_t r = feature_at(p->plugin, p->feat_type, image_ptr(ds, sm->img), ds->width[sm->img],
                             ds->height[sm->img], ds->n_channels, sm->x, sm->y, feats + (size_t)n * D, &tv);
      snode[s] = lc[n] + (r <= thrs[n] ? 0 : 1);
    }
    for (uint32_t i = 0; i < nf; i++) split_now[frontier[i]] = 0;
    if (actx && depth + 1 < end_depth) {
      /* the next depth's node map: labelled pixels at split nodes move on
       * (predict.cl:36-85 over the label image as mask) */
#pragma omp parallel for schedule(dynamic, 1) NT(n_threads)
      for (int64_t i = 0; i < (int64_t)ds->n_images; i++) {
        const uint32_t w = ds->width[i], h = ds->height[i];
        const int32_t *mi = map + moff[i];
        int32_t *mo = map2 + moff[i];
        const uint8_t *lab = ds->labels + ds->lab_off[i];
        tree_view tv = {mi, lc, posts, K, (int32_t)depth - 1, (int32_t)n_nodes};
        for (uint64_t q = 0; q < (uint64_t)w * h; q++) {
          const int32_t n = mi[q], c = lab[q] ? lc[n] : -1;
          if (c < 0) {
            mo[q] = n;
            continue;
          }
          int32_t r = feature_at(p->plugin, p->feat_type, image_ptr(ds, (uint32_t)i), w, h, ds->n_channels,
                                 (int32_t)(q % w), (int32_t)(q / w), feats + (size_t)n * D, &tv);
          mo[q] = c + (r <= thrs[n] ? 0 : 1);
        }
      }
      int32_t *sw = map;
      map = map2;
      map2 = sw;
    }
  }
  if (sample_leaf) memcpy(sample_leaf, snode, sizeof(int32_t) * S);
  if (stats) *stats = st;
  free(frontier); free(split_now); free(L); free(class_tot); free(node_tot); free(snode); free(smp);
  free(moff); free(map); free(map2);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* a10 + a11: traversal and forest posterior.                               */
/* kernels/predict.cl:36-117 and cl_classifier_impl.hpp:478-552.             */
/* ------------------------------------------------------------------------ */
static inline int32_t traverse(const or_params *p, const void *img, uint32_t w, uint32_t h, uint32_t nch,
                               int32_t x, int32_t y, uint32_t depth, const int32_t *lc,
                               const int32_t *feats, const int32_t *thrs) {
  int32_t node = 0;
  for (uint32_t d = 1; d < depth; d++) {
    int32_t c = lc[node];
    if (c < 0) break; /* leaf (-1); an absent root (-2) also stops */
    int32_t r = or_feature(p->plugin, p->feat_type, img, w, h, nch, x, y, feats + (size_t)node * p->feat_dim);
    node = c + (r <= thrs[node] ? 0 : 1);
  }
  return node;
}

/* The node map of one tree over an image for a feature that reads the tree:
 * all pixels at the root, then depth-1 synchronous steps of the pixels inside
 * the mask (cl_classifier_impl.hpp:478-520, predict.cl:36-85); out[q] = the
 * pixel's leaf (0 outside the mask). */
static void tree_node_map(const or_params *p, const void *img, uint32_t w, uint32_t h, uint32_t nch,
                          const uint8_t *mask, uint32_t depth, const int32_t *lc, const int32_t *feats,
                          const int32_t *thrs, const float *posts, int32_t *out, int32_t *tmp, int n_threads) {
  const size_t P = (size_t)w * h;
  memset(out, 0, sizeof(int32_t) * P);
  for (uint32_t d = 1; d < depth; d++) {
    tree_view tv = {out, lc, posts, (uint32_t)p->n_classes, (int32_t)d - 1, (int32_t)((1u << depth) - 1u)};
#pragma omp parallel for schedule(static) NT(n_threads)
    for (int64_t q = 0; q < (int64_t)P; q++) {
      const int32_t n = out[q], c = (mask && !mask[q]) ? -1 : lc[n];
      if (c < 0) {
        tmp[q] = n;
        continue;
      }
      int32_t r = feature_at(p->plugin, p->feat_type, img, w, h, nch, (int32_t)(q % w), (int32_t)(q / w),
                             feats + (size_t)n * p->feat_dim, &tv);
      tmp[q] = c + (r <= thrs[n] ? 0 : 1);
    }
    memcpy(out, tmp, sizeof(int32_t) * P);
  }
}

int or_predict_posterior(const or_params *p, const void *img, uint32_t w, uint32_t h,
                         uint32_t nch, const uint8_t *mask, uint32_t n_trees,
                         const uint32_t *depth, const uint64_t *node_off,
                         const int32_t *lc, const int32_t *feats, const int32_t *thrs,
                         const float *posts, float *out, int n_threads) {
  const uint32_t K = (uint32_t)p->n_classes;
  const size_t P = (size_t)w * h;
  memset(out, 0, sizeof(float) * P * K);
  if (p->plugin == OR_PLUGIN_AUTO_CONTEXT) {
    int32_t *m = (int32_t *)malloc(sizeof(int32_t) * (P + 1)), *tmp = (int32_t *)malloc(sizeof(int32_t) * (P + 1));
    for (uint32_t t = 0; t < n_trees; t++) {
      const uint64_t o = node_off[t];
      tree_node_map(p, img, w, h, nch, mask, depth[t], lc + o, feats + o * p->feat_dim, thrs + o, posts + o * K, m,
                    tmp, n_threads);
      for (size_t q = 0; q < P; q++) {
        if (mask && !mask[q]) continue;
        for (uint32_t l = 0; l < K; l++) out[(size_t)l * P + q] += posts[(o + (uint64_t)m[q]) * K + l];
      }
    }
    free(m);
    free(tmp);
    for (size_t i = 0; i < P * K; i++) out[i] /= (float)n_trees;
    return 0;
  }
#pragma omp parallel for schedule(static) NT(n_threads)
  for (int64_t q = 0; q < (int64_t)P; q++) {
    if (mask && !mask[q]) continue;
    int32_t x = (int32_t)(q % w), y = (int32_t)(q / w);
    for (uint32_t t = 0; t < n_trees; t++) {
      uint64_t o = node_off[t];
      int32_t leaf = traverse(p, img, w, h, nch, x, y, depth[t], lc + o, feats + o * p->feat_dim, thrs + o);
      for (uint32_t l = 0; l < K; l++) out[(size_t)l * P + q] += posts[(o + (uint64_t)leaf) * K + l];
    }
  }
  for (size_t i = 0; i < P * K; i++) out[i] /= (float)n_trees;
  return 0;
}

int or_predict_leaf(const or_params *p, const void *img, uint32_t w, uint32_t h,
                    uint32_t nch, const uint8_t *mask, uint32_t depth,
                    const int32_t *lc, const int32_t *feats, const int32_t *thrs,
                    int32_t *out, int n_threads) {
  const size_t P = (size_t)w * h;
  if (p->plugin == OR_PLUGIN_AUTO_CONTEXT) return -1; /* needs the posteriors: or_predict_leaf_tree */
#pragma omp parallel for schedule(static) NT(n_threads)
  for (int64_t q = 0; q < (int64_t)P; q++) {
    if (mask && !mask[q]) { out[q] = 0; continue; }
    out[q] = traverse(p, img, w, h, nch, (int32_t)(q % w), (int32_t)(q / w), depth, lc, feats, thrs);
  }
  return 0;
}

int or_predict_leaf_tree(const or_params *p, const void *img, uint32_t w, uint32_t h, uint32_t nch,
                         const uint8_t *mask, uint32_t depth, const int32_t *lc, const int32_t *feats,
                         const int32_t *thrs, const float *posts, int32_t *out, int n_threads) {
  if (p->plugin != OR_PLUGIN_AUTO_CONTEXT)
    return or_predict_leaf(p, img, w, h, nch, mask, depth, lc, feats, thrs, out, n_threads);
  int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * ((size_t)w * h + 1));
  tree_node_map(p, img, w, h, nch, mask, depth, lc, feats, thrs, posts, out, tmp, n_threads);
  free(tmp);
  return 0;
}
