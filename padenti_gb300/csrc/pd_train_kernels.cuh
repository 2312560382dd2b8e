// Device kernels of one training depth: candidate table, class histograms,
// best split with FP64 recheck, reassignment and the stable regrouping of the
// active samples by frontier slot.
#pragma once

#if defined(__CUDACC_RTC__)
#define FLT_MAX 3.402823466e+38F
#define DBL_MAX 1.7976931348623158e+308
#define LLONG_MAX 9223372036854775807LL
#define LLONG_MIN (-LLONG_MAX - 1LL)
#else
#include <cfloat>
#include <climits>
#endif

#include "pd_log2.cuh"
#include "pd_plugins.cuh"
#include "pd_propose.cuh"
#include "pd_rng.cuh"

namespace pd {

constexpr int kHistThreads = 256;  // 8 warps, each on its own samples
constexpr int kScanItems = 4096;   // active samples per scan block (256 threads x 16)
// FP32 gain window rechecked in FP64.  Each FP32 entropy term -p log2 p (fast
// reciprocal and log2) is within about 2e-7 of its exact value and each of the
// ~K additions of an entropy adds at most 2.4e-7, so |gain32 - gain64| stays
// below eps(K) = (3K + 3) * 4.4e-7; a candidate within 2*eps of the FP32 maximum
// can be the exact winner.  The window is 4.5x that.
PD_HD float recheck_delta(uint32_t K) { return (3.0f * (float)K + 3.0f) * 4.0e-6f; }

// Filter of the fused split (nodes of N <= 65535 samples, so 1e6*c > N for every
// c >= 1 and the cutoff never applies).  The exact split maximises -(S_L + S_R),
// S(c, n) = n log2 n - sum_l c_l log2 c_l, the canonical gain times N minus a
// per-node constant.  In FP32 with the table X[c] = fl(c log2 c) and sequential
// sums the error is at most (K + 3) u N log2 N (u = 2^-24): per side K + 1
// table roundings of terms whose magnitudes add up to at most 2 n log2 n, K
// additions of partial sums bounded by n log2 n, and one final addition, with
// nL log2 nL + nR log2 nR <= N log2 N.  The exact winner is therefore within
// 2 (K + 3) u N log2 N of the FP32 maximum; the window is 2 (2K + 5) u N log2 N.
constexpr uint32_t kXlog2Len = 65536;
constexpr uint32_t kRecheckList = 512;  // recheck list of a fused split (pairs, u16)
PD_D float fused_window(uint32_t K, uint32_t N) {
  return 2.0f * (2.0f * (float)K + 5.0f) * 5.9604645e-8f * (float)N * log2f((float)N);
}

struct CandBounds {
  int32_t low[PD_MAX_FEAT_DIM];
  int32_t up[PD_MAX_FEAT_DIM];
  int32_t thr_lo, thr_hi;
  uint32_t f_base;  // candidate f of a table is the node's candidate f_base + f (candidate-sharded training)
};

// One histogram work item: candidates [tile*64, tile*64+64) of frontier slot
// `slot` over the active samples act[begin, end) (end - begin <= 65535).
// multi = 0: the only work item of its rows, stores them; 1: other work items
// add into the same rows (atomics); 2: the only work item of its rows, and the
// node's split is fused into the kernel (no rows are written).
struct WorkItem {
  uint32_t slot, tile, begin, end, multi, pad0, pad1, pad2;
};

struct DevSet {
  const uint32_t *magic;
  const uint8_t *pixels;
  const uint64_t *img_off;
  const uint32_t *img_wh;
  const uint32_t *s_xy;
  const uint32_t *s_img;
  const uint8_t *s_label;
  // for features that read the tree (P::kUsesTree): the node map of the depth
  // being trained (int32 per pixel, image i from map_off[i]; null when none is
  // kept), the device tree, its class count, the map's level (the depth being
  // trained, root 0) and the tree's node count
  const int32_t *nodes;
  const uint64_t *map_off;
  const int32_t *tree_lc;
  const float *tree_post;
  uint32_t n_classes;
  int32_t tree_level, tree_nodes;
};

// The tree-reading fields of an image reference (a no-op for other plugins).
template <class P, class ImgT>
PD_D void attach_tree(ImageRef<ImgT> &im, const DevSet &ds, uint64_t map_off) {
  if constexpr (P::kUsesTree) {
    im.nodes = ds.nodes ? ds.nodes + map_off : nullptr;
    im.tree_lc = ds.tree_lc;
    im.tree_post = ds.tree_post;
    im.n_classes = ds.n_classes;
    im.tree_level = ds.tree_level;
    im.tree_nodes = ds.tree_nodes;
  }
}

// What the kernels need of a sample, in one 16-byte word: its position, image
// and class, and the plugin's preload words of its pixel (static per sample).
// The active samples of a depth are kept as these records, in slot order, so a
// warp reads 32 samples with one coalesced load.
struct __align__(16) SampleRec {
  uint32_t xy;       // x | y << 16
  uint32_t img_lab;  // image | class << 24
  uint32_t pre[2];   // P::preload words (kPreWords <= 2)
};

// Brings the line holding p to L2 (no register result, no wait).
PD_D void prefetch_l2(const void *p) {
#if defined(__CUDA_ARCH__)
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
#endif
}

template <typename T>
PD_D T max_of() {
  return (T)(sizeof(T) == 2 ? 32767 : 2147483647);
}

// ------------------------------------------------------ candidate table ----
// Thread per (slot, candidate).  Thresholds are written sorted ascending with
// their original index, so a response needs one binary search instead of T
// comparisons and the split can prefix-sum the counts back.  The insertion
// sort runs in the thread's own shared-memory column (conflict-free), and the
// sorted column is written out row by row, coalesced across candidates.
constexpr int kCandThreads = 128;

// Column c of slot n holds candidate ord[n][c] (c itself when ord is null).
// PACKED (threshold range below 2^24): value and original index sort as one
// word (v - lo) << 8 | t, whose order is the stable order of the values; else
// two shared-memory columns.
// With prop.out set, candidates f < prop.n_prop of slot n are drawn from the
// proposal network's mixture for that slot (pd_propose.cuh) instead of MD5.
template <typename FeatT, bool PACKED>
__global__ void __launch_bounds__(kCandThreads) k_candidates(const int32_t *__restrict__ nodes, uint32_t n_nodes,
                                                             uint32_t tree, uint32_t F, uint32_t T, int D,
                                                             CandBounds b, const uint32_t *__restrict__ ord,
                                                             FeatT *__restrict__ feat,
                                                             FeatT *__restrict__ thr_sorted,
                                                             uint8_t *__restrict__ perm, PropSrc prop) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t *sk = reinterpret_cast<uint32_t *>(smem_raw);                         // PACKED: [T][128]
  FeatT *sv = reinterpret_cast<FeatT *>(smem_raw);                               // [T][128]
  uint8_t *si = reinterpret_cast<uint8_t *>(sv + (size_t)T * kCandThreads);      // [T][128]
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = idx < (uint64_t)n_nodes * F;
  const uint32_t n = active ? (uint32_t)(idx / F) : 0u, c = active ? (uint32_t)(idx % F) : 0u;
  if (active) {
    const uint32_t node = (uint32_t)nodes[n];
    const uint32_t f = ord ? ord[(size_t)n * F + c] : c;
    const uint32_t fg = b.f_base + f;  // the candidate's index among all of the node's candidates
    const bool net = prop.out != nullptr && f < prop.n_prop;
    uint64_t stream = 0;
    uint32_t g = 0;
    FeatT fv[PD_MAX_FEAT_DIM];
    if (net) {
      stream = prop_stream(prop.seed, tree, node, f);
      g = prop_component(prop, n, stream);
      for (int d = 0; d < D; d++) fv[d] = (FeatT)prop_draw(prop, n, g, (uint32_t)d, stream, (uint32_t)d);
    } else {
      candidate_feature<FeatT>(tree, node, fg, D, b.low, b.up, fv);
    }
    for (int d = 0; d < D; d++) feat[((size_t)n * D + d) * F + c] = fv[d];
    uint32_t *k = sk + threadIdx.x;
    FeatT *v = sv + threadIdx.x;
    uint8_t *id = si + threadIdx.x;
    uint32_t seed[4] = {tree, node, fg, 1u}, st[4] = {0u, 0u, 0u, 0u};
    for (uint32_t t = 0; t < T; t++) {
      if (!net && (t & 3u) == 0) {
        md5_block(seed, st);
        seed[0] = st[0];
        seed[1] = st[1];
        seed[2] = st[2];
        seed[3] = st[3];
      }
      const FeatT x = net ? (FeatT)prop_draw(prop, n, g, (uint32_t)D, stream, (uint32_t)D + 1u + t)
                          : draw<FeatT>(st[t & 3u], b.thr_lo, b.thr_hi);
      // stable insertion
      uint32_t j = t;
      if (PACKED) {
        const uint32_t key = ((uint32_t)((int32_t)x - b.thr_lo) << 8) | t;
        while (j > 0 && k[(j - 1) * kCandThreads] > key) {
          k[j * kCandThreads] = k[(j - 1) * kCandThreads];
          j--;
        }
        k[j * kCandThreads] = key;
      } else {
        while (j > 0 && v[(j - 1) * kCandThreads] > x) {
          v[j * kCandThreads] = v[(j - 1) * kCandThreads];
          id[j * kCandThreads] = id[(j - 1) * kCandThreads];
          j--;
        }
        v[j * kCandThreads] = x;
        id[j * kCandThreads] = (uint8_t)t;
      }
    }
  }
  __syncwarp();
  if (!active) return;
  for (uint32_t j = 0; j < T; j++) {
    if (PACKED) {
      const uint32_t key = sk[j * kCandThreads + threadIdx.x];
      thr_sorted[((size_t)n * T + j) * F + c] = (FeatT)((int32_t)(key >> 8) + b.thr_lo);
      perm[((size_t)n * T + j) * F + c] = (uint8_t)(key & 0xffu);
    } else {
      thr_sorted[((size_t)n * T + j) * F + c] = sv[j * kCandThreads + threadIdx.x];
      perm[((size_t)n * T + j) * F + c] = si[j * kCandThreads + threadIdx.x];
    }
  }
}

// The same table with packed keys and at most TP thresholds (TP = 16, 32 or 64):
// the keys of a candidate live in registers (padded with 0xffffffff, above every
// key since t < TP) and are sorted by a bitonic network with compile-time
// indices -- branch-free min/max pairs in place of the insertion sort, whose
// data-dependent shifts diverge across a warp.  Same output as
// k_candidates<FeatT, true>, proposal source included.
template <int N>
PD_D void bitonic_sort_regs(uint32_t (&k)[N]) {
#pragma unroll
  for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int j = i ^ stride;
        if (j > i) {
          const uint32_t a = k[i], c = k[j];
          const uint32_t lo = min(a, c), hi = max(a, c);
          if ((i & size) == 0) {
            k[i] = lo;
            k[j] = hi;
          } else {
            k[i] = hi;
            k[j] = lo;
          }
        }
      }
    }
  }
}

template <typename FeatT, int TP>
__global__ void __launch_bounds__(kCandThreads) k_candidates_reg(const int32_t *__restrict__ nodes, uint32_t n_nodes,
                                                                 uint32_t tree, uint32_t F, uint32_t T, int D,
                                                                 CandBounds b, const uint32_t *__restrict__ ord,
                                                                 FeatT *__restrict__ feat,
                                                                 FeatT *__restrict__ thr_sorted,
                                                                 uint8_t *__restrict__ perm, PropSrc prop) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)n_nodes * F) return;
  const uint32_t n = (uint32_t)(idx / F), c = (uint32_t)(idx % F);
  const uint32_t node = (uint32_t)nodes[n];
  const uint32_t f = ord ? ord[(size_t)n * F + c] : c;
  const uint32_t fg = b.f_base + f;
  const bool net = prop.out != nullptr && f < prop.n_prop;
  uint64_t stream = 0;
  uint32_t g = 0;
  {
    FeatT fv[PD_MAX_FEAT_DIM];
    if (net) {
      stream = prop_stream(prop.seed, tree, node, f);
      g = prop_component(prop, n, stream);
      for (int d = 0; d < D; d++) fv[d] = (FeatT)prop_draw(prop, n, g, (uint32_t)d, stream, (uint32_t)d);
    } else {
      candidate_feature<FeatT>(tree, node, fg, D, b.low, b.up, fv);
    }
    for (int d = 0; d < D; d++) feat[((size_t)n * D + d) * F + c] = fv[d];
  }
  uint32_t key[TP];
  uint32_t seed[4] = {tree, node, fg, 1u}, st[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int t = 0; t < TP; t++) {
    if ((uint32_t)t < T) {
      FeatT x;
      if (net) {
        x = (FeatT)prop_draw(prop, n, g, (uint32_t)D, stream, (uint32_t)D + 1u + (uint32_t)t);
      } else {
        if ((t & 3) == 0) {
          md5_block(seed, st);
          seed[0] = st[0];
          seed[1] = st[1];
          seed[2] = st[2];
          seed[3] = st[3];
        }
        x = draw<FeatT>(st[t & 3], b.thr_lo, b.thr_hi);
      }
      key[t] = ((uint32_t)((int32_t)x - b.thr_lo) << 8) | (uint32_t)t;
    } else {
      key[t] = 0xffffffffu;
    }
  }
  bitonic_sort_regs<TP>(key);
#pragma unroll
  for (int j = 0; j < TP; j++) {
    if ((uint32_t)j < T) {
      thr_sorted[((size_t)n * T + j) * F + c] = (FeatT)((int32_t)(key[j] >> 8) + b.thr_lo);
      perm[((size_t)n * T + j) * F + c] = (uint8_t)(key[j] & 0xffu);
    }
  }
}

// ------------------------------------------------------ candidate order ----
// Column order of a node's candidate table: the candidates sorted row-major by
// their first probe offset (feature dims kOrderDim + 1 = y, then kOrderDim = x,
// each scaled to 10 bits over its bounds).  The 32 lanes of a histogram warp
// then probe pixels of few image rows and share cache sectors (a sector is 16
// pixels of one row: row-major groups beat square ones).  Only the placement
// changes: split decisions use the original index f (ties to the lowest
// t*F + f).  Block per slot; bitonic sort of (code << 32 | f) in shared memory
// over the next power of two of F.
constexpr uint32_t kOrderMaxF = 8192;
constexpr int kOrderThreads = 512;

PD_D uint32_t order_quant10(int32_t v, int32_t lo, int32_t up) {
  const int64_t span = (int64_t)up - lo + 1, x = (int64_t)v - lo;
  const int64_t q = span > 0 ? x * 1024 / span : 0;
  return (uint32_t)(q < 0 ? 0 : (q > 1023 ? 1023 : q));
}
// With prop.out set, candidates f < prop.n_prop are the proposal network's
// draws (the same values k_candidates puts in the table).
template <class P>
__global__ void __launch_bounds__(kOrderThreads) k_cand_order(const int32_t *__restrict__ nodes, uint32_t tree,
                                                              uint32_t F, CandBounds b, uint32_t *__restrict__ ord,
                                                              PropSrc prop) {
  using FeatT = typename P::feat_t;
  constexpr int D = P::kFeatDim, X = P::kOrderDim;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long *key = reinterpret_cast<unsigned long long *>(smem_raw);  // [N]
  const uint32_t n = blockIdx.x, node = (uint32_t)nodes[n];
  uint32_t N = 1;
  while (N < F) N <<= 1;
  for (uint32_t f = threadIdx.x; f < N; f += blockDim.x) {
    unsigned long long k = ~0ull;  // padding sorts last
    if (f < F) {
      int32_t vx, vy;
      if (prop.out != nullptr && f < prop.n_prop) {
        const uint64_t stream = prop_stream(prop.seed, tree, node, f);
        const uint32_t g = prop_component(prop, n, stream);
        vx = (int32_t)(FeatT)prop_draw(prop, n, g, (uint32_t)X, stream, (uint32_t)X);
        vy = (int32_t)(FeatT)prop_draw(prop, n, g, (uint32_t)X + 1u, stream, (uint32_t)X + 1u);
      } else {
        FeatT fv[D];
        candidate_feature<FeatT>(tree, node, b.f_base + f, D, b.low, b.up, fv);
        vx = (int32_t)fv[X];
        vy = (int32_t)fv[X + 1];
      }
      const uint32_t qx = order_quant10(vx, b.low[X], b.up[X]);
      const uint32_t qy = order_quant10(vy, b.low[X + 1], b.up[X + 1]);
      k = ((unsigned long long)((qy << 10) | qx) << 32) | f;
    }
    key[f] = k;
  }
  __syncthreads();
  for (uint32_t size = 2; size <= N; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < N / 2; i += blockDim.x) {
        const uint32_t lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
        const bool ascending = (lo & size) == 0;
        const unsigned long long a = key[lo], c = key[hi];
        if ((a > c) == ascending) {
          key[lo] = c;
          key[hi] = a;
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t c = threadIdx.x; c < F; c += blockDim.x) ord[(size_t)n * F + c] = (uint32_t)key[c];
}

// ---------------------------------------------------------------- split ----
struct SplitOut {
  int32_t t, f, j;  // original threshold and candidate of the winner, its sorted position
  int32_t col;      // its column in the candidate table (-1: no split)
  double gain;
};
// Best candidate of one column range of one node.
struct SplitPart {
  double gain;
  long long idx;  // t*F + f (f the original candidate index)
  int32_t j;      // sorted threshold position
  int32_t col;    // column of the candidate table
};

constexpr int kSplitCols = 128;  // threads of a split CTA, one column each per pass
constexpr int kSplitRows = 4;    // histogram rows loaded together in pass 1

// Reference-formula FP32 entropy (kernels/learn_best_feature.cl:75-93) with the
// p <= 1e-6 cutoff as the integer test 1e6*c <= n; fast intrinsics, error well
// inside recheck_delta(K)/2.
template <int KM, bool RIGHT>
PD_D float ent32(const uint32_t *tot, const uint32_t *c, uint32_t K, uint32_t n) {
  if (n == 0) return 0.0f;
  const float inv = __frcp_rn((float)n);
  float s = 0.0f;
#pragma unroll
  for (int l = 0; l < KM; l++) {
    if ((uint32_t)l < K) {
      const uint32_t cl = RIGHT ? tot[l] - c[l] : c[l];
      if (cl != 0u && (uint64_t)cl * 1000000ull > n) {
        const float p = (float)cl * inv;
        s -= p * __log2f(p);
      }
    }
  }
  return s;
}
// Exact n*entropy: sum over classes of c (log2 n - log2 c), one IEEE double
// operation at a time with the shared log2 table (the oracle's sum64).
template <int KM, bool RIGHT>
PD_D double sum64(const uint32_t *tot, const uint32_t *c, uint32_t K, uint32_t n, const double *L) {
  double s = 0.0;
  if (n == 0) return s;
  const double ln = L[n];
#pragma unroll
  for (int l = 0; l < KM; l++) {
    if ((uint32_t)l < K) {
      const uint32_t cl = RIGHT ? tot[l] - c[l] : c[l];
      if (cl != 0u && (uint64_t)cl * 1000000ull > n) s = dadd(s, dmul((double)cl, dsub(ln, L[cl])));
    }
  }
  return s;
}

struct SplitArgs {
  const uint32_t *hist;       // [slots][K][T][F]: rank space, or cumulative when CUM
  const uint8_t *perm;        // [slots][T][F] original threshold of sorted position (null: identity)
  const uint32_t *class_tot;  // [slots][K]
  float *g32;                 // scratch [slots][T][F]
  const double *L;
  uint64_t L_len;
  uint32_t F, T, K;
  float delta;
  uint32_t cols;              // columns per part
  uint32_t parts;             // parts per node
  unsigned *node_max;         // [slots] order-preserving bits of the FP32 maximum
  unsigned *done;             // [slots] finished parts
  SplitPart *part_best;       // [slots][parts]
  SplitOut *out;
  uint32_t *out_cl;           // [slots][K] left class counts of the winner
  unsigned long long *rechecked;
  const uint32_t *slot_list;  // slots to process (null: blockIdx.y)
  const uint32_t *ord;        // [slots][F] original index of each column (null: identity)
};

PD_D unsigned f2ord(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
PD_D float ord2f(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }
// int64 key whose order is the order of the (non-NaN) doubles
PD_D long long gain_order_key(double g) {
  const long long b = __double_as_longlong(g);
  return b < 0 ? (LLONG_MIN - b - 1) : b;
}

// ------------------------------------------------------------ histogram ----
// Each CTA owns one (slot, 64-candidate tile, sample chunk).  Lane l evaluates
// candidates l and l+32 of the tile; each warp walks its own samples.  Per
// evaluation: the plugin response, a branch-free lower_bound over the sorted
// thresholds of the candidate (padded with +max to a power of two, column-major
// in shared memory so every lane hits its own bank), and one shared atomic into
// bin [label][rank] of a word that packs the two candidates of the lane as
// 16-bit counters (rank = number of thresholds below the response; rank T counts
// for no threshold and is dropped).  A chunk has at most 65535 samples, so a
// 16-bit counter never carries.  The tile histogram then goes to global memory
// in rank space as uint32.
constexpr int kCandPerLane = 2;
constexpr int kTileF = 32 * kCandPerLane;
constexpr uint32_t kMaxChunk = 65535;

// The sample loop of k_hist: each warp walks its samples SPI at a time (their
// probe loads in flight together) and adds both candidates of the lane into the
// shared histogram.
template <class P, uint32_t TP, bool FAST, int SPI>
PD_D void hist_samples(const DevSet &ds, const SampleRec *__restrict__ rec, const WorkItem &w,
                       const typename P::Cand &ca, const typename P::Cand &cb, uint32_t *sh_hist,
                       const typename P::feat_t *sh_thr, uint32_t T) {
  using FeatT = typename P::feat_t;
  using ImgT = typename P::img_t;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the lane's two threshold columns (rows of 32 entries, like the histogram)
  const FeatT *ta = sh_thr + lane, *tb = sh_thr + TP * 32 + lane;
  uint32_t *hl = sh_hist + lane;
  // the first levels of each column's search in registers -- two at 8 rows,
  // three from 16 rows up (3 pivots, then 4 more per column): that many shared
  // loads fewer per evaluation.  Not at 2 samples per iteration, whose register
  // budget (3 CTAs per SM) has no room for them.
  constexpr bool kPivots = TP >= 8 && SPI >= 4;
  FeatT a_p1 = 0, a_p2 = 0, a_p3 = 0, b_p1 = 0, b_p2 = 0, b_p3 = 0;
  FeatT a_q[4] = {0, 0, 0, 0}, b_q[4] = {0, 0, 0, 0};
  if constexpr (kPivots && TP >= 16) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      a_q[k] = ta[((2 * k + 1) * TP / 8 - 1) * 32];
      b_q[k] = tb[((2 * k + 1) * TP / 8 - 1) * 32];
    }
  }
  if constexpr (kPivots) {
    a_p1 = ta[(TP / 2 - 1) * 32];
    a_p2 = ta[(TP / 4 - 1) * 32];
    a_p3 = ta[(3 * TP / 4 - 1) * 32];
    b_p1 = tb[(TP / 2 - 1) * 32];
    b_p2 = tb[(TP / 4 - 1) * 32];
    b_p3 = tb[(3 * TP / 4 - 1) * 32];
  }
  const uint32_t class_words = (T + 1) * 32;
  constexpr int PW = P::kPreWords;
  const unsigned full = 0xffffffffu;
  // one evaluation pair (both candidates of the lane) on warp sample i
  struct Eval {
    FeatT ra, rb;
    uint32_t row;  // class * (T + 1) * 32: the class block of the histogram
  };
  // samples per warp batch: 32, or for an item of fewer than 256 samples an equal
  // share (rounded up to SPI) so that every warp of the CTA has samples
  const uint32_t n_item = w.end - w.begin;
  const uint32_t share = (n_item + kHistThreads / 32 - 1) / (kHistThreads / 32);
  const uint32_t bs = n_item >= kHistThreads ? 32u : min(32u, (share + SPI - 1) / SPI * SPI);
  for (uint32_t base = w.begin + warp * bs; base < w.end; base += bs * (kHistThreads / 32)) {
    const uint32_t n_here = min(bs, w.end - base);
    // lane-parallel preload of 32 samples: position, class, image, pixel words
    uint32_t my_xy = 0, my_wh = 0, my_row = 0, my_pre[PW];
    uint64_t my_off = 0, my_moff = 0;
#pragma unroll
    for (int k = 0; k < PW; k++) my_pre[k] = 0u;
    if ((uint32_t)lane < n_here) {
      const uint4 r = ldg(reinterpret_cast<const uint4 *>(rec + base + lane));
      my_xy = r.x;
      my_row = (r.y >> 24) * class_words;
      const uint32_t imi = r.y & 0xffffffu;
      my_pre[0] = r.z;
      if (PW > 1) my_pre[PW - 1] = r.w;
      my_off = ds.img_off[imi];
      my_wh = ds.img_wh[imi];
      if constexpr (P::kUsesTree) my_moff = ds.map_off ? ds.map_off[imi] : 0ull;
    }
    auto eval_at = [&](uint32_t i) -> Eval {
      const uint32_t xy = __shfl_sync(full, my_xy, i);
      const uint32_t wh = __shfl_sync(full, my_wh, i);
      const uint64_t off = __shfl_sync(full, my_off, i);
      uint32_t pre[PW];
#pragma unroll
      for (int k = 0; k < PW; k++) pre[k] = __shfl_sync(full, my_pre[k], i);
      ImageRef<ImgT> im;
      im.data = reinterpret_cast<const ImgT *>(ds.pixels + off);
      im.w = (int32_t)(wh & 0xffffu);
      im.h = (int32_t)(wh >> 16);
      im.magic = ds.magic;
      if constexpr (P::kUsesTree) attach_tree<P>(im, ds, __shfl_sync(full, my_moff, i));
      const auto prep = P::prepare(im, (int32_t)(xy & 0xffffu), (int32_t)(xy >> 16), pre);
      Eval e;
      e.ra = P::template eval_train<FAST>(prep, ca);
      e.rb = P::template eval_train<FAST>(prep, cb);
      e.row = __shfl_sync(full, my_row, i);
      return e;
    };
    auto accumulate = [&](const Eval &e) {
      // lower_bound over the padded sorted column: k = #thresholds < r
      const FeatT *pa = ta, *pb = tb;
      if constexpr (kPivots) {
        uint32_t ka = a_p1 < e.ra ? TP / 2 : 0u, kb = b_p1 < e.rb ? TP / 2 : 0u;
        const FeatT qa = ka ? a_p3 : a_p2, qb = kb ? b_p3 : b_p2;
        ka += qa < e.ra ? TP / 4 : 0u;
        kb += qb < e.rb ? TP / 4 : 0u;
        constexpr uint32_t first = TP >= 16 ? (TP >> 4) : (TP >> 3);
        if constexpr (TP >= 16) {
          // third level: the pivot of the quarter reached so far
          const uint32_t ia = ka / (TP / 4), ib = kb / (TP / 4);
          const FeatT ra = ia & 2 ? (ia & 1 ? a_q[3] : a_q[2]) : (ia & 1 ? a_q[1] : a_q[0]);
          const FeatT rb = ib & 2 ? (ib & 1 ? b_q[3] : b_q[2]) : (ib & 1 ? b_q[1] : b_q[0]);
          ka += ra < e.ra ? TP / 8 : 0u;
          kb += rb < e.rb ? TP / 8 : 0u;
        }
        pa += ka * 32;
        pb += kb * 32;
#pragma unroll
        for (uint32_t step = first; step > 0; step >>= 1) {
          if (pa[(step - 1) * 32] < e.ra) pa += step * 32;
          if (pb[(step - 1) * 32] < e.rb) pb += step * 32;
        }
      } else {
#pragma unroll
        for (uint32_t step = TP >> 1; step > 0; step >>= 1) {
          if (pa[(step - 1) * 32] < e.ra) pa += step * 32;
          if (pb[(step - 1) * 32] < e.rb) pb += step * 32;
        }
      }
      // rank k = (pa - ta) / 32 in [0, T]; histogram rows also hold 32 words,
      // so the word of rank k is (pa - ta) words into the class block.  Rank T
      // (no threshold >= r) and the columns past F (all-max thresholds, rank
      // 0) land in words that are never read.
      uint32_t *row = hl + e.row;
      atomicAdd(row + (pa - ta), 1u);
      atomicAdd(row + (pb - tb), 0x10000u);
    };
    // SPI samples per iteration: their probe loads are in flight together
    uint32_t i = 0;
    for (; i + SPI <= n_here; i += SPI) {
      Eval e[SPI];
#pragma unroll
      for (int k = 0; k < SPI; k++) e[k] = eval_at(i + k);
#pragma unroll
      for (int k = 0; k < SPI; k++) accumulate(e[k]);
    }
    for (; i < n_here; i++) accumulate(eval_at(i));
  }
}

// Split of a node whose samples all went through one work item, fused into the
// histogram CTA: the tile histogram (packed pairs of 16-bit counters) is
// prefix-summed in place over the ranks, so word (l, j, lane) holds the left
// counts of sorted position j; the FP32 filter -(S_L + S_R) of every
// (j, candidate) goes to shared memory; every candidate within fused_window of
// the tile's own FP32 maximum is re-evaluated with the exact FP64 gain.  The
// window holds the tile's exact best (and its ties), so the best of the tiles'
// rechecked candidates is the node's winner.  The last tile of the node to
// finish reduces the tiles.
struct FusedSplit {
  const uint32_t *class_tot;  // [slots][K]
  const uint8_t *perm;        // [slots][T][F]
  const double *L;
  uint64_t L_len;
  const float *xlog2;         // c log2 c for c < kXlog2Len (fused nodes have N <= 65535)
  const double *parent;       // [slots] parent term of the exact gain (k_parent_term)
  uint32_t tiles;             // tiles per slot
  SplitPart *part_best;       // [slots][tiles]
  uint32_t *part_cl;          // [slots][tiles][K]
  unsigned *done;             // [slots]
  SplitOut *out;
  uint32_t *out_cl;           // [slots][K]
  unsigned long long *rechecked;
  const uint32_t *ord;        // [slots][F] original index of each column (null: identity)
};

PD_D uint32_t half16(uint32_t word, uint32_t c) { return (word >> ((c >> 5) * 16)) & 0xffffu; }


PD_D void fused_split(const FusedSplit &fs, const WorkItem &w, uint32_t *sh_hist, float *sh_g, uint32_t *sh_nl,
                      uint32_t F, uint32_t T, uint32_t K) {
  __shared__ uint32_t s_tot[PD_MAX_CLASSES];
  __shared__ float s_red[kHistThreads / 32];
  __shared__ double s_g[kHistThreads / 32];
  __shared__ long long s_i[kHistThreads / 32];
  __shared__ int s_j[kHistThreads / 32];
  __shared__ int s_c[kHistThreads / 32];
  __shared__ bool s_last;
  __shared__ uint32_t s_nlist;
  __shared__ uint16_t s_list[kRecheckList];
  __shared__ unsigned long long s_pmin;
  __shared__ int s_j0;
  __shared__ uint8_t s_cls[PD_MAX_CLASSES];  // the classes present in the node, in class order
  __shared__ uint32_t s_nc;
  const uint32_t slot = w.slot, f0 = w.tile * kTileF;
  const uint32_t TS = T + 1;  // histogram rows per class
  for (uint32_t l = threadIdx.x; l < K; l += blockDim.x) s_tot[l] = fs.class_tot[(size_t)slot * K + l];
  __syncthreads();
  if (threadIdx.x == 0) {
    s_nlist = 0u;
    s_pmin = ~0ull;
    s_j0 = 0;
    uint32_t nc = 0;
    for (uint32_t l = 0; l < K; l++)
      if (s_tot[l]) s_cls[nc++] = (uint8_t)l;
    s_nc = nc;
  }
  __syncthreads();
  // Only the classes present in the node: the item holds all of the node's
  // samples, so an absent class's rows were never counted (nor zeroed, hist_item)
  // and every term they would add is c log2 c of 0, or skipped as c = 0.
  const uint32_t nc = s_nc;
  // in-place prefix over the ranks of each (present class, packed column), eight
  // rows loaded together
  for (uint32_t q = threadIdx.x; q < nc * 32; q += blockDim.x) {
    uint32_t *h = sh_hist + (s_cls[q >> 5] * TS) * 32 + (q & 31);
    uint32_t run = 0, j = 0;
    for (; j + 8 <= T; j += 8) {
      uint32_t v[8];
#pragma unroll
      for (int k = 0; k < 8; k++) v[k] = h[(j + k) * 32];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        run += v[k];
        h[(j + k) * 32] = run;
      }
    }
    for (; j < T; j++) {
      run += h[j * 32];
      h[j * 32] = run;
    }
  }
  __syncthreads();
  uint32_t N = 0, classes = 0;
  for (uint32_t l = 0; l < K; l++) {
    N += s_tot[l];
    classes += s_tot[l] != 0u;
  }
  const bool ok = N != 0 && (uint64_t)N < fs.L_len;
  double best = -DBL_MAX;
  long long best_idx = LLONG_MAX;
  int best_j = -1, best_c = -1;
  unsigned long long n_checked = 0;
  if (ok && classes == 1) {
    // A pure node: every exact gain is 0 (each term is c (log2 n - log2 c) with
    // c = n), so the winner is the lowest index t*F + f, the original threshold
    // 0 of the tile's lowest original candidate; its counts are those of the
    // sorted position of that threshold.
    for (uint32_t c = threadIdx.x; c < kTileF; c += blockDim.x) {
      const uint32_t f = f0 + c;
      if (f < F) atomicMin(&s_pmin, ((unsigned long long)(fs.ord ? fs.ord[(size_t)slot * F + f] : f) << 8) | c);
    }
    __syncthreads();
    const uint32_t c = (uint32_t)(s_pmin & 0xffu), f = f0 + c;
    for (uint32_t t = threadIdx.x; t < T; t += blockDim.x)
      if (fs.perm[((size_t)slot * T + t) * F + f] == 0) s_j0 = (int)t;
    __syncthreads();
    best = 0.0;
    best_idx = (long long)(s_pmin >> 8);
    best_j = s_j0;
    best_c = (int)f;
  } else {
    // packed left totals of every (position, column pair)
    for (uint32_t q = threadIdx.x; q < T * 32; q += blockDim.x) {
      const uint32_t j = q >> 5, col = q & 31;
      uint32_t n = 0;
      for (uint32_t i = 0; i < nc; i++) n += sh_hist[(s_cls[i] * TS + j) * 32 + col];
      sh_nl[q] = n;
    }
    __syncthreads();
    const uint32_t pairs = T * kTileF;
    // FP32 filter -(S_L + S_R) from the c log2 c table (fused_window) and the tile
    // maximum.  Thread (column c, quarter) walks a run of consecutive positions j of
    // its column, so the previous position's left total stays in a register; the
    // 32 lanes of a warp share j and read 32 consecutive words.
    static_assert(kHistThreads == 4 * kTileF, "four threads per candidate column");
    float lmax = -FLT_MAX;
    if (ok) {
      const float *X = fs.xlog2;
      const uint32_t c = threadIdx.x & (kTileF - 1), col = c & 31, hs = (c >> 5) * 16;
      const uint32_t per = (T + 3) / 4, jb = (threadIdx.x / kTileF) * per, je = min(T, jb + per);
      const bool valid = f0 + c < F;
      uint32_t prev = jb > 0 && jb < je ? (sh_nl[(jb - 1) * 32 + col] >> hs) & 0xffffu : 0xffffffffu;
      for (uint32_t j = jb; j < je; j++) {
        const uint32_t nL = (sh_nl[j * 32 + col] >> hs) & 0xffffu;
        float g = -FLT_MAX;  // duplicates of the previous position stay -max
        // counts are monotone in j: an equal total means equal counts
        if (valid && nL != prev) {
          float sl = __ldg(X + nL), sr = __ldg(X + (N - nL));
          const uint32_t *hj = sh_hist + j * 32 + col;
          for (uint32_t i = 0; i < nc; i++) {
            const uint32_t l = s_cls[i];
            const uint32_t cl = (hj[l * TS * 32] >> hs) & 0xffffu;
            sl -= __ldg(X + cl);
            sr -= __ldg(X + (s_tot[l] - cl));
          }
          g = -(sl + sr);
        }
        prev = nL;
        sh_g[j * kTileF + c] = g;
        lmax = fmaxf(lmax, g);
      }
    }
    for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = lmax;
    __syncthreads();
    float tmax = s_red[0];
    for (int i = 1; i < kHistThreads / 32; i++) tmax = fmaxf(tmax, s_red[i]);
    const float cut = tmax - fused_window(K, N);
    // exact FP64 gains of the near-maximum candidates
    if (ok) {
      const double *L = fs.L;
      const double hp64 = fs.parent[slot];
      auto recheck = [&](uint32_t q) {
        const uint32_t j = q / kTileF, c = q % kTileF;
        n_checked++;
        const uint32_t nL = half16(sh_nl[j * 32 + (c & 31)], c);
        const uint32_t nR = N - nL;
        // both sides in one loop (two independent chains; each sums in class order)
        const double Ll = L[nL], Lr = L[nR];
        double sl = 0.0, sr = 0.0;
#pragma unroll 3
        for (uint32_t i = 0; i < nc; i++) {
          const uint32_t l = s_cls[i];
          const uint32_t cl = half16(sh_hist[(l * TS + j) * 32 + (c & 31)], c), cr = s_tot[l] - cl;
          if (cl != 0u && (uint64_t)cl * 1000000ull > nL) sl = dadd(sl, dmul((double)cl, dsub(Ll, L[cl])));
          if (cr != 0u && (uint64_t)cr * 1000000ull > nR) sr = dadd(sr, dmul((double)cr, dsub(Lr, L[cr])));
        }
        const double g = dsub(hp64, ddiv(dadd(sl, sr), (double)N));
        const uint32_t f = f0 + c;
        // the positions j..je share these counts: the lowest original threshold
        // wins (the run's end first, then its loads all in flight together)
        const uint32_t orig = fs.ord ? fs.ord[(size_t)slot * F + f] : f;
        uint32_t je = j + 1;
        while (je < T && half16(sh_nl[je * 32 + (c & 31)], c) == nL) je++;
        uint32_t t = 0xffu;
#pragma unroll 4
        for (uint32_t jj = j; jj < je; jj++) t = min(t, (uint32_t)fs.perm[((size_t)slot * T + jj) * F + f]);
        const long long idx = (long long)t * F + orig;
        if (g > best || (g == best && idx < best_idx)) {
          best = g;
          best_idx = idx;
          best_j = (int)j;
          best_c = (int)f;
        }
      };
      // The pairs within the window cluster in few columns, i.e. in few threads of
      // the pair loop: list them first, then deal the list out over all threads
      // (the winner does not depend on the order).  A list that overflows falls
      // back to the pair loop.
      for (uint32_t q = threadIdx.x; q < pairs; q += blockDim.x) {
        if (sh_g[q] >= cut) {  // within the window (duplicate positions hold -max)
          const uint32_t i = atomicAdd(&s_nlist, 1u);
          if (i < kRecheckList) s_list[i] = (uint16_t)q;
        }
      }
      __syncthreads();
      const uint32_t n_list = s_nlist;
      if (n_list <= kRecheckList) {
        for (uint32_t i = threadIdx.x; i < n_list; i += blockDim.x) recheck(s_list[i]);
      } else {
        for (uint32_t q = threadIdx.x; q < pairs; q += blockDim.x)
          if (sh_g[q] >= cut) recheck(q);
      }
    }
  }
  if (n_checked) atomicAdd(fs.rechecked, n_checked);
  // warp reduction on integer keys of the gains (no FP64 compares: the FP64
  // pipe is narrow); gains are never -0 (hp >= 0), so the keys order as the doubles
  long long best_key = gain_order_key(best);
  for (int o = 16; o > 0; o >>= 1) {
    const long long okey = __shfl_xor_sync(0xffffffffu, best_key, o);
    const double og = __shfl_xor_sync(0xffffffffu, best, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, best_idx, o);
    const int oj = __shfl_xor_sync(0xffffffffu, best_j, o);
    const int oc = __shfl_xor_sync(0xffffffffu, best_c, o);
    if (okey > best_key || (okey == best_key && oi < best_idx)) {
      best_key = okey;
      best = og;
      best_idx = oi;
      best_j = oj;
      best_c = oc;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    s_g[threadIdx.x >> 5] = best;
    s_i[threadIdx.x >> 5] = best_idx;
    s_j[threadIdx.x >> 5] = best_j;
    s_c[threadIdx.x >> 5] = best_c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kHistThreads / 32; i++) {
      if (s_g[i] > s_g[0] || (s_g[i] == s_g[0] && s_i[i] < s_i[0])) {
        s_g[0] = s_g[i];
        s_i[0] = s_i[i];
        s_j[0] = s_j[i];
        s_c[0] = s_c[i];
      }
    }
    SplitPart pb;
    pb.gain = s_g[0];
    pb.idx = s_i[0];
    pb.j = s_j[0];
    pb.col = s_c[0];
    const size_t pi = (size_t)slot * fs.tiles + w.tile;
    fs.part_best[pi] = pb;
    if (pb.idx != LLONG_MAX) {
      const uint32_t c = (uint32_t)pb.col - f0;
      for (uint32_t l = 0; l < K; l++)
        fs.part_cl[pi * K + l] = s_tot[l] ? half16(sh_hist[(l * TS + pb.j) * 32 + (c & 31)], c) : 0u;
    }
    __threadfence();
    s_last = atomicAdd(fs.done + slot, 1u) == fs.tiles - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  size_t bi = (size_t)slot * fs.tiles;
  SplitPart b = fs.part_best[bi];
  for (uint32_t i = 1; i < fs.tiles; i++) {
    const SplitPart q = fs.part_best[(size_t)slot * fs.tiles + i];
    if (q.gain > b.gain || (q.gain == b.gain && q.idx < b.idx)) {
      b = q;
      bi = (size_t)slot * fs.tiles + i;
    }
  }
  SplitOut o;
  if (b.idx == LLONG_MAX) {
    o.t = o.f = o.j = o.col = -1;
    o.gain = 0.0;
  } else {
    o.t = (int32_t)(b.idx / F);
    o.f = (int32_t)(b.idx % F);
    o.j = b.j;
    o.col = b.col;
    o.gain = b.gain;
    for (uint32_t l = 0; l < K; l++) fs.out_cl[(size_t)slot * K + l] = fs.part_cl[bi * K + l];
  }
  fs.out[slot] = o;
}

// One work item of the histogram kernel (the whole CTA).
template <class P, uint32_t TP, int SPI>
__device__ __forceinline__ void hist_item(const DevSet &ds, const SampleRec *__restrict__ rec, const WorkItem w,
                                          const typename P::feat_t *__restrict__ cand_feat,
                                          const typename P::feat_t *__restrict__ cand_thr,
                                          uint32_t *__restrict__ hist, uint32_t F, uint32_t T, uint32_t K,
                                          const FusedSplit &fs) {
  using FeatT = typename P::feat_t;
  using ImgT = typename P::img_t;
  constexpr int D = P::kFeatDim;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t *sh_hist = reinterpret_cast<uint32_t *>(smem_raw);                   // [K][T+1][32] packed
  FeatT *sh_thr = reinterpret_cast<FeatT *>(sh_hist + (size_t)K * (T + 1) * 32);  // [2][TP][32]
  // fused split scratch, over the threshold table (dead after the sample loop):
  // sh_g [T][64] gains, sh_nl [T][32] packed left totals
  float *sh_g = reinterpret_cast<float *>(sh_thr);
  uint32_t *sh_nl = reinterpret_cast<uint32_t *>(sh_g + (size_t)T * kTileF);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t f0 = w.tile * kTileF;
  const uint32_t fa = f0 + lane, fb = f0 + 32 + lane;
  const bool va = fa < F, vb = fb < F;

  // sorted thresholds: column c of the tile at [c / 32][t][c % 32]; padding rows
  // and candidates past F hold the maximum, which no response exceeds
  for (uint32_t j = threadIdx.x; j < TP * kTileF; j += blockDim.x) {
    const uint32_t t = j / kTileF, c = j % kTileF, ff = f0 + c;
    sh_thr[(c >> 5) * (TP * 32) + t * 32 + (c & 31)] =
        (t < T && ff < F) ? cand_thr[((size_t)w.slot * T + t) * F + ff] : max_of<FeatT>();
  }
  if (w.multi == 2) {
    // a fused item: only the rows of the classes present in the node are counted and read
    for (uint32_t l = 0; l < K; l++)
      if (fs.class_tot[(size_t)w.slot * K + l])
        for (uint32_t j = threadIdx.x; j < (T + 1) * 32; j += blockDim.x) sh_hist[l * (T + 1) * 32 + j] = 0u;
  } else {
    for (uint32_t j = threadIdx.x; j < K * (T + 1) * 32; j += blockDim.x) sh_hist[j] = 0u;
  }
  if (w.multi == 2) {
    // the fused split reads the tile's threshold permutation and column order
    // at the end; bring them to L2 now
    const uint32_t last = min(F - 1, f0 + kTileF - 1);  // the tile's last column
    if (threadIdx.x < T) {
      const uint8_t *r = fs.perm + ((size_t)w.slot * T + threadIdx.x) * F;
      prefetch_l2(r + f0);
      prefetch_l2(r + last);
    } else if (fs.ord && threadIdx.x < T + 2) {
      prefetch_l2(fs.ord + (size_t)w.slot * F + (threadIdx.x == T ? f0 : last));
    }
  }
  typename P::Cand ca, cb;
  {
    FeatT fva[D], fvb[D];
#pragma unroll
    for (int d = 0; d < D; d++) {
      fva[d] = va ? cand_feat[((size_t)w.slot * D + d) * F + fa] : (FeatT)0;
      fvb[d] = vb ? cand_feat[((size_t)w.slot * D + d) * F + fb] : (FeatT)0;
    }
    ca = P::candidate(fva);
    cb = P::candidate(fvb);
  }
  // the exact-division fast path when every candidate of the tile allows it
  const bool fast = __syncthreads_and(P::fast(ca) && P::fast(cb));
  if (fast) hist_samples<P, TP, true, SPI>(ds, rec, w, ca, cb, sh_hist, sh_thr, T);
  else hist_samples<P, TP, false, SPI>(ds, rec, w, ca, cb, sh_hist, sh_thr, T);

  __syncthreads();
  if (w.multi == 2) {
    fused_split(fs, w, sh_hist, sh_g, sh_nl, F, T, K);
    return;
  }
  for (uint32_t l = 0; l < K; l++) {
    for (uint32_t q = threadIdx.x; q < T * 32; q += blockDim.x) {
      const uint32_t v = sh_hist[l * (T + 1) * 32 + q];
      const uint32_t c = q & 31;
      uint32_t *dst = hist + ((size_t)w.slot * K * T + l * T + (q >> 5)) * F + f0 + c;
      if (f0 + c < F) {
        if (w.multi) {
          if (v & 0xffffu) atomicAdd(dst, v & 0xffffu);
        } else {
          *dst = v & 0xffffu;
        }
      }
      if (f0 + 32 + c < F) {
        if (w.multi) {
          if (v >> 16) atomicAdd(dst + 32, v >> 16);
        } else {
          dst[32] = v >> 16;
        }
      }
    }
  }
}

// The histogram kernel over a work list.  queue == null: one CTA per item
// (blockIdx.x).  Otherwise a persistent grid (a few CTAs per SM) whose CTAs
// take items k = 0, 1, ... in list order from the counter *queue (an atomic
// add, no wait), so a list sorted largest first keeps every SM busy to the end.
template <class P, uint32_t TP, int SPI>
__global__ void __launch_bounds__(kHistThreads, SPI <= 2 ? 3 : 2) k_hist(DevSet ds, const SampleRec *__restrict__ rec,
                                                       const WorkItem *__restrict__ items, uint32_t n_items,
                                                       unsigned *__restrict__ queue,
                                                       const typename P::feat_t *__restrict__ cand_feat,
                                                       const typename P::feat_t *__restrict__ cand_thr,
                                                       uint32_t *__restrict__ hist, uint32_t F,
                                                       uint32_t T, uint32_t K, FusedSplit fs) {
  if (queue == nullptr) {
    hist_item<P, TP, SPI>(ds, rec, items[blockIdx.x], cand_feat, cand_thr, hist, F, T, K, fs);
    return;
  }
  __shared__ uint32_t s_next;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t k = s_next;
    __syncthreads();  // read by every thread before thread 0 takes the next item
    if (k >= n_items) return;
    hist_item<P, TP, SPI>(ds, rec, items[k], cand_feat, cand_thr, hist, F, T, K, fs);
    __syncthreads();  // the item's shared memory is free again
  }
}

static __global__ void k_zero_slots(uint32_t *__restrict__ hist, const uint32_t *__restrict__ slots, uint32_t n,
                             uint64_t per_slot) {
  const uint64_t total = (uint64_t)n * per_slot;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = i / per_slot;
    hist[(uint64_t)slots[s] * per_slot + (i - s * per_slot)] = 0u;
  }
}

// Split parameters of the winners read from the candidate tables: the D
// feature values of column `col` and the threshold of original index t (the
// sorted entry whose permutation is t) -- the values candidate_feature and
// candidate_threshold regenerate from MD5.  params [n][D + 1]; slots without a
// split are left as they are.
template <typename FeatT>
__global__ void k_split_params(const SplitOut *__restrict__ out, uint32_t n, const FeatT *__restrict__ cand_feat,
                               const FeatT *__restrict__ cand_thr, const uint8_t *__restrict__ perm, uint32_t F,
                               uint32_t T, int D, FeatT *__restrict__ params) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SplitOut o = out[i];
  if (o.t < 0 || o.col < 0) return;
  const uint32_t col = (uint32_t)o.col;
  for (int d = 0; d < D; d++) params[(size_t)i * (D + 1) + d] = cand_feat[((size_t)i * D + d) * F + col];
  for (uint32_t j = 0; j < T; j++)
    if (perm[((size_t)i * T + j) * F + col] == (uint8_t)o.t) params[(size_t)i * (D + 1) + D] = cand_thr[((size_t)i * T + j) * F + col];
}

// The parent term S(tot, N) / N of the exact FP64 gain of every slot, the same
// IEEE operation sequence as sum64 (0 for an empty slot or one beyond the table).
static __global__ void k_parent_term(const uint32_t *__restrict__ class_tot, uint32_t n, uint32_t K,
                                     const double *__restrict__ L, uint64_t L_len, double *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t *tot = class_tot + (size_t)i * K;
  uint32_t N = 0;
  for (uint32_t l = 0; l < K; l++) N += tot[l];
  double h = 0.0;
  if (N != 0 && (uint64_t)N < L_len) {
    for (uint32_t l = 0; l < K; l++) {
      const uint32_t cl = tot[l];
      if (cl != 0u && (uint64_t)cl * 1000000ull > N) h = dadd(h, dmul((double)cl, dsub(L[N], L[cl])));
    }
    h = ddiv(h, (double)N);
  }
  out[i] = h;
}

// Rank-space counts -> the reference layout hist[n][l][t][f] (number of
// samples with response <= threshold t).
static __global__ void k_hist_to_ref(const uint32_t *__restrict__ rank_hist, const uint8_t *__restrict__ perm,
                              uint32_t *__restrict__ out, uint32_t n_nodes, uint32_t K, uint32_t T,
                              uint32_t F) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)n_nodes * K * F) return;
  const uint32_t f = (uint32_t)(idx % F);
  const uint64_t nl = idx / F;
  const uint32_t n = (uint32_t)(nl / K);
  uint32_t c = 0;
  for (uint32_t j = 0; j < T; j++) {
    c += rank_hist[(nl * T + j) * F + f];
    out[(nl * T + perm[((size_t)n * T + j) * F + f]) * F + f] = c;
  }
}

// Loads the counts of sorted position j of column f into c (prefix-summed in
// rank space, copied when cumulative); returns whether they changed.
template <int KM, bool CUM>
PD_D bool step_counts(const uint32_t *H, uint32_t K, uint32_t T, uint32_t F, uint32_t j, uint32_t f, uint32_t *c,
                      uint32_t &nL) {
  bool changed = false;
  nL = 0;
#pragma unroll
  for (int l = 0; l < KM; l++) {
    if ((uint32_t)l < K) {
      const uint32_t h = H[((size_t)l * T + j) * F + f];
      if (CUM) {
        changed |= h != c[l];
        c[l] = h;
      } else {
        changed |= h != 0u;
        c[l] += h;
      }
      nL += c[l];
    }
  }
  return changed;
}

template <int KM>
PD_D void load_tot(const SplitArgs &a, uint32_t slot, uint32_t *tot, uint32_t &N) {
  for (uint32_t l = threadIdx.x; l < KM; l += blockDim.x) tot[l] = l < a.K ? a.class_tot[(size_t)slot * a.K + l] : 0u;
  __syncthreads();
  N = 0;
#pragma unroll
  for (int l = 0; l < KM; l++) N += tot[l];
}

// Pass 1: FP32 gain of every (t,f) of a column range, kept in scratch, and the
// node maximum (atomic over the parts of the node).  A sorted position whose
// rank bin is empty has the counts, hence the gain, of the previous one.
template <int KM, bool CUM>
__global__ void __launch_bounds__(kSplitCols) k_split_g32(SplitArgs a) {
  const uint32_t slot = a.slot_list ? a.slot_list[blockIdx.y] : blockIdx.y, part = blockIdx.x;
  const uint32_t F = a.F, T = a.T, K = a.K;
  __shared__ uint32_t tot[KM];
  __shared__ float red[kSplitCols / 32];
  uint32_t N;
  load_tot<KM>(a, slot, tot, N);
  if (N == 0 || (uint64_t)N >= a.L_len) return;
  const float hp32 = ent32<KM, false>(tot, tot, K, N);
  const float invN = __frcp_rn((float)N);
  const uint32_t *H = a.hist + (size_t)slot * K * T * F;
  float *G = a.g32 + (size_t)slot * T * F;
  const uint32_t fb = part * a.cols, fe = min(F, fb + a.cols);
  float lmax = -FLT_MAX;
  for (uint32_t f = fb + threadIdx.x; f < fe; f += blockDim.x) {
    uint32_t c[KM];
#pragma unroll
    for (int l = 0; l < KM; l++) c[l] = 0u;
    float g = 0.0f;
    // rows are loaded kSplitRows at a time so their loads are in flight together
    for (uint32_t j0 = 0; j0 < T; j0 += kSplitRows) {
      uint32_t h[kSplitRows][KM];
#pragma unroll
      for (int r = 0; r < kSplitRows; r++)
#pragma unroll
        for (int l = 0; l < KM; l++)
          h[r][l] = ((uint32_t)l < K && j0 + r < T) ? H[((size_t)l * T + j0 + r) * F + f] : 0u;
#pragma unroll
      for (int r = 0; r < kSplitRows; r++) {
        const uint32_t j = j0 + r;
        if (j >= T) break;
        bool changed = false;
        uint32_t nL = 0;
#pragma unroll
        for (int l = 0; l < KM; l++) {
          if ((uint32_t)l < K) {
            if (CUM) {
              changed |= h[r][l] != c[l];
              c[l] = h[r][l];
            } else {
              changed |= h[r][l] != 0u;
              c[l] += h[r][l];
            }
            nL += c[l];
          }
        }
        if (j == 0 || changed) {
          const uint32_t nR = N - nL;
          const float hl = ent32<KM, false>(tot, c, K, nL);
          const float hr = ent32<KM, true>(tot, c, K, nR);
          g = hp32 - ((float)nL * invN * hl + (float)nR * invN * hr);
        }
        G[(size_t)j * F + f] = g;
        lmax = fmaxf(lmax, g);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = red[0];
    for (int i = 1; i < kSplitCols / 32; i++) m = fmaxf(m, red[i]);
    atomicMax(a.node_max + slot, f2ord(m));
  }
}

// Pass 2: candidates within delta of the node's FP32 maximum are re-evaluated
// with the exact FP64 gain S(tot,N)/N - (S(L)+S(R))/N; the largest exact gain
// wins, ties to the lowest t*F+f (the first-max rule of
// learn_best_feature.cl:96-101 + std::max_element).  The last part of a node to
// finish reduces the parts and writes the winner with its left class counts.
template <int KM, bool CUM>
__global__ void __launch_bounds__(kSplitCols) k_split_pick(SplitArgs a) {
  const uint32_t slot = a.slot_list ? a.slot_list[blockIdx.y] : blockIdx.y, part = blockIdx.x;
  const uint32_t F = a.F, T = a.T, K = a.K;
  __shared__ uint32_t tot[KM];
  __shared__ double red_g[kSplitCols / 32];
  __shared__ long long red_i[kSplitCols / 32];
  __shared__ int red_j[kSplitCols / 32];
  __shared__ int red_c[kSplitCols / 32];
  __shared__ bool last;
  uint32_t N;
  load_tot<KM>(a, slot, tot, N);
  if (N == 0 || (uint64_t)N >= a.L_len) {
    if (part == 0 && threadIdx.x == 0) {
      SplitOut o;
      o.t = o.f = o.j = o.col = -1;
      o.gain = 0.0;
      a.out[slot] = o;
    }
    return;
  }
  const float cut = ord2f(a.node_max[slot]) - a.delta;
  const double hp64 = ddiv(sum64<KM, false>(tot, tot, K, N, a.L), (double)N);
  const uint32_t *H = a.hist + (size_t)slot * K * T * F;
  const float *G = a.g32 + (size_t)slot * T * F;
  const uint32_t fb = part * a.cols, fe = min(F, fb + a.cols);
  double best = -DBL_MAX;
  long long best_idx = LLONG_MAX;
  int best_j = -1, best_c = -1;
  unsigned long long n_checked = 0;
  for (uint32_t f = fb + threadIdx.x; f < fe; f += blockDim.x) {
    int jmax = -1;
    for (uint32_t j = 0; j < T; j++)
      if (G[(size_t)j * F + f] >= cut) jmax = (int)j;
    if (jmax < 0) continue;
    uint32_t c[KM];
#pragma unroll
    for (int l = 0; l < KM; l++) c[l] = 0u;
    bool dirty = true;
    double g = 0.0;
    for (int j = 0; j <= jmax; j++) {
      uint32_t nL;
      dirty |= step_counts<KM, CUM>(H, K, T, F, (uint32_t)j, f, c, nL);
      if (!(G[(size_t)j * F + f] >= cut)) continue;
      if (dirty) {
        n_checked++;
        const uint32_t nR = N - nL;
        const double sl = sum64<KM, false>(tot, c, K, nL, a.L);
        const double sr = sum64<KM, true>(tot, c, K, nR, a.L);
        g = dsub(hp64, ddiv(dadd(sl, sr), (double)N));
        dirty = false;
      }
      const uint32_t t = a.perm ? a.perm[((size_t)slot * T + j) * F + f] : (uint32_t)j;
      const long long idx = (long long)t * F + (a.ord ? a.ord[(size_t)slot * F + f] : f);
      if (g > best || (g == best && idx < best_idx)) {
        best = g;
        best_idx = idx;
        best_j = j;
        best_c = (int)f;
      }
    }
  }
  if (n_checked) atomicAdd(a.rechecked, n_checked);
  // warp reduction on integer keys of the gains (no FP64 compares: the FP64
  // pipe is narrow); gains are never -0 (hp >= 0), so the keys order as the doubles
  long long best_key = gain_order_key(best);
  for (int o = 16; o > 0; o >>= 1) {
    const long long okey = __shfl_xor_sync(0xffffffffu, best_key, o);
    const double og = __shfl_xor_sync(0xffffffffu, best, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, best_idx, o);
    const int oj = __shfl_xor_sync(0xffffffffu, best_j, o);
    const int oc = __shfl_xor_sync(0xffffffffu, best_c, o);
    if (okey > best_key || (okey == best_key && oi < best_idx)) {
      best_key = okey;
      best = og;
      best_idx = oi;
      best_j = oj;
      best_c = oc;
    }
  }
  if ((threadIdx.x & 31) == 0) {
    red_g[threadIdx.x >> 5] = best;
    red_i[threadIdx.x >> 5] = best_idx;
    red_j[threadIdx.x >> 5] = best_j;
    red_c[threadIdx.x >> 5] = best_c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kSplitCols / 32; i++) {
      if (red_g[i] > red_g[0] || (red_g[i] == red_g[0] && red_i[i] < red_i[0])) {
        red_g[0] = red_g[i];
        red_i[0] = red_i[i];
        red_j[0] = red_j[i];
        red_c[0] = red_c[i];
      }
    }
    SplitPart pb;
    pb.gain = red_g[0];
    pb.idx = red_i[0];
    pb.j = red_j[0];
    pb.col = red_c[0];
    a.part_best[(size_t)slot * a.parts + part] = pb;
    __threadfence();
    last = atomicAdd(a.done + slot, 1u) == a.parts - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  SplitPart b = a.part_best[(size_t)slot * a.parts];
  for (uint32_t i = 1; i < a.parts; i++) {
    const SplitPart q = a.part_best[(size_t)slot * a.parts + i];
    if (q.gain > b.gain || (q.gain == b.gain && q.idx < b.idx)) b = q;
  }
  SplitOut o;
  if (b.idx == LLONG_MAX) {
    o.t = o.f = o.j = o.col = -1;
    o.gain = 0.0;
  } else {
    o.t = (int32_t)(b.idx / F);
    o.f = (int32_t)(b.idx % F);
    o.j = b.j;
    o.col = b.col;
    o.gain = b.gain;
    const uint32_t col = (uint32_t)b.col;
    for (uint32_t l = 0; l < K; l++) {
      uint32_t c = 0;
      if (CUM) {
        c = H[((size_t)l * T + o.j) * F + col];
      } else {
        for (int j = 0; j <= o.j; j++) c += H[((size_t)l * T + j) * F + col];
      }
      a.out_cl[(size_t)slot * K + l] = c;
    }
  }
  a.out[slot] = o;
}

// ------------------------------------------------------------ reassign ----
// kernels/predict.cl:36-85 as used by the trainer: a sample on a node that has
// just been split moves to leftChild + (response > threshold).  flags: 1 = goes
// to a left child that is on the next frontier, 2 = right child on the next
// frontier, 0 = leaves the active set.
struct SlotNext {
  long long adj_l, adj_r;  // next position base (next offset of child - samples of earlier parents)
  int32_t k_l, k_r;        // next frontier slot of each child or -1
};

template <class P>
__global__ void k_reassign(DevSet ds, const uint32_t *__restrict__ act, const SampleRec *__restrict__ rec,
                           const uint32_t *__restrict__ act_slot,
                           uint32_t n_act, int32_t *__restrict__ snode, const int32_t *__restrict__ lc,
                           const typename P::feat_t *__restrict__ feat,
                           const typename P::feat_t *__restrict__ thr, const SlotNext *__restrict__ nxt,
                           uint8_t *__restrict__ flags) {
  using FeatT = typename P::feat_t;
  using ImgT = typename P::img_t;
  constexpr int D = P::kFeatDim;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_act) return;
  const uint32_t s = act[i];
  const int32_t n = snode[s];
  const int32_t c = lc[n];
  uint8_t flag = 0;
  if (c >= 0) {
    const SampleRec r = rec[i];
    const uint32_t xy = r.xy, im_i = r.img_lab & 0xffffffu;
    const uint32_t wh = ds.img_wh[im_i];
    ImageRef<ImgT> im;
    im.data = reinterpret_cast<const ImgT *>(ds.pixels + ds.img_off[im_i]);
    im.w = (int32_t)(wh & 0xffffu);
    im.h = (int32_t)(wh >> 16);
    im.magic = ds.magic;
    if constexpr (P::kUsesTree) attach_tree<P>(im, ds, ds.map_off ? ds.map_off[im_i] : 0ull);
    FeatT fv[D];
#pragma unroll
    for (int d = 0; d < D; d++) fv[d] = feat[(size_t)n * D + d];
    const auto prep = P::prepare(im, (int32_t)(xy & 0xffffu), (int32_t)(xy >> 16), r.pre);
    const FeatT resp = P::eval(prep, fv);
    const bool right = resp > thr[n];
    snode[s] = c + (right ? 1 : 0);
    const SlotNext sn = nxt[act_slot[i]];
    if (right) flag = sn.k_r >= 0 ? 2 : 0;
    else flag = sn.k_l >= 0 ? 1 : 0;
  }
  flags[i] = flag;
}

// Per scan block: number of flags equal to 1 (low 32 bits) and 2 (high 32).
static __global__ void __launch_bounds__(256) k_scan_reduce(const uint8_t *__restrict__ flags, uint32_t n,
                                                     unsigned long long *__restrict__ bsum) {
  const uint32_t b0 = blockIdx.x * kScanItems;
  unsigned long long acc = 0;
  for (uint32_t i = b0 + threadIdx.x; i < min(n, b0 + kScanItems); i += blockDim.x) {
    const uint8_t fl = flags[i];
    acc += fl == 1 ? 1ull : (fl == 2 ? (1ull << 32) : 0ull);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ unsigned long long red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int i = 0; i < 8; i++) s += red[i];
    bsum[blockIdx.x] = s;
  }
}

// Exclusive scan of the block sums in one CTA (any count).
static __global__ void __launch_bounds__(1024) k_scan_blocks(unsigned long long *__restrict__ bsum, uint32_t nb,
                                                      unsigned long long *__restrict__ total) {
  const uint32_t per = (nb + blockDim.x - 1) / blockDim.x;
  const uint32_t b = threadIdx.x * per, e = min(nb, b + per);
  unsigned long long s = 0;
  for (uint32_t i = b; i < e; i++) s += bsum[i];
  __shared__ unsigned long long sh[1024];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t o = 1; o < blockDim.x; o <<= 1) {
    const unsigned long long v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned long long run = sh[threadIdx.x] - s;
  for (uint32_t i = b; i < e; i++) {
    const unsigned long long v = bsum[i];
    bsum[i] = run;
    run += v;
  }
  if (threadIdx.x == blockDim.x - 1) *total = sh[threadIdx.x];
}

// Stable regrouping: sample i of parent slot p goes to
// adj[p] + (number of earlier samples with the same flag).  Because parents are
// in slot order and their children in the same order, this keeps every child's
// samples in their previous (image-major) order.
static __global__ void __launch_bounds__(256) k_scatter(const uint8_t *__restrict__ flags, uint32_t n,
                                                 const unsigned long long *__restrict__ bsum,
                                                 const uint32_t *__restrict__ act,
                                                 const uint32_t *__restrict__ act_slot,
                                                 const SlotNext *__restrict__ nxt, uint32_t n_next,
                                                 uint32_t *__restrict__ act_out,
                                                 uint32_t *__restrict__ slot_out,
                                                 const SampleRec *__restrict__ rec,
                                                 SampleRec *__restrict__ rec_out,
                                                 uint32_t *__restrict__ err) {
  constexpr int PER = kScanItems / 256;
  const uint32_t b0 = blockIdx.x * kScanItems + threadIdx.x * PER;
  uint8_t fl[PER];
  unsigned long long mine = 0;
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const uint32_t i = b0 + k;
    fl[k] = i < n ? flags[i] : 0;
    mine += fl[k] == 1 ? 1ull : (fl[k] == 2 ? (1ull << 32) : 0ull);
  }
  // block exclusive scan of per-thread counts
  __shared__ unsigned long long sh[256];
  sh[threadIdx.x] = mine;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const unsigned long long v = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned long long run = bsum[blockIdx.x] + sh[threadIdx.x] - mine;
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const uint32_t i = b0 + k;
    if (fl[k] == 0) continue;
    const SlotNext sn = nxt[act_slot[i]];
    long long pos;
    uint32_t kslot;
    if (fl[k] == 1) {
      pos = sn.adj_l + (long long)(run & 0xffffffffull);
      kslot = (uint32_t)sn.k_l;
      run += 1ull;
    } else {
      pos = sn.adj_r + (long long)(run >> 32);
      kslot = (uint32_t)sn.k_r;
      run += 1ull << 32;
    }
    if (pos < 0 || pos >= (long long)n_next) {
      atomicAdd(err, 1u);
      continue;
    }
    act_out[pos] = act[i];
    slot_out[pos] = kslot;
    rec_out[pos] = rec[i];
  }
}

// rec[i] = the static record of sample act[i].
static __global__ void k_gather_rec(const uint32_t *__restrict__ act, uint32_t n, const SampleRec *__restrict__ all,
                                    SampleRec *__restrict__ rec) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rec[i] = all[act[i]];
}

// The static record of every uploaded sample (after the plugin's image mapping).
template <class P>
__global__ void k_build_rec(DevSet ds, uint32_t n, SampleRec *__restrict__ rec) {
  using ImgT = typename P::img_t;
  static_assert(P::kPreWords <= 2, "a sample record holds two preload words");
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  SampleRec r;
  r.xy = ds.s_xy[s];
  const uint32_t imi = ds.s_img[s];
  r.img_lab = imi | ((uint32_t)ds.s_label[s] << 24);
  const uint32_t wh = ds.img_wh[imi];
  ImageRef<ImgT> im;
  im.data = reinterpret_cast<const ImgT *>(ds.pixels + ds.img_off[imi]);
  im.w = (int32_t)(wh & 0xffffu);
  im.h = (int32_t)(wh >> 16);
  im.magic = ds.magic;
  uint32_t pre[2] = {0u, 0u};
  P::preload(im, (int32_t)(r.xy & 0xffffu), (int32_t)(r.xy >> 16), pre);
  r.pre[0] = pre[0];
  r.pre[1] = pre[1];
  rec[s] = r;
}

static __global__ void k_iota(uint32_t *__restrict__ a, uint32_t *__restrict__ slot, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    a[i] = i;
    slot[i] = 0u;
  }
}

// The trainer's copy of uint16 depth images with 0 stored as the background
// depth (plugins with kTrainMapsZero read both alike).
static __global__ void k_zero_to_background(uint16_t *__restrict__ px, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (px[i] == 0) px[i] = (uint16_t)kBgDepth;
}

static __global__ void k_magic_table(uint32_t *__restrict__ out) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < 65536u) out[d] = d ? RoundDiv::multiplier(d) : 0u;
}

static __global__ void k_log2_table(double *__restrict__ out, uint64_t n, DD inv_ln2) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = dd_log2_u32((uint32_t)i, inv_ln2);
}

// c*log2(c) rounded to float (0 for c = 0), from the exact log2 table.
static __global__ void k_xlog2_table(float *__restrict__ out, const double *__restrict__ L, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i ? __double2float_rn(dmul((double)i, L[i])) : 0.0f;
}

}  // namespace pd
