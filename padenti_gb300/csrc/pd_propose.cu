// The proposal network of learned candidate proposals (no reference
// counterpart; the reference draws candidates uniformly,
// kernels/hist_update.cl:62-184).
//
// A BF16 MLP -- input row of a node (depth, log-count, class frequencies), three
// hidden layers of 256 with GELU, and a head giving a 16-component Gaussian
// mixture over the normalised (feature values, threshold) space -- trained on
// the GPU by this file's own kernels from the records the plain trainer emits
// (one per split node: its statistics and its winning candidate).  Matrix
// products run on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
// accumulation) with the bias, GELU and GELU-derivative fused into the
// epilogue; weight gradients are reduced over the batch in fixed-order split-K
// partials, so a training run is deterministic.  Master weights and Adam state
// are FP32; the GEMMs read BF16 copies.
//
// Parameter vector (FP32, in this order): W1 [H][IN], b1 [H], W2 [H][H], b2,
// W3 [H][H], b3, Wo [OUT][H], bo [OUT].  Output row: G logits, G x DY means,
// G x DY log standard deviations (component-major), DY = FeatDim + 1.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pd_ctx.cuh"
#include "pd_propose.cuh"

using bf16 = __nv_bfloat16;

namespace pd {

constexpr int kGemmTM = 64, kGemmTN = 64, kGemmMaxStage = 256, kGemmPad = 8;
constexpr int kSplits = 8;  // batch splits of the weight-gradient products

enum { EPI_GELU = 0, EPI_LINEAR = 1, EPI_DGELU = 2, EPI_PARTIAL = 3 };

// C(i, j) = sum_k A(i, k) B(k, j) over k in this CTA's split range, with
// A(i, k) = A[i * a_i + k * a_k] and B(k, j) = B[k * b_k + j * b_j].
struct GemmArgs {
  const bf16 *A;
  int64_t a_i, a_k;
  const bf16 *B;
  int64_t b_k, b_j;
  int M, N, K, k_split;
  const float *bias;   // EPI_GELU, EPI_LINEAR
  float *outf;         // z (EPI_GELU), output (EPI_LINEAR), partials (EPI_PARTIAL)
  bf16 *outb;          // GELU(z) (EPI_GELU), dz (EPI_DGELU)
  const float *zin;    // z of the layer (EPI_DGELU)
  int64_t ldo;         // row pitch of outf / outb / zin
  int64_t split_stride;  // EPI_PARTIAL: floats between the partials of two splits
  float *bias_part;      // EPI_PARTIAL: row sums of A over the split (the bias gradient), written by the
                         // CTAs of the first column tile (null: none)
  // 16-byte loads of 8 elements along the contiguous index of A / B (set by
  // gemm() when that index's extent, the other stride, the split length and
  // the base pointer allow it)
  int vec_a, vec_b;
  int kstage;  // reduction columns staged in shared memory at a time (a multiple of 32, <= 256)
};

PD_D float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
PD_D float gelu_d(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

PD_D void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int kGemmThreads = 256;  // 8 warps: 4 x 2 warps of 16 x 32 outputs
constexpr int kStageBatch = 8;     // 16-byte loads per thread per operand in flight

// The 16-byte loads of one operand tile: rows [r0, r0 + 64) x columns
// [k0, k0 + kn) of X(r, k) = X[r * s_r + k * s_k], 8 elements each along the
// contiguous index (s_k == 1: along k; s_r == 1: along r); zero outside r < R,
// k < ke.  Load and store are separate so that both operands' loads are in
// flight before the first store.
struct TileLoads {
  uint4 v[kStageBatch];
};
PD_D void tile_load(TileLoads &L, int e0, const bf16 *__restrict__ X, int64_t s_r, int64_t s_k, int r0, int R,
                    int k0, int kn, int ke) {
  const bool along_k = s_k == 1;
  const int total = kGemmTM * kn / 8;
#pragma unroll
  for (int b = 0; b < kStageBatch; b++) {
    const int e = e0 + b * kGemmThreads;
    const int r = along_k ? e / (kn / 8) : (e % (kGemmTM / 8)) * 8, c = along_k ? (e % (kn / 8)) * 8 : e / (kGemmTM / 8);
    const int gr = r0 + r, gk = k0 + c;
    L.v[b] = make_uint4(0u, 0u, 0u, 0u);
    if (e < total && gr < R && gk < ke) L.v[b] = *reinterpret_cast<const uint4 *>(X + (int64_t)gr * s_r + (int64_t)gk * s_k);
  }
}
PD_D void tile_store(const TileLoads &L, int e0, bf16 *S, int ld, bool along_k, int kn) {
  const int total = kGemmTM * kn / 8;
#pragma unroll
  for (int b = 0; b < kStageBatch; b++) {
    const int e = e0 + b * kGemmThreads;
    if (e >= total) break;
    if (along_k) {
      *reinterpret_cast<uint4 *>(S + (e / (kn / 8)) * ld + (e % (kn / 8)) * 8) = L.v[b];
    } else {
      const int r = (e % (kGemmTM / 8)) * 8, c = e / (kGemmTM / 8);
      const bf16 *pv = reinterpret_cast<const bf16 *>(&L.v[b]);
#pragma unroll
      for (int q = 0; q < 8; q++) S[(r + q) * ld + c] = pv[q];
    }
  }
}
// Element-wise staging for layouts that do not allow 16-byte loads.
PD_D void tile_scalar(bf16 *S, int ld, const bf16 *__restrict__ X, int64_t s_r, int64_t s_k, int r0, int R, int k0,
                      int kn, int ke, int tid) {
  const bf16 zero = __float2bfloat16(0.0f);
  const int total = kGemmTM * kn;
  for (int e0 = tid; e0 < total; e0 += kGemmThreads * kStageBatch) {
    bf16 v[kStageBatch];
#pragma unroll
    for (int b = 0; b < kStageBatch; b++) {
      const int e = e0 + b * kGemmThreads;
      const int r = s_k == 1 ? e / kn : e % kGemmTM, c = s_k == 1 ? e % kn : e / kGemmTM;
      const int gr = r0 + r, gk = k0 + c;
      v[b] = (e < total && gr < R && gk < ke) ? X[(int64_t)gr * s_r + (int64_t)gk * s_k] : zero;
    }
#pragma unroll
    for (int b = 0; b < kStageBatch; b++) {
      const int e = e0 + b * kGemmThreads;
      if (e >= total) break;
      const int r = s_k == 1 ? e / kn : e % kGemmTM, c = s_k == 1 ? e % kn : e / kGemmTM;
      S[r * ld + c] = v[b];
    }
  }
}

// 64 x 64 output tile per CTA, 8 warps of 16 x 32 (1 x 4 mma tiles each).  The
// reduction range is staged in shared memory kstage (<= 256) at a time -- for
// every product of the network one stage holds it all, and with 256 threads a
// full stage is one batch of 8 loads per thread and operand, issued for both
// operands before any store -- as an A tile [i][k] and a B tile [j][k] (k
// contiguous, so every fragment register is one aligned 32-bit load).
template <int EPI>
__global__ void __launch_bounds__(kGemmThreads) k_prop_gemm(GemmArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ks = g.kstage, ld = ks + kGemmPad;  // row pitch in elements (a multiple of 8)
  bf16 *As = reinterpret_cast<bf16 *>(smem_raw);
  bf16 *Bs = As + kGemmTM * ld;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1, gq = lane >> 2, tq = lane & 3;
  const int i0 = blockIdx.y * kGemmTM, j0 = blockIdx.x * kGemmTN;
  const int kb = blockIdx.z * g.k_split, ke = min(g.K, kb + g.k_split);
  float bsum = 0.0f;  // EPI_PARTIAL with bias_part: this thread's row sum
  float acc[4][4];
#pragma unroll
  for (int b = 0; b < 4; b++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[b][c] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += ks) {
    const int kn = min(ks, ke - k0 + 31) / 32 * 32;  // columns of this stage, a multiple of 32
    // A(i, k) for i in [i0, i0 + 64); B(k, j) staged as rows j in [j0, j0 + 64)
    if (g.vec_a && g.vec_b) {
      for (int e0 = tid; e0 < kGemmTM * kn / 8; e0 += kGemmThreads * kStageBatch) {
        TileLoads la, lb;
        tile_load(la, e0, g.A, g.a_i, g.a_k, i0, g.M, k0, kn, ke);
        tile_load(lb, e0, g.B, g.b_j, g.b_k, j0, g.N, k0, kn, ke);
        tile_store(la, e0, As, ld, g.a_k == 1, kn);
        tile_store(lb, e0, Bs, ld, g.b_k == 1, kn);
      }
    } else {
      if (g.vec_a) {
        for (int e0 = tid; e0 < kGemmTM * kn / 8; e0 += kGemmThreads * kStageBatch) {
          TileLoads la;
          tile_load(la, e0, g.A, g.a_i, g.a_k, i0, g.M, k0, kn, ke);
          tile_store(la, e0, As, ld, g.a_k == 1, kn);
        }
      } else {
        tile_scalar(As, ld, g.A, g.a_i, g.a_k, i0, g.M, k0, kn, ke, tid);
      }
      if (g.vec_b) {
        for (int e0 = tid; e0 < kGemmTN * kn / 8; e0 += kGemmThreads * kStageBatch) {
          TileLoads lb;
          tile_load(lb, e0, g.B, g.b_j, g.b_k, j0, g.N, k0, kn, ke);
          tile_store(lb, e0, Bs, ld, g.b_k == 1, kn);
        }
      } else {
        tile_scalar(Bs, ld, g.B, g.b_j, g.b_k, j0, g.N, k0, kn, ke, tid);
      }
    }
    __syncthreads();
    if (EPI == EPI_PARTIAL && g.bias_part && blockIdx.x == 0 && tid < kGemmTM) {
      // row sums of the staged A tile, in column order
      for (int c = 0; c < kn; c++) bsum += __bfloat162float(As[tid * ld + c]);
    }
    for (int kk = 0; kk < kn; kk += 16) {
      uint32_t a[4], b[4][2];
      const bf16 *r0 = As + (wm * 16 + gq) * ld + kk + tq * 2;
      a[0] = *reinterpret_cast<const uint32_t *>(r0);
      a[1] = *reinterpret_cast<const uint32_t *>(r0 + 8 * ld);
      a[2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
      a[3] = *reinterpret_cast<const uint32_t *>(r0 + 8 * ld + 8);
#pragma unroll
      for (int nt = 0; nt < 4; nt++) {
        const bf16 *c0 = Bs + (wn * 32 + nt * 8 + gq) * ld + kk + tq * 2;
        b[nt][0] = *reinterpret_cast<const uint32_t *>(c0);
        b[nt][1] = *reinterpret_cast<const uint32_t *>(c0 + 8);
      }
#pragma unroll
      for (int nt = 0; nt < 4; nt++) mma_bf16(acc[nt], a, b[nt]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int nt = 0; nt < 4; nt++)
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int row = i0 + wm * 16 + gq + h * 8, col = j0 + wn * 32 + nt * 8 + tq * 2 + e;
        if (row >= g.M || col >= g.N) continue;
        const float v = acc[nt][h * 2 + e];
        const int64_t o = (int64_t)row * g.ldo + col;
        if (EPI == EPI_GELU) {
          const float z = v + g.bias[col];
          g.outf[o] = z;
          g.outb[o] = __float2bfloat16(gelu_f(z));
        } else if (EPI == EPI_LINEAR) {
          g.outf[o] = v + g.bias[col];
        } else if (EPI == EPI_DGELU) {
          g.outb[o] = __float2bfloat16(v * gelu_d(g.zin[o]));
        } else {
          g.outf[(int64_t)blockIdx.z * g.split_stride + o] = v;
        }
      }
  if (EPI == EPI_PARTIAL && g.bias_part && blockIdx.x == 0 && tid < kGemmTM && i0 + tid < g.M)
    g.bias_part[(int64_t)blockIdx.z * g.split_stride + i0 + tid] = bsum;
}

// Mixture negative log-likelihood of each row's target and its gradient with
// respect to the network output.  Half a warp per row, one lane per mixture
// component (log-sum-exps by shuffles within the 16 lanes).  Rows are weighted
// by w[i] * inv_wsum (the loss is the weighted mean); a log-sd outside the
// clamp gets no gradient.
__global__ void __launch_bounds__(128) k_prop_mdn(const float *__restrict__ out, uint32_t ldo,
                                                  const float *__restrict__ y, const float *__restrict__ w,
                                                  uint32_t B, uint32_t DY, const float *__restrict__ inv_wsum,
                                                  bf16 *__restrict__ dout, float *__restrict__ loss_rows) {
  static_assert(kPropG == 16, "one half-warp lane per component");
  const uint32_t lane = threadIdx.x & 31u, gk = lane & 15u;
  const uint32_t i = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2u + (lane >> 4);
  const bool live = i < B;
  const uint32_t ii = live ? i : 0u;  // every lane takes part in the shuffles
  const float *o = out + (size_t)ii * ldo;
  const float *yi = y + (size_t)ii * DY;
  const float logit = o[gk];
  float lmax = logit;
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, off));
  float lsum = expf(logit - lmax);
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  const float lse_logits = lmax + logf(lsum);
  float ll = 0.0f;
  for (uint32_t dd = 0; dd < DY; dd++) {
    const float mu = o[kPropG + gk * DY + dd];
    const float s = fminf(fmaxf(o[kPropG + kPropG * DY + gk * DY + dd], kPropSMin), kPropSMax);
    const float q = (yi[dd] - mu) * expf(-s);
    ll += -0.5f * q * q - s - 0.91893853320467274f;
  }
  const float a = logit - lse_logits + ll;
  float amax = a;
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
  float asum = expf(a - amax);
#pragma unroll
  for (int off = 8; off > 0; off >>= 1) asum += __shfl_xor_sync(0xffffffffu, asum, off);
  if (!live) return;
  const float lse = amax + logf(asum);
  const float ws = (w ? w[i] : 1.0f) * inv_wsum[0];
  if (gk == 0) loss_rows[i] = -lse * ws;
  bf16 *d = dout + (size_t)i * ldo;
  const float r = expf(a - lse), pi = expf(logit - lse_logits);
  d[gk] = __float2bfloat16(ws * (pi - r));
  for (uint32_t dd = 0; dd < DY; dd++) {
    const float mu = o[kPropG + gk * DY + dd];
    const float sraw = o[kPropG + kPropG * DY + gk * DY + dd];
    const float s = fminf(fmaxf(sraw, kPropSMin), kPropSMax);
    const float inv = expf(-s), q = (yi[dd] - mu) * inv;
    d[kPropG + gk * DY + dd] = __float2bfloat16(-ws * r * q * inv);
    const bool grad_s = sraw > kPropSMin && sraw < kPropSMax;
    d[kPropG + kPropG * DY + gk * DY + dd] = __float2bfloat16(grad_s ? -ws * r * (q * q - 1.0f) : 0.0f);
  }
  for (uint32_t j = (uint32_t)kPropG * (1u + 2u * DY) + gk; j < ldo; j += 16u) d[j] = __float2bfloat16(0.0f);
}

// Sums the split partials of every parameter in split order (the gradient).
__global__ void k_prop_grad_sum(const float *__restrict__ part, uint64_t P, float *__restrict__ grad) {
  const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float g = 0.0f;
  for (int s = 0; s < kSplits; s++) g += part[(uint64_t)s * P + p];
  grad[p] = g;
}

// Adam on the FP32 master parameters; the step count lives on the device so
// that one captured training step can be replayed.
__global__ void k_prop_adam(const float *__restrict__ part, uint64_t P, float *__restrict__ w, float *__restrict__ m,
                            float *__restrict__ v, bf16 *__restrict__ wb, const uint32_t *__restrict__ step, float lr) {
  const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float g = 0.0f;
  for (int s = 0; s < kSplits; s++) g += part[(uint64_t)s * P + p];
  const float b1 = 0.9f, b2 = 0.999f;
  const float t = (float)(step[0] + 1u);  // this step's number (the loss kernel advances the counter)
  const float mm = b1 * m[p] + (1.0f - b1) * g, vv = b2 * v[p] + (1.0f - b2) * g * g;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.0f - powf(b1, t)), vh = vv / (1.0f - powf(b2, t));
  const float nw = w[p] - lr * mh / (sqrtf(vh) + 1e-8f);
  w[p] = nw;
  wb[p] = __float2bfloat16(nw);
}

__global__ void k_prop_to_bf16(const float *__restrict__ x, uint64_t n, bf16 *__restrict__ y) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// The loss of one step: sum of the rows' weighted losses, in a fixed order;
// the last kernel of a step, it advances the step counter.
__global__ void __launch_bounds__(256) k_prop_loss(const float *__restrict__ rows, uint32_t B,
                                                   uint32_t *__restrict__ step, float *__restrict__ hist,
                                                   uint32_t hist_len) {
  __shared__ float s[256];
  float a = 0.0f;
  for (uint32_t i = threadIdx.x; i < B; i += 256) a += rows[i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const uint32_t t = step[0];
    if (t < hist_len) hist[t] = s[0];
    step[0] = t + 1u;
  }
}

// Network inputs and targets of the records (thread per record).
__global__ void k_prop_records(const pd_record *__restrict__ rec, uint32_t n, uint32_t K, uint32_t IN, uint32_t D,
                               PropSrc norm, bf16 *__restrict__ x, float *__restrict__ y, float *__restrict__ w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const pd_record &r = rec[i];
  for (uint32_t j = 0; j < IN; j++)
    x[(size_t)i * IN + j] = __float2bfloat16(prop_input(j, r.depth, r.count, r.class_count, K));
  for (uint32_t d = 0; d <= D; d++) {
    const float v = d < D ? (float)r.feat[d] : (float)r.thr;
    y[(size_t)i * (D + 1) + d] = norm.span[d] > 0.0f ? 2.0f * (v - norm.lo[d]) / norm.span[d] - 1.0f : 0.0f;
  }
  w[i] = 1.0f;
}

// The batch of one step: rows drawn uniformly from the records by a hash of
// (seed, step, row).
__global__ void k_prop_gather(const bf16 *__restrict__ rx, const float *__restrict__ ry, const float *__restrict__ rw,
                              uint32_t n, uint32_t IN, uint32_t DY, uint32_t B, uint64_t seed,
                              const uint32_t *__restrict__ step, bf16 *__restrict__ x, float *__restrict__ y,
                              float *__restrict__ w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const uint32_t k = (uint32_t)(prop_mix(seed ^ prop_mix(((uint64_t)(step[0] + 1u) << 32) | i)) % n);
  for (uint32_t j = 0; j < IN; j++) x[(size_t)i * IN + j] = rx[(size_t)k * IN + j];
  for (uint32_t d = 0; d < DY; d++) y[(size_t)i * DY + d] = ry[(size_t)k * DY + d];
  w[i] = rw[k];
}

// Inputs of the frontier nodes of a slice from their class totals.
__global__ void k_prop_node_inputs(const uint32_t *__restrict__ ctot, uint32_t n, uint32_t K, uint32_t IN,
                                   uint32_t depth, bf16 *__restrict__ x) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t count = 0;
  for (uint32_t l = 0; l < K; l++) count += ctot[(size_t)i * K + l];
  for (uint32_t j = 0; j < IN; j++)
    x[(size_t)i * IN + j] = __float2bfloat16(prop_input(j, depth, count, ctot + (size_t)i * K, K));
}

}  // namespace pd

using namespace pd;

struct pd_proposer {
  pd_ctx *ctx = nullptr;
  uint32_t K = 0, D = 0, DY = 0, IN = 0, OUT = 0;
  uint64_t seed = 0;
  PropSrc norm{};  // value ranges of the drawn dimensions
  uint64_t P = 0;
  uint64_t off_w[4] = {}, off_b[4] = {};
  uint32_t din[4] = {}, dout[4] = {};
  DevBuf master, m, v, wb, part, grad;
  // activations and gradients of a batch of up to `rows` rows
  uint32_t rows = 0;
  DevBuf x, z[3], act[3], out, dout_b, dz[2], y, w, loss_rows;
  DevBuf wsum;  // 1 / sum of the batch weights
  DevBuf step, loss_hist;
  DevBuf rec, rec_x, rec_y, rec_w;
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_rows = 0, graph_n = 0;
  float graph_lr = 0.0f;
  ~pd_proposer() {
    if (graph) cudaGraphExecDestroy(graph);
    DevBuf *bufs[] = {&master, &m, &v, &wb, &part, &grad, &x, &z[0], &z[1], &z[2], &act[0], &act[1], &act[2],
                      &out, &dout_b, &dz[0], &dz[1], &y, &w, &loss_rows, &wsum, &step, &loss_hist, &rec, &rec_x,
                      &rec_y, &rec_w};
    for (DevBuf *b : bufs) b->release();
  }
};

namespace pd {

static int prop_ensure_rows(pd_proposer *p, uint32_t rows) {
  if (rows <= p->rows) return PD_OK;
  const uint32_t H = kPropH;
  PD_TRY(p->x.ensure((size_t)rows * p->IN * 2));
  for (int l = 0; l < 3; l++) {
    PD_TRY(p->z[l].ensure((size_t)rows * H * 4));
    PD_TRY(p->act[l].ensure((size_t)rows * H * 2));
  }
  PD_TRY(p->out.ensure((size_t)rows * p->OUT * 4));
  PD_TRY(p->dout_b.ensure((size_t)rows * p->OUT * 2));
  for (int l = 0; l < 2; l++) PD_TRY(p->dz[l].ensure((size_t)rows * H * 2));
  PD_TRY(p->y.ensure((size_t)rows * p->DY * 4));
  PD_TRY(p->w.ensure((size_t)rows * 4));
  PD_TRY(p->loss_rows.ensure((size_t)rows * 4));
  p->rows = rows;
  if (p->graph) {
    cudaGraphExecDestroy(p->graph);
    p->graph = nullptr;
  }
  return PD_OK;
}

template <int EPI>
static int gemm(cudaStream_t st, GemmArgs g, int splits = 1) {
  auto al16 = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
  // along k: every row start and every k-range start (k0 steps by 32 from a split start) is a multiple of 8
  const bool kfit = g.K % 8 == 0 && g.k_split % 8 == 0;
  g.vec_a = al16(g.A) && ((g.a_k == 1 && g.a_i % 8 == 0 && kfit) || (g.a_i == 1 && g.a_k % 8 == 0 && g.M % 8 == 0));
  g.vec_b = al16(g.B) && ((g.b_k == 1 && g.b_j % 8 == 0 && kfit) || (g.b_j == 1 && g.b_k % 8 == 0 && g.N % 8 == 0));
  const int krange = std::min(g.K, g.k_split);
  g.kstage = std::min(kGemmMaxStage, (krange + 31) / 32 * 32);
  const size_t smem = (size_t)(kGemmTM + kGemmTN) * (g.kstage + kGemmPad) * sizeof(bf16);
  const dim3 grid((unsigned)((g.N + kGemmTN - 1) / kGemmTN), (unsigned)((g.M + kGemmTM - 1) / kGemmTM),
                  (unsigned)splits);
  k_prop_gemm<EPI><<<grid, kGemmThreads, smem, st>>>(g);
  PD_CUDA(cudaGetLastError());
  return PD_OK;
}

// Opts the product kernels into the shared memory of a full stage (done when a
// network is created on a device, before any capture of a training step).
static int gemm_setup() {
  const int bytes = (int)((kGemmTM + kGemmTN) * (kGemmMaxStage + kGemmPad) * sizeof(bf16));
  PD_CUDA(cudaFuncSetAttribute(k_prop_gemm<EPI_GELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  PD_CUDA(cudaFuncSetAttribute(k_prop_gemm<EPI_LINEAR>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  PD_CUDA(cudaFuncSetAttribute(k_prop_gemm<EPI_DGELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  PD_CUDA(cudaFuncSetAttribute(k_prop_gemm<EPI_PARTIAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  return PD_OK;
}

static GemmArgs gargs(const bf16 *A, int64_t a_i, int64_t a_k, const bf16 *B, int64_t b_k, int64_t b_j, int M, int N,
                      int K) {
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.A = A;
  g.a_i = a_i;
  g.a_k = a_k;
  g.B = B;
  g.b_k = b_k;
  g.b_j = b_j;
  g.M = M;
  g.N = N;
  g.K = K;
  g.k_split = K;
  return g;
}

// Forward pass of n rows of p->x into p->out (and z / act for the backward pass).
static int prop_forward(pd_proposer *p, uint32_t n, cudaStream_t st) {
  const bf16 *wb = p->wb.as<bf16>();
  const float *wm = p->master.as<float>();
  const bf16 *in = p->x.as<bf16>();
  for (int l = 0; l < 4; l++) {
    const uint32_t di = p->din[l], dn = p->dout[l];
    // out(i, j) = sum_k in(i, k) W[j][k]
    GemmArgs g = gargs(in, di, 1, wb + p->off_w[l], 1, di, (int)n, (int)dn, (int)di);
    g.bias = wm + p->off_b[l];
    g.ldo = dn;
    if (l < 3) {
      g.outf = p->z[l].as<float>();
      g.outb = p->act[l].as<bf16>();
      PD_TRY(gemm<EPI_GELU>(st, g));
      in = p->act[l].as<bf16>();
    } else {
      g.outf = p->out.as<float>();
      PD_TRY(gemm<EPI_LINEAR>(st, g));
    }
  }
  return PD_OK;
}

// Backward pass of a batch of n rows (after prop_forward and k_prop_mdn wrote
// dout_b): weight and bias gradient partials into p->part.
static int prop_backward(pd_proposer *p, uint32_t n, cudaStream_t st) {
  const bf16 *wb = p->wb.as<bf16>();
  float *part = p->part.as<float>();
  const uint32_t per = (n + kSplits - 1) / kSplits;
  const bf16 *d = p->dout_b.as<bf16>();  // gradient w.r.t. the output of layer l
  int cur = 0;
  for (int l = 3; l >= 0; l--) {
    const uint32_t di = p->din[l], dn = p->dout[l];
    const bf16 *in = l == 0 ? p->x.as<bf16>() : p->act[l - 1].as<bf16>();
    // dW[j][k] = sum_i d(i, j) in(i, k): A(j, i) = d[i * dn + j], B(i, k) = in[i * di + k]
    GemmArgs g = gargs(d, 1, dn, in, di, 1, (int)dn, (int)di, (int)n);
    g.k_split = (int)per;
    g.outf = part + p->off_w[l];
    g.ldo = di;
    g.split_stride = (int64_t)p->P;
    g.bias_part = part + p->off_b[l];  // db[j] = sum_i d(i, j), from the same staged tiles
    PD_TRY(gemm<EPI_PARTIAL>(st, g, kSplits));
    if (l == 0) break;
    // d(in)(i, k) = sum_j d(i, j) W[j][k], times GELU'(z of layer l - 1)
    GemmArgs h = gargs(d, dn, 1, wb + p->off_w[l], di, 1, (int)n, (int)di, (int)dn);
    h.zin = p->z[l - 1].as<float>();
    h.outb = p->dz[cur].as<bf16>();
    h.ldo = di;
    PD_TRY(gemm<EPI_DGELU>(st, h));
    d = p->dz[cur].as<bf16>();
    cur ^= 1;
  }
  return PD_OK;
}

// Loss and gradient partials of the batch already in x / y / w.
static int prop_loss_grad(pd_proposer *p, uint32_t n, cudaStream_t st) {
  PD_TRY(prop_forward(p, n, st));
  k_prop_mdn<<<(n + 7) / 8, 128, 0, st>>>(p->out.as<float>(), p->OUT, p->y.as<float>(), p->w.as<float>(), n,
                                          p->DY, p->wsum.as<float>(), p->dout_b.as<bf16>(),
                                          p->loss_rows.as<float>());
  PD_CUDA(cudaGetLastError());
  return prop_backward(p, n, st);
}

int proposer_infer(pd_proposer *p, const uint32_t *d_ctot, uint32_t n, uint32_t depth, uint32_t n_prop, PropSrc *src) {
  cudaStream_t st = p->ctx->stream;
  PD_TRY(prop_ensure_rows(p, std::max<uint32_t>(n, 64)));
  if (n) {
    k_prop_node_inputs<<<(n + 127) / 128, 128, 0, st>>>(d_ctot, n, p->K, p->IN, depth, p->x.as<bf16>());
    PD_CUDA(cudaGetLastError());
    PD_TRY(prop_forward(p, n, st));
    p->ctx->launches += 5;
  }
  *src = p->norm;
  src->out = p->out.as<float>();
  src->ldo = p->OUT;
  src->DY = p->DY;
  src->n_prop = n_prop;
  src->seed = p->seed;
  return PD_OK;
}

// Deterministic initial parameters: Glorot-uniform weights from a hash of
// (seed, index); zero biases except the head's means (spread over [-0.8, 0.8])
// and log-sds (log 0.5).
static void prop_init(pd_proposer *p, std::vector<float> &h) {
  h.assign(p->P, 0.0f);
  for (int l = 0; l < 4; l++) {
    const float a = std::sqrt(6.0f / (float)(p->din[l] + p->dout[l])) * (l == 3 ? 0.1f : 1.0f);
    for (uint64_t k = 0; k < (uint64_t)p->din[l] * p->dout[l]; k++) {
      const float u = prop_unit(prop_mix(p->seed ^ prop_mix(((uint64_t)l << 56) | k)));
      h[p->off_w[l] + k] = (2.0f * u - 1.0f) * a;
    }
  }
  float *bo = h.data() + p->off_b[3];
  for (uint32_t gk = 0; gk < (uint32_t)kPropG; gk++)
    for (uint32_t d = 0; d < p->DY; d++) {
      const float u = prop_unit(prop_mix(p->seed ^ prop_mix((7ull << 56) | (gk * 64 + d))));
      bo[kPropG + gk * p->DY + d] = (2.0f * u - 1.0f) * 0.8f;
      bo[kPropG + kPropG * p->DY + gk * p->DY + d] = std::log(0.5f);
    }
}

static int prop_upload_params(pd_proposer *p, const float *h) {
  cudaStream_t st = p->ctx->stream;
  PD_CUDA(cudaMemcpyAsync(p->master.ptr, h, p->P * 4, cudaMemcpyHostToDevice, st));
  PD_CUDA(cudaMemsetAsync(p->m.ptr, 0, p->P * 4, st));
  PD_CUDA(cudaMemsetAsync(p->v.ptr, 0, p->P * 4, st));
  k_prop_to_bf16<<<(unsigned)((p->P + 255) / 256), 256, 0, st>>>(p->master.as<float>(), p->P, p->wb.as<bf16>());
  PD_CUDA(cudaGetLastError());
  PD_CUDA(cudaStreamSynchronize(st));
  return PD_OK;
}

static int check_proposer(const pd_proposer *p) {
  PD_CHECK(p && p->ctx, PD_ERR_INVALID, "null proposer");
  PD_CUDA(cudaSetDevice(p->ctx->device));
  return PD_OK;
}

}  // namespace pd

extern "C" int pd_proposer_create(pd_ctx *ctx, const pd_train_params *bounds, uint64_t seed, pd_proposer **out) {
  PD_CHECK(ctx && bounds && out, PD_ERR_INVALID, "null argument");
  PD_CUDA(cudaSetDevice(ctx->device));
  auto *p = new pd_proposer();
  p->ctx = ctx;
  p->K = (uint32_t)ctx->cfg.n_classes;
  p->D = (uint32_t)ctx->cfg.feat_dim;
  p->DY = p->D + 1;
  p->IN = prop_in_dim(p->K);
  p->OUT = prop_out_dim(p->DY);
  p->seed = seed;
  memset(&p->norm, 0, sizeof(p->norm));
  for (uint32_t d = 0; d < p->D; d++) {
    p->norm.lo[d] = (float)bounds->feat_low[d];
    p->norm.span[d] = (float)((int64_t)bounds->feat_up[d] - bounds->feat_low[d]);
  }
  p->norm.lo[p->D] = (float)bounds->thr_low;
  p->norm.span[p->D] = (float)((int64_t)bounds->thr_up - bounds->thr_low);
  const uint32_t H = kPropH;
  const uint32_t din[4] = {p->IN, H, H, H}, dn[4] = {H, H, H, p->OUT};
  uint64_t o = 0;
  for (int l = 0; l < 4; l++) {
    p->din[l] = din[l];
    p->dout[l] = dn[l];
    p->off_w[l] = o;
    o += (uint64_t)din[l] * dn[l];
    p->off_b[l] = o;
    o += dn[l];
  }
  p->P = o;
  int rc = gemm_setup();
  if (rc == PD_OK) rc = p->master.ensure(p->P * 4);
  if (rc == PD_OK) rc = p->m.ensure(p->P * 4);
  if (rc == PD_OK) rc = p->v.ensure(p->P * 4);
  if (rc == PD_OK) rc = p->wb.ensure(p->P * 2);
  if (rc == PD_OK) rc = p->part.ensure((size_t)kSplits * p->P * 4);
  if (rc == PD_OK) rc = p->grad.ensure(p->P * 4);
  if (rc == PD_OK) rc = p->step.ensure(16);
  if (rc == PD_OK) rc = p->wsum.ensure(16);
  if (rc == PD_OK) {
    std::vector<float> h;
    prop_init(p, h);
    rc = prop_upload_params(p, h.data());
  }
  if (rc != PD_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return PD_OK;
}

extern "C" int pd_proposer_destroy(pd_proposer *p) {
  if (!p) return PD_OK;
  cudaSetDevice(p->ctx->device);
  delete p;
  return PD_OK;
}

extern "C" int pd_proposer_dims(pd_proposer *p, uint32_t dims[6], uint64_t *n_params) {
  PD_TRY(check_proposer(p));
  if (dims) {
    dims[0] = p->IN;
    dims[1] = kPropH;
    dims[2] = kPropLayers;
    dims[3] = p->OUT;
    dims[4] = kPropG;
    dims[5] = p->DY;
  }
  if (n_params) *n_params = p->P;
  return PD_OK;
}

extern "C" int pd_proposer_get_params(pd_proposer *p, float *out) {
  PD_TRY(check_proposer(p));
  PD_CHECK(out, PD_ERR_INVALID, "null argument");
  PD_CUDA(cudaMemcpyAsync(out, p->master.ptr, p->P * 4, cudaMemcpyDeviceToHost, p->ctx->stream));
  PD_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return PD_OK;
}

extern "C" int pd_proposer_set_params(pd_proposer *p, const float *in) {
  PD_TRY(check_proposer(p));
  PD_CHECK(in, PD_ERR_INVALID, "null argument");
  return prop_upload_params(p, in);
}

extern "C" int pd_proposer_forward(pd_proposer *p, const float *x, uint32_t n, float *out) {
  PD_TRY(check_proposer(p));
  PD_CHECK(x && out, PD_ERR_INVALID, "null argument");
  if (!n) return PD_OK;
  cudaStream_t st = p->ctx->stream;
  PD_TRY(prop_ensure_rows(p, n));
  PD_TRY(p->grad.ensure(std::max<size_t>(p->P, (size_t)n * p->IN) * 4));
  PD_CUDA(cudaMemcpyAsync(p->grad.ptr, x, (size_t)n * p->IN * 4, cudaMemcpyHostToDevice, st));
  k_prop_to_bf16<<<(unsigned)(((uint64_t)n * p->IN + 255) / 256), 256, 0, st>>>(p->grad.as<float>(),
                                                                                (uint64_t)n * p->IN, p->x.as<bf16>());
  PD_CUDA(cudaGetLastError());
  PD_TRY(prop_forward(p, n, st));
  PD_CUDA(cudaMemcpyAsync(out, p->out.ptr, (size_t)n * p->OUT * 4, cudaMemcpyDeviceToHost, st));
  PD_CUDA(cudaStreamSynchronize(st));
  return PD_OK;
}

extern "C" int pd_proposer_loss_grad(pd_proposer *p, const float *x, const float *y, const float *w, uint32_t n,
                                     float *loss, float *grad) {
  PD_TRY(check_proposer(p));
  PD_CHECK(x && y && loss && grad && n, PD_ERR_INVALID, "null argument or no rows");
  cudaStream_t st = p->ctx->stream;
  PD_TRY(prop_ensure_rows(p, n));
  PD_TRY(p->grad.ensure(std::max<size_t>(p->P, (size_t)n * p->IN) * 4));
  PD_CUDA(cudaMemcpyAsync(p->grad.ptr, x, (size_t)n * p->IN * 4, cudaMemcpyHostToDevice, st));
  k_prop_to_bf16<<<(unsigned)(((uint64_t)n * p->IN + 255) / 256), 256, 0, st>>>(p->grad.as<float>(),
                                                                                (uint64_t)n * p->IN, p->x.as<bf16>());
  PD_CUDA(cudaGetLastError());
  PD_CUDA(cudaMemcpyAsync(p->y.ptr, y, (size_t)n * p->DY * 4, cudaMemcpyHostToDevice, st));
  std::vector<float> hw(n, 1.0f);
  if (w) memcpy(hw.data(), w, (size_t)n * 4);
  double ws = 0.0;
  for (float v : hw) ws += v;
  PD_CHECK(ws > 0.0, PD_ERR_INVALID, "row weights sum to zero");
  const float inv = (float)(1.0 / ws);
  PD_CUDA(cudaMemcpyAsync(p->w.ptr, hw.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
  PD_CUDA(cudaMemcpyAsync(p->wsum.ptr, &inv, 4, cudaMemcpyHostToDevice, st));
  PD_TRY(prop_loss_grad(p, n, st));
  k_prop_grad_sum<<<(unsigned)((p->P + 255) / 256), 256, 0, st>>>(p->part.as<float>(), p->P, p->grad.as<float>());
  PD_CUDA(cudaGetLastError());
  std::vector<float> rows(n);
  PD_CUDA(cudaMemcpyAsync(rows.data(), p->loss_rows.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  PD_CUDA(cudaMemcpyAsync(grad, p->grad.ptr, p->P * 4, cudaMemcpyDeviceToHost, st));
  PD_CUDA(cudaStreamSynchronize(st));
  double l = 0.0;
  for (float r : rows) l += r;
  *loss = (float)l;
  return PD_OK;
}

extern "C" int pd_proposer_fit(pd_proposer *p, const pd_record *records, uint64_t n, uint32_t steps, uint32_t batch,
                               float lr, float *loss_out, float *ms_out) {
  PD_TRY(check_proposer(p));
  PD_CHECK(records && n >= 1 && n < (1ull << 31), PD_ERR_INVALID, "need between 1 and 2^31-1 records");
  PD_CHECK(batch >= 64 && batch <= (1u << 20), PD_ERR_INVALID, "batch %u outside [64, 2^20]", batch);
  PD_CHECK(steps >= 1, PD_ERR_INVALID, "steps must be >= 1");
  cudaStream_t st = p->ctx->stream;
  PD_TRY(prop_ensure_rows(p, batch));
  PD_TRY(p->rec.ensure(n * sizeof(pd_record)));
  PD_TRY(p->rec_x.ensure(n * p->IN * 2));
  PD_TRY(p->rec_y.ensure(n * p->DY * 4));
  PD_TRY(p->rec_w.ensure(n * 4));
  PD_TRY(p->loss_hist.ensure((size_t)steps * 4));
  cudaEvent_t e0 = p->ctx->ev[6], e1 = p->ctx->ev[7];
  PD_CUDA(cudaEventRecord(e0, st));
  PD_CUDA(cudaMemcpyAsync(p->rec.ptr, records, n * sizeof(pd_record), cudaMemcpyHostToDevice, st));
  k_prop_records<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(p->rec.as<pd_record>(), (uint32_t)n, p->K, p->IN, p->D,
                                                              p->norm, p->rec_x.as<bf16>(), p->rec_y.as<float>(),
                                                              p->rec_w.as<float>());
  PD_CUDA(cudaGetLastError());
  const float inv = 1.0f / (float)batch;
  PD_CUDA(cudaMemcpyAsync(p->wsum.ptr, &inv, 4, cudaMemcpyHostToDevice, st));
  PD_CUDA(cudaMemsetAsync(p->step.ptr, 0, 4, st));
  PD_CUDA(cudaMemsetAsync(p->loss_hist.ptr, 0, (size_t)steps * 4, st));
  // one training step, captured once per (batch, record count, rate) and replayed
  if (!p->graph || p->graph_rows != batch || p->graph_n != (uint32_t)n || p->graph_lr != lr) {
    if (p->graph) {
      cudaGraphExecDestroy(p->graph);
      p->graph = nullptr;
    }
    PD_CUDA(cudaStreamSynchronize(st));
    cudaGraph_t g = nullptr;
    PD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = PD_OK;
    k_prop_gather<<<(batch + 127) / 128, 128, 0, st>>>(p->rec_x.as<bf16>(), p->rec_y.as<float>(),
                                                       p->rec_w.as<float>(), (uint32_t)n, p->IN, p->DY, batch,
                                                       p->seed, p->step.as<uint32_t>(), p->x.as<bf16>(),
                                                       p->y.as<float>(), p->w.as<float>());
    if (rc == PD_OK) rc = prop_loss_grad(p, batch, st);
    k_prop_adam<<<(unsigned)((p->P + 255) / 256), 256, 0, st>>>(p->part.as<float>(), p->P, p->master.as<float>(),
                                                              p->m.as<float>(), p->v.as<float>(), p->wb.as<bf16>(),
                                                              p->step.as<uint32_t>(), lr);
    k_prop_loss<<<1, 256, 0, st>>>(p->loss_rows.as<float>(), batch, p->step.as<uint32_t>(),
                                   p->loss_hist.as<float>(), steps);
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    PD_TRY(rc);
    PD_CUDA(ce);
    const cudaError_t ie = cudaGraphInstantiate(&p->graph, g, 0);
    cudaGraphDestroy(g);
    PD_CUDA(ie);
    p->graph_rows = batch;
    p->graph_n = (uint32_t)n;
    p->graph_lr = lr;
  }
  for (uint32_t s = 0; s < steps; s++) PD_CUDA(cudaGraphLaunch(p->graph, st));
  PD_CUDA(cudaEventRecord(e1, st));
  PD_CUDA(cudaStreamSynchronize(st));
  if (loss_out) {
    PD_CUDA(cudaMemcpy(loss_out, p->loss_hist.ptr, (size_t)steps * 4, cudaMemcpyDeviceToHost));
  }
  if (ms_out) {
    float ms = 0.f;
    PD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    *ms_out = ms;
  }
  p->ctx->launches += (uint64_t)steps * 15;  // gather, 4 forward and 7 backward products, loss, Adam, loss sum
  return PD_OK;
}
