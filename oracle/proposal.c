/*
 * TEST INFRASTRUCTURE ONLY: a CPU restatement of the proposal network of the
 * library's learned candidate proposals (padenti_gb300/csrc/pd_propose.cu; no
 * counterpart in the reference), to check its forward pass and its gradients.
 *
 * Same parameter layout (W1 [H][IN], b1, W2 [H][H], b2, W3 [H][H], b3,
 * Wo [OUT][H], bo), GELU (erf form), mixture negative log-likelihood with the
 * log-sd clamp [-6, 3], weighted mean over the rows.  Arithmetic in double.
 * With bf16 = 1 the values the GPU stores as BF16 are rounded to BF16
 * (round-to-nearest-even) at the same points: the inputs, the weights, every
 * hidden activation, the output gradient and every hidden-layer gradient; with
 * bf16 = 0 nothing is rounded (the exact function, for finite differences).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "padenti_oracle.h"

#define PR_G 16
#define PR_SMIN (-6.0)
#define PR_SMAX 3.0

static double pr_bf16(double v, int on) {
  if (!on) return v;
  float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return v; /* inf / nan unchanged */
  u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
  memcpy(&f, &u, 4);
  return (double)f;
}
static double pr_gelu(double z) { return 0.5 * z * (1.0 + erf(z * 0.70710678118654752)); }
static double pr_dgelu(double z) {
  return 0.5 * (1.0 + erf(z * 0.70710678118654752)) + z * exp(-0.5 * z * z) * 0.39894228040143268;
}

typedef struct {
  uint32_t in[4], out[4];
  uint64_t ow[4], ob[4], P;
} pr_layout;

static void pr_layout_of(uint32_t IN, uint32_t H, uint32_t OUT, pr_layout *L) {
  const uint32_t din[4] = {IN, H, H, H}, dn[4] = {H, H, H, OUT};
  uint64_t o = 0;
  for (int l = 0; l < 4; l++) {
    L->in[l] = din[l];
    L->out[l] = dn[l];
    L->ow[l] = o;
    o += (uint64_t)din[l] * dn[l];
    L->ob[l] = o;
    o += dn[l];
  }
  L->P = o;
}

/* Forward of n rows; z[l] (pre-activations) and a[l] (activations, a[0] = x)
 * are kept for the backward pass when non-NULL. */
static void pr_forward(const float *params, const pr_layout *L, const float *x, uint32_t n, int bf16, double *out,
                       double **z, double **a) {
  double *cur = (double *)malloc(sizeof(double) * (size_t)n * L->in[0]);
  for (size_t i = 0; i < (size_t)n * L->in[0]; i++) cur[i] = pr_bf16(x[i], bf16);
  if (a) memcpy(a[0], cur, sizeof(double) * (size_t)n * L->in[0]);
  for (int l = 0; l < 4; l++) {
    const uint32_t di = L->in[l], dn = L->out[l];
    double *nx = (double *)malloc(sizeof(double) * (size_t)n * dn);
    for (uint32_t i = 0; i < n; i++)
      for (uint32_t j = 0; j < dn; j++) {
        double s = 0.0;
        for (uint32_t k = 0; k < di; k++)
          s += cur[(size_t)i * di + k] * pr_bf16(params[L->ow[l] + (size_t)j * di + k], bf16);
        const double zz = s + params[L->ob[l] + j];
        if (l < 3) {
          if (z) z[l][(size_t)i * dn + j] = zz;
          nx[(size_t)i * dn + j] = pr_bf16(pr_gelu(zz), bf16);
        } else {
          out[(size_t)i * dn + j] = zz;
        }
      }
    free(cur);
    cur = nx;
    if (l < 3 && a) memcpy(a[l + 1], cur, sizeof(double) * (size_t)n * dn);
  }
  free(cur);
}

int or_prop_forward(const float *params, uint32_t IN, uint32_t H, uint32_t OUT, const float *x, uint32_t n,
                    int bf16, float *out) {
  pr_layout L;
  pr_layout_of(IN, H, OUT, &L);
  double *o = (double *)malloc(sizeof(double) * (size_t)n * OUT);
  pr_forward(params, &L, x, n, bf16, o, NULL, NULL);
  for (size_t i = 0; i < (size_t)n * OUT; i++) out[i] = (float)o[i];
  free(o);
  return 0;
}

int or_prop_loss_grad(const float *params, uint32_t IN, uint32_t H, uint32_t OUT, uint32_t DY, const float *x,
                      const float *y, const float *w, uint32_t n, int bf16, double *loss, double *grad) {
  pr_layout L;
  pr_layout_of(IN, H, OUT, &L);
  double *z[3], *a[4];
  for (int l = 0; l < 3; l++) z[l] = (double *)malloc(sizeof(double) * (size_t)n * H);
  a[0] = (double *)malloc(sizeof(double) * (size_t)n * IN);
  for (int l = 1; l < 4; l++) a[l] = (double *)malloc(sizeof(double) * (size_t)n * H);
  double *o = (double *)malloc(sizeof(double) * (size_t)n * OUT);
  pr_forward(params, &L, x, n, bf16, o, z, a);
  double wsum = 0.0;
  for (uint32_t i = 0; i < n; i++) wsum += w ? w[i] : 1.0;
  double *d = (double *)calloc((size_t)n * OUT, sizeof(double));
  double tot = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    const double *oi = o + (size_t)i * OUT;
    const double ws = (w ? w[i] : 1.0) / wsum;
    double lmax = oi[0];
    for (int g = 1; g < PR_G; g++) lmax = oi[g] > lmax ? oi[g] : lmax;
    double ls = 0.0;
    for (int g = 0; g < PR_G; g++) ls += exp(oi[g] - lmax);
    const double lse_l = lmax + log(ls);
    double av[PR_G], amax = -INFINITY;
    for (int g = 0; g < PR_G; g++) {
      double ll = 0.0;
      for (uint32_t dd = 0; dd < DY; dd++) {
        const double mu = oi[PR_G + g * DY + dd];
        double s = oi[PR_G + PR_G * DY + g * DY + dd];
        s = s < PR_SMIN ? PR_SMIN : (s > PR_SMAX ? PR_SMAX : s);
        const double q = (y[(size_t)i * DY + dd] - mu) * exp(-s);
        ll += -0.5 * q * q - s - 0.91893853320467274;
      }
      av[g] = oi[g] - lse_l + ll;
      if (av[g] > amax) amax = av[g];
    }
    double as = 0.0;
    for (int g = 0; g < PR_G; g++) as += exp(av[g] - amax);
    const double lse = amax + log(as);
    tot += -lse * ws;
    double *di = d + (size_t)i * OUT;
    for (int g = 0; g < PR_G; g++) {
      const double r = exp(av[g] - lse), pi = exp(oi[g] - lse_l);
      di[g] = pr_bf16(ws * (pi - r), bf16);
      for (uint32_t dd = 0; dd < DY; dd++) {
        const double mu = oi[PR_G + g * DY + dd];
        const double sraw = oi[PR_G + PR_G * DY + g * DY + dd];
        const double s = sraw < PR_SMIN ? PR_SMIN : (sraw > PR_SMAX ? PR_SMAX : sraw);
        const double inv = exp(-s), q = (y[(size_t)i * DY + dd] - mu) * inv;
        di[PR_G + g * DY + dd] = pr_bf16(-ws * r * q * inv, bf16);
        const int live = sraw > PR_SMIN && sraw < PR_SMAX;
        di[PR_G + PR_G * DY + g * DY + dd] = pr_bf16(live ? -ws * r * (q * q - 1.0) : 0.0, bf16);
      }
    }
  }
  *loss = tot;
  memset(grad, 0, sizeof(double) * L.P);
  double *cur = d;
  for (int l = 3; l >= 0; l--) {
    const uint32_t di = L.in[l], dn = L.out[l];
    const double *in = a[l];
    for (uint32_t j = 0; j < dn; j++) {
      double bsum = 0.0;
      for (uint32_t i = 0; i < n; i++) bsum += cur[(size_t)i * dn + j];
      grad[L.ob[l] + j] = bsum;
      for (uint32_t k = 0; k < di; k++) {
        double s = 0.0;
        for (uint32_t i = 0; i < n; i++) s += cur[(size_t)i * dn + j] * in[(size_t)i * di + k];
        grad[L.ow[l] + (size_t)j * di + k] = s;
      }
    }
    if (l == 0) break;
    double *nx = (double *)malloc(sizeof(double) * (size_t)n * di);
    for (uint32_t i = 0; i < n; i++)
      for (uint32_t k = 0; k < di; k++) {
        double s = 0.0;
        for (uint32_t j = 0; j < dn; j++)
          s += cur[(size_t)i * dn + j] * pr_bf16(params[L.ow[l] + (size_t)j * di + k], bf16);
        nx[(size_t)i * di + k] = pr_bf16(s * pr_dgelu(z[l - 1][(size_t)i * di + k]), bf16);
      }
    if (cur != d) free(cur);
    cur = nx;
  }
  if (cur != d) free(cur);
  free(d);
  free(o);
  for (int l = 0; l < 3; l++) free(z[l]);
  for (int l = 0; l < 4; l++) free(a[l]);
  return 0;
}
