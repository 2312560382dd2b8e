// Exact-reproducible log2 of integers for the split's FP64 recheck.
//
// The best split must be identical to the CPU oracle's, so the gain of a
// candidate is evaluated from integer counts with one table of log2(n) shared
// by both sides.  The table is computed in double-double arithmetic (Dekker's
// exact product with 27-bit splitting, Knuth's two-sum, and the Hida-Li-Bailey
// double-double add/mul/div), with ln(m) = 2 atanh((m-1)/(m+1)) and
// ln 2 = 2 atanh(1/3).  Only correctly rounded IEEE +,-,*,/ are used, in a fixed
// order, so every IEEE machine produces the same table bit for bit.
#pragma once

#include "pd_common.cuh"

namespace pd {

struct DD {
  double hi, lo;
};

PD_HD DD dd_two_sum(double a, double b) {
  const double s = dadd(a, b);
  const double bb = dsub(s, a);
  const double e = dadd(dsub(a, dsub(s, bb)), dsub(b, bb));
  return DD{s, e};
}
PD_HD DD dd_quick_two_sum(double a, double b) {
  const double s = dadd(a, b);
  const double e = dsub(b, dsub(s, a));
  return DD{s, e};
}
PD_HD void dd_split(double a, double &hi, double &lo) {
  const double t = dmul(134217729.0, a);
  hi = dsub(t, dsub(t, a));
  lo = dsub(a, hi);
}
PD_HD DD dd_two_prod(double a, double b) {
  const double p = dmul(a, b);
  double ah, al, bh, bl;
  dd_split(a, ah, al);
  dd_split(b, bh, bl);
  const double e = dadd(dadd(dadd(dsub(dmul(ah, bh), p), dmul(ah, bl)), dmul(al, bh)), dmul(al, bl));
  return DD{p, e};
}
PD_HD DD dd_add(DD a, DD b) {
  DD s = dd_two_sum(a.hi, b.hi);
  const DD t = dd_two_sum(a.lo, b.lo);
  s.lo = dadd(s.lo, t.hi);
  s = dd_quick_two_sum(s.hi, s.lo);
  s.lo = dadd(s.lo, t.lo);
  return dd_quick_two_sum(s.hi, s.lo);
}
PD_HD DD dd_mul(DD a, DD b) {
  DD p = dd_two_prod(a.hi, b.hi);
  p.lo = dadd(p.lo, dadd(dmul(a.hi, b.lo), dmul(a.lo, b.hi)));
  return dd_quick_two_sum(p.hi, p.lo);
}
PD_HD DD dd_mul_d(DD a, double b) {
  DD p = dd_two_prod(a.hi, b);
  p.lo = dadd(p.lo, dmul(a.lo, b));
  return dd_quick_two_sum(p.hi, p.lo);
}
PD_HD DD dd_div(DD a, DD b) {
  const double q1 = ddiv(a.hi, b.hi);
  DD r = dd_add(a, dd_mul_d(b, -q1));
  const double q2 = ddiv(r.hi, b.hi);
  r = dd_add(r, dd_mul_d(b, -q2));
  const double q3 = ddiv(r.hi, b.hi);
  const DD q = dd_quick_two_sum(q1, q2);
  return dd_add(q, DD{q3, 0.0});
}
// 2*(z + z^3/3 + z^5/5 + ...) with a fixed number of terms.
PD_HD DD dd_2atanh(DD z, int terms) {
  const DD z2 = dd_mul(z, z);
  DD term = z, sum = z;
  for (int k = 1; k <= terms; k++) {
    term = dd_mul(term, z2);
    sum = dd_add(sum, dd_div(term, DD{(double)(2 * k + 1), 0.0}));
  }
  return dd_mul_d(sum, 2.0);
}
PD_HD DD dd_inv_ln2() {
  const DD ln2 = dd_2atanh(dd_div(DD{1.0, 0.0}, DD{3.0, 0.0}), 40);
  return dd_div(DD{1.0, 0.0}, ln2);
}
PD_HD double dd_log2_u32(uint32_t n, DD inv_ln2) {
  if (n <= 1u) return 0.0;
  int e = 31;
  while (!((n >> e) & 1u)) e--;
  double m = ddiv((double)n, (double)(1u << e));  // exact, in [1,2)
  if (m > 1.4142135623730951) {
    m = dmul(m, 0.5);
    e += 1;
  }
  const DD num = DD{dsub(m, 1.0), 0.0};  // exact (Sterbenz)
  const DD den = dd_two_sum(m, 1.0);     // exact pair
  const DD z = dd_div(num, den);
  const DD ln_m = dd_2atanh(z, 24);
  const DD r = dd_add(DD{(double)e, 0.0}, dd_mul(ln_m, inv_ln2));
  return r.hi;
}

}  // namespace pd
