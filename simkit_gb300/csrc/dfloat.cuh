// Double-float arithmetic: a value hi + lo held as two FP32 numbers with
// |lo| <= ulp(hi) / 2, about 48 significant bits.  GB300's FP64 rate is a small
// fraction of its FP32 rate, so the force kernel of the mixed-precision stepper
// evaluates the stress in this form instead of FP64 (relative error of a few
// 1e-14 per operation, far below the 1e-6 residual the Newton loop resolves).
//
// The algorithms are the classical error-free transformations: Knuth's two-sum,
// Dekker's fast two-sum (|a| >= |b|), and the FMA form of the exact product
// (p = a b, e = fma(a, b, -p)), combined as in the double-double literature
// (Hida, Li and Bailey, "Library for double-double and quad-double arithmetic",
// 2000): the "accurate" addition and the product with cross terms.
#pragma once

#include <math.h>

#include "snh_math.cuh"

namespace skg {

struct DF {
  float hi, lo;
  DF() = default;
  SK_HD constexpr DF(float h, float l) : hi(h), lo(l) {}
  SK_HD DF(double x) : hi(float(x)), lo(float(x - double(float(x)))) {}
  SK_HD DF(int x) : hi(float(x)), lo(0.f) {}
  SK_HD double to_double() const { return double(hi) + double(lo); }
};

SK_HD void df_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
SK_HD void df_fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

SK_HD DF operator+(DF a, DF b) {
  float s1, s2, t1, t2;
  df_two_sum(a.hi, b.hi, s1, s2);
  df_two_sum(a.lo, b.lo, t1, t2);
  s2 += t1;
  df_fast_two_sum(s1, s2, s1, s2);
  s2 += t2;
  df_fast_two_sum(s1, s2, s1, s2);
  return DF(s1, s2);
}
SK_HD DF operator-(DF a) { return DF(-a.hi, -a.lo); }
SK_HD DF operator-(DF a, DF b) { return a + (-b); }
SK_HD DF operator*(DF a, DF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  float s, t;
  df_fast_two_sum(p, e, s, t);
  return DF(s, t);
}
// quotient by two correction steps of the FP32 quotient of the leading parts
SK_HD DF operator/(DF a, DF b) {
  const float q1 = a.hi / b.hi;
  DF r = a - DF(q1, 0.f) * b;
  const float q2 = r.hi / b.hi;
  r = r - DF(q2, 0.f) * b;
  const float q3 = r.hi / b.hi;
  float s, t;
  df_fast_two_sum(q1, q2, s, t);
  return DF(s, t) + DF(q3, 0.f);
}
SK_HD DF& operator+=(DF& a, DF b) { return a = a + b; }
SK_HD DF& operator-=(DF& a, DF b) { return a = a - b; }
SK_HD DF& operator*=(DF& a, DF b) { return a = a * b; }

}  // namespace skg
