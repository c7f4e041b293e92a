// FP64 functions for GB300, whose FP64 pipe issues one warp instruction per
// ~20 SM cycles (about 1/64 of the FP32 rate): the parts that only need a
// few significant bits run on the FP32 pipe, the rest in FP64.
//
//  * ExpFast: P. T. P. Tang, "Table-driven implementation of the exponential
//    function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989.
//    x = (64 m + j) ln2/256 + r with |r| <= ln2/512 (+ a small slack from the
//    FP32 rounding of N), exp(x) = 2^m * T_j * (1 + expm1(r)),
//    T_j = 2^(j/256) (a table computed on the host in extended precision),
//    expm1(r) = r + r^2/2 in FP64 plus r^3/6 + r^4/24 + r^5/120 in FP32
//    (|r^3/6| < 4.2e-10, so FP32 rounding adds < 2e-16 relative).
//    About 7 FP64 instructions instead of ~20 for the library exp. Error
//    within a few ulp; |x| >= 700 and non-finite inputs use exp().
//  * RcpFast: an FP32 reciprocal seed refined by two Newton steps
//    y <- y + y (1 - d y) in FP64 (quadratic convergence: 2^-22 -> 2^-44 ->
//    below double rounding). Inputs outside the FP32 range use 1.0 / d.
//
// Conversions between FP64 and FP32 are done with integer operations (the
// FP32 values only seed or correct FP64 quantities, truncation is enough).
#pragma once

#include <cstdint>

namespace lmc {

constexpr int kExpTableSize = 256;

// Truncates a double to a float (zero below the FP32 normal range; callers
// keep the magnitude below the FP32 maximum).
__device__ __forceinline__ float DoubleToFloatTrunc(double d) {
  const int hi = __double2hiint(d);
  const unsigned lo = static_cast<unsigned>(__double2loint(d));
  const int e = ((hi >> 20) & 0x7FF) - 896;  // rebias 1023 -> 127
  const unsigned bits = (static_cast<unsigned>(hi) & 0x80000000u) | (static_cast<unsigned>(e) << 23) |
                        ((static_cast<unsigned>(hi) & 0xFFFFFu) << 3) | (lo >> 29);
  return e > 0 ? __uint_as_float(bits) : 0.0f;
}

// Exact float -> double (zero for FP32 subnormals).
__device__ __forceinline__ double FloatToDouble(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xFFFFFu);
  return e ? __hiloint2double(static_cast<int>(hi), static_cast<int>(u << 29)) : 0.0;
}

struct ExpConsts {
  const double *tab;  // 2^(j/256), j = 0..255
  double l1, l2;      // ln2/256 = l1 + l2, l1 with at most 34 significant bits
};

__device__ __forceinline__ double ExpFast(double x, const ExpConsts &c) {
  const int hi = __double2hiint(x);
  if ((hi & 0x7FFFFFFF) >= 0x4085E000) return exp(x);  // |x| >= 700, inf, nan
  // N = round(x * 256 / ln2) in FP32 (an error of one in N only widens |r|)
  const float tf = fmaf(DoubleToFloatTrunc(x), 369.329930467574632f, 12582912.0f);  // + 1.5 * 2^23
  const int n = __float_as_int(tf) - 0x4B400000;
  const double nd = __longlong_as_double(0x4338000000000000LL + n) - 6755399441055744.0;  // (double) n, exact
  double r = fma(-nd, c.l1, x);  // exact: n * l1 has at most 53 bits
  r = fma(-nd, c.l2, r);
  const float rf = DoubleToFloatTrunc(r);
  const float tail = rf * rf * rf * fmaf(rf, fmaf(rf, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f);
  const double p = fma(r, 0.5 * r, r) + FloatToDouble(tail);  // expm1(r)
  const int j = n & (kExpTableSize - 1), m = n >> 8;           // n = 256 m + j
  const double tj = c.tab[j];
  const double v = fma(tj, p, tj);
  return __hiloint2double(__double2hiint(v) + (m << 20), __double2loint(v));
}

__device__ __forceinline__ double RcpFast(double d) {
  const int e = (__double2hiint(d) >> 20) & 0x7FF;
  if (e < 1023 - 120 || e > 1023 + 120) return 1.0 / d;  // outside the FP32 range (and 0, inf, nan)
  float yf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(DoubleToFloatTrunc(d)));
  double y = FloatToDouble(yf);
  y = fma(y, fma(-d, y, 1.0), y);
  y = fma(y, fma(-d, y, 1.0), y);
  return y;
}

}  // namespace lmc
