// tdy_ff.h -- double-float ("float-float") arithmetic for Jacobian products.
//
// On GB300 the FP64 pipe issues about 1.6 FMA per SM per clock, and float <->
// double conversion instructions run on that same pipe, while FP32 FMA issues
// about 115.  The Jacobian products w_r * T_rc are therefore formed as
// unevaluated sums of two floats (hi + lo, about 48 significant bits) with
//   * error-free products (Dekker; the rounding error of hi*hi from one FMA,
//     cross terms in FP32),
//   * Knuth's TwoSum for the running sums, errors collected in a float,
//   * double -> (hi, lo) splits and (hi, lo) -> double conversions done with
//     integer bit operations (no conversion instructions), a power-of-two
//     scale folded into the exponent field so every octant's sum sits near 1.
// The relative error of one product is below 2^-45 and of a sum of n terms
// below (n + 2) * 2^-46 of the sum of their magnitudes.  Every floating-point
// operation is an explicit _rn intrinsic, so the compiler neither contracts
// nor reassociates them and all entry points produce the same bits.
#pragma once

#include <cuda_runtime.h>

namespace tdy {

struct ff {
  float h, l;
};

// biased exponent field of a double (0 for zero and subnormal numbers)
__device__ __forceinline__ int d_bexp(double x) { return (int)(((unsigned)__double2hiint(x) >> 20) & 0x7ffu); }

// x * 2^s as hi + lo: hi is x truncated to 24 significant bits, lo the
// remainder truncated to 24 bits (|error| < 2^-47 |x|).  Results below the
// float normal range flush to signed zero; above it, hi saturates.
__device__ __forceinline__ ff ff_split(double x, int s) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned sign = hw & 0x80000000u;
  const int ef = (int)((hw >> 20) & 0x7ffu);
  const int fe = ef + s - 896;  // float biased exponent of hi
  ff r;
  if (ef == 0 || fe <= 0) {
    r.h = __uint_as_float(sign);
    r.l = 0.0f;
    return r;
  }
  if (fe >= 255) {
    r.h = __uint_as_float(sign | 0x7f7fffffu);
    r.l = 0.0f;
    return r;
  }
  r.h = __uint_as_float(sign | ((unsigned)fe << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  const unsigned rem = lw & 0x1fffffffu;  // the 29 significand bits below hi
  const int lz = __clz(rem);              // 32 when rem == 0
  const int lfe = fe - 21 - lz;           // float biased exponent of lo
  const unsigned m = (rem << (lz & 31)) >> 8;
  r.l = (rem == 0u || lfe <= 0) ? __uint_as_float(sign) : __uint_as_float(sign | ((unsigned)lfe << 23) | (m & 0x7fffffu));
  return r;
}

// x * 2^s as hi + lo for the Jacobian products, given bx = d_bexp(x) and
// the scale s, with fewer operations than ff_split: hi is x truncated to 24
// bits, lo the next 23 significand bits (unnormalised), so |error| < 2^-46
// |x|.  Callers choose s so that |x| 2^s < 4; parts that fall below the float
// normal range come out as subnormal or zero floats of magnitude < 2^-126.
__device__ __forceinline__ ff ff_split_scaled(double x, int bx, int s) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned sign = hw & 0x80000000u;
  const int fe = bx ? max(bx + s - 896, 0) : 0;  // float biased exponent of hi
  ff r;
  r.h = __uint_as_float(sign | ((unsigned)fe << 23) | (__funnelshift_l(lw, hw, 3) & 0x7fffffu));
  // (the 23 bits below hi) * 2^-23 exactly, in [0, 1)
  const float frac = __fadd_rn(__uint_as_float(0x3f800000u | ((lw >> 6) & 0x7fffffu)), -1.0f);
  r.l = __fmul_rn(frac, __uint_as_float(sign | ((unsigned)max(fe - 23, 0) << 23)));
  return r;
}

// exact float -> double times 2^s (zero, subnormal and underflowing inputs
// give signed zero)
__device__ __forceinline__ double ff_f2d(float f, int s) {
  const unsigned u = __float_as_uint(f);
  const int e = (int)((u >> 23) & 0xffu);
  const unsigned sign = u & 0x80000000u;
  const int de = e + 896 + s;
  if (e == 0 || de <= 0) return __hiloint2double((int)sign, 0);
  return __hiloint2double((int)(sign | ((unsigned)de << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
}

// (hi + lo) * 2^s rounded once to double
__device__ __forceinline__ double ff_to_d(ff a, int s) { return __dadd_rn(ff_f2d(a.h, s), ff_f2d(a.l, s)); }

__device__ __forceinline__ ff ff_neg(ff a) {
  ff r;
  r.h = __uint_as_float(__float_as_uint(a.h) ^ 0x80000000u);
  r.l = __uint_as_float(__float_as_uint(a.l) ^ 0x80000000u);
  return r;
}

// a * b: hi*hi rounded, its exact error by FMA, plus the cross terms
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  ff p;
  p.h = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p.h);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  p.l = e;
  return p;
}

// s += p (TwoSum on the high parts, low parts and the sum's error collected
// in s.l)
__device__ __forceinline__ void ff_acc(ff &s, ff p) {
  const float t = __fadd_rn(s.h, p.h);
  const float bp = __fadd_rn(t, -s.h);
  const float ap = __fadd_rn(t, -bp);
  const float err = __fadd_rn(__fadd_rn(s.h, -ap), __fadd_rn(p.h, -bp));
  s.l = __fadd_rn(s.l, __fadd_rn(err, p.l));
  s.h = t;
}

}  // namespace tdy
