// Double-float ("dd") arithmetic on the FP32 pipes.
//
// GB300 executes FP64 FMA/ADD at about 1.6 operations per clock per SM, against
// about 113 for FP32 (measured), so an FP64 FFT is bound by the FP64 unit at a
// small fraction of the HBM roofline.  A dd value holds an unevaluated sum
// hi + lo of two floats (48-bit significand).  Sums use the error-free
// two-sum, products the FMA-based two-product; both keep the lo part lazily
// (no renormalisation after each operation) and renorm() restores
// |lo| <= ulp(hi)/2 where needed.  Relative error per operation is about
// 2^-47 of the operand magnitudes.
//
// Conversions between IEEE doubles and dd use integer and FP32 operations
// only (no FP64 instruction: GB300 runs F2F.F64 conversions at the FP64 rate):
// d2dd splits the 53-bit significand into a 24-bit hi and the rounded
// remainder; dd2d rebuilds the double from hi's significand plus lo counted in
// units of the double's last place.  A power-of-two scale (an exponent
// offset) keeps any finite double range inside the float exponent range.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PFGB_HD __host__ __device__ __forceinline__
#else
#define PFGB_HD inline
#endif

namespace pfgb {

#if defined(__CUDA_ARCH__)
PFGB_HD float f_add(float a, float b) { return __fadd_rn(a, b); }
PFGB_HD float f_sub(float a, float b) { return __fsub_rn(a, b); }
PFGB_HD float f_mul(float a, float b) { return __fmul_rn(a, b); }
PFGB_HD float f_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
PFGB_HD float f_add(float a, float b) { volatile float r = a + b; return r; }
PFGB_HD float f_sub(float a, float b) { volatile float r = a - b; return r; }
PFGB_HD float f_mul(float a, float b) { volatile float r = a * b; return r; }
PFGB_HD float f_fma(float a, float b, float c) { return __builtin_fmaf(a, b, c); }
#endif

struct dd {
  float h, l;
  dd() = default;
  PFGB_HD constexpr dd(float hi, float lo) : h(hi), l(lo) {}
  // Compile-time split of a double constant (folded by the compiler).
  PFGB_HD constexpr explicit dd(double c) : h((float)c), l((float)(c - (double)(float)c)) {}
  PFGB_HD constexpr explicit dd(int c) : h((float)c), l(0.0f) {}
};

// s + e == a + b exactly (Knuth two-sum, 6 flops).
PFGB_HD void two_sum(float a, float b, float& s, float& e) {
  s = f_add(a, b);
  float bb = f_sub(s, a);
  e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
}

PFGB_HD dd operator+(dd a, dd b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return dd(s, f_add(e, f_add(a.l, b.l)));
}
PFGB_HD dd operator-(dd a) { return dd(-a.h, -a.l); }
PFGB_HD dd operator-(dd a, dd b) {
  float s, e;
  two_sum(a.h, -b.h, s, e);
  return dd(s, f_add(e, f_sub(a.l, b.l)));
}
PFGB_HD dd operator*(dd a, dd b) {
  float p = f_mul(a.h, b.h);
  float e = f_fma(a.h, b.h, -p);
  e = f_fma(a.h, b.l, e);
  e = f_fma(a.l, b.h, e);
  return dd(p, e);
}
// |lo| <= ulp(hi)/2 afterwards (fast two-sum).
PFGB_HD dd renorm(dd a) {
  float s = f_add(a.h, a.l);
  return dd(s, f_sub(a.l, f_sub(s, a.h)));
}

// ---------------------------------------------------------------------------
// Integer conversions (device): double <-> dd with a power-of-two scale.
// ---------------------------------------------------------------------------
#if defined(__CUDACC__)
// Biased exponent field of a double's bit pattern (0 for zero/subnormal).
__device__ __forceinline__ int dexp_bits(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// x * 2^(1023 - emax) as dd.  hi keeps the top 24 significand bits of x, lo
// the remaining 29 bits rounded to a float (I2F, then an exact power-of-two
// scale).  Values more than 2^126 below 2^(emax-1023) become zero; emax is
// the largest biased exponent of the data being converted.
__device__ __forceinline__ dd d2dd(double x, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FF);
  const unsigned sign = hi32 & 0x80000000u;
  const int ef = e - emax + 127;  // biased float exponent of the scaled value
  const unsigned m23 = __funnelshift_l(lo32, hi32, 3) & 0x7FFFFFu;
  float h = __uint_as_float(sign | ((unsigned)ef << 23) | m23);
  const float r = __uint2float_rn(lo32 & 0x1FFFFFFFu);
  const float sc = __uint_as_float((unsigned)max(ef - 52, 0) << 23);  // 2^(ef - 179), 0 if ef <= 52
  float l = __uint_as_float(__float_as_uint(__fmul_rn(r, sc)) | sign);
  if (ef <= 0 || e == 0) { h = 0.0f; l = 0.0f; }
  if (e == 0x7FF) h = __uint_as_float(0x7FC00000u);
  return dd(h, l);
}

// (v.h + v.l) * 2^(emax - 1023) as a double.  After a renormalisation
// (|lo| <= ulp_float(hi)/2) the double bit pattern of hi is built with integer
// operations, and lo, converted to an integer count of the double's last place
// (scale by 2^(179 - eh), F2I), is added to that 64-bit pattern: IEEE bit
// patterns are monotonic in magnitude, and |lo| is at most 2^28 last places,
// so the sum stays inside hi's binade except below an exact power of two,
// where the last place halves (the count is doubled there).
__device__ __forceinline__ double dd2d(dd v, int emax) {
  v = renorm(v);
  const unsigned hb = __float_as_uint(v.h), lb = __float_as_uint(v.l);
  const int eh = (int)((hb >> 23) & 0xFF);
  const int E = eh - 127 + emax;  // biased double exponent of hi
  const unsigned hw = (hb & 0x80000000u) | ((unsigned)(E & 0xFFF) << 20) | ((hb & 0x7FFFFFu) >> 3);
  const unsigned lw = hb << 29;
  const float su = __uint_as_float((unsigned)min(max(306 - eh, 1), 254) << 23);  // 2^(179 - eh)
  int li = __float2int_rn(__fmul_rn(v.l, su));
  if (eh < 52) li = 0;
  int lm = ((hb ^ lb) & 0x80000000u) ? -abs(li) : abs(li);  // change of |value|
  if ((hb & 0x7FFFFFu) == 0 && lm < 0) lm *= 2;
  unsigned long long bits = (((unsigned long long)hw << 32) | lw) + (unsigned long long)(long long)lm;
  if (eh == 0 || E <= 0) bits = (unsigned long long)(hb & 0x80000000u) << 32;
  if (eh == 0xFF || E >= 0x7FF) bits = 0x7FF8000000000000ull;
  return __longlong_as_double((long long)bits);
}
#endif

}  // namespace pfgb
