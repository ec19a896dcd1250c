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
// Conversions between IEEE doubles and dd use integer operations only (no FP64
// instruction): d2dd splits the 53-bit significand into a 24-bit hi and the
// correctly rounded remainder; dd2d rebuilds the double from the two
// significands.  A power-of-two scale (an exponent offset) keeps any finite
// double range inside the float exponent range.
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

// x * 2^(1023 - emax) as dd.  Values more than 2^126 below 2^(emax-1023)
// become zero; emax is the largest biased exponent of the tile.
__device__ __forceinline__ dd d2dd(double x, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FF);
  const unsigned sign = hi32 & 0x80000000u;
  const int ef = e - emax + 127;  // biased float exponent of the scaled value
  if (e == 0 || ef <= 0) return dd(0.0f, 0.0f);
  if (e == 0x7FF) return dd(__uint_as_float(0x7FC00000u), 0.0f);
  const unsigned m23 = ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29);
  const float h = __uint_as_float(sign | ((unsigned)ef << 23) | m23);
  // remainder: low 29 significand bits, value r29 * 2^(ef - 127 - 52)
  const unsigned r29 = lo32 & 0x1FFFFFFFu;
  float l = 0.0f;
  if (ef > 52 && r29 != 0) {
    // correctly rounded float(r29) with two exact 16-bit halves and one FMA
    const float fh = __uint_as_float(0x4B000000u | (r29 >> 15)) - 8388608.0f;
    const float fl = __uint_as_float(0x4B000000u | (r29 & 0x7FFFu)) - 8388608.0f;
    const float r = __fmaf_rn(fh, 32768.0f, fl);
    l = __fmul_rn(r, __uint_as_float((unsigned)(ef - 52) << 23));
    l = __uint_as_float(__float_as_uint(l) | sign);
  }
  return dd(h, l);
}

// (v.h + v.l) * 2^(emax - 1023) as a double (truncating the last bit at worst).
__device__ __forceinline__ double dd2d(dd v, int emax) {
  v = renorm(v);
  const unsigned hb = __float_as_uint(v.h), lb = __float_as_uint(v.l);
  const int eh = (int)((hb >> 23) & 0xFF);
  if (eh == 0) return 0.0;
  if (eh == 0xFF) return __longlong_as_double(0x7FF8000000000000ll);
  const int el = (int)((lb >> 23) & 0xFF);
  long long M = (long long)(0x800000u | (hb & 0x7FFFFFu)) << 29;  // bit 52 set
  if (el != 0) {
    const long long ml = (long long)(0x800000u | (lb & 0x7FFFFFu));
    const int sh = el - eh + 29;
    long long t;
    if (sh >= 0) t = ml << sh;
    else t = (sh > -40) ? (ml >> (-sh)) : 0;
    M = ((hb ^ lb) & 0x80000000u) ? M - t : M + t;
  }
  int E = eh - 127 + emax;  // biased double exponent
  if (M >> 53) { M >>= 1; ++E; }
  else if (!(M >> 52)) { M <<= 1; --E; }
  if (E <= 0) return 0.0;
  if (E >= 0x7FF) E = 0x7FF, M = 0;
  const unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) |
                                  ((unsigned long long)E << 52) |
                                  ((unsigned long long)M & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}
#endif

}  // namespace pfgb
