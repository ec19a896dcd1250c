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

// Rare cases of d2dd and dd2d, out of line: inlined at every conversion
// site they would only add instruction-cache footprint.
static __device__ __noinline__ dd d2dd_rare(unsigned hi32, unsigned fs, int e, int c) {
  const unsigned sign = hi32 & 0x80000000u;
  const int ef = e + c;
  if (e == 0x7FF) return dd(__uint_as_float(0x7FC00000u), 0.0f);
  if (e == 0 || ef <= 0) return dd(0.0f, 0.0f);
  return dd(__uint_as_float(sign | ((unsigned)ef << 23) | (fs & 0x7FFFFFu)), 0.0f);
}
static __device__ __noinline__ double dd2d_rare(unsigned sb, int es, int off) {
  if (es == 255 || es + off >= 0x7FF) return __longlong_as_double(0x7FF8000000000000ll);
  return __longlong_as_double((long long)((unsigned long long)(sb & 0x80000000u) << 32));
}

// x * 2^(1023 - emax) as dd.  hi keeps the top 24 significand bits of x, lo
// the remaining 29 bits rounded to a float (I2F, then an exact power-of-two
// scale).  emax is the largest biased exponent of the data being converted.
// Common case (finite nonzero x whose scaled float exponent ef lies in
// [53, 254]): the float pattern of hi is the funnel-shifted word (low 9
// exponent bits : 23 significand bits) plus (127 - emax) << 23, since
// (e + 127 - emax) mod 512 = ef.  Rare cases: zero, subnormal and values
// more than 2^126 below 2^(emax-1023) become zero, Inf/NaN become NaN, and
// values 2^74..2^126 below keep hi only.

__device__ __forceinline__ dd d2dd(double x, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FF);
  const int c = 127 - emax;  // ef = e + c
  const int lo = max(53 - c, 1), hi = min(254 - c, 2046);
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned fs = __funnelshift_l(lo32, hi32, 3);
  if ((unsigned)(e - lo) <= (unsigned)(hi - lo)) {
    const unsigned hx = fs + ((unsigned)c << 23);
    const float r = __uint2float_rn(lo32 & 0x1FFFFFFFu);
    const float sc = __uint_as_float((hx & 0x7F800000u) - (52u << 23));  // 2^(ef - 179)
    return dd(__uint_as_float(hx | sign), __uint_as_float(__float_as_uint(__fmul_rn(r, sc)) | sign));
  }
  return d2dd_rare(hi32, fs, e, c);
}

// (v.h + v.l) * 2^(emax - 1023) as a double, within one unit in the last
// place.  The renormalised pair s + e (fast two-sum, |e| <= ulp_float(s)/2)
// gives the double bit pattern of s by integer operations, and e, converted
// to a signed count of the double's last place (scale by +-2^(179 - es), F2I),
// is added to that 64-bit pattern: IEEE bit patterns are monotonic in
// magnitude and |count| <= 2^28, so the sum stays inside s's binade except
// below an exact power of two, where the last place halves (the count is
// doubled there).  Rare cases (checked once): s zero or subnormal and
// results below the double range give zero, Inf/NaN and overflow give NaN.
__device__ __forceinline__ double dd2d(dd v, int emax) {
  const float s = __fadd_rn(v.h, v.l);
  const float e = __fsub_rn(v.l, __fsub_rn(s, v.h));
  const unsigned sb = __float_as_uint(s);
  const unsigned esx = sb & 0x7F800000u;  // float exponent << 23
  const int es = (int)(esx >> 23);
  const int off = emax - 127;             // double exponent E = es + off
  const int lo = max(1 - off, 1), hi = min(2046 - off, 254);
  const unsigned sign = sb & 0x80000000u;
  if ((unsigned)(es - lo) <= (unsigned)(hi - lo)) {
    const unsigned hw = (((sb & 0x7FFFFFFFu) >> 3) + ((unsigned)off << 20)) | sign;
    const unsigned sux = (0x99000000u - max(esx, 52u << 23)) | sign;  // +-2^(179 - es)
    int li = __float2int_rn(__fmul_rn(e, __uint_as_float(sux)));
    if (li < 0 && (sb & 0x7FFFFFu) == 0) li *= 2;
    const unsigned long long bits = (((unsigned long long)hw << 32) | (sb << 29)) + (unsigned long long)(long long)li;
    return __longlong_as_double((long long)bits);
  }
  return dd2d_rare(sb, es, off);
}
#endif

}  // namespace pfgb
