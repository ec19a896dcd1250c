// Block floating point ("fx") arithmetic for Float64 passes: 64-bit integer
// components, one power-of-two scale per line (PFGB_PRECISION_BLOCK_FLOAT).
//
// The dd form spends eight FP32 instructions on every sum (error-free
// two-sum plus the low parts), and sums are most of an FFT.  On GB300 this
// form still measures slower than dd (512^3 round trip 4.82 against 4.46 ms):
// integer instructions issue at half the FP32 rate, and the 64-bit splits,
// shifts and carries leave the instruction count near dd's.  Here a pass
// keeps line values as int64 multiples of 2^S, S fixed per line: sums are
// exact 64-bit integer adds (two 32-bit instructions), and a product with a
// twiddle w (|w| <= 1, held as W = round(w 2^60)) is formed from three
// 32 x 32 -> 64-bit multiply-adds on the halves a = ah 2^31 + al,
// W = wh 2^31 + wl:
//   a W / 2^60 = 4 ah wh + (ah wl + al wh) / 2^29 + al wl / 2^60,
// the last term (in [0, 4) units) replaced by its mean in the rounding
// constant: a product is within 4 units, a complex twiddle product within 7.
// Headroom: a pass scales each line so that its components lie below 2^H,
// H = 59 - log2 M (one bit less for c2r, whose input sums two half
// spectra), so that every value of the transform stays below 2^61 and the
// cross terms cannot overflow; relative precision is 2^-H of the line's
// largest component (2^-50 for 512-point lines), and the FFT's growth is
// absorbed by renormalising each output line to 2^61 before it is stored.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PFGB_FX __host__ __device__ __forceinline__
#else
#define PFGB_FX inline
#endif

namespace pfgb {

struct fx {
  long long v;
  fx() = default;
  PFGB_FX constexpr explicit fx(long long x) : v(x) {}
  // the integer 0 (the kernels' R(0))
  PFGB_FX constexpr explicit fx(int x) : v(x) {}
  // a constant c, |c| <= 1, as round(c 2^60) (clamped below 2^60): the
  // right-hand operand of a product
  PFGB_FX constexpr explicit fx(double c)
      : v(c >= 1.0 ? (1ll << 60) - 1
                   : (long long)(c * 1152921504606846976.0 + (c >= 0 ? 0.5 : -0.5))) {}
};

PFGB_FX fx operator+(fx a, fx b) { return fx(a.v + b.v); }
PFGB_FX fx operator-(fx a, fx b) { return fx(a.v - b.v); }
PFGB_FX fx operator-(fx a) { return fx(-a.v); }

// a * c for a data value a (|a| < 2^61) and a constant c (fx(double)).
PFGB_FX fx operator*(fx a, fx c) {
  const int ah = (int)(a.v >> 31), al = (int)(a.v & 0x7FFFFFFFll);
  const int ch = (int)(c.v >> 31), cl = (int)(c.v & 0x7FFFFFFFll);
  // rounding: half a unit of the shift plus the mean of the dropped al cl term
  long long x = (3ll << 28) + (long long)ah * cl + (long long)al * ch;
  return fx((x >> 29) + (long long)ah * (ch * 4));
}

// Twiddle table entry of the fast kernel for Float64 plans: W = round(w 2^60)
// for the real and imaginary parts, each as (4 * (W >> 31), W & (2^31 - 1)).
struct fx_tw {
  int rh4, rl, ih4, il;
};

// a * w for a twiddle w of the pass's table (the pass's sign already applied).
// |a.re|, |a.im| < 2^61: each cross-term sum stays below 6 * 2^60.
PFGB_FX void fx_twiddle(fx& re, fx& im, fx_tw w) {
  const int arh = (int)(re.v >> 31), arl = (int)(re.v & 0x7FFFFFFFll);
  const int aih = (int)(im.v >> 31), ail = (int)(im.v & 0x7FFFFFFFll);
  const int wrh = w.rh4 >> 2, wih = w.ih4 >> 2;
  // rounding constants: half a unit of the shift, plus the means of the dropped
  // low products (+ for ar wr and ai wr / ar wi, - for ai wi)
  long long xr = (1ll << 28) + (long long)arh * w.rl + (long long)arl * wrh;
  xr -= (long long)aih * w.il + (long long)ail * wih;
  long long xi = (5ll << 28) + (long long)arh * w.il + (long long)arl * wih;
  xi += (long long)aih * w.rl + (long long)ail * wrh;
  const long long rr = (xr >> 29) + (long long)arh * w.rh4 - (long long)aih * w.ih4;
  const long long ri = (xi >> 29) + (long long)arh * w.ih4 + (long long)aih * w.rh4;
  re = fx(rr);
  im = fx(ri);
}

// Exponent words of stored fx lines: a line's values are its int64 components
// times 2^(te - 61), all below 2^te in magnitude.  All-zero lines and lines
// holding a NaN or an infinity carry these markers.
constexpr int kTeZero = -(1 << 24);
constexpr int kTeNaN = 1 << 24;

// Headroom bits of the components at the start of a pass (see above).
PFGB_FX constexpr int fx_head(int logm, bool c2r) {
  return (59 - logm - (c2r ? 1 : 0)) < 52 ? (59 - logm - (c2r ? 1 : 0)) : 52;
}

// Bit casts and leading-zero count for both host and device compilation.
PFGB_FX long long fx_dbits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
PFGB_FX double fx_bitsd(long long b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}
PFGB_FX int fx_clz(unsigned long long u) {  // 64 for u == 0
#if defined(__CUDA_ARCH__)
  return __clzll((long long)u);
#else
  return u ? __builtin_clzll(u) : 64;
#endif
}

// x (a double of a line whose largest biased exponent is eb) as a multiple of
// 2^(eb - 1022 - H): the significand shifted right by base - e, base =
// eb + 53 - H (>= 1 above e since H <= 52), rounded to nearest.
PFGB_FX long long d2fx(double x, int base) {
  const unsigned long long b = (unsigned long long)fx_dbits(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  const int r0 = base - (e > 1 ? e : 1);
  const int r = r0 < 63 ? r0 : 63;
  const unsigned long long q = (m + ((1ull << r) >> 1)) >> r;
  return (long long)b < 0 ? -(long long)q : (long long)q;
}

// v * 2^s as a double (|v| < 2^62), rounded to nearest; values below the
// double range give zero, above it infinity.
PFGB_FX double fx2d(long long v, int s) {
  const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
  const unsigned long long u = (unsigned long long)(v < 0 ? -v : v);
  const int lz = fx_clz(u) & 63;
  const unsigned long long n = u << lz;  // leading one at bit 63
  const unsigned long long mant = (n >> 11) + ((n >> 10) & 1ull);
  const int eb = 1023 + s + 63 - lz;     // biased exponent of the result
  const unsigned long long bits =
      eb >= 2047 ? 0x7FF0000000000000ull : (((unsigned long long)(eb - 1) << 52) + mant);
  return fx_bitsd((long long)((u != 0 && eb > 0) ? (bits | sgn) : 0ull));
}

// x >> s for a stored component (|x| <= 2^61), s >= 1, truncated; s >= 63
// gives 0 or -1.
PFGB_FX long long fx_shr(long long x, int s) { return x >> (s < 63 ? s : 63); }

}  // namespace pfgb
