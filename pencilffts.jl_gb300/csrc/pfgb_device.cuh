// Device code of the generic transform pass.
//
// One launch performs one 1D transform along one axis of an N-D array (one
// "pass" of the reference's per-dimension loop, src/operations.jl:227-254),
// with the pencil re-layout of PencilArrays' transpose! fused into the same
// pass: a CTA loads a tile of lines into shared memory with coalesced reads
// in the input layout, transforms every line there (Stockham autosort or
// Bluestein), and stores the tile with coalesced writes in the output layout.
//
// The arithmetic type R is a template parameter (float or double here); the
// complex element type in memory is Cx<R>.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pencilfft_gb300.h"
#include "pfgb_div31.h"

namespace pfgb {

constexpr int kMaxStages = 8;
constexpr int kMaxDevicesConfigured = 64;  // devices per process the launchers track
constexpr int kMaxOuter = 12;
constexpr int kMaxTerms = 3;  // sources of a fused sum of spectral derivatives

// Operation performed by a pass.
enum PassOp : int {
  OP_C2C = 0,    // complex -> complex DFT (sign in PassArgs::sign)
  OP_R2C = 1,    // two real lines packed in one complex DFT, n -> n/2+1
  OP_C2R = 2,    // two Hermitian half-spectra packed in one complex DFT, m -> n
  OP_R2R_C = 3,  // real-to-real kind applied to complex data
  OP_R2R_R = 4,  // real-to-real kind applied to real data (two lines packed)
  // register Stockham pass only: REDFT00 / RODFT00 as a complex DFT of the
  // even / odd extension (length a power of two), on complex lines (X00C) or
  // on two real lines packed in one complex line (X00R)
  OP_X00C = 5,
  OP_X00R = 6,
  // register Stockham pass only: a c2c pass whose input is the sum over up
  // to kMaxTerms sources of c_t i k_t src_t (fused divergence / curl)
  OP_CSUM = 7,
  // register Stockham pass only: the first pass of a line split in two
  // (lines longer than one pass takes): c2c along n2 whose outputs are
  // multiplied by W_M^(n1 k2), n1 the index along the line's other part
  OP_C2CT = 8,
  // register Stockham pass only: REDFT10 / RODFT10 (D2) and REDFT01 / RODFT01
  // (D3) of a power-of-two length n through one n-point complex DFT, on
  // complex lines (D2C, D3C) or on two real lines packed in one complex line
  // (D2R, D3R).  D2: the DFT of v[m] = x[2m], v[n-1-m] = x[2m+1] (m < n/2),
  // then Y[k] = w_k V[k] + conj(w_k) V[n-k], w_k = exp(-i pi k / (2n)).  D3:
  // the inverse DFT of conj(w_k) (y[k] - i y[n-k]) (y[n] = 0), then
  // out[2m] = v[m], out[2m+1] = v[n-1-m].  The odd kinds (RODFT10 / RODFT01)
  // alternate the sign of the even kind's input (D2) or output (D3) and
  // reverse its output (D2) or input (D3).  The DHT is D2 without the
  // reordering and with w_k = (1 + i) / 2 (H[k] = Re F[k] - Im F[k] for real
  // lines, by linearity for complex ones).
  OP_D2C = 9,
  OP_D2R = 10,
  OP_D3C = 11,
  OP_D3R = 12,
  // register Stockham pass only: REDFT11 / RODFT11 (D4) of a power-of-two
  // length n through one 2n-point DFT: V = DFT_2n of x[j] c_j (j < n, zero
  // above; c_j = exp(-i pi j / (2n))), then with d_k = exp(-i pi (2k+1) / (4n))
  // REDFT11: Y[k] = d_k V[k] + conj(d_k) V[2n-1-k], RODFT11: i (d_k V[k] -
  // conj(d_k) V[2n-1-k]), k < n; complex lines (D4C) or two real lines packed
  // in one (D4R)
  OP_D4C = 13,
  OP_D4R = 14,
};

// FFTW r2r kind codes.
enum R2RKind : int {
  K_DHT = 2, K_REDFT00 = 3, K_REDFT01 = 4, K_REDFT10 = 5, K_REDFT11 = 6,
  K_RODFT00 = 7, K_RODFT01 = 8, K_RODFT10 = 9, K_RODFT11 = 10
};

// Kernel argument block (host fills it, passed by value).
struct PassArgs {
  const void* in;
  void* out;
  const void* tw;     // core twiddles: Lc entries exp(-2 pi i m / Lc)
  const void* chirp;  // Bluestein chirp (M entries) for this pass's sign
  const void* bfilt;  // Bluestein filter spectrum / L (L entries) for this sign
  const void* r2rtw;  // r2r twiddles exp(-i pi m / (4 n)), m in [0, 4n]
  int op, r2r_kind, sign, scale_on;
  int n_in, n_out;    // line length (elements) in input / output
  int M;              // DFT length
  int L;              // Bluestein convolution length (0: direct Stockham of M)
  int nst;            // number of Stockham stages of the core length
  int rad[kMaxStages];
  int lines;          // array lines per tile (input lines)
  int clines;         // complex lines per tile (lines or lines/2 when packed)
  int bpl;            // threads per complex line in the core
  int lp;             // shared-memory pitch of one complex line (elements)
  int zero_fill;      // clear the tile before the load
  int in_tfast, out_tfast;  // tile dimension has stride 1 in input / output
  int nouter;
  int64_t nt;         // extent of the tile dimension
  int64_t ntiles;     // ceil(nt / lines)
  int64_t in_sa, in_st, out_sa, out_st;  // axis and tile strides (elements)
  int64_t osz[kMaxOuter], in_so[kMaxOuter], out_so[kMaxOuter];
  double scale;
  // spectral derivative (c2c passes), as in FastArgs: multiply the input
  // (deriv == 1) or the output (deriv == 2) by i k0 f(index)
  int deriv, deriv_role, deriv_half;
  int64_t deriv_n;
  double k0;
  // fused sum of spectral derivatives (c2c passes, nterm > 0): the input of
  // the pass is sum_t i k_t(idx) tsrc[t], k_t = tk0[t] f with f the
  // frequency of the index along the dimension of role trole[t] (0 axis, 1
  // tile dimension, 2 + o outer dimension o); tsrc[t] has the layout of in
  int nterm;
  const void* tsrc[kMaxTerms];
  int trole[kMaxTerms], thalf[kMaxTerms];
  int64_t tn[kMaxTerms];
  double tk0[kMaxTerms];
};

template <typename R>
struct Cx {
  R re, im;
};

template <typename R>
__device__ __forceinline__ Cx<R> mk(R a, R b) {
  Cx<R> z;
  z.re = a;
  z.im = b;
  return z;
}
template <typename R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a) { return mk(-a.re, -a.im); }
template <typename R>
__device__ __forceinline__ Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename R>
__device__ __forceinline__ Cx<R> scal(Cx<R> a, R s) { return mk(a.re * s, a.im * s); }
template <typename R>
__device__ __forceinline__ Cx<R> conj(Cx<R> a) { return mk(a.re, -a.im); }
// multiply by i
template <typename R>
__device__ __forceinline__ Cx<R> mul_i(Cx<R> a) { return mk(-a.im, a.re); }
// multiply by -i
template <typename R>
__device__ __forceinline__ Cx<R> mul_mi(Cx<R> a) { return mk(a.im, -a.re); }
// multiply by the quarter-turn root exp(SIGN * i pi / 2)
template <int SIGN, typename R>
__device__ __forceinline__ Cx<R> mul_w4(Cx<R> a) { return SIGN < 0 ? mul_mi(a) : mul_i(a); }

template <typename R>
__device__ __forceinline__ Cx<R> ldtw(const void* t, int m) {
  return reinterpret_cast<const Cx<R>*>(t)[m];
}
// exp(SIGN * 2 pi i m / Lc) from the table of exp(-2 pi i m / Lc).
template <int SIGN, typename R>
__device__ __forceinline__ Cx<R> twid(const void* t, int m) {
  Cx<R> w = ldtw<R>(t, m);
  return SIGN < 0 ? w : conj(w);
}

// ---------------------------------------------------------------------------
// Small DFT butterflies, y_k = sum_j v_j exp(SIGN 2 pi i jk / RAD), in place.
// ---------------------------------------------------------------------------
template <int SIGN, typename R>
__device__ __forceinline__ void dft2(Cx<R>& a, Cx<R>& b) {
  Cx<R> t = a;
  a = t + b;
  b = t - b;
}

template <int SIGN, typename R>
__device__ __forceinline__ void dft4(Cx<R>& x0, Cx<R>& x1, Cx<R>& x2, Cx<R>& x3) {
  Cx<R> t0 = x0 + x2, t1 = x0 - x2, t2 = x1 + x3, t3 = mul_w4<SIGN>(x1 - x3);
  x0 = t0 + t2;
  x2 = t0 - t2;
  x1 = t1 + t3;
  x3 = t1 - t3;
}

// x * exp(SIGN i pi m / 8) for the compile-time exponent m in [0, 16).
template <int SIGN, int m, typename R>
__device__ __forceinline__ Cx<R> w16mul(Cx<R> x) {
  constexpr int mm = m & 15;
  if constexpr (mm == 0) {
    return x;
  } else if constexpr (mm == 4) {
    return mul_w4<SIGN>(x);
  } else if constexpr (mm == 8) {
    return -x;
  } else if constexpr (mm == 12) {
    return mul_w4<-SIGN>(x);
  } else if constexpr ((mm & 3) == 2) {
    // odd multiples of pi/4: (c, s) = h (+-1, +-1), h = cos(pi/4)
    const R h = R(0.70710678118654752440);
    constexpr int cs = (mm == 2 || mm == 14) ? 1 : -1;                      // sign of cos
    constexpr int ss = ((mm == 2 || mm == 6) ? 1 : -1) * (SIGN < 0 ? -1 : 1);  // sign of sin
    // (re c - im s, re s + im c) with |c| = |s| = h
    R a = (cs > 0) ? x.re : -x.re;
    R b = (ss > 0) ? x.im : -x.im;
    R c2 = (ss > 0) ? x.re : -x.re;
    R d2 = (cs > 0) ? x.im : -x.im;
    return mk((a - b) * h, (c2 + d2) * h);
  } else {
    const R c1 = R(0.92387953251128675613);  // cos(pi/8)
    const R s1 = R(0.38268343236508977173);  // sin(pi/8)
    // angle pi mm / 8 for the odd mm: cos and sin as +-c1 / +-s1
    constexpr bool swap = (mm == 3 || mm == 5 || mm == 11 || mm == 13);
    constexpr int cs = (mm == 1 || mm == 3 || mm == 13 || mm == 15) ? 1 : -1;
    constexpr int ss0 = (mm < 8) ? 1 : -1;
    constexpr int ss = ss0 * (SIGN < 0 ? -1 : 1);
    R c = swap ? s1 : c1;
    R s = swap ? c1 : s1;
    if constexpr (cs < 0) c = -c;
    if constexpr (ss < 0) s = -s;
    return mk(x.re * c - x.im * s, x.re * s + x.im * c);
  }
}

template <int SIGN, typename R>
__device__ __forceinline__ void dft8(Cx<R>* v) {
  // n = n1 + 2 n2, k = k2 + 4 k1
  dft4<SIGN>(v[0], v[2], v[4], v[6]);
  dft4<SIGN>(v[1], v[3], v[5], v[7]);
  v[3] = w16mul<SIGN, 2>(v[3]);
  v[5] = w16mul<SIGN, 4>(v[5]);
  v[7] = w16mul<SIGN, 6>(v[7]);
  // a[n1][k2] sits at v[n1 + 2 k2]
  Cx<R> y[8];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    Cx<R> a0 = v[2 * k2], a1 = v[2 * k2 + 1];
    y[k2] = a0 + a1;
    y[k2 + 4] = a0 - a1;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = y[i];
}

// dft4 / dft8 of inputs whose upper half is zero (x2 = x3 = 0; v[4..7] = 0),
// which are not read: the first stage of a zero-padded transform
template <int SIGN, typename R>
__device__ __forceinline__ void dft4_zh(Cx<R>& x0, Cx<R>& x1, Cx<R>& x2, Cx<R>& x3) {
  const Cx<R> a = x0, t3 = mul_w4<SIGN>(x1);
  x0 = a + x1;
  x2 = a - x1;
  x3 = a - t3;
  x1 = a + t3;
}
template <int SIGN, typename R>
__device__ __forceinline__ void dft8_zh(Cx<R>* v) {
  dft4_zh<SIGN>(v[0], v[2], v[4], v[6]);
  dft4_zh<SIGN>(v[1], v[3], v[5], v[7]);
  v[3] = w16mul<SIGN, 2>(v[3]);
  v[5] = w16mul<SIGN, 4>(v[5]);
  v[7] = w16mul<SIGN, 6>(v[7]);
  Cx<R> y[8];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    Cx<R> a0 = v[2 * k2], a1 = v[2 * k2 + 1];
    y[k2] = a0 + a1;
    y[k2 + 4] = a0 - a1;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = y[i];
}

template <int SIGN, typename R>
__device__ __forceinline__ void dft16(Cx<R>* v) {
  // n = n1 + 4 n2, k = k2 + 4 k1; a[n1][k2] lives in v[n1 + 4 k2]
  dft4<SIGN>(v[0], v[4], v[8], v[12]);
  dft4<SIGN>(v[1], v[5], v[9], v[13]);
  dft4<SIGN>(v[2], v[6], v[10], v[14]);
  dft4<SIGN>(v[3], v[7], v[11], v[15]);
  v[5] = w16mul<SIGN, 1>(v[5]);
  v[9] = w16mul<SIGN, 2>(v[9]);
  v[13] = w16mul<SIGN, 3>(v[13]);
  v[6] = w16mul<SIGN, 2>(v[6]);
  v[10] = w16mul<SIGN, 4>(v[10]);
  v[14] = w16mul<SIGN, 6>(v[14]);
  v[7] = w16mul<SIGN, 3>(v[7]);
  v[11] = w16mul<SIGN, 6>(v[11]);
  v[15] = w16mul<SIGN, 9>(v[15]);
  Cx<R> y[16];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    Cx<R> a0 = v[4 * k2], a1 = v[4 * k2 + 1], a2 = v[4 * k2 + 2], a3 = v[4 * k2 + 3];
    dft4<SIGN>(a0, a1, a2, a3);
    y[k2] = a0;
    y[k2 + 4] = a1;
    y[k2 + 8] = a2;
    y[k2 + 12] = a3;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = y[i];
}

// Odd prime radix via the symmetric real/imaginary split; the roots of unity
// come from the core twiddle table (RAD divides the core length Lc).
template <int RAD, int SIGN, typename R>
__device__ __forceinline__ void dft_odd(Cx<R>* v, const void* tw, int Lc) {
  constexpr int H = (RAD - 1) / 2;
  const int step = Lc / RAD;
  Cx<R> s[H], d[H];
  Cx<R> y0 = v[0];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = v[j] + v[RAD - j];
    d[j - 1] = v[j] - v[RAD - j];
    y0 = y0 + s[j - 1];
  }
  Cx<R> y[RAD];
  y[0] = y0;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    Cx<R> a = v[0], b = mk(R(0), R(0));
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % RAD;
      Cx<R> w = ldtw<R>(tw, m * step);  // (cos t, -sin t), t = 2 pi m / RAD
      a = a + scal(s[j - 1], w.re);
      b = b + scal(d[j - 1], -w.im);    // sum d_j sin t
    }
    // sign -1: y_k = a - i b, y_{RAD-k} = a + i b
    Cx<R> ib = mul_i(b);
    if (SIGN < 0) {
      y[k] = a - ib;
      y[RAD - k] = a + ib;
    } else {
      y[k] = a + ib;
      y[RAD - k] = a - ib;
    }
  }
#pragma unroll
  for (int i = 0; i < RAD; ++i) v[i] = y[i];
}

template <int RAD, int SIGN, typename R>
__device__ __forceinline__ void dft_any(Cx<R>* v, const void* tw, int Lc) {
  if constexpr (RAD == 2) {
    dft2<SIGN>(v[0], v[1]);
  } else if constexpr (RAD == 4) {
    dft4<SIGN>(v[0], v[1], v[2], v[3]);
  } else if constexpr (RAD == 8) {
    dft8<SIGN>(v);
  } else if constexpr (RAD == 16) {
    dft16<SIGN>(v);
  } else {
    dft_odd<RAD, SIGN>(v, tw, Lc);
  }
}

// One Stockham stage of radix RAD on every complex line of the tile.
// Line length Lc, already-transformed sub-length Ls.  Thread (p, b) does
// butterfly b of line p: reads z[b + r T], writes z[(b - j) RAD + j + r Ls],
// j = b mod Ls, T = Lc / RAD.
template <int RAD, int SIGN, typename R>
__device__ __forceinline__ void stage(Cx<R>* zl, bool line_ok, int b, int Lc, int Ls,
                                      const void* tw) {
  const int T = Lc / RAD;
  const bool act = line_ok && b < T;
  Cx<R> v[RAD];
  int j = 0;
  if (act) {
    j = b % Ls;
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[r] = zl[b + r * T];
    if (Ls > 1) {
      const int tstep = j * (Lc / (Ls * RAD));
#pragma unroll
      for (int r = 1; r < RAD; ++r) v[r] = v[r] * twid<SIGN, R>(tw, r * tstep);
    }
    dft_any<RAD, SIGN>(v, tw, Lc);
  }
  __syncthreads();
  if (act) {
    const int base = (b - j) * RAD + j;
#pragma unroll
    for (int r = 0; r < RAD; ++r) zl[base + r * Ls] = v[r];
  }
  __syncthreads();
}

template <int SIGN, typename R>
__device__ void stockham(Cx<R>* z, const PassArgs& a, int Lc) {
  const int p = threadIdx.x / a.bpl;
  const int b = threadIdx.x % a.bpl;
  const bool line_ok = p < a.clines;
  Cx<R>* zl = z + (size_t)(line_ok ? p : 0) * a.lp;
  int Ls = 1;
  for (int s = 0; s < a.nst; ++s) {
    const int rd = a.rad[s];
    switch (rd) {
      case 2: stage<2, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 3: stage<3, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 4: stage<4, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 5: stage<5, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 7: stage<7, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 8: stage<8, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 11: stage<11, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      case 13: stage<13, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
      default: stage<16, SIGN, R>(zl, line_ok, b, Lc, Ls, a.tw); break;
    }
    Ls *= rd;
  }
}

// ---------------------------------------------------------------------------
// Pre-op: place one complex input value x (array line p of the tile, index j)
// into the complex DFT line zl (length M).
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void r2r_pre(Cx<R>* zl, const PassArgs& a, int j, Cx<R> x) {
  const int n = a.n_in;
  const int M = a.M;
  switch (a.r2r_kind) {
    case K_DHT:
      zl[j] = x;
      break;
    case K_REDFT00:
      zl[j] = x;
      if (j >= 1 && j <= n - 2) zl[M - j] = x;
      break;
    case K_RODFT00:
      zl[j + 1] = x;
      zl[M - 1 - j] = -x;
      break;
    case K_REDFT10:
      zl[j] = x;
      zl[2 * n - 1 - j] = x;
      break;
    case K_RODFT10:
      zl[j] = x;
      zl[2 * n - 1 - j] = -x;
      break;
    case K_REDFT11:
      zl[j] = x * ldtw<R>(a.r2rtw, 2 * j);
      zl[2 * n - 1 - j] = -(x * ldtw<R>(a.r2rtw, 2 * (2 * n - 1 - j)));
      break;
    case K_RODFT11:
      zl[j] = x * ldtw<R>(a.r2rtw, 2 * j);
      zl[2 * n - 1 - j] = x * ldtw<R>(a.r2rtw, 2 * (2 * n - 1 - j));
      break;
    case K_REDFT01: {
      Cx<R> y = x * ldtw<R>(a.r2rtw, 2 * j);
      zl[j] = j == 0 ? scal(y, R(0.5)) : y;
      break;
    }
    default: {  // K_RODFT01
      Cx<R> y = mul_i(x * ldtw<R>(a.r2rtw, 2 * (j + 1)));
      zl[j + 1] = j == n - 1 ? scal(y, R(0.5)) : y;
      break;
    }
  }
}

// R2R post-op: output k of line zl (length M).
template <typename R>
__device__ __forceinline__ Cx<R> r2r_post(const Cx<R>* zl, const PassArgs& a, int k) {
  const int n = a.n_out;
  const int M = a.M;
  switch (a.r2r_kind) {
    case K_DHT: {
      Cx<R> f = zl[k], g = zl[k == 0 ? 0 : M - k];
      // ((1+i) f + (1-i) g) / 2
      Cx<R> s = f + g, d = f - g;
      return scal(s + mul_i(d), R(0.5));
    }
    case K_REDFT00:
      return zl[k];
    case K_RODFT00:
      return mul_i(zl[k + 1]);
    case K_REDFT10:
      return ldtw<R>(a.r2rtw, 2 * k) * zl[k];
    case K_RODFT10:
      return mul_i(ldtw<R>(a.r2rtw, 2 * (k + 1)) * zl[k + 1]);
    case K_REDFT11:
      return ldtw<R>(a.r2rtw, 2 * k + 1) * zl[k];
    case K_RODFT11:
      return mul_i(ldtw<R>(a.r2rtw, 2 * k + 1) * zl[k]);
    case K_REDFT01:
      return zl[k] + zl[2 * n - 1 - k];
    default:  // K_RODFT01
      return zl[k] - zl[2 * n - 1 - k];
  }
}

// ---------------------------------------------------------------------------
// The pass kernel.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(1024) pass_kernel(const PassArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Cx<R>* z = reinterpret_cast<Cx<R>*>(smem_raw);
  const int nth = blockDim.x;
  const int tid = threadIdx.x;

  // Tile decode: tile index along the tile dimension, then outer indices.
  int64_t bid = blockIdx.x;
  const int64_t tile = bid % a.ntiles;
  int64_t rest = bid / a.ntiles;
  const int64_t t0 = tile * a.lines;
  int64_t ioff = t0 * a.in_st, ooff = t0 * a.out_st;
  int64_t didx = 0;
  int64_t tdidx[kMaxTerms] = {0, 0, 0};
  for (int d = 0; d < a.nouter; ++d) {
    const int64_t idx = rest % a.osz[d];
    rest /= a.osz[d];
    ioff += idx * a.in_so[d];
    ooff += idx * a.out_so[d];
    if (a.deriv && a.deriv_role == 2 + d) didx = idx;
    for (int t = 0; t < a.nterm; ++t)
      if (a.trole[t] == 2 + d) tdidx[t] = idx;
  }
  auto ik = [&](Cx<R> y, int64_t idx) {
    const int64_t f = (a.deriv_half || idx <= (a.deriv_n - 1) / 2) ? idx : idx - a.deriv_n;
    const R k = R(a.k0 * (double)f);
    return mk(-(y.im * k), y.re * k);
  };
  auto ik_t = [&](int t, Cx<R> y, int64_t idx) {
    const int64_t f = (a.thalf[t] || idx <= (a.tn[t] - 1) / 2) ? idx : idx - a.tn[t];
    const R k = R(a.tk0[t] * (double)f);
    return mk(-(y.im * k), y.re * k);
  };
  const int nvalid = (int)min((int64_t)a.lines, a.nt - t0);
  const int Lc = a.L > 0 ? a.L : a.M;

  if (a.zero_fill) {
    const int tot = a.clines * a.lp;
    for (int e = tid; e < tot; e += nth) z[e] = mk(R(0), R(0));
    __syncthreads();
  }

  // ---- load ----
  const int op = a.op;
  if (op == OP_C2C || op == OP_R2R_C) {
    const Cx<R>* in = reinterpret_cast<const Cx<R>*>(a.in) + ioff;
    const int tot = a.lines * a.n_in;
    for (int e = tid; e < tot; e += nth) {
      int i, j;
      if (a.in_tfast) { i = e % a.lines; j = e / a.lines; } else { j = e % a.n_in; i = e / a.n_in; }
      Cx<R> x = mk(R(0), R(0));
      if (a.nterm > 0) {
        for (int t = 0; t < a.nterm && i < nvalid; ++t) {
          const Cx<R> y = reinterpret_cast<const Cx<R>*>(a.tsrc[t])[ioff + (int64_t)j * a.in_sa + (int64_t)i * a.in_st];
          x = x + ik_t(t, y, a.trole[t] == 0 ? (int64_t)j : a.trole[t] == 1 ? t0 + i : tdidx[t]);
        }
      } else if (i < nvalid) {
        x = in[(int64_t)j * a.in_sa + (int64_t)i * a.in_st];
      }
      if (a.deriv == 1)
        x = ik(x, a.deriv_role == 0 ? (int64_t)j : a.deriv_role == 1 ? t0 + i : didx);
      Cx<R>* zl = z + (size_t)i * a.lp;
      if (op == OP_C2C) zl[j] = x; else r2r_pre(zl, a, j, x);
    }
  } else if (op == OP_R2C || op == OP_R2R_R) {
    const R* in = reinterpret_cast<const R*>(a.in) + ioff;
    const int tot = a.clines * a.n_in;
    for (int e = tid; e < tot; e += nth) {
      int p, j;
      if (a.in_tfast) { p = e % a.clines; j = e / a.clines; } else { j = e % a.n_in; p = e / a.n_in; }
      const int i0 = 2 * p, i1 = 2 * p + 1;
      R xr = R(0), xi = R(0);
      if (i0 < nvalid) xr = in[(int64_t)j * a.in_sa + (int64_t)i0 * a.in_st];
      if (i1 < nvalid) xi = in[(int64_t)j * a.in_sa + (int64_t)i1 * a.in_st];
      Cx<R>* zl = z + (size_t)p * a.lp;
      if (op == OP_R2C) zl[j] = mk(xr, xi); else r2r_pre(zl, a, j, mk(xr, xi));
    }
  } else {  // OP_C2R
    const Cx<R>* in = reinterpret_cast<const Cx<R>*>(a.in) + ioff;
    const int n = a.M, m = a.n_in;
    const int tot = a.clines * m;
    for (int e = tid; e < tot; e += nth) {
      int p, k;
      if (a.in_tfast) { p = e % a.clines; k = e / a.clines; } else { k = e % m; p = e / m; }
      const int i0 = 2 * p, i1 = 2 * p + 1;
      Cx<R> A = mk(R(0), R(0)), B = mk(R(0), R(0));
      if (i0 < nvalid) A = in[(int64_t)k * a.in_sa + (int64_t)i0 * a.in_st];
      if (i1 < nvalid) B = in[(int64_t)k * a.in_sa + (int64_t)i1 * a.in_st];
      if (k == 0 || 2 * k == n) { A.im = R(0); B.im = R(0); }
      Cx<R>* zl = z + (size_t)p * a.lp;
      zl[k] = mk(A.re - B.im, A.im + B.re);                        // A + i B
      if (k >= 1 && k <= n - m) zl[n - k] = mk(A.re + B.im, B.re - A.im);  // conj(A) + i conj(B)
    }
  }
  __syncthreads();

  // ---- core DFT ----
  if (a.L == 0) {
    if (a.sign < 0) stockham<-1, R>(z, a, Lc); else stockham<1, R>(z, a, Lc);
  } else {
    const Cx<R>* chirp = reinterpret_cast<const Cx<R>*>(a.chirp);
    const Cx<R>* bf = reinterpret_cast<const Cx<R>*>(a.bfilt);
    const int tot = a.clines * Lc;
    for (int e = tid; e < tot; e += nth) {
      const int p = e / Lc, j = e % Lc;
      Cx<R>* zl = z + (size_t)p * a.lp;
      zl[j] = j < a.M ? zl[j] * chirp[j] : mk(R(0), R(0));
    }
    __syncthreads();
    stockham<-1, R>(z, a, Lc);
    for (int e = tid; e < tot; e += nth) {
      const int p = e / Lc, j = e % Lc;
      Cx<R>* zl = z + (size_t)p * a.lp;
      zl[j] = zl[j] * bf[j];
    }
    __syncthreads();
    stockham<1, R>(z, a, Lc);
    const int tot2 = a.clines * a.M;
    for (int e = tid; e < tot2; e += nth) {
      const int p = e / a.M, j = e % a.M;
      Cx<R>* zl = z + (size_t)p * a.lp;
      zl[j] = zl[j] * chirp[j];
    }
    __syncthreads();
  }

  // ---- store ----
  const R sc = a.scale_on ? R(a.scale) : R(1);
  if (op == OP_C2C || op == OP_R2R_C) {
    Cx<R>* out = reinterpret_cast<Cx<R>*>(a.out) + ooff;
    const int tot = a.lines * a.n_out;
    for (int e = tid; e < tot; e += nth) {
      int i, k;
      if (a.out_tfast) { i = e % a.lines; k = e / a.lines; } else { k = e % a.n_out; i = e / a.n_out; }
      if (i >= nvalid) continue;
      const Cx<R>* zl = z + (size_t)i * a.lp;
      Cx<R> y = op == OP_C2C ? zl[k] : r2r_post(zl, a, k);
      if (a.scale_on) y = scal(y, sc);
      if (a.deriv == 2)
        y = ik(y, a.deriv_role == 0 ? (int64_t)k : a.deriv_role == 1 ? t0 + i : didx);
      out[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = y;
    }
  } else if (op == OP_R2C) {
    Cx<R>* out = reinterpret_cast<Cx<R>*>(a.out) + ooff;
    const int n = a.M, m = a.n_out;
    const int tot = a.clines * m;
    for (int e = tid; e < tot; e += nth) {
      int p, k;
      if (a.out_tfast) { p = e % a.clines; k = e / a.clines; } else { k = e % m; p = e / m; }
      const Cx<R>* zl = z + (size_t)p * a.lp;
      const Cx<R> f = zl[k], g = conj(zl[k == 0 ? 0 : n - k]);
      Cx<R> A = scal(f + g, R(0.5));
      Cx<R> B = scal(mul_mi(f - g), R(0.5));
      if (a.scale_on) { A = scal(A, sc); B = scal(B, sc); }
      const int i0 = 2 * p, i1 = 2 * p + 1;
      if (i0 < nvalid) out[(int64_t)k * a.out_sa + (int64_t)i0 * a.out_st] = A;
      if (i1 < nvalid) out[(int64_t)k * a.out_sa + (int64_t)i1 * a.out_st] = B;
    }
  } else {  // OP_C2R and OP_R2R_R: real output, two lines per complex line
    R* out = reinterpret_cast<R*>(a.out) + ooff;
    const int tot = a.clines * a.n_out;
    for (int e = tid; e < tot; e += nth) {
      int p, k;
      if (a.out_tfast) { p = e % a.clines; k = e / a.clines; } else { k = e % a.n_out; p = e / a.n_out; }
      const Cx<R>* zl = z + (size_t)p * a.lp;
      Cx<R> y = op == OP_C2R ? zl[k] : r2r_post(zl, a, k);
      if (a.scale_on) y = scal(y, sc);
      const int i0 = 2 * p, i1 = 2 * p + 1;
      if (i0 < nvalid) out[(int64_t)k * a.out_sa + (int64_t)i0 * a.out_st] = y.re;
      if (i1 < nvalid) out[(int64_t)k * a.out_sa + (int64_t)i1 * a.out_st] = y.im;
    }
  }
}

// ---------------------------------------------------------------------------
// Permuted copy (NoTransform passes): out (memory order) <- in (strided).
// Bit-exact unless a scale is requested.
// ---------------------------------------------------------------------------
struct CopyArgs {
  const void* in;
  void* out;
  int nd;
  int64_t total;
  int64_t osz[kMaxOuter];   // output sizes in output memory order (fastest first)
  int64_t ist[kMaxOuter];   // input strides of those dims (elements)
  int64_t ost[kMaxOuter];   // output strides of those dims (elements)
  double scale;
  int scale_on;
  int real_is_double;       // element real type for scaling
};

// Real lines longer than one register pass: two real lines x1, x2 of n
// points (neighbours along the pair dimension of the real-side layout,
// index 2c and 2c + 1) travel as one complex line z = x1 + i x2 through an
// n-point c2c transform; these four element maps go either side of it.
// The complex side holds one line per pair (the pair dimension halved,
// rounded up: the last pair of an odd count has no second line).  The two
// layouts of a map usually share their memory order; where the c2c passes
// cannot carry a change of order, the separating map does (strided reads).
enum LPackMode : int {
  LP_R2C_PACK = 0,    // x -> z[k] = x[k, 2c] + i x[k, 2c+1], k < n
  LP_R2C_SEP = 1,     // Z -> X[k, 2c] = (Z[k] + conj Z[n-k]) / 2,
                      //      X[k, 2c+1] = (Z[k] - conj Z[n-k]) / 2i, k <= n/2
  LP_C2R_HPACK = 2,   // X -> Z[k] = X[k, 2c] + i X[k, 2c+1] and
                      //      Z[n-k] = conj X[k, 2c] + i conj X[k, 2c+1], k <= n/2
                      //      (imaginary parts at k = 0 and k = n/2 dropped)
  LP_C2R_UNPACK = 3,  // z -> x[k, 2c] = Re z[k], x[k, 2c+1] = Im z[k], k < n
  // R2R lines whose extension (m points) is longer than one pass: the
  // extension gathered from the line (two real lines packed when `packed`),
  // an m-point c2c transform, and the outputs read from its result, as
  // r2r_pre / r2r_post do in shared memory (tab: exp(-i pi q / (4n)), q <= 4n + 1)
  LP_R2R_PRE = 4,     // y -> z[j], j < m (every point written)
  LP_R2R_POST = 5,    // Z -> y[k], k < n
  // c2c lines of n points without a split, as a Bluestein convolution of
  // length m (a power of two): chirp product and zero padding, the m-point
  // transform, the product with the filter spectrum (divided by m), the
  // inverse m-point transform, chirp product and truncation
  LP_CHIRP_PRE = 6,   // x -> z[j] = x[j] c[j] (j < n), 0 (n <= j < m); tab = c
  LP_MUL = 7,         // z -> z[j] f[j], j < m (in place allowed); tab = f
  LP_CHIRP_POST = 8,  // Z -> y[k] = Z[k] c[k], k < n; tab = c
};

struct LPackArgs {
  const void* in;
  void* out;
  int mode, nd;
  int qa, qp;      // positions of the line axis and of the pair dimension (-1: none)
  int64_t n;       // complex DFT length
  int64_t npair;   // full extent of the pair dimension
  int64_t total;   // iteration points (product of ext)
  int64_t ext[kMaxOuter];  // iteration extents in memory order (fastest first)
  int64_t ist[kMaxOuter], ost[kMaxOuter];  // strides (elements) per iteration coordinate
  Div31 dext[kMaxOuter];   // division by ext (total < 2^31)
  int64_t ist_a, ost_a;    // strides of the line axis
  int64_t in_pst, out_pst; // offset of a pair's second line on the side that holds both
  int64_t m;               // extension / convolution length (R2R and chirp maps)
  int kind;                // R2RKind of the R2R maps
  int packed;              // R2R maps: the data side holds real pairs
  const void* tab;         // complex table (element type of the plan)
};

template <typename E>
__global__ void copy_kernel(const CopyArgs a) {
  const E* in = reinterpret_cast<const E*>(a.in);
  E* out = reinterpret_cast<E*>(a.out);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = e, io = 0, oo = 0;
    for (int d = 0; d < a.nd; ++d) {
      const int64_t idx = rem % a.osz[d];
      rem /= a.osz[d];
      io += idx * a.ist[d];
      oo += idx * a.ost[d];
    }
    out[oo] = in[io];
  }
}

int fail_cuda(cudaError_t e, const char* what);

// Shared-memory opt-in of a kernel on the current device, once per device.
// Plans call every launcher once with grid == 0 at creation ("configure
// only"), so kernel launches recorded into a CUDA graph never configure.
template <typename K>
inline int ensure_smem_attr(K* kernel, int bytes, bool* done, const char* what) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevicesConfigured) return fail_cuda(cudaErrorInvalidDevice, what);
  if (!done[dev]) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return fail_cuda(e, what);
    done[dev] = true;
  }
  return PFGB_OK;
}

}  // namespace pfgb
