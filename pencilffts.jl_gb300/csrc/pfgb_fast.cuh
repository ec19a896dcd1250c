// Register-resident Stockham pass for power-of-two lines (8 <= M <= 4096).
//
// Same pass semantics as pass_kernel (one 1D transform along one axis, the
// pencil re-layout fused into the store), specialised for the common
// lengths: every thread keeps 8 points of one line in registers; radix-8
// stages (plus one radix-2/4 stage when log2 M is not a multiple of 3) run in
// registers and exchange through shared memory between stages only.  The
// first stage reads its inputs straight from global memory and, when the
// output layout allows it, the last stage writes straight to global memory:
// thread (line p, index b) handles elements b + r*(M/8), so warps read and
// write contiguous runs along either the line (axis-contiguous layouts) or
// the tile dimension (axis-strided layouts).
//
// R is the arithmetic type: float for Float32 data; for Float64 data dd
// (double-float on the FP32 pipes, the default) or fx (64-bit integers with
// a per-line power-of-two scale, PFGB_PRECISION_BLOCK_FLOAT).  dd data are scaled by powers of two
// (each line's largest exponent in the first pass of a run, the run's
// largest afterwards) so that any finite double range fits the float
// exponent range; fx lines carry their own scale from pass to pass.
#pragma once

#include <type_traits>

#include "pfgb_dd.cuh"
#include "pfgb_device.cuh"
#include "pfgb_fx.cuh"

namespace pfgb {

struct FastArgs {
  const void* in;
  void* out;
  const void* tw;  // M entries exp(-2 pi i m / M) as Cx<R>
  const void* tw2; // mixed-radix pass (mr_pass): R0 N entries exp(-2 pi i m / (R0 N)); tw has N
  // Bluestein pass (bs_pass): DFT length, chirp w[j] (bs_m entries), filter
  // spectrum (L entries, 1/L included), divisor of its store loop
  int bs_m;
  const void* bs_chirp;
  const void* bs_filt;
  Div31 div_m;
  // OP_C2CT (first pass of a split line of M = M1 * M2 points): outputs times
  // exp(sign 2 pi i n1 k2 / M) from t4_tab (M entries), n1 the index along
  // the dimension of role t4_role (1 tile, 2 + o outer)
  const void* t4_tab;
  int t4_role;
  int op;          // OP_C2C, OP_R2C, OP_C2R, OP_X00C, OP_X00R, OP_D2C ...
  int r2r_odd;     // OP_X00C / R, OP_D2C / R, OP_D3C / R: 0 the REDFT kind, 1 the RODFT kind, 2 DHT (D2)
  // OP_D2* / OP_D3*: w_k = exp(-i pi k / (2n)), k < n (DHT: (1 + i) / 2); OP_D4*:
  // c_j = exp(-i pi j / (2n)), j < n, then d_k = exp(-i pi (2k+1) / (4n)), k < n; as Cx<R>
  const void* d23_tab;
  int n_in, n_out;
  int lmap_tile;     // lanes along the tile dimension (tile dim contiguous in input)
  int store_direct;  // store from registers with the load mapping
  int out_tfast;     // tile dimension contiguous in the output (smem store loop)
  int vec2;          // float r2c: lines 2j, 2j+1 adjacent and 16-byte aligned in the output
  int scale_on;
  float scale_h, scale_l;  // ldiv! normalisation as hi + lo
  // Float64 (dd) passes: the input / output of a pass between two dd passes is
  // kept in dd form (re.hi, re.lo, im.hi, im.lo floats), scaled by the power
  // of two 2^(1023 - *emax), *emax the run exponent (see self_scale below).
  int in_dd, out_dd;
  const int* emax_ptr;
  // added to the run exponent for the double outputs of the pass: the ldiv!
  // normalisation when it is a power of two (scale_on is then 0)
  int emax_shift;
  // Run exponent without a separate reduction: the first pass of a run
  // (self_scale) scales each complex line by its own largest exponent (the
  // tile's, when lines lie across the thread index), stores it in te[line]
  // (line = t0 / pk + p + te_ncl * outer index, pk = 2 real lines per
  // complex line when packed) and folds it into *emax_ptr (atomicMax; zeroed
  // before the run); the second pass (te_rescale) multiplies each loaded
  // element by 2^(te[line1] - *emax_ptr), line1 = sum over its roles (axis,
  // tile dimension, outer dimension o) of (coordinate >> te_sh) * te_mul, the
  // first-pass line of that element.  Later passes use *emax_ptr.
  int self_scale, te_rescale;
  int* te;
  int64_t te_ncl;
  int te_sh[2 + kMaxOuter];
  unsigned te_mul[2 + kMaxOuter];
  int nouter;
  int64_t nt, ntiles;
  int64_t in_sa, in_st, out_sa, out_st;
  int64_t osz[kMaxOuter], in_so[kMaxOuter], out_so[kMaxOuter];
  // the tile decode's divisors (ntiles, osz[d]) as multiply-and-shift pairs;
  // tile indices are below 2^31 (checked at launch)
  Div31 div_tiles, div_osz[kMaxOuter];
  // Spectral derivative fused into the pass (c2c passes): multiply the input
  // (deriv == 1) or the output (deriv == 2) by i k, k = k0 * f, where f is the
  // signed frequency of the element's index along one logical dimension
  // (AbstractFFTs fftfreq/rfftfreq convention).  deriv_role locates that
  // dimension: 0 the pass axis, 1 the tile dimension, 2 + o outer dimension o.
  int deriv, deriv_role, deriv_half;
  int64_t deriv_n;  // physical length of the dimension (frequency wrap)
  float k0_h, k0_l;
  // OP_CSUM: the pass input is sum_t i k_t(idx) tsrc[t] (k_t = tk0[t] f, f
  // the frequency along the dimension of role trole[t], as deriv_role); the
  // sources have the layout of the pass input
  int nterm;
  const void* tsrc[kMaxTerms];
  int trole[kMaxTerms], thalf[kMaxTerms];
  int64_t tn[kMaxTerms];
  float tk0_h[kMaxTerms], tk0_l[kMaxTerms];
  // persistent forms (fast_pass_tma, tc_pass): tiles of the pass and an error
  // word set when a bounded wait gives up
  int64_t total;
  int* err;
  // test of the give-up path (pfgb_plan_set_wait_test): > 0 makes the first
  // data wait of every CTA poll, this many times, an mbarrier that nothing
  // signals, so that it gives up
  int wait_test;
  // tensor-core split form: the DFT matrices' tf32 hi / lo parts in the
  // shared-memory operand layout (tc_pass)
  const void* tcb;
  // fx passes (R = fx): exponent words of the input lines (te_in, indexed as
  // te above, present when the input is in fx form) and of the output lines
  // (te_out, when the output is); the ldiv! normalisation's significand as
  // round(m 2^60), m in [0.5, 1) (its exponent is in emax_shift)
  const int* te_in;
  int* te_out;
  long long scale_fx;
};

// i k y for the frequency of index idx (fftfreq: idx - n above (n-1)/2,
// except along a half-spectrum dimension)
template <typename R>
__device__ __forceinline__ Cx<R> mul_ik(Cx<R> y, int64_t idx, int half, int64_t n, float k0h, float k0l) {
  const int64_t f = (half || idx <= (n - 1) / 2) ? idx : idx - n;
  R k;
  if constexpr (std::is_same<R, dd>::value) k = dd(k0h, k0l) * dd((float)f, 0.0f);
  else k = k0h * (float)f;
  return mk(-(y.im * k), y.re * k);
}

// Threads per CTA of the fast pass (8 points of one line per thread) and
// CTAs per SM, measured on GB300 (512^3 round trip):
//   dd:    256 threads, 4 CTAs/SM (64 registers): the CTAs' load and
//          compute phases interleave (two CTAs: 5.87 ms against 6.58 ms with
//          one 512-thread CTA; three: 5.43 ms against 5.63 ms with two; four:
//          4.70 ms against 4.91 ms with three; 128-thread CTAs: 5.81 ms);
//          512 threads when a line needs them (M = 4096).
//   float: 512 threads, 3 CTAs/SM (register cap 42): 1.75 ms against 1.84 ms
//          with 2 CTAs/SM and 1.80 ms with four 256-thread CTAs.
#ifndef PFGB_FAST_THREADS_F32
#define PFGB_FAST_THREADS_F32 512
#endif
#ifndef PFGB_FAST_THREADS_DD
#define PFGB_FAST_THREADS_DD 256
#endif
// float lines of 1024 points and more (c2c, r2c): CTAs of 1024 threads, so
// that a tile still holds 8 lines (64-byte runs per position on strided
// axes); measured on the 1024^3 Float32 round trip, y passes 2.45 -> 2.28 ms,
// first backward pass 3.31 -> 2.79 ms.  c2r keeps 512 threads (at 1024 it
// spills or runs one CTA per SM: 2.65 -> 3.42 ms).
#ifndef PFGB_FAST_THREADS_F32_LONG
#define PFGB_FAST_THREADS_F32_LONG 1024
#endif
// Points per thread: 8, or 16 for Float32 lines of 2^PFGB_FAST_P16_LOGM
// points and more.  With 16, the stages are radix-16 (dft16) and a 1024-point
// line takes two shared-memory exchanges instead of three: the Float32
// 1024-point passes are bound by those exchanges (MIO throttle, short
// scoreboard and barrier stalls, 34-43% of DRAM throughput with 8 points).
// Double-float lines keep 8 (their registers are full).
#ifndef PFGB_FAST_P16_LOGM
#define PFGB_FAST_P16_LOGM 10
#endif
// CTA size of the 16-point Float32 passes (8 lines of 1024 points a tile)
#ifndef PFGB_FAST_THREADS_F32_P16
#define PFGB_FAST_THREADS_F32_P16 512
#endif
template <typename R>
__host__ __device__ constexpr int fast_pts(int logm) {
  return sizeof(R) == 4 && logm >= PFGB_FAST_P16_LOGM ? 16 : 8;
}

// Operations of the fast pass that pack two real lines in one complex line.
__host__ __device__ constexpr bool fast_packed(int op) {
  return op == OP_R2C || op == OP_C2R || op == OP_X00R || op == OP_D2R || op == OP_D3R || op == OP_D4R;
}
// REDFT11 / RODFT11 through one DFT of twice their length
__host__ __device__ constexpr bool fast_d4(int op) { return op == OP_D4C || op == OP_D4R; }
// REDFT10 / 01 and RODFT10 / 01 through one DFT of their length
__host__ __device__ constexpr bool fast_d23(int op) {
  return op == OP_D2C || op == OP_D2R || op == OP_D3C || op == OP_D3R;
}

template <typename R>
__host__ __device__ constexpr int fast_threads(int logm, int op = OP_C2C) {
  return sizeof(R) == 4
             ? (fast_pts<R>(logm) == 16
                    ? ((1 << logm) / 16 > PFGB_FAST_THREADS_F32_P16 ? (1 << logm) / 16 : PFGB_FAST_THREADS_F32_P16)
                : logm >= 10 && op != OP_C2R ? PFGB_FAST_THREADS_F32_LONG
                                             : PFGB_FAST_THREADS_F32)
             : ((1 << logm) / 8 > PFGB_FAST_THREADS_DD ? (1 << logm) / 8 : PFGB_FAST_THREADS_DD);
}
// complex lines per CTA for a line of 2^logm points (one line at least)
template <typename R>
__host__ __device__ constexpr int fast_tw(int logm, int op = OP_C2C) {
  return (fast_threads<R>(logm, op) * fast_pts<R>(logm)) >> logm > 0
             ? ((fast_threads<R>(logm, op) * fast_pts<R>(logm)) >> logm)
             : 1;
}
// Shared-memory padding of the exchange buffer: one pad slot every 2^shift
// elements plus `extra` slots per line.  Chosen from a bank model of the stage
// writes/reads for both thread mappings; the best extra depends on the element
// size and on the lines per CTA (tw).  8-byte elements: <= 1.25 wavefronts
// per access for M >= 128; 16-byte elements: conflict-free for M >= 64.
__host__ __device__ constexpr int fast_pad_shift(int logm, int ebytes) {
  return ebytes == 16 ? (logm <= 5 ? 2 : 3) : (logm <= 6 ? 2 : 4);
}
__host__ __device__ constexpr int fast_pitch_extra(int tw, int ebytes) {
  return ebytes == 16 ? (tw >= 8 ? 1 : tw == 4 ? 2 : tw == 2 ? 4 : 0)
                      : (tw >= 16 ? 1 : tw == 8 ? 2 : tw == 4 ? 4 : tw == 2 ? 8 : 0);
}
// bytes of one element of the exchange layout
template <typename R>
__host__ __device__ constexpr int fast_xbytes() {
  return (int)sizeof(Cx<R>);
}
template <typename R>
__host__ __device__ constexpr int fast_pitch(int logm, int op = OP_C2C) {
  return (1 << logm) + ((1 << logm) >> fast_pad_shift(logm, fast_xbytes<R>())) +
         fast_pitch_extra(fast_tw<R>(logm, op), fast_xbytes<R>());
}
template <typename R>
__host__ __device__ constexpr size_t fast_smem(int logm, int op = OP_C2C) {
  return (size_t)fast_tw<R>(logm, op) * fast_pitch<R>(logm, op) * sizeof(Cx<R>);
}

template <typename R>
struct FastIO;

template <>
struct FastIO<float> {
  using MR = float;
  using MC = float2;
  static constexpr bool kDD = false;
  static constexpr bool kFX = false;
};
template <>
struct FastIO<dd> {
  using MR = double;
  using MC = double2;
  static constexpr bool kDD = true;
  static constexpr bool kFX = false;
};
template <>
struct FastIO<fx> {
  using MR = double;
  using MC = double2;
  static constexpr bool kDD = false;
  static constexpr bool kFX = true;
};

template <typename R>
__device__ __forceinline__ Cx<R> ldg_tw(const void* t, int m) {
  if constexpr (std::is_same<R, dd>::value) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(t) + m);
    return mk(dd(q.x, q.y), dd(q.z, q.w));
  } else {
    const float2 q = __ldg(reinterpret_cast<const float2*>(t) + m);
    return mk(q.x, q.y);
  }
}

template <typename R>
__device__ __forceinline__ R half(R x) {
  if constexpr (std::is_same<R, dd>::value) return dd(x.h * 0.5f, x.l * 0.5f);
  else if constexpr (std::is_same<R, fx>::value) return fx(x.v >> 1);
  else return x * 0.5f;
}

// v * exp(SIGN 2 pi i m / M) from the pass's twiddle table (fx tables hold
// the pass's sign already)
template <typename R, int SIGN>
__device__ __forceinline__ Cx<R> tw_mul(Cx<R> v, const void* tw, int m) {
  if constexpr (std::is_same<R, fx>::value) {
    const int4 q = __ldg(reinterpret_cast<const int4*>(tw) + m);
    fx_twiddle(v.re, v.im, fx_tw{q.x, q.y, q.z, q.w});
    return v;
  } else {
    Cx<R> w = ldg_tw<R>(tw, m);
    if (SIGN > 0) w = conj(w);
    return v * w;
  }
}

// Shared-memory slot of element pos of complex line p (padding avoids bank
// conflicts for the strided stage writes and the across-line accesses).
template <typename R, int LOGM>
__host__ __device__ constexpr int padded(int pos) {
  return pos + (pos >> fast_pad_shift(LOGM, fast_xbytes<R>()));
}
template <typename R, int LOGM, int OP>
__device__ __forceinline__ int sidx(int p, int pos) {
  return p * fast_pitch<R>(LOGM, OP) + padded<R, LOGM>(pos);
}
// Exchange element i of a tile's shared-memory buffer z.
template <typename R, int LOGM, int OP>
__device__ __forceinline__ void xst(Cx<R>* z, int i, const Cx<R>& v) {
  z[i] = v;
}
template <typename R, int LOGM, int OP>
__device__ __forceinline__ Cx<R> xld(const Cx<R>* z, int i) {
  return z[i];
}
// The padding is additive over the exchange patterns: with all sizes powers
// of two, padded(p0 + r L) = padded(p0) + padded(r L) for 0 <= r < 8 when
// p0 = b < T = M/8 and L = T (stage reads), and when p0 = 8 Ls m + j with
// j < Ls and L = Ls (stage writes): a thread forms one base address and
// reaches its 8 slots at compile-time offsets.

// Barrier of a stage exchange.  Each thread reads and writes only its own
// line's slots, so with lines along the thread index (line p = threads
// p T .. p T + T - 1) the T threads of a line synchronise alone: a named
// barrier per line (ids 1..lines, T a multiple of 32) or a warp barrier when
// a warp holds whole lines.  With lines across the thread index (strided
// axis, lanes along the tile dimension) every warp holds every line.
template <typename R, int LOGM, int OP, int P = 8>
__device__ __forceinline__ void line_sync(bool lanes_across_lines, int p) {
  constexpr int T = (1 << LOGM) / P;
  if (lanes_across_lines || T == fast_threads<R>(LOGM, OP)) {
    __syncthreads();
  } else if constexpr (T <= 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + p), "r"(T) : "memory");
  }
}

// The register stages of a line of M = 2^LOGM points, P points a thread
// (positions b + r M/P): radix-P stages (dft8 or dft16), then one radix-2,
// 4 or 8 stage when log2 M is not a multiple of log2 P; outputs left in
// natural order at the same positions.  ZH: the inputs at positions M/2 and
// above are zero (v[4..7] with P = 8) and are not read.
template <typename R, int LOGM, int SIGN, int OP, int P = 8, bool ZH = false>
__device__ __forceinline__ void fast_stages(Cx<R> (&v)[P], Cx<R>* z, int p, int b, const void* tw,
                                            bool lanes_across_lines) {
  static_assert(!ZH || P == 8, "zero upper half: 8 points a thread");
  constexpr int M = 1 << LOGM;
  constexpr int T = M / P;
  constexpr int LP = P == 16 ? 4 : 3;
  constexpr int SP = LOGM / LP;
  constexpr int REM = LOGM % LP;
  constexpr int NST = SP + (REM ? 1 : 0);
  int Ls = 1;
#pragma unroll
  for (int s = 0; s < NST; ++s) {
    const bool last = (s == NST - 1);
    if (s < SP) {
      const int j = b & (Ls - 1);
      if (Ls > 1) {
        const int step = j * (M / (P * Ls));
#pragma unroll
        for (int r = 1; r < P; ++r) v[r] = tw_mul<R, SIGN>(v[r], tw, r * step);
      }
      if constexpr (P == 16) dft16<SIGN>(v);
      else if (ZH && s == 0) dft8_zh<SIGN>(v);
      else dft8<SIGN>(v);
      if (!last) {
        const int zw = sidx<R, LOGM, OP>(p, (b - j) * P + j);
#pragma unroll
        for (int r = 0; r < P; ++r) xst<R, LOGM, OP>(z, zw + padded<R, LOGM>(r * Ls), v[r]);
      }
      Ls *= P;
    } else {
      // final radix-2, 4 or 8 stage, Ls = M / RS: butterfly beta = b + r1 T
      constexpr int RS = 1 << (REM ? REM : 1);
      constexpr int G = P / RS;
#pragma unroll
      for (int r1 = 0; r1 < G; ++r1) {
        const int beta = b + r1 * T;
#pragma unroll
        for (int q = 1; q < RS; ++q) v[r1 + q * G] = tw_mul<R, SIGN>(v[r1 + q * G], tw, q * beta);
        if constexpr (RS == 2) {
          dft2<SIGN>(v[r1], v[r1 + G]);
        } else if constexpr (RS == 4) {
          dft4<SIGN>(v[r1], v[r1 + G], v[r1 + 2 * G], v[r1 + 3 * G]);
        } else {
          Cx<R> t[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) t[q] = v[r1 + q * G];
          dft8<SIGN>(t);
#pragma unroll
          for (int q = 0; q < 8; ++q) v[r1 + q * G] = t[q];
        }
      }
    }
    if (!last) {
      line_sync<R, LOGM, OP, P>(lanes_across_lines, p);
      const int zr = sidx<R, LOGM, OP>(p, b);
#pragma unroll
      for (int r = 0; r < P; ++r) v[r] = xld<R, LOGM, OP>(z, zr + padded<R, LOGM>(r * T));
      line_sync<R, LOGM, OP, P>(lanes_across_lines, p);
    }
  }
}

template <typename R>
__device__ __forceinline__ R mkr(typename FastIO<R>::MR x, int emax) {
  if constexpr (FastIO<R>::kDD) return d2dd(x, emax);
  else return x;
}
template <typename R>
__device__ __forceinline__ typename FastIO<R>::MR outr(R x, int emax) {
  if constexpr (FastIO<R>::kDD) return dd2d(x, emax);
  else return x;
}

// dd form of a complex value in memory: (re.hi, re.lo, im.hi, im.lo)
template <typename R>
__device__ __forceinline__ Cx<R> ld_dd4(float4 q) {
  if constexpr (std::is_same<R, dd>::value) return mk(dd(q.x, q.y), dd(q.z, q.w));
  else return mk(q.x, q.z);
}
template <typename R>
__device__ __forceinline__ float4 st_dd4(Cx<R> y) {
  if constexpr (std::is_same<R, dd>::value) return make_float4(y.re.h, y.re.l, y.im.h, y.im.l);
  else return make_float4(y.re, 0.f, y.im, 0.f);
}

template <typename R>
__device__ __forceinline__ Cx<R> apply_scale(Cx<R> y, const FastArgs& a) {
  if (!a.scale_on) return y;
  if constexpr (std::is_same<R, fx>::value) {
    const fx s(a.scale_fx);
    return mk(y.re * s, y.im * s);
  } else if constexpr (std::is_same<R, dd>::value) {
    const dd s(a.scale_h, a.scale_l);
    return mk(y.re * s, y.im * s);
  } else {
    return mk(y.re * a.scale_h, y.im * a.scale_h);
  }
}

// float CTAs of 512 threads: four per SM (32 registers, no spill) for c2c
// and r2c kernels, three (40 registers) for c2r, which spills at 32
#ifndef PFGB_FAST_F32_MINBLOCKS
#define PFGB_FAST_F32_MINBLOCKS 4
#endif
// dd CTAs of 256 threads: four per SM (64 registers), measured per 512^3
// round trip: 4.52 ms against 4.63 ms with five (48 registers, 20-56 bytes of
// spill) and 4.91 ms with three (80 registers); in an earlier build three
// against two (123 registers) gave 5.43 against 5.63 ms: this issue-bound
// kernel gains from resident warps until spills take over.  The variants
// (operation, dd or double input, dd or double output) are separate kernels
// so that each allocates registers for its own paths only (at 64 registers
// 0-16 bytes of spill, against 96-140 with all paths in one kernel).  A c2r
// pass with double input would spill 0.4-0.6 KB at 48 registers and stays at
// four when more are asked for.  0 selects 128 registers a thread.
#ifndef PFGB_FAST_DD_MINBLOCKS
#define PFGB_FAST_DD_MINBLOCKS 4
#endif
// kernel variant: operation OP and IOM = dd input (bit 0) | dd output (bit 1)
template <typename R>
__host__ __device__ constexpr int fast_min_blocks(int logm, int op, int iom) {
  return sizeof(R) == 4 && fast_pts<R>(logm) == 16
             ? (fast_threads<R>(logm, op) >= 1024 ? 1 : 2)  // 16 points: 64 registers a thread
         : sizeof(R) == 4 && (op == OP_CSUM || fast_d23(op) || fast_d4(op))
             // the sum's terms; the two loads a position of D3: ~0.2-0.5 KB of spill at 32 registers
             ? (fast_threads<R>(logm, op) >= 1024 ? 1 : 2)
         : sizeof(R) == 4
             ? (op == OP_C2R && fast_threads<R>(logm, op) >= 1024
                    ? 1  // c2r at 1024 threads spills heavily at 32 registers
                    : ((op == OP_C2R && PFGB_FAST_F32_MINBLOCKS > 3 ? 3 : PFGB_FAST_F32_MINBLOCKS) <
                               2048 / fast_threads<R>(logm, op)
                           ? (op == OP_C2R && PFGB_FAST_F32_MINBLOCKS > 3 ? 3 : PFGB_FAST_F32_MINBLOCKS)
                           : 2048 / fast_threads<R>(logm, op)))
         : fast_threads<R>(logm, op) >= 512 ? 1
         : (fast_d23(op) || fast_d4(op)) ? 3  // two loads a position (D3) or two real lines (D2R / D3R): ~0.2-0.5 KB of spill at 64 registers
         : PFGB_FAST_DD_MINBLOCKS <= 0 ? 512 / fast_threads<R>(logm, op)
         : (op == OP_C2R && !(iom & 1) && PFGB_FAST_DD_MINBLOCKS > 4) ? 4
                                                                     : PFGB_FAST_DD_MINBLOCKS;
}

// Origin of tile `bid` (< 2^31) of a pass: first line t0 along the tile
// dimension, element offsets of the tile in the pass input and output, and
// the index along the derivative dimension when that is an outer one.  The
// divisions are multiply-and-shift pairs prepared on the host.
struct TileOrigin {
  int64_t t0, ioff, ooff, didx;
  unsigned tebase;  // te_rescale: the outer dimensions' part of the first-pass tile index
};
__device__ __forceinline__ TileOrigin tile_origin(const FastArgs& a, unsigned bid, int lines) {
  unsigned rest = div31(bid, a.div_tiles);
  const unsigned tile = bid - rest * (unsigned)a.ntiles;
  TileOrigin o;
  o.t0 = (int64_t)tile * lines;
  o.ioff = o.t0 * a.in_st;
  o.ooff = o.t0 * a.out_st;
  o.didx = 0;
  o.tebase = 0;
  for (int d = 0; d < a.nouter; ++d) {
    const unsigned q = div31(rest, a.div_osz[d]);
    const int64_t idx = rest - q * (unsigned)a.osz[d];
    rest = q;
    o.ioff += idx * a.in_so[d];
    o.ooff += idx * a.out_so[d];
    if (a.deriv && a.deriv_role == 2 + d) o.didx = idx;
    o.tebase += ((unsigned)idx >> a.te_sh[2 + d]) * a.te_mul[2 + d];
  }
  return o;
}

// Scale exponent of the thread's complex line in the first pass of a run
// (self_scale): the largest biased exponent over the line (over the tile when
// lines lie across the thread index).  The lines' leaders record it for the
// next pass and fold it into the run's exponent word.  Called by all threads.
template <typename R, int LOGM, int OP, int P = 8>
__device__ __forceinline__ int line_exponent(unsigned emx, const FastArgs& a, unsigned bid, int64_t t0,
                                             int p, int nvalid_cl, bool lanes_across_lines) {
  constexpr int T = (1 << LOGM) / P;
  constexpr int TW = (fast_threads<R>(LOGM, OP) * P) >> LOGM > 0 ? (fast_threads<R>(LOGM, OP) * P) >> LOGM : 1;
  __shared__ unsigned wmax[32];
  unsigned e;
  bool leader;
  if (lanes_across_lines || T == fast_threads<R>(LOGM, OP)) {
    emx = __reduce_max_sync(0xFFFFFFFFu, emx);
    const int nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = emx;
    __syncthreads();
    e = 0;
    for (int w = 0; w < nw; ++w) e = max(e, wmax[w]);
    __syncthreads();  // wmax is reused by the next tile of a persistent CTA
    leader = lanes_across_lines ? (int)threadIdx.x < TW : threadIdx.x == 0;
  } else if constexpr (T <= 32) {
    const unsigned mask = (T == 32 ? 0xFFFFFFFFu : ((1u << T) - 1u)) << ((p * T) & 31);
    e = __reduce_max_sync(mask, emx);
    leader = (threadIdx.x % T) == 0;
  } else {
    emx = __reduce_max_sync(0xFFFFFFFFu, emx);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = emx;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + p), "r"(T) : "memory");
    e = 0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) e = max(e, wmax[p * (T / 32) + w]);
    leader = (threadIdx.x % T) == 0;
  }
  // leader of line q: line p in the per-line branches, thread q in the
  // tile-wide branch (all lines share e)
  const int q = (lanes_across_lines && !(T == fast_threads<R>(LOGM, OP))) ? (int)threadIdx.x
                : (T == fast_threads<R>(LOGM, OP) ? 0 : p);
  if (leader && q < nvalid_cl) {
    constexpr int pk = fast_packed(OP) ? 2 : 1;
    const unsigned rest = div31(bid, a.div_tiles);
    if (a.te) a.te[t0 / pk + q + a.te_ncl * rest] = (int)e;
    if ((int)e > *reinterpret_cast<const volatile int*>(a.emax_ptr)) atomicMax(const_cast<int*>(a.emax_ptr), (int)e);
  }
  return (int)e;
}
__device__ __forceinline__ unsigned dexp_u(double x) {
  return (unsigned)(__double_as_longlong(x) >> 52) & 0x7FFu;
}
// First-pass line of the element at axis coordinate pos of the line at
// coordinate line along the tile dimension (te_rescale), its recorded
// exponent, and 2^(d) for the difference d to the run exponent (d <= 0).
__device__ __forceinline__ unsigned te_index(const FastArgs& a, unsigned tebase, int64_t line, int pos) {
  return tebase + ((unsigned)line >> a.te_sh[1]) * a.te_mul[1] + ((unsigned)pos >> a.te_sh[0]) * a.te_mul[0];
}
// Index along outer dimension d of tile `bid` (the multiply-and-shift decode
// of tile_origin).
__device__ __forceinline__ int64_t outer_index(const FastArgs& a, unsigned bid, int d) {
  unsigned rest = div31(bid, a.div_tiles);
  for (int q = 0; q < d; ++q) rest = div31(rest, a.div_osz[q]);
  return (int64_t)(rest - div31(rest, a.div_osz[d]) * (unsigned)a.osz[d]);
}
__device__ __forceinline__ float pow2_le0(int d) {
  return d >= -126 ? __uint_as_float((unsigned)(d + 127) << 23) : 0.0f;
}
__device__ __forceinline__ float te_factor(const FastArgs& a, unsigned tebase, int64_t line, int pos, int erun) {
  return pow2_le0(__ldg(a.te + te_index(a, tebase, line, pos)) - erun);
}
template <typename R>
__device__ __forceinline__ Cx<R> scale_pow2(Cx<R> y, float f) {
  if constexpr (std::is_same<R, dd>::value) return mk(dd(y.re.h * f, y.re.l * f), dd(y.im.h * f, y.im.l * f));
  else return mk(y.re * f, y.im * f);
}

// Element pos of the extension (length M) of a REDFT00 line (even: x[0..n-1],
// n = M/2 + 1, then x[n-2..1]) or of a RODFT00 line (odd: 0, x[0..n-1], 0,
// -x[n-1..0], n = M/2 - 1): returns the input index and sets its sign s (0:
// the element is zero).
__device__ __forceinline__ int x00_src(int pos, int M, int odd, int& s) {
  const int h = M >> 1;
  if (!odd) {
    s = 1;
    return pos <= h ? pos : M - pos;
  }
  if (pos == 0 || pos == h) {
    s = 0;
    return 0;
  }
  s = pos < h ? 1 : -1;
  return pos < h ? pos - 1 : M - pos - 1;
}
// Output k of a REDFT00 / RODFT00 line (k < n): the extension's DFT Z at k
// (even), i Z at k + 1 (odd); the register position of the store-direct path
// holds output pos (even) or pos - 1 (odd).
template <typename R>
__device__ __forceinline__ Cx<R> x00_out(Cx<R> z, int odd) {
  return odd ? mul_i(z) : z;
}

// State of one tile of the register pass between its load and its store.
struct FastTile {
  TileOrigin o;
  int64_t t0, ooff, didx, ioff;
  int nvalid, ncl_valid;  // lines (complex lines) of the tile with data
  int emax, emax_out;     // dd: exponent of the loaded values, of the outputs
};

// Tile `bid` of the pass (valid == false: a tile without lines, whose loads
// and stores are all masked)
template <typename R, int LOGM, int OP>
__device__ __forceinline__ FastTile fast_tile_begin(const FastArgs& a, int64_t bid, int64_t soff, bool valid) {
  constexpr bool packed = fast_packed(OP);
  constexpr int TW = fast_tw<R>(LOGM, OP);
  const int lines = packed ? 2 * TW : TW;
  FastTile s;
  s.o = tile_origin(a, (unsigned)bid, lines);
  s.t0 = s.o.t0;
  s.ooff = s.o.ooff;
  s.didx = s.o.didx;
  s.ioff = soff >= 0 ? soff : s.o.ioff;
  s.nvalid = valid ? (int)min((int64_t)lines, a.nt - s.t0) : 0;
  s.ncl_valid = packed ? (s.nvalid + 1) / 2 : s.nvalid;
  s.emax = s.emax_out = 0;
  return s;
}

// Load of a tile: v[r] = line p, element b + r T (the stage-1 Stockham
// inputs), converted to the arithmetic type; dd: the tile's exponents in s.
template <typename R, int LOGM, int SIGN, int OP, int IOM>
__device__ __forceinline__ void fast_tile_load(const FastArgs& a, int64_t bid, const void* src, int64_t ssa,
                                               int64_t sst, int p, int b, FastTile& s,
                                               Cx<R> (&v)[fast_pts<R>(LOGM)]) {
  using IO = FastIO<R>;
  constexpr bool IN_DD = IO::kDD && (IOM & 1) != 0;   // input in dd form
  constexpr bool OUT_DD = IO::kDD && (IOM & 2) != 0;  // output in dd form
  using MR = typename IO::MR;
  using MC = typename IO::MC;
  constexpr int M = 1 << LOGM;
  constexpr int P = fast_pts<R>(LOGM);  // points a thread
  constexpr int T = M / P;
  constexpr int TW = fast_tw<R>(LOGM, OP);
  const TileOrigin& o = s.o;
  const int64_t t0 = s.t0, didx = s.didx, ioff = s.ioff;
  const int nvalid = s.nvalid, ncl_valid = s.ncl_valid;
  int& emax = s.emax;
  int& emax_out = s.emax_out;
  if constexpr (IO::kDD) {
    if (!a.self_scale) {
      emax = *a.emax_ptr;
      emax_out = emax + a.emax_shift;
    }
  }
  if constexpr (OP == OP_C2C || OP == OP_C2CT) {
    if (IO::kDD && IN_DD) {
      const float4* in = reinterpret_cast<const float4*>(src) + ioff + (int64_t)p * sst;
      // exponents of the elements' first-pass lines, loaded ahead of the data
      int tev[P];
      if (IO::kDD && a.te_rescale) {
#pragma unroll
        for (int r = 0; r < P; ++r) tev[r] = p < nvalid ? __ldg(a.te + te_index(a, o.tebase, t0 + p, b + r * T)) : emax;
      }
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const float4 q = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : make_float4(0.f, 0.f, 0.f, 0.f);
        v[r] = ld_dd4<R>(q);
      }
      if (IO::kDD && a.te_rescale) {
        bool off = false;
#pragma unroll
        for (int r = 0; r < P; ++r) off |= tev[r] != emax;
        if (__any_sync(0xFFFFFFFFu, off)) {  // lines below the run exponent in this warp
#pragma unroll
          for (int r = 0; r < P; ++r) v[r] = scale_pow2(v[r], pow2_le0(tev[r] - emax));
        }
      }
    } else {
      // all loads first, conversions after: the conversion's rare-case
      // branch must not serialise the loads
      const MC* in = reinterpret_cast<const MC*>(src) + ioff + (int64_t)p * sst;
      MC raw[P];
#pragma unroll
      for (int r = 0; r < P; ++r) raw[r] = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : MC{0, 0};
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < P; ++r) emx = max(emx, max(dexp_u(raw[r].x), dexp_u(raw[r].y)));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < P; ++r) v[r] = mk(mkr<R>(raw[r].x, emax), mkr<R>(raw[r].y, emax));
    }
    if (a.deriv == 1) {
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int64_t idx = a.deriv_role == 0 ? (int64_t)(b + r * T) : a.deriv_role == 1 ? t0 + p : didx;
        v[r] = mul_ik(v[r], idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
      }
    }
  } else if constexpr (OP == OP_CSUM) {
    // sum over the terms of i k_t(idx) src_t, converted with one line
    // exponent over all terms (first loop: exponents only; second: values)
    int64_t tidx[kMaxTerms];
#pragma unroll
    for (int t = 0; t < kMaxTerms; ++t)
      tidx[t] = (t < a.nterm && a.trole[t] >= 2) ? outer_index(a, (unsigned)bid, a.trole[t] - 2) : 0;
    if constexpr (IO::kDD) {
      if (a.self_scale) {
        unsigned emx = 0;
        for (int t = 0; t < a.nterm; ++t) {
          const MC* in = reinterpret_cast<const MC*>(a.tsrc[t]) + ioff + (int64_t)p * sst;
#pragma unroll
          for (int r = 0; r < P; ++r) {
            const MC q = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : MC{0, 0};
            emx = max(emx, max(dexp_u(q.x), dexp_u(q.y)));
          }
        }
        emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
        emax_out = emax + a.emax_shift;
      }
    }
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = mk(R(0), R(0));
    for (int t = 0; t < a.nterm; ++t) {
      const MC* in = reinterpret_cast<const MC*>(a.tsrc[t]) + ioff + (int64_t)p * sst;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const MC q = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : MC{0, 0};
        const int64_t idx = a.trole[t] == 0 ? (int64_t)(b + r * T) : a.trole[t] == 1 ? t0 + p : tidx[t];
        v[r] = v[r] + mul_ik(mk(mkr<R>(q.x, emax), mkr<R>(q.y, emax)), idx, a.thalf[t], a.tn[t],
                             a.tk0_h[t], a.tk0_l[t]);
      }
    }
  } else if constexpr (OP == OP_X00C) {
    // complex lines through the even / odd extension
    const int odd = a.r2r_odd;
    if (IO::kDD && IN_DD) {
      const float4* in = reinterpret_cast<const float4*>(src) + ioff + (int64_t)p * sst;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        int sg;
        const int k = x00_src(b + r * T, M, odd, sg);
        const float4 q = (p < nvalid && sg) ? in[(int64_t)k * ssa] : make_float4(0.f, 0.f, 0.f, 0.f);
        Cx<R> y = ld_dd4<R>(q);
        if (IO::kDD && a.te_rescale && p < nvalid && sg) y = scale_pow2(y, te_factor(a, o.tebase, t0 + p, k, emax));
        v[r] = sg < 0 ? -y : y;
      }
    } else {
      const MC* in = reinterpret_cast<const MC*>(src) + ioff + (int64_t)p * sst;
      MC raw[P];
      int sgs[P];
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int k = x00_src(b + r * T, M, odd, sgs[r]);
        raw[r] = (p < nvalid && sgs[r]) ? in[(int64_t)k * ssa] : MC{0, 0};
      }
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < P; ++r) emx = max(emx, max(dexp_u(raw[r].x), dexp_u(raw[r].y)));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const Cx<R> y = mk(mkr<R>(raw[r].x, emax), mkr<R>(raw[r].y, emax));
        v[r] = sgs[r] < 0 ? -y : y;
      }
    }
  } else if constexpr (OP == OP_X00R) {
    // two real lines (2p, 2p + 1) through the even / odd extension; double input
    const int odd = a.r2r_odd;
    const MR* in = reinterpret_cast<const MR*>(src) + ioff;
    const int i0 = 2 * p, i1 = 2 * p + 1;
    MR ra[P], rb[P];
    int sgs[P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const int k = x00_src(b + r * T, M, odd, sgs[r]);
      const int64_t off = (int64_t)k * ssa;
      ra[r] = (i0 < nvalid && sgs[r]) ? in[off + (int64_t)i0 * sst] : MR(0);
      rb[r] = (i1 < nvalid && sgs[r]) ? in[off + (int64_t)i1 * sst] : MR(0);
    }
    if constexpr (IO::kDD) {
      if (a.self_scale) {
        unsigned emx = 0;
#pragma unroll
        for (int r = 0; r < P; ++r) emx = max(emx, max(dexp_u(ra[r]), dexp_u(rb[r])));
        emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
        emax_out = emax + a.emax_shift;
      }
    }
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const Cx<R> y = mk(mkr<R>(ra[r], emax), mkr<R>(rb[r], emax));
      v[r] = sgs[r] < 0 ? -y : y;
    }
  } else if constexpr (fast_d23(OP)) {
    // REDFT10 / RODFT10 / DHT (D2) and REDFT01 / RODFT01 (D3) through one
    // M-point DFT (the identities at OP_D2C in pfgb_device.cuh), on complex
    // lines or two real lines packed in one.  Register r holds the DFT input
    // at position pos = b + r T: D2 the source x[ja] (negated at odd ja for
    // RODFT10; ja = pos for the DHT), D3 conj(w_pos) (y[ja] - i y[jb])
    // (jb < 0: y[M] = 0).
    constexpr bool D3 = OP == OP_D3C || OP == OP_D3R;
    constexpr bool PK = OP == OP_D2R || OP == OP_D3R;
    const int odd = a.r2r_odd;
    int ja[P], jb[P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const int pos = b + r * T;
      if constexpr (!D3) {
        ja[r] = odd == 2 ? pos : pos < M / 2 ? 2 * pos : 2 * (M - 1 - pos) + 1;  // DHT: in order
        jb[r] = -1;
      } else {
        ja[r] = odd ? M - 1 - pos : pos;
        jb[r] = pos == 0 ? -1 : (odd ? pos - 1 : M - pos);
      }
    }
    Cx<R> ya[P], yb[P];
    if constexpr (PK) {
      const MR* in = reinterpret_cast<const MR*>(src) + ioff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
      MR a0[P], a1[P], b0[P], b1[P];
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int64_t oa = (int64_t)ja[r] * ssa, ob = (int64_t)(jb[r] < 0 ? 0 : jb[r]) * ssa;
        a0[r] = i0 < nvalid ? in[oa + (int64_t)i0 * sst] : MR(0);
        a1[r] = i1 < nvalid ? in[oa + (int64_t)i1 * sst] : MR(0);
        b0[r] = (D3 && jb[r] >= 0 && i0 < nvalid) ? in[ob + (int64_t)i0 * sst] : MR(0);
        b1[r] = (D3 && jb[r] >= 0 && i1 < nvalid) ? in[ob + (int64_t)i1 * sst] : MR(0);
      }
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < P; ++r)
            emx = max(emx, max(max(dexp_u(a0[r]), dexp_u(a1[r])), max(dexp_u(b0[r]), dexp_u(b1[r]))));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < P; ++r) {
        ya[r] = mk(mkr<R>(a0[r], emax), mkr<R>(a1[r], emax));
        yb[r] = mk(mkr<R>(b0[r], emax), mkr<R>(b1[r], emax));
      }
    } else if (IO::kDD && IN_DD) {
      const float4* in = reinterpret_cast<const float4*>(src) + ioff + (int64_t)p * sst;
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int r = 0; r < P; ++r) {
        ya[r] = ld_dd4<R>(p < nvalid ? in[(int64_t)ja[r] * ssa] : z4);
        yb[r] = ld_dd4<R>((D3 && jb[r] >= 0 && p < nvalid) ? in[(int64_t)jb[r] * ssa] : z4);
        if (IO::kDD && a.te_rescale && p < nvalid) {
          ya[r] = scale_pow2(ya[r], te_factor(a, o.tebase, t0 + p, ja[r], emax));
          if (D3 && jb[r] >= 0) yb[r] = scale_pow2(yb[r], te_factor(a, o.tebase, t0 + p, jb[r], emax));
        }
      }
    } else {
      const MC* in = reinterpret_cast<const MC*>(src) + ioff + (int64_t)p * sst;
      MC ra[P], rb[P];
#pragma unroll
      for (int r = 0; r < P; ++r) {
        ra[r] = p < nvalid ? in[(int64_t)ja[r] * ssa] : MC{0, 0};
        rb[r] = (D3 && jb[r] >= 0 && p < nvalid) ? in[(int64_t)jb[r] * ssa] : MC{0, 0};
      }
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < P; ++r)
            emx = max(emx, max(max(dexp_u(ra[r].x), dexp_u(ra[r].y)), max(dexp_u(rb[r].x), dexp_u(rb[r].y))));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < P; ++r) {
        ya[r] = mk(mkr<R>(ra[r].x, emax), mkr<R>(ra[r].y, emax));
        yb[r] = mk(mkr<R>(rb[r].x, emax), mkr<R>(rb[r].y, emax));
      }
    }
#pragma unroll
    for (int r = 0; r < P; ++r) {
      if constexpr (!D3) {
        v[r] = (odd == 1 && (ja[r] & 1)) ? -ya[r] : ya[r];
      } else {
        const Cx<R> u = mk(ya[r].re + yb[r].im, ya[r].im - yb[r].re);  // y[ja] - i y[jb]
        v[r] = u * conj(ldg_tw<R>(a.d23_tab, b + r * T));
      }
    }
  } else if constexpr (fast_d4(OP)) {
    // REDFT11 / RODFT11: the M-point DFT (M = 2n) of x[pos] c_pos, pos < n
    // (registers r < H = P / 2: pos = b + r T < H T = n), zero above (with
    // 8 points a thread the first stage does not read registers r >= 4)
    constexpr bool PK = OP == OP_D4R;
    constexpr int H = P / 2;
    Cx<R> y[H];
    if constexpr (PK) {
      const MR* in = reinterpret_cast<const MR*>(src) + ioff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
      MR a0[H], a1[H];
#pragma unroll
      for (int r = 0; r < H; ++r) {
        const int64_t off = (int64_t)(b + r * T) * ssa;
        a0[r] = i0 < nvalid ? in[off + (int64_t)i0 * sst] : MR(0);
        a1[r] = i1 < nvalid ? in[off + (int64_t)i1 * sst] : MR(0);
      }
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < H; ++r) emx = max(emx, max(dexp_u(a0[r]), dexp_u(a1[r])));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < H; ++r) y[r] = mk(mkr<R>(a0[r], emax), mkr<R>(a1[r], emax));
    } else if (IO::kDD && IN_DD) {
      const float4* in = reinterpret_cast<const float4*>(src) + ioff + (int64_t)p * sst;
#pragma unroll
      for (int r = 0; r < H; ++r) {
        const int pos = b + r * T;
        y[r] = ld_dd4<R>(p < nvalid ? in[(int64_t)pos * ssa] : make_float4(0.f, 0.f, 0.f, 0.f));
        if (IO::kDD && a.te_rescale && p < nvalid) y[r] = scale_pow2(y[r], te_factor(a, o.tebase, t0 + p, pos, emax));
      }
    } else {
      const MC* in = reinterpret_cast<const MC*>(src) + ioff + (int64_t)p * sst;
      MC ra[H];
#pragma unroll
      for (int r = 0; r < H; ++r) ra[r] = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : MC{0, 0};
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < H; ++r) emx = max(emx, max(dexp_u(ra[r].x), dexp_u(ra[r].y)));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
#pragma unroll
      for (int r = 0; r < H; ++r) y[r] = mk(mkr<R>(ra[r].x, emax), mkr<R>(ra[r].y, emax));
    }
#pragma unroll
    for (int r = 0; r < P; ++r)
      v[r] = r < H ? y[r < H ? r : 0] * ldg_tw<R>(a.d23_tab, b + r * T) : mk(R(0), R(0));
  } else if constexpr (OP == OP_R2C) {
    const MR* in = reinterpret_cast<const MR*>(src) + ioff;
    const int i0 = 2 * p, i1 = 2 * p + 1;
    MR ra[P], rb[P];
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const int64_t off = (int64_t)(b + r * T) * ssa;
      ra[r] = i0 < nvalid ? in[off + (int64_t)i0 * sst] : MR(0);
      rb[r] = i1 < nvalid ? in[off + (int64_t)i1 * sst] : MR(0);
    }
    if constexpr (IO::kDD) {
      if (a.self_scale) {
        unsigned emx = 0;
#pragma unroll
        for (int r = 0; r < P; ++r) emx = max(emx, max(dexp_u(ra[r]), dexp_u(rb[r])));
        emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
        emax_out = emax + a.emax_shift;
      }
    }
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = mk(mkr<R>(ra[r], emax), mkr<R>(rb[r], emax));
  } else {  // OP_C2R: Hermitian extension of two half spectra, n = M
    // m = n_in = M/2 + 1 (power-of-two M): the extension's case distinctions
    // are compile-time for every register but r = 0 and r = 4
    constexpr int m = M / 2 + 1;
    const int i0 = 2 * p, i1 = 2 * p + 1;
    MC ra[P], rb[P];
    if (!(IO::kDD && IN_DD)) {
      const MC* in = reinterpret_cast<const MC*>(src) + ioff;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int pos = b + r * T;
        const int64_t off = (int64_t)(pos < m ? pos : M - pos) * ssa;
        ra[r] = i0 < nvalid ? in[off + (int64_t)i0 * sst] : MC{0, 0};
        rb[r] = i1 < nvalid ? in[off + (int64_t)i1 * sst] : MC{0, 0};
      }
      if constexpr (IO::kDD) {
        if (a.self_scale) {
          unsigned emx = 0;
#pragma unroll
          for (int r = 0; r < P; ++r)
            emx = max(emx, max(max(dexp_u(ra[r].x), dexp_u(ra[r].y)), max(dexp_u(rb[r].x), dexp_u(rb[r].y))));
          emax = line_exponent<R, LOGM, OP, P>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
          emax_out = emax + a.emax_shift;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const int pos = b + r * T;
      const int k = pos < m ? pos : M - pos;
      const int64_t off = (int64_t)k * ssa;
      Cx<R> A, B;
      if (IO::kDD && IN_DD) {
        const float4* in = reinterpret_cast<const float4*>(src) + ioff;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        A = ld_dd4<R>(i0 < nvalid ? in[off + (int64_t)i0 * sst] : z4);
        B = ld_dd4<R>(i1 < nvalid ? in[off + (int64_t)i1 * sst] : z4);
        if (IO::kDD && a.te_rescale) {
          if (i0 < nvalid) A = scale_pow2(A, te_factor(a, o.tebase, t0 + i0, k, emax));
          if (i1 < nvalid) B = scale_pow2(B, te_factor(a, o.tebase, t0 + i1, k, emax));
        }
      } else {
        A = mk(mkr<R>(ra[r].x, emax), mkr<R>(ra[r].y, emax));
        B = mk(mkr<R>(rb[r].x, emax), mkr<R>(rb[r].y, emax));
      }
      if (k == 0 || 2 * k == M) { A.im = R(0); B.im = R(0); }
      // pos < m: A + iB ; else conj(A) + i conj(B): one formula with the
      // imaginary parts negated for the mirrored half (a free sign flip)
      if (pos >= m) { A.im = -A.im; B.im = -B.im; }
      v[r] = mk(A.re - B.im, A.im + B.re);
    }
  }
}

// Store of a tile from the stage outputs v (directly, or through z in
// shared memory for the transposed layouts and the r2c split); lexp: the
// per-line exponents of a self-scaled dd pass.
template <typename R, int LOGM, int SIGN, int OP, int IOM>
__device__ __forceinline__ void fast_tile_store(const FastArgs& a, int64_t bid, int p, int b, const FastTile& s,
                                                Cx<R> (&v)[fast_pts<R>(LOGM)], Cx<R>* z, const int* lexp) {
  using IO = FastIO<R>;
  constexpr bool IN_DD = IO::kDD && (IOM & 1) != 0;   // input in dd form
  constexpr bool OUT_DD = IO::kDD && (IOM & 2) != 0;  // output in dd form
  using MR = typename IO::MR;
  using MC = typename IO::MC;
  constexpr int M = 1 << LOGM;
  constexpr int P = fast_pts<R>(LOGM);  // points a thread
  constexpr int T = M / P;
  constexpr int TW = fast_tw<R>(LOGM, OP);
  const int tid = threadIdx.x;
  const int64_t t0 = s.t0, ooff = s.ooff, didx = s.didx;
  const int nvalid = s.nvalid;
  const int emax_out = s.emax_out;
  // ---- store ----
  if (a.deriv == 2 && a.store_direct && OP == OP_C2C) {
#pragma unroll
    for (int r = 0; r < P; ++r) {
      const int64_t idx = a.deriv_role == 0 ? (int64_t)(b + r * T) : a.deriv_role == 1 ? t0 + p : didx;
      v[r] = mul_ik(v[r], idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
    }
  }
  if constexpr (OP == OP_C2CT) {
    // the split line's twiddles W_M^(n1 k2), k2 = b + r T, before any store
    const int64_t n1 = a.t4_role == 1 ? t0 + p : outer_index(a, (unsigned)bid, a.t4_role - 2);
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = tw_mul<R, SIGN>(v[r], a.t4_tab, (int)(n1 * (int64_t)(b + r * T)));
  }
  if (a.store_direct && OP != OP_R2C && !fast_d23(OP) && !fast_d4(OP)) {
    if constexpr (OP == OP_C2C || OP == OP_CSUM || OP == OP_C2CT) {
      if (p < nvalid) {
        if (IO::kDD && OUT_DD) {
          float4* out = reinterpret_cast<float4*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < P; ++r) out[(int64_t)(b + r * T) * a.out_sa] = st_dd4(apply_scale(v[r], a));
        } else {
          MC* out = reinterpret_cast<MC*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < P; ++r) {
            const Cx<R> y = apply_scale(v[r], a);
            MC o;
            o.x = outr<R>(y.re, emax_out);
            o.y = outr<R>(y.im, emax_out);
            out[(int64_t)(b + r * T) * a.out_sa] = o;
          }
        }
      }
    } else if constexpr (OP == OP_X00C) {
      // outputs k < n: register r holds k = pos (even) or pos - 1 (odd)
      const int odd = a.r2r_odd, n = a.n_out;
      if (p < nvalid) {
#pragma unroll
        for (int r = 0; r < P; ++r) {
          const int k = b + r * T - odd;
          if (k < 0 || k >= n) continue;
          const Cx<R> y = apply_scale(x00_out(v[r], odd), a);
          if (IO::kDD && OUT_DD) {
            reinterpret_cast<float4*>(a.out)[ooff + (int64_t)p * a.out_st + (int64_t)k * a.out_sa] = st_dd4(y);
          } else {
            MC o;
            o.x = outr<R>(y.re, emax_out);
            o.y = outr<R>(y.im, emax_out);
            reinterpret_cast<MC*>(a.out)[ooff + (int64_t)p * a.out_st + (int64_t)k * a.out_sa] = o;
          }
        }
      }
    } else if constexpr (OP == OP_X00R) {
      const int odd = a.r2r_odd, n = a.n_out;
      MR* out = reinterpret_cast<MR*>(a.out) + ooff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const int k = b + r * T - odd;
        if (k < 0 || k >= n) continue;
        const Cx<R> y = apply_scale(x00_out(v[r], odd), a);
        const int64_t off = (int64_t)k * a.out_sa;
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, emax_out);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, emax_out);
      }
    } else {  // C2R, real outputs of lines 2p and 2p+1
      MR* out = reinterpret_cast<MR*>(a.out) + ooff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
#pragma unroll
      for (int r = 0; r < P; ++r) {
        const Cx<R> y = apply_scale(v[r], a);
        const int64_t off = (int64_t)(b + r * T) * a.out_sa;
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, emax_out);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, emax_out);
      }
    }
    return;
  }

  // via shared memory: transposed layouts and the r2c split
  {
    Cx<R>* zw = z + sidx<R, LOGM, OP>(p, b);
#pragma unroll
    for (int r = 0; r < P; ++r) zw[padded<R, LOGM>(r * T)] = v[r];
  }
  __syncthreads();
  // the launch's thread count (fast_pass and fast_pass_tma launch
  // fast_threads(LOGM, OP)); as a compile-time constant for dd, whose store
  // loops then get constant trip counts and index steps (r2c and c2r passes
  // of the 512^3 Float64 round trip 0.788 -> 0.778 and 0.885 -> 0.877 ms),
  // read at run time for float, whose 32-register kernels spill with the
  // unrolled loops (Float32 round trip 1.457 -> 1.504 ms)
  const int nth = sizeof(R) == 4 ? (int)blockDim.x : fast_threads<R>(LOGM, OP);
  // output exponent of complex line i (the first pass of a run scales lines
  // separately; the loops below write other threads' lines)
  auto line_emax_out = [&](int i) { return IO::kDD && a.self_scale ? lexp[i] + a.emax_shift : emax_out; };
  if constexpr (OP == OP_C2C || OP == OP_CSUM || OP == OP_C2CT) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { k = e % M; i = e / M; }
      if (i >= nvalid) continue;
      Cx<R> y = apply_scale(z[sidx<R, LOGM, OP>(i, k)], a);
      if (a.deriv == 2) {
        const int64_t idx = a.deriv_role == 0 ? (int64_t)k : a.deriv_role == 1 ? t0 + i : didx;
        y = mul_ik(y, idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
      }
      if (IO::kDD && OUT_DD) {
        reinterpret_cast<float4*>(out)[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = st_dd4(y);
      } else {
        const int eo = line_emax_out(i);
        MC o;
        o.x = outr<R>(y.re, eo);
        o.y = outr<R>(y.im, eo);
        out[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = o;
      }
    }
  } else if constexpr (OP == OP_R2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    constexpr int m = M / 2 + 1;  // n_out of a power-of-two r2c line
    const int tot = TW * m;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % m; q = e / m; }
      const Cx<R> f = z[sidx<R, LOGM, OP>(q, k)];
      const Cx<R> g = conj(z[sidx<R, LOGM, OP>(q, k == 0 ? 0 : M - k)]);
      Cx<R> A = f + g, B = mul_mi(f - g);
      if constexpr (!IO::kDD) {
        A = mk(half(A.re), half(A.im));
        B = mk(half(B.re), half(B.im));
      }  // dd: the factor 1/2 is one less in the run's output exponent (emax_shift)
      A = apply_scale(A, a);
      B = apply_scale(B, a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (IO::kDD && OUT_DD) {
        float4* o4 = reinterpret_cast<float4*>(out);
        if (i0 < nvalid) o4[off + (int64_t)i0 * a.out_st] = st_dd4(A);
        if (i1 < nvalid) o4[off + (int64_t)i1 * a.out_st] = st_dd4(B);
      } else if (!IO::kDD && a.vec2 && i1 < nvalid) {  // lines 2q, 2q+1 in one 16-byte store
        *reinterpret_cast<float4*>(out + off + i0) =
            make_float4(outr<R>(A.re, 0), outr<R>(A.im, 0), outr<R>(B.re, 0), outr<R>(B.im, 0));
      } else {
        const int eo = line_emax_out(q);
        if (i0 < nvalid) {
          MC o;
          o.x = outr<R>(A.re, eo);
          o.y = outr<R>(A.im, eo);
          out[off + (int64_t)i0 * a.out_st] = o;
        }
        if (i1 < nvalid) {
          MC o;
          o.x = outr<R>(B.re, eo);
          o.y = outr<R>(B.im, eo);
          out[off + (int64_t)i1 * a.out_st] = o;
        }
      }
    }
  } else if constexpr (OP == OP_X00C) {
    const int odd = a.r2r_odd, n = a.n_out;
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    const int tot = TW * n;
    for (int e = tid; e < tot; e += nth) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { k = e % n; i = e / n; }
      if (i >= nvalid) continue;
      const Cx<R> y = apply_scale(x00_out(z[sidx<R, LOGM, OP>(i, k + odd)], odd), a);
      if (IO::kDD && OUT_DD) {
        reinterpret_cast<float4*>(out)[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = st_dd4(y);
      } else {
        const int eo = line_emax_out(i);
        MC o;
        o.x = outr<R>(y.re, eo);
        o.y = outr<R>(y.im, eo);
        out[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = o;
      }
    }
  } else if constexpr (OP == OP_X00R) {
    const int odd = a.r2r_odd, n = a.n_out;
    MR* out = reinterpret_cast<MR*>(a.out) + ooff;
    const int tot = TW * n;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % n; q = e / n; }
      const Cx<R> y = apply_scale(x00_out(z[sidx<R, LOGM, OP>(q, k + odd)], odd), a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      const int eo = line_emax_out(q);
      if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, eo);
      if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, eo);
    }
  } else if constexpr (fast_d23(OP)) {
    // D2: Y[kk] = w_kk V[kk] + conj(w_kk) V[M - kk] at output k = kk (REDFT10)
    // or M - 1 - kk (RODFT10); D3: out[k] = v[k / 2] (k even) or
    // v[M - 1 - (k - 1) / 2] (k odd), negated at odd k for RODFT01
    constexpr bool D3 = OP == OP_D3C || OP == OP_D3R;
    constexpr bool PK = OP == OP_D2R || OP == OP_D3R;
    const int odd = a.r2r_odd;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % M; q = e / M; }
      if (!PK && q >= nvalid) continue;
      Cx<R> y;
      if constexpr (!D3) {
        const int kk = odd == 1 ? M - 1 - k : k;
        const Cx<R> f = z[sidx<R, LOGM, OP>(q, kk)];
        const Cx<R> g = z[sidx<R, LOGM, OP>(q, (M - kk) & (M - 1))];
        const Cx<R> w = ldg_tw<R>(a.d23_tab, kk);
        y = f * w + g * conj(w);
      } else {
        y = z[sidx<R, LOGM, OP>(q, (k & 1) ? M - 1 - (k >> 1) : (k >> 1))];
        if (odd && (k & 1)) y = -y;
      }
      y = apply_scale(y, a);
      const int64_t off = (int64_t)k * a.out_sa;
      if constexpr (PK) {
        MR* out = reinterpret_cast<MR*>(a.out) + ooff;
        const int i0 = 2 * q, i1 = 2 * q + 1;
        const int eo = line_emax_out(q);
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, eo);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, eo);
      } else if (IO::kDD && OUT_DD) {
        reinterpret_cast<float4*>(a.out)[ooff + off + (int64_t)q * a.out_st] = st_dd4(y);
      } else {
        const int eo = line_emax_out(q);
        MC o;
        o.x = outr<R>(y.re, eo);
        o.y = outr<R>(y.im, eo);
        reinterpret_cast<MC*>(a.out)[ooff + off + (int64_t)q * a.out_st] = o;
      }
    }
  } else if constexpr (fast_d4(OP)) {
    // outputs k < n = M / 2: d_k V[k] + conj(d_k) V[M-1-k] (REDFT11), i times
    // d_k V[k] - conj(d_k) V[M-1-k] (RODFT11); d_k at table entry n + k
    constexpr bool PK = OP == OP_D4R;
    constexpr int N = M / 2;
    const int odd = a.r2r_odd;
    const int tot = TW * N;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % N; q = e / N; }
      if (!PK && q >= nvalid) continue;
      const Cx<R> f = z[sidx<R, LOGM, OP>(q, k)] * ldg_tw<R>(a.d23_tab, N + k);
      const Cx<R> g = z[sidx<R, LOGM, OP>(q, M - 1 - k)] * conj(ldg_tw<R>(a.d23_tab, N + k));
      Cx<R> y = odd ? mul_i(f - g) : f + g;
      y = apply_scale(y, a);
      const int64_t off = (int64_t)k * a.out_sa;
      if constexpr (PK) {
        MR* out = reinterpret_cast<MR*>(a.out) + ooff;
        const int i0 = 2 * q, i1 = 2 * q + 1;
        const int eo = line_emax_out(q);
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, eo);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, eo);
      } else if (IO::kDD && OUT_DD) {
        reinterpret_cast<float4*>(a.out)[ooff + off + (int64_t)q * a.out_st] = st_dd4(y);
      } else {
        const int eo = line_emax_out(q);
        MC o;
        o.x = outr<R>(y.re, eo);
        o.y = outr<R>(y.im, eo);
        reinterpret_cast<MC*>(a.out)[ooff + off + (int64_t)q * a.out_st] = o;
      }
    }
  } else {  // C2R with a transposed output layout
    MR* out = reinterpret_cast<MR*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % M; q = e / M; }
      const Cx<R> y = apply_scale(z[sidx<R, LOGM, OP>(q, k)], a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      const int eo = line_emax_out(q);
      if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, eo);
      if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, eo);
    }
  }
}

// One tile of the register pass for float and dd (fx: fast_tile_fx): load
// (from `src`: the pass input in global memory, or a copy of the tile's input
// lines in shared memory), stages, store.  `src` is addressed as
// src[soff + pos * ssa + line * sst] (soff < 0: the tile's offset in the pass
// input).
template <typename R, int LOGM, int SIGN, int OP, int IOM>
__device__ __forceinline__ void fast_tile_std(const FastArgs& a, int64_t bid, Cx<R>* z, const void* src,
                                              int64_t soff, int64_t ssa, int64_t sst) {
  using IO = FastIO<R>;
  constexpr int P = fast_pts<R>(LOGM);
  constexpr int T = (1 << LOGM) / P;
  constexpr int TW = fast_tw<R>(LOGM, OP);
  const int tid = threadIdx.x;
  int p, b;
  if (a.lmap_tile) { p = tid % TW; b = tid / TW; } else { b = tid % T; p = tid / T; }
  FastTile s = fast_tile_begin<R, LOGM, OP>(a, bid, soff, true);
  Cx<R> v[P];
  fast_tile_load<R, LOGM, SIGN, OP, IOM>(a, bid, src, ssa, sst, p, b, s, v);
  // per-line exponents of a self-scaled pass, for the stores of other lines
  __shared__ int lexp[TW];
  if (IO::kDD && a.self_scale && b == 0) lexp[p] = s.emax;
  // (REDFT11 / RODFT11: the upper half of the DFT input is the zero padding)
  fast_stages<R, LOGM, SIGN, OP, P, fast_d4(OP) && P == 8>(v, z, p, b, a.tw, a.lmap_tile != 0);
  fast_tile_store<R, LOGM, SIGN, OP, IOM>(a, bid, p, b, s, v, z, lexp);
}

// One tile of an fx pass (R = fx).  Load: each complex line gets the scale
// 2^(et - H), et its largest exponent (values below 2^et): from the doubles'
// exponents, or from the exponent words of the fx lines its elements come
// from, each element shifted to the line's scale.  Store: double outputs are
// converted from the line's scale; fx outputs are shifted so that the line's
// largest component reaches bit 61 (bit length by a per-line OR), and the
// line's exponent word is recorded for the next pass.
template <int LOGM, int SIGN, int OP, int IOM>
__device__ __forceinline__ void fast_tile_fx(const FastArgs& a, int64_t bid, Cx<fx>* z, const void* src,
                                             int64_t soff, int64_t ssa, int64_t sst) {
  constexpr bool IN_FX = (IOM & 1) != 0;
  constexpr bool OUT_FX = (IOM & 2) != 0;
  constexpr int M = 1 << LOGM;
  constexpr int T = M / 8;
  constexpr int TW = fast_tw<fx>(LOGM, OP);
  constexpr int H = fx_head(LOGM, OP == OP_C2R);

  const int tid = threadIdx.x;
  int p, b;
  if (a.lmap_tile) { p = tid % TW; b = tid / TW; } else { b = tid % T; p = tid / T; }
  const bool packed = OP != OP_C2C;
  const int lines = packed ? 2 * TW : TW;
  const TileOrigin o = tile_origin(a, (unsigned)bid, lines);
  const int64_t t0 = o.t0, ooff = o.ooff;
  const int64_t ioff = soff >= 0 ? soff : o.ioff;
  const int nvalid = (int)min((int64_t)lines, a.nt - t0);
  const int ncl_valid = packed ? (nvalid + 1) / 2 : nvalid;

  // per complex line: [0] largest input exponent (biased double exponent, or
  // the largest exponent word), [1] bit length of the output components
  __shared__ int red[2][TW];
  if (tid < TW) {
    red[0][tid] = kTeZero;
    red[1][tid] = 0;
  }
  __syncthreads();
  // largest exponent et of complex line i (values below 2^et)
  auto line_et = [&](int i) {
    const int x = red[0][i];
    return IN_FX ? x : (x == 0x7FF ? kTeNaN : x - 1022);
  };

  Cx<fx> v[8];
  if constexpr (OP == OP_C2C) {
    if constexpr (IN_FX) {
      const longlong2* in = reinterpret_cast<const longlong2*>(src) + ioff + (int64_t)p * sst;
      longlong2 q[8];
      int tev[8];
      int tm = kTeZero;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const bool ok = p < nvalid;
        q[r] = ok ? in[(int64_t)(b + r * T) * ssa] : make_longlong2(0, 0);
        tev[r] = ok ? __ldg(a.te_in + te_index(a, o.tebase, t0 + p, b + r * T)) : kTeZero;
        tm = max(tm, tev[r]);
      }
      atomicMax(&red[0][p], tm);
      __syncthreads();
      const int sb = red[0][p] - H + 61;
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = mk(fx(fx_shr(q[r].x, sb - tev[r])), fx(fx_shr(q[r].y, sb - tev[r])));
    } else {
      const double2* in = reinterpret_cast<const double2*>(src) + ioff + (int64_t)p * sst;
      double2 raw[8];
      unsigned emx = 0;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        raw[r] = p < nvalid ? in[(int64_t)(b + r * T) * ssa] : make_double2(0.0, 0.0);
        emx = max(emx, max(dexp_u(raw[r].x), dexp_u(raw[r].y)));
      }
      atomicMax(&red[0][p], (int)emx);
      __syncthreads();
      const int base = red[0][p] + 53 - H;
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = mk(fx(d2fx(raw[r].x, base)), fx(d2fx(raw[r].y, base)));
    }
  } else if constexpr (OP == OP_R2C) {
    // two real lines (2p, 2p+1) as one complex line; always double input
    const double* in = reinterpret_cast<const double*>(src) + ioff;
    const int i0 = 2 * p, i1 = 2 * p + 1;
    double ra[8], rb[8];
    unsigned emx = 0;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int64_t off = (int64_t)(b + r * T) * ssa;
      ra[r] = i0 < nvalid ? in[off + (int64_t)i0 * sst] : 0.0;
      rb[r] = i1 < nvalid ? in[off + (int64_t)i1 * sst] : 0.0;
      emx = max(emx, max(dexp_u(ra[r]), dexp_u(rb[r])));
    }
    atomicMax(&red[0][p], (int)emx);
    __syncthreads();
    const int base = red[0][p] + 53 - H;
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = mk(fx(d2fx(ra[r], base)), fx(d2fx(rb[r], base)));
  } else {  // OP_C2R: Hermitian extension of two half spectra, n = M, m = n_in
    // exponents first (input lines' words, or the doubles' exponents), then
    // load, convert and combine after the line's scale is known (the second
    // reads hit L1); holding the raw values across the barrier would spill
    constexpr int m = M / 2 + 1;
    const int i0 = 2 * p, i1 = 2 * p + 1;
    int tm = kTeZero;
    unsigned emx = 0;
    int ta[8], tb[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int pos = b + r * T;
      const int k = pos < m ? pos : M - pos;
      if constexpr (IN_FX) {
        ta[r] = i0 < nvalid ? __ldg(a.te_in + te_index(a, o.tebase, t0 + i0, k)) : kTeZero;
        tb[r] = i1 < nvalid ? __ldg(a.te_in + te_index(a, o.tebase, t0 + i1, k)) : kTeZero;
        tm = max(tm, max(ta[r], tb[r]));
      } else {
        const double2* in = reinterpret_cast<const double2*>(src) + ioff;
        const int64_t off = (int64_t)k * ssa;
        const double2 qa = i0 < nvalid ? in[off + (int64_t)i0 * sst] : make_double2(0.0, 0.0);
        const double2 qb = i1 < nvalid ? in[off + (int64_t)i1 * sst] : make_double2(0.0, 0.0);
        emx = max(emx, max(max(dexp_u(qa.x), dexp_u(qa.y)), max(dexp_u(qb.x), dexp_u(qb.y))));
      }
    }
    atomicMax(&red[0][p], IN_FX ? tm : (int)emx);
    __syncthreads();
    const int sb = red[0][p] - H + 61;      // fx input: shift base
    const int base = red[0][p] + 53 - H;   // double input: conversion base
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int pos = b + r * T;
      const int k = pos < m ? pos : M - pos;
      const int64_t off = (int64_t)k * ssa;
      Cx<fx> A, B;
      if constexpr (IN_FX) {
        const longlong2* in = reinterpret_cast<const longlong2*>(src) + ioff;
        const longlong2 qa = i0 < nvalid ? in[off + (int64_t)i0 * sst] : make_longlong2(0, 0);
        const longlong2 qb = i1 < nvalid ? in[off + (int64_t)i1 * sst] : make_longlong2(0, 0);
        A = mk(fx(fx_shr(qa.x, sb - ta[r])), fx(fx_shr(qa.y, sb - ta[r])));
        B = mk(fx(fx_shr(qb.x, sb - tb[r])), fx(fx_shr(qb.y, sb - tb[r])));
      } else {
        const double2* in = reinterpret_cast<const double2*>(src) + ioff;
        const double2 qa = i0 < nvalid ? in[off + (int64_t)i0 * sst] : make_double2(0.0, 0.0);
        const double2 qb = i1 < nvalid ? in[off + (int64_t)i1 * sst] : make_double2(0.0, 0.0);
        A = mk(fx(d2fx(qa.x, base)), fx(d2fx(qa.y, base)));
        B = mk(fx(d2fx(qb.x, base)), fx(d2fx(qb.y, base)));
      }
      if (k == 0 || 2 * k == M) { A.im = fx(0); B.im = fx(0); }
      // pos < m: A + iB ; else conj(A) + i conj(B)
      if (pos >= m) { A.im = -A.im; B.im = -B.im; }
      v[r] = mk(A.re - B.im, A.im + B.re);
    }
  }

  // ---- stages ----
  fast_stages<fx, LOGM, SIGN, OP>(v, z, p, b, a.tw, a.lmap_tile != 0);

  // ---- store ----
  // exponent word of complex line i of the output (the line's scale is
  // 2^(et - H); shifted left by 61 - bl its values lie below 2^(et - H + bl))
  auto te_word = [&](int i) {
    const int et = line_et(i), bl = red[1][i];
    return et >= kTeNaN ? kTeNaN : bl == 0 ? kTeZero : et - H + bl;
  };
  // scale exponent of complex line i for double outputs
  auto out_shift = [&](int i) { return line_et(i) - H + a.emax_shift; };
  auto out_nan = [&](int i) { return line_et(i) >= kTeNaN; };
  if constexpr (OUT_FX) {
    unsigned long long orv = 0;
#pragma unroll
    for (int r = 0; r < 8; ++r)
      orv |= (unsigned long long)(v[r].re.v ^ (v[r].re.v >> 63)) | (unsigned long long)(v[r].im.v ^ (v[r].im.v >> 63));
    const int bl = orv ? 64 - __clzll((long long)orv) : 0;
    atomicMax(&red[1][p], bl);
  }
  const double qnan = __longlong_as_double(0x7FF8000000000000ll);
  if (a.store_direct && OP != OP_R2C) {
    if constexpr (OP == OP_C2C) {
      if constexpr (OUT_FX) {
        __syncthreads();
        const int sh = 61 - red[1][p];
        if (p < nvalid) {
          longlong2* out = reinterpret_cast<longlong2*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < 8; ++r)
            out[(int64_t)(b + r * T) * a.out_sa] = make_longlong2(v[r].re.v << sh, v[r].im.v << sh);
        }
      } else {
        const int so = out_shift(p);
        const bool nan = out_nan(p);
        if (p < nvalid) {
          double2* out = reinterpret_cast<double2*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            const Cx<fx> y = apply_scale(v[r], a);
            out[(int64_t)(b + r * T) * a.out_sa] =
                nan ? make_double2(qnan, qnan) : make_double2(fx2d(y.re.v, so), fx2d(y.im.v, so));
          }
        }
      }
    } else {  // C2R, real outputs of lines 2p and 2p+1
      double* out = reinterpret_cast<double*>(a.out) + ooff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
      const int so = out_shift(p);
      const bool nan = out_nan(p);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const Cx<fx> y = apply_scale(v[r], a);
        const int64_t off = (int64_t)(b + r * T) * a.out_sa;
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = nan ? qnan : fx2d(y.re.v, so);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = nan ? qnan : fx2d(y.im.v, so);
      }
    }
    if constexpr (OUT_FX) {
      if (b == 0 && p < ncl_valid)
        a.te_out[t0 / (packed ? 2 : 1) + p + a.te_ncl * div31((unsigned)bid, a.div_tiles)] = te_word(p);
    }
    return;
  }

  // via shared memory: transposed layouts and the r2c split
  {
    Cx<fx>* zw = z + sidx<fx, LOGM, OP>(p, b);
#pragma unroll
    for (int r = 0; r < 8; ++r) zw[padded<fx, LOGM>(r * T)] = v[r];
  }
  __syncthreads();
  if constexpr (OUT_FX) {
    if (b == 0 && p < ncl_valid)
      a.te_out[t0 / (packed ? 2 : 1) + p + a.te_ncl * div31((unsigned)bid, a.div_tiles)] = te_word(p);
  }
  constexpr int nth = fast_threads<fx>(LOGM, OP);  // the launch's thread count
  if constexpr (OP == OP_C2C) {
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { k = e % M; i = e / M; }
      if (i >= nvalid) continue;
      const Cx<fx> y = z[sidx<fx, LOGM, OP>(i, k)];
      const int64_t off = (int64_t)k * a.out_sa + (int64_t)i * a.out_st;
      if constexpr (OUT_FX) {
        const int sh = 61 - red[1][i];
        reinterpret_cast<longlong2*>(a.out)[ooff + off] = make_longlong2(y.re.v << sh, y.im.v << sh);
      } else {
        const Cx<fx> ys = apply_scale(y, a);
        const int so = out_shift(i);
        reinterpret_cast<double2*>(a.out)[ooff + off] =
            out_nan(i) ? make_double2(qnan, qnan) : make_double2(fx2d(ys.re.v, so), fx2d(ys.im.v, so));
      }
    }
  } else if constexpr (OP == OP_R2C) {
    constexpr int m = M / 2 + 1;
    const int tot = TW * m;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % m; q = e / m; }
      const Cx<fx> f = z[sidx<fx, LOGM, OP>(q, k)];
      const Cx<fx> g = conj(z[sidx<fx, LOGM, OP>(q, k == 0 ? 0 : M - k)]);
      Cx<fx> A = f + g, B = mul_mi(f - g);
      A = mk(half(A.re), half(A.im));
      B = mk(half(B.re), half(B.im));
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if constexpr (OUT_FX) {
        const int sh = 61 - red[1][q];
        longlong2* o2 = reinterpret_cast<longlong2*>(a.out) + ooff;
        if (i0 < nvalid) o2[off + (int64_t)i0 * a.out_st] = make_longlong2(A.re.v << sh, A.im.v << sh);
        if (i1 < nvalid) o2[off + (int64_t)i1 * a.out_st] = make_longlong2(B.re.v << sh, B.im.v << sh);
      } else {
        A = apply_scale(A, a);
        B = apply_scale(B, a);
        const int so = out_shift(q);
        const bool nan = out_nan(q);
        double2* o2 = reinterpret_cast<double2*>(a.out) + ooff;
        if (i0 < nvalid)
          o2[off + (int64_t)i0 * a.out_st] = nan ? make_double2(qnan, qnan) : make_double2(fx2d(A.re.v, so), fx2d(A.im.v, so));
        if (i1 < nvalid)
          o2[off + (int64_t)i1 * a.out_st] = nan ? make_double2(qnan, qnan) : make_double2(fx2d(B.re.v, so), fx2d(B.im.v, so));
      }
    }
  } else {  // C2R with a transposed output layout
    double* out = reinterpret_cast<double*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % M; q = e / M; }
      const Cx<fx> y = apply_scale(z[sidx<fx, LOGM, OP>(q, k)], a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      const int so = out_shift(q);
      const bool nan = out_nan(q);
      if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = nan ? qnan : fx2d(y.re.v, so);
      if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = nan ? qnan : fx2d(y.im.v, so);
    }
  }
}

template <typename R, int LOGM, int SIGN, int OP, int IOM>
__device__ __forceinline__ void fast_tile(const FastArgs& a, int64_t bid, Cx<R>* z, const void* src,
                                          int64_t soff, int64_t ssa, int64_t sst) {
  if constexpr (FastIO<R>::kFX) fast_tile_fx<LOGM, SIGN, OP, IOM>(a, bid, z, src, soff, ssa, sst);
  else fast_tile_std<R, LOGM, SIGN, OP, IOM>(a, bid, z, src, soff, ssa, sst);
}

// One kernel per variant (operation c2c / r2c / c2r, dd or double input and
// output): each keeps only its own load and store paths, which frees
// registers (c2c at 64 registers: 8-16 bytes of spill against 96-140 bytes
// with all three operations in one kernel).
template <typename R, int LOGM, int SIGN, int OP, int IOM>
__global__ void __launch_bounds__(fast_threads<R>(LOGM, OP), fast_min_blocks<R>(LOGM, OP, IOM))
    fast_pass(const FastArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  fast_tile<R, LOGM, SIGN, OP, IOM>(a, blockIdx.x, reinterpret_cast<Cx<R>*>(smem_raw), a.in, -1, a.in_sa, a.in_st);
}

// ---------------------------------------------------------------------------
// Persistent form fed by TMA bulk copies.
//
// For passes whose input lines are contiguous (the transformed axis has
// stride 1) and 16-byte aligned, each CTA walks tiles with a stride of the
// grid; one thread issues a cp.async.bulk copy per input line of the *next*
// tile into a shared-memory buffer (two buffers, one mbarrier each), so the
// HBM reads of tile i+1 proceed while tile i is transformed; the loads of the
// stage-1 values then come from shared memory.  Waits on the mbarriers are
// bounded: after ~2^22 polls a CTA records an error in *a.err, waits (bounded)
// for the copy it issued and leaves.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* ptr) {
  return (unsigned)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// polls of a bounded wait before it gives up
constexpr int kWaitPolls = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  int polls = kWaitPolls) {
  for (int i = 0; i < polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// bytes of one input line and lines of a tile, per operation
template <typename R, int LOGM>
__host__ __device__ constexpr int tma_line_bytes(int op) {
  return op == OP_C2C ? (1 << LOGM) * 2 * (int)sizeof(typename FastIO<R>::MR)
       : op == OP_R2C ? (1 << LOGM) * (int)sizeof(typename FastIO<R>::MR)
                      : ((1 << LOGM) / 2 + 1) * 2 * (int)sizeof(typename FastIO<R>::MR);
}
template <typename R, int LOGM>
__host__ __device__ constexpr int tma_tile_bytes(int op) {
  return ((op == OP_C2C ? fast_tw<R>(LOGM, OP_C2R) : 2 * fast_tw<R>(LOGM, OP_C2R)) * tma_line_bytes<R, LOGM>(op) + 127) /
         128 * 128;
}
template <typename R, int LOGM>
__host__ __device__ constexpr size_t tma_smem(int op) {
  return (fast_smem<R>(LOGM, OP_C2R) + 127) / 128 * 128 + 2 * (size_t)tma_tile_bytes<R, LOGM>(op);
}

template <typename R, int LOGM>
__device__ __forceinline__ void tma_issue(const FastArgs& a, int64_t bid, unsigned char* buf,
                                          unsigned long long* bar) {
  constexpr int TW = fast_tw<R>(LOGM, OP_C2R);
  const int lines = a.op == OP_C2C ? TW : 2 * TW;
  const int lb = tma_line_bytes<R, LOGM>(a.op);
  const int esz = a.op == OP_R2C ? (int)sizeof(typename FastIO<R>::MR) : 2 * (int)sizeof(typename FastIO<R>::MR);
  const int64_t tt = bid % a.ntiles;
  int64_t rest = bid / a.ntiles;
  const int64_t t0 = tt * lines;
  int64_t ioff = t0 * a.in_st;
  for (int d = 0; d < a.nouter; ++d) {
    const int64_t idx = rest % a.osz[d];
    rest /= a.osz[d];
    ioff += idx * a.in_so[d];
  }
  const int nvalid = (int)min((int64_t)lines, a.nt - t0);
  mbar_expect_tx(bar, (unsigned)(nvalid * lb));
  const unsigned char* in = reinterpret_cast<const unsigned char*>(a.in);
  for (int i = 0; i < nvalid; ++i)
    tma_load_1d(buf + i * lb, in + (ioff + (int64_t)i * a.in_st) * esz, (unsigned)lb, bar);
}

template <typename R>
__host__ __device__ constexpr int tma_min_blocks(int logm) {
  return sizeof(R) == 4 ? 2 : (fast_threads<R>(logm, OP_C2R) <= 256 ? 2 : 1);
}

template <typename R, int LOGM, int SIGN, int IOM>
__global__ void __launch_bounds__(fast_threads<R>(LOGM, OP_C2R), tma_min_blocks<R>(LOGM)) fast_pass_tma(const FastArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // bars[0..1]: the two tile buffers' copies; bars[2]: never signalled (the
  // give-up test's wait)
  __shared__ __align__(8) unsigned long long bars[3];
  __shared__ int s_fail;
  Cx<R>* z = reinterpret_cast<Cx<R>*>(smem_raw);
  const size_t zb = (fast_smem<R>(LOGM, OP_C2R) + 127) / 128 * 128;
  const int tb = tma_tile_bytes<R, LOGM>(a.op);
  unsigned char* buf0 = smem_raw + zb;
  const int line_elems = a.op == OP_C2R ? (1 << LOGM) / 2 + 1 : (1 << LOGM);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  __syncthreads();
  int64_t tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < a.total) tma_issue<R, LOGM>(a, tile, buf0, &bars[0]);
  int it = 0;
  for (; tile < a.total; tile += gridDim.x, ++it) {
    const int64_t nxt = tile + gridDim.x;
    if (threadIdx.x == 0 && nxt < a.total)
      tma_issue<R, LOGM>(a, nxt, buf0 + ((it + 1) & 1) * tb, &bars[(it + 1) & 1]);
    const bool ok = a.wait_test > 0 ? mbar_wait_bounded(&bars[2], 0, a.wait_test)
                                    : mbar_wait_bounded(&bars[it & 1], (it >> 1) & 1);
    if (!ok) s_fail = 1;
    __syncthreads();
    if (s_fail) break;
    fast_tile<R, LOGM, SIGN, OP_C2R, IOM>(a, tile, z, buf0 + (it & 1) * tb, 0, 1, line_elems);
    __syncthreads();
  }
  if (s_fail && threadIdx.x == 0) {
    atomicOr(a.err, 1);
    // the copies this CTA issued may still be in flight (the tile whose wait
    // gave up, and the next tile): wait for both, bounded, before the CTA's
    // shared memory is released; bit 4 if one of them does not complete
    bool drained = mbar_wait_bounded(&bars[it & 1], (it >> 1) & 1);
    const int64_t nxt = tile + gridDim.x;
    if (nxt < a.total) drained = mbar_wait_bounded(&bars[(it + 1) & 1], ((it + 1) >> 1) & 1) && drained;
    if (!drained) atomicOr(a.err, 4);
  }
}

}  // namespace pfgb
