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
// R is the arithmetic type: float, or dd (double-float on the FP32 pipes) for
// Float64 data; dd tiles are scaled by a power of two (the tile's largest
// exponent) so that any finite double range fits the float exponent range.
#pragma once

#include <type_traits>

#include "pfgb_dd.cuh"
#include "pfgb_device.cuh"

namespace pfgb {

struct FastArgs {
  const void* in;
  void* out;
  const void* tw;  // M entries exp(-2 pi i m / M) as Cx<R>
  int op;          // OP_C2C, OP_R2C, OP_C2R
  int n_in, n_out;
  int lmap_tile;     // lanes along the tile dimension (tile dim contiguous in input)
  int store_direct;  // store from registers with the load mapping
  int out_tfast;     // tile dimension contiguous in the output (smem store loop)
  int scale_on;
  float scale_h, scale_l;  // ldiv! normalisation as hi + lo
  // Float64 (dd) passes: the input / output of a pass between two dd passes is
  // kept in dd form (re.hi, re.lo, im.hi, im.lo floats), scaled by the run's
  // power of two 2^(1023 - *emax) where *emax is the largest biased exponent of
  // the run's double input (computed by emax_kernel before the run).
  int in_dd, out_dd;
  const int* emax_ptr;
  int nouter;
  int64_t nt, ntiles;
  int64_t in_sa, in_st, out_sa, out_st;
  int64_t osz[kMaxOuter], in_so[kMaxOuter], out_so[kMaxOuter];
};

// Threads per CTA of the fast pass (8 points of one line per thread) and
// CTAs per SM, measured on GB300 (512^3 round trip):
//   dd:    256 threads, 2 CTAs/SM (~125 registers): the two CTAs' load and
//          compute phases interleave (5.87 ms against 6.58 ms with one
//          512-thread CTA); 512 threads when a line needs them (M = 4096).
//   float: 512 threads, 3 CTAs/SM (register cap 42): 1.75 ms against 1.84 ms
//          with 2 CTAs/SM and 1.80 ms with four 256-thread CTAs.
#ifndef PFGB_FAST_THREADS_F32
#define PFGB_FAST_THREADS_F32 512
#endif
#ifndef PFGB_FAST_THREADS_DD
#define PFGB_FAST_THREADS_DD 256
#endif
template <typename R>
__host__ __device__ constexpr int fast_threads(int logm) {
  return sizeof(R) == 4 ? PFGB_FAST_THREADS_F32
                        : ((1 << logm) / 8 > PFGB_FAST_THREADS_DD ? (1 << logm) / 8 : PFGB_FAST_THREADS_DD);
}
// complex lines per CTA for a line of 2^logm points (one line at least)
template <typename R>
__host__ __device__ constexpr int fast_tw(int logm) {
  return (fast_threads<R>(logm) * 8) >> logm > 0 ? ((fast_threads<R>(logm) * 8) >> logm) : 1;
}
__host__ __device__ constexpr int fast_pad_shift(int logm, int ebytes) {
  return ebytes == 16 ? (logm <= 5 ? 2 : 3) : (logm <= 6 ? 2 : 4);
}
__host__ __device__ constexpr int fast_pitch_extra(int logm, int ebytes) {
  return ebytes == 16 ? (logm == 10 ? 2 : logm == 11 ? 4 : logm == 12 ? 0 : 1)
                      : (logm == 9 ? 2 : logm == 10 ? 4 : logm == 11 ? 8 : logm == 12 ? 0 : 1);
}
__host__ __device__ constexpr int fast_pitch(int logm, int ebytes) {
  return (1 << logm) + ((1 << logm) >> fast_pad_shift(logm, ebytes)) + fast_pitch_extra(logm, ebytes);
}
template <typename R>
__host__ __device__ constexpr size_t fast_smem(int logm) {
  return (size_t)fast_tw<R>(logm) * fast_pitch(logm, (int)sizeof(Cx<R>)) * sizeof(Cx<R>);
}

template <typename R>
struct FastIO;

template <>
struct FastIO<float> {
  using MR = float;
  using MC = float2;
  static constexpr bool kDD = false;
};
template <>
struct FastIO<dd> {
  using MR = double;
  using MC = double2;
  static constexpr bool kDD = true;
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
  else return x * 0.5f;
}

// Shared-memory slot of element pos of complex line p (padding avoids bank
// conflicts for the strided stage writes and the across-line accesses).
template <int LOGM, int EB>
__device__ __forceinline__ int sidx(int p, int pos) {
  return p * fast_pitch(LOGM, EB) + pos + (pos >> fast_pad_shift(LOGM, EB));
}

template <typename R, int LOGM, int SIGN>
__device__ __forceinline__ void fast_stages(Cx<R> (&v)[8], Cx<R>* z, int p, int b, const void* tw) {
  constexpr int M = 1 << LOGM;
  constexpr int T = M / 8;
  constexpr int S8 = LOGM / 3;
  constexpr int REM = LOGM % 3;
  constexpr int NST = S8 + (REM ? 1 : 0);
  int Ls = 1;
#pragma unroll
  for (int s = 0; s < NST; ++s) {
    const bool last = (s == NST - 1);
    if (s < S8) {
      const int j = b & (Ls - 1);
      if (Ls > 1) {
        const int step = j * (M / (8 * Ls));
#pragma unroll
        for (int r = 1; r < 8; ++r) {
          Cx<R> w = ldg_tw<R>(tw, r * step);
          if (SIGN > 0) w = conj(w);
          v[r] = v[r] * w;
        }
      }
      dft8<SIGN>(v);
      if (!last) {
        const int base = (b - j) * 8 + j;
#pragma unroll
        for (int r = 0; r < 8; ++r) z[sidx<LOGM, (int)sizeof(Cx<R>)>(p, base + r * Ls)] = v[r];
      }
      Ls *= 8;
    } else {
      // final radix-2 or radix-4 stage, Ls = M / RS: butterfly beta = b + r1 T
      constexpr int RS = 1 << (REM ? REM : 1);
      constexpr int G = 8 / RS;
#pragma unroll
      for (int r1 = 0; r1 < G; ++r1) {
        const int beta = b + r1 * T;
#pragma unroll
        for (int q = 1; q < RS; ++q) {
          Cx<R> w = ldg_tw<R>(tw, q * beta);
          if (SIGN > 0) w = conj(w);
          v[r1 + q * G] = v[r1 + q * G] * w;
        }
        if constexpr (RS == 2) {
          dft2<SIGN>(v[r1], v[r1 + G]);
        } else {
          dft4<SIGN>(v[r1], v[r1 + G], v[r1 + 2 * G], v[r1 + 3 * G]);
        }
      }
    }
    if (!last) {
      __syncthreads();
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = z[sidx<LOGM, (int)sizeof(Cx<R>)>(p, b + r * T)];
      __syncthreads();
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
  if constexpr (std::is_same<R, dd>::value) {
    const dd s(a.scale_h, a.scale_l);
    return mk(y.re * s, y.im * s);
  } else {
    return mk(y.re * a.scale_h, y.im * a.scale_h);
  }
}

#ifndef PFGB_FAST_F32_MINBLOCKS
#define PFGB_FAST_F32_MINBLOCKS 3
#endif
template <typename R>
__host__ __device__ constexpr int fast_min_blocks(int logm) {
  return sizeof(R) == 4 ? PFGB_FAST_F32_MINBLOCKS : (fast_threads<R>(logm) <= 256 ? 2 : 1);
}

template <typename R, int LOGM, int SIGN>
__global__ void __launch_bounds__(fast_threads<R>(LOGM), fast_min_blocks<R>(LOGM)) fast_pass(const FastArgs a) {
  using IO = FastIO<R>;
  using MR = typename IO::MR;
  using MC = typename IO::MC;
  constexpr int M = 1 << LOGM;
  constexpr int T = M / 8;
  constexpr int TW = fast_tw<R>(LOGM);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<R>* z = reinterpret_cast<Cx<R>*>(smem_raw);

  const int tid = threadIdx.x;
  int p, b;
  if (a.lmap_tile) { p = tid % TW; b = tid / TW; } else { b = tid % T; p = tid / T; }

  // tile decode
  int64_t bid = blockIdx.x;
  const int64_t tile = bid % a.ntiles;
  int64_t rest = bid / a.ntiles;
  const bool packed = a.op != OP_C2C;
  const int lines = packed ? 2 * TW : TW;
  const int64_t t0 = tile * lines;
  int64_t ioff = t0 * a.in_st, ooff = t0 * a.out_st;
  for (int d = 0; d < a.nouter; ++d) {
    const int64_t idx = rest % a.osz[d];
    rest /= a.osz[d];
    ioff += idx * a.in_so[d];
    ooff += idx * a.out_so[d];
  }
  const int nvalid = (int)min((int64_t)lines, a.nt - t0);

  // ---- load: v[r] = line p, element b + r T (stage-1 Stockham inputs) ----
  Cx<R> v[8];
  int emax = 0;
  if constexpr (IO::kDD) emax = *a.emax_ptr;
  if (a.op == OP_C2C) {
    if (IO::kDD && a.in_dd) {
      const float4* in = reinterpret_cast<const float4*>(a.in) + ioff + (int64_t)p * a.in_st;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const float4 q = p < nvalid ? in[(int64_t)(b + r * T) * a.in_sa] : make_float4(0.f, 0.f, 0.f, 0.f);
        v[r] = ld_dd4<R>(q);
      }
    } else {
      const MC* in = reinterpret_cast<const MC*>(a.in) + ioff + (int64_t)p * a.in_st;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const MC raw = p < nvalid ? in[(int64_t)(b + r * T) * a.in_sa] : MC{0, 0};
        v[r] = mk(mkr<R>(raw.x, emax), mkr<R>(raw.y, emax));
      }
    }
  } else if (a.op == OP_R2C) {
    const MR* in = reinterpret_cast<const MR*>(a.in) + ioff;
    const int i0 = 2 * p, i1 = 2 * p + 1;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int64_t off = (int64_t)(b + r * T) * a.in_sa;
      const MR ra = i0 < nvalid ? in[off + (int64_t)i0 * a.in_st] : MR(0);
      const MR rb = i1 < nvalid ? in[off + (int64_t)i1 * a.in_st] : MR(0);
      v[r] = mk(mkr<R>(ra, emax), mkr<R>(rb, emax));
    }
  } else {  // OP_C2R: Hermitian extension of two half spectra, n = M, m = n_in
    const int m = a.n_in;
    const int i0 = 2 * p, i1 = 2 * p + 1;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int pos = b + r * T;
      const int k = pos < m ? pos : M - pos;
      const int64_t off = (int64_t)k * a.in_sa;
      Cx<R> A, B;
      if (IO::kDD && a.in_dd) {
        const float4* in = reinterpret_cast<const float4*>(a.in) + ioff;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        A = ld_dd4<R>(i0 < nvalid ? in[off + (int64_t)i0 * a.in_st] : z4);
        B = ld_dd4<R>(i1 < nvalid ? in[off + (int64_t)i1 * a.in_st] : z4);
      } else {
        const MC* in = reinterpret_cast<const MC*>(a.in) + ioff;
        const MC ra = i0 < nvalid ? in[off + (int64_t)i0 * a.in_st] : MC{0, 0};
        const MC rb = i1 < nvalid ? in[off + (int64_t)i1 * a.in_st] : MC{0, 0};
        A = mk(mkr<R>(ra.x, emax), mkr<R>(ra.y, emax));
        B = mk(mkr<R>(rb.x, emax), mkr<R>(rb.y, emax));
      }
      if (k == 0 || 2 * k == M) { A.im = R(0); B.im = R(0); }
      // pos < m: A + iB ; else conj(A) + i conj(B): one formula with the
      // imaginary parts negated for the mirrored half (a free sign flip)
      if (pos >= m) { A.im = -A.im; B.im = -B.im; }
      v[r] = mk(A.re - B.im, A.im + B.re);
    }
  }

  // ---- stages ----
  fast_stages<R, LOGM, SIGN>(v, z, p, b, a.tw);

  // ---- store ----
  if (a.store_direct && a.op != OP_R2C) {
    if (a.op == OP_C2C) {
      if (p < nvalid) {
        if (IO::kDD && a.out_dd) {
          float4* out = reinterpret_cast<float4*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < 8; ++r) out[(int64_t)(b + r * T) * a.out_sa] = st_dd4(apply_scale(v[r], a));
        } else {
          MC* out = reinterpret_cast<MC*>(a.out) + ooff + (int64_t)p * a.out_st;
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            const Cx<R> y = apply_scale(v[r], a);
            MC o;
            o.x = outr<R>(y.re, emax);
            o.y = outr<R>(y.im, emax);
            out[(int64_t)(b + r * T) * a.out_sa] = o;
          }
        }
      }
    } else {  // C2R, real outputs of lines 2p and 2p+1
      MR* out = reinterpret_cast<MR*>(a.out) + ooff;
      const int i0 = 2 * p, i1 = 2 * p + 1;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const Cx<R> y = apply_scale(v[r], a);
        const int64_t off = (int64_t)(b + r * T) * a.out_sa;
        if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, emax);
        if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, emax);
      }
    }
    return;
  }

  // via shared memory: transposed layouts and the r2c split
#pragma unroll
  for (int r = 0; r < 8; ++r) z[sidx<LOGM, (int)sizeof(Cx<R>)>(p, b + r * T)] = v[r];
  __syncthreads();
  const int nth = blockDim.x;
  if (a.op == OP_C2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { k = e % M; i = e / M; }
      if (i >= nvalid) continue;
      const Cx<R> y = apply_scale(z[sidx<LOGM, (int)sizeof(Cx<R>)>(i, k)], a);
      if (IO::kDD && a.out_dd) {
        reinterpret_cast<float4*>(out)[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = st_dd4(y);
      } else {
        MC o;
        o.x = outr<R>(y.re, emax);
        o.y = outr<R>(y.im, emax);
        out[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = o;
      }
    }
  } else if (a.op == OP_R2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    const int m = a.n_out;
    const int tot = TW * m;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % m; q = e / m; }
      const Cx<R> f = z[sidx<LOGM, (int)sizeof(Cx<R>)>(q, k)];
      const Cx<R> g = conj(z[sidx<LOGM, (int)sizeof(Cx<R>)>(q, k == 0 ? 0 : M - k)]);
      Cx<R> A = f + g, B = mul_mi(f - g);
      A = apply_scale(mk(half(A.re), half(A.im)), a);
      B = apply_scale(mk(half(B.re), half(B.im)), a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (IO::kDD && a.out_dd) {
        float4* o4 = reinterpret_cast<float4*>(out);
        if (i0 < nvalid) o4[off + (int64_t)i0 * a.out_st] = st_dd4(A);
        if (i1 < nvalid) o4[off + (int64_t)i1 * a.out_st] = st_dd4(B);
      } else {
        if (i0 < nvalid) {
          MC o;
          o.x = outr<R>(A.re, emax);
          o.y = outr<R>(A.im, emax);
          out[off + (int64_t)i0 * a.out_st] = o;
        }
        if (i1 < nvalid) {
          MC o;
          o.x = outr<R>(B.re, emax);
          o.y = outr<R>(B.im, emax);
          out[off + (int64_t)i1 * a.out_st] = o;
        }
      }
    }
  } else {  // C2R with a transposed output layout
    MR* out = reinterpret_cast<MR*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += nth) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % M; q = e / M; }
      const Cx<R> y = apply_scale(z[sidx<LOGM, (int)sizeof(Cx<R>)>(q, k)], a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, emax);
      if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, emax);
    }
  }
}

}  // namespace pfgb
