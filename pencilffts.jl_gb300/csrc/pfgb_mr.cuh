// Register pass for mixed-radix lines of M = R0 * N points (R0 = 3 or 5,
// N = 2^LOGN >= 8): one 1D transform per line, any input / output layout,
// the pencil re-layout fused into the store.
//
// Decomposition n = n1 + N n2 (n1 < N, n2 < R0), k = k2 + R0 k1:
//   X[k2 + R0 k1] = sum_n1 W_N^(n1 k1) [ W_M^(n1 k2) sum_n2 x[n1 + N n2] W_R0^(n2 k2) ].
// Phase A: thread (line p, index b) holds the positions n1 = b + r N/8
// (r < 8) of its line; for each r it loads the R0 inputs x[n1 + N n2],
// computes their R0-point DFT in registers (symmetric split; roots of unity
// from the M-point table), multiplies by the twiddles W_M^(n1 k2) and parks
// value k2 in sub-line k2 of shared memory.  Phase B: each sub-line is an
// N-point transform computed by the power-of-two register stages
// (fast_stages), its outputs X[k2 + R0 k1] left in the sub-line at k1.
// Store: one loop over the tile's outputs through shared memory (c2c, the
// r2c split of two packed real lines, or the two real outputs of a c2r
// line), coalesced along the output's contiguous dimension.
//
// Float64 data compute in double-float (dd) with one power-of-two scale per
// complex line (its largest input exponent), doubles in and out; Float32 in
// FP32.
#pragma once

#include "pfgb_fast.cuh"

namespace pfgb {

// threads per CTA and lines (complex) per tile
template <typename R>
__host__ __device__ constexpr int mr_threads(int logn) {
  return ((1 << logn) / 8) > 256 ? (1 << logn) / 8 : 256;
}
template <typename R>
__host__ __device__ constexpr int mr_tw(int logn) {
  return mr_threads<R>(logn) / ((1 << logn) / 8);
}
// sub-line pitch in elements (the exchange layout of fast_stages)
template <typename R, int LOGN, int OP>
__host__ __device__ constexpr int mr_pitch() {
  return fast_pitch<R>(LOGN, OP);
}
template <typename R>
__host__ __device__ constexpr size_t mr_smem(int r0, int logn, int op) {
  return (size_t)r0 * mr_tw<R>(logn) * fast_pitch<R>(logn, op) * sizeof(Cx<R>);
}

// y_k = sum_j v_j exp(SIGN 2 pi i j k / R0) for odd R0, from the table of
// exp(-2 pi i m / M), M = R0 N (the R0-th roots at multiples of N)
template <int R0, int SIGN, typename R>
__device__ __forceinline__ void mr_dft_odd(Cx<R> (&v)[R0], const void* tw2, int N) {
  constexpr int H = (R0 - 1) / 2;
  Cx<R> s[H], d[H];
  Cx<R> y0 = v[0];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = v[j] + v[R0 - j];
    d[j - 1] = v[j] - v[R0 - j];
    y0 = y0 + s[j - 1];
  }
  Cx<R> y[R0];
  y[0] = y0;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    Cx<R> a = v[0], b = mk(R(0), R(0));
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const Cx<R> w = ldg_tw<R>(tw2, ((j * k) % R0) * N);  // (cos t, -sin t)
      a = a + mk(s[j - 1].re * w.re, s[j - 1].im * w.re);
      b = b - mk(d[j - 1].re * w.im, d[j - 1].im * w.im);  // sum d_j sin t
    }
    const Cx<R> ib = mul_i(b);
    if (SIGN < 0) {
      y[k] = a - ib;
      y[R0 - k] = a + ib;
    } else {
      y[k] = a + ib;
      y[R0 - k] = a - ib;
    }
  }
#pragma unroll
  for (int i = 0; i < R0; ++i) v[i] = y[i];
}

// NT threads (mr_threads by default; the persistent batch kernel runs the
// tile with its own CTA size), NT / (N / 8) complex lines a tile.
template <typename R, int R0, int LOGN, int SIGN, int OP, int NT = mr_threads<R>(LOGN)>
__device__ __forceinline__ void mr_tile(const FastArgs& a, int64_t bid, Cx<R>* z) {
  using IO = FastIO<R>;
  using MR = typename IO::MR;
  using MC = typename IO::MC;
  constexpr int N = 1 << LOGN;
  constexpr int M = R0 * N;
  constexpr int T = N / 8;
  constexpr int TW = NT / T;
  static_assert(NT % T == 0 && TW >= 1, "mr_tile: threads must hold whole lines");
  constexpr int PITCH = mr_pitch<R, LOGN, OP>();
  constexpr bool packed = OP == OP_R2C || OP == OP_C2R;

  const int tid = threadIdx.x;
  int p, b;
  if (a.lmap_tile) { p = tid % TW; b = tid / TW; } else { b = tid % T; p = tid / T; }
  const int lines = packed ? 2 * TW : TW;
  const TileOrigin o = tile_origin(a, (unsigned)bid, lines);
  const int64_t t0 = o.t0, ooff = o.ooff, ioff = o.ioff, didx = o.didx;
  const int nvalid = (int)min((int64_t)lines, a.nt - t0);
  const int ncl_valid = packed ? (nvalid + 1) / 2 : nvalid;
  const int64_t ssa = a.in_sa, sst = a.in_st;
  auto sub = [&](int s) { return z + (size_t)s * TW * PITCH; };  // sub-line region s

  // ---- line exponent (dd): largest input exponent of the complex line ----
  int emax = 0;
  __shared__ int lexp[TW];
  if constexpr (IO::kDD) {
    unsigned emx = 0;
#pragma unroll 1
    for (int r = 0; r < 8; ++r) {
#pragma unroll
      for (int n2 = 0; n2 < R0; ++n2) {
        const int n = b + r * T + N * n2;
        if constexpr (OP == OP_C2C) {
          for (int t = 0; t < (a.nterm > 0 ? a.nterm : 1); ++t) {
            const void* src = a.nterm > 0 ? a.tsrc[t] : a.in;
            const MC q = p < nvalid ? reinterpret_cast<const MC*>(src)[ioff + (int64_t)n * ssa + (int64_t)p * sst] : MC{0, 0};
            emx = max(emx, max(dexp_u(q.x), dexp_u(q.y)));
          }
        } else if constexpr (OP == OP_R2C) {
          const MR* in = reinterpret_cast<const MR*>(a.in) + ioff + (int64_t)n * ssa;
          const MR qa = 2 * p < nvalid ? in[(int64_t)(2 * p) * sst] : MR(0);
          const MR qb = 2 * p + 1 < nvalid ? in[(int64_t)(2 * p + 1) * sst] : MR(0);
          emx = max(emx, max(dexp_u(qa), dexp_u(qb)));
        } else {
          const int k = n <= M / 2 ? n : M - n;
          const MC* in = reinterpret_cast<const MC*>(a.in) + ioff + (int64_t)k * ssa;
          const MC qa = 2 * p < nvalid ? in[(int64_t)(2 * p) * sst] : MC{0, 0};
          const MC qb = 2 * p + 1 < nvalid ? in[(int64_t)(2 * p + 1) * sst] : MC{0, 0};
          emx = max(emx, max(max(dexp_u(qa.x), dexp_u(qa.y)), max(dexp_u(qb.x), dexp_u(qb.y))));
        }
      }
    }
    emax = line_exponent<R, LOGN, OP>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
    if (b == 0) lexp[p] = emax;
  }

  // ---- phase A: R0-point DFTs, twiddles, park in the sub-lines (a loop:
  // nothing is held in registers across r) ----
#pragma unroll 1
  for (int r = 0; r < 8; ++r) {
    const int n1 = b + r * T;
    Cx<R> u[R0];
#pragma unroll
    for (int n2 = 0; n2 < R0; ++n2) {
      const int n = n1 + N * n2;
      if constexpr (OP == OP_C2C) {
        if (a.nterm > 0) {  // sum of i k_t src_t (fused divergence / curl)
          u[n2] = mk(R(0), R(0));
          for (int t = 0; t < a.nterm; ++t) {
            const MC q = p < nvalid ? reinterpret_cast<const MC*>(a.tsrc[t])[ioff + (int64_t)n * ssa + (int64_t)p * sst]
                                    : MC{0, 0};
            const int64_t idx = a.trole[t] == 0   ? (int64_t)n
                                : a.trole[t] == 1 ? t0 + p
                                                  : outer_index(a, (unsigned)bid, a.trole[t] - 2);
            u[n2] = u[n2] + mul_ik(mk(mkr<R>(q.x, emax), mkr<R>(q.y, emax)), idx, a.thalf[t], a.tn[t],
                                   a.tk0_h[t], a.tk0_l[t]);
          }
        } else {
          const MC q = p < nvalid ? reinterpret_cast<const MC*>(a.in)[ioff + (int64_t)n * ssa + (int64_t)p * sst] : MC{0, 0};
          u[n2] = mk(mkr<R>(q.x, emax), mkr<R>(q.y, emax));
        }
        if (a.deriv == 1) {
          const int64_t idx = a.deriv_role == 0 ? (int64_t)n : a.deriv_role == 1 ? t0 + p : didx;
          u[n2] = mul_ik(u[n2], idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
        }
      } else if constexpr (OP == OP_R2C) {
        const MR* in = reinterpret_cast<const MR*>(a.in) + ioff + (int64_t)n * ssa;
        const MR qa = 2 * p < nvalid ? in[(int64_t)(2 * p) * sst] : MR(0);
        const MR qb = 2 * p + 1 < nvalid ? in[(int64_t)(2 * p + 1) * sst] : MR(0);
        u[n2] = mk(mkr<R>(qa, emax), mkr<R>(qb, emax));
      } else {  // C2R: Hermitian extension of two half spectra (m = M/2 + 1 inputs)
        const int k = n <= M / 2 ? n : M - n;
        const MC* in = reinterpret_cast<const MC*>(a.in) + ioff + (int64_t)k * ssa;
        const MC qa = 2 * p < nvalid ? in[(int64_t)(2 * p) * sst] : MC{0, 0};
        const MC qb = 2 * p + 1 < nvalid ? in[(int64_t)(2 * p + 1) * sst] : MC{0, 0};
        Cx<R> A = mk(mkr<R>(qa.x, emax), mkr<R>(qa.y, emax));
        Cx<R> B = mk(mkr<R>(qb.x, emax), mkr<R>(qb.y, emax));
        if (k == 0 || 2 * k == M) { A.im = R(0); B.im = R(0); }
        if (n > M / 2) { A.im = -A.im; B.im = -B.im; }
        u[n2] = mk(A.re - B.im, A.im + B.re);
      }
    }
    mr_dft_odd<R0, SIGN>(u, a.tw2, N);
#pragma unroll
    for (int k2 = 0; k2 < R0; ++k2) {
      const Cx<R> y = k2 == 0 ? u[0] : tw_mul<R, SIGN>(u[k2], a.tw2, n1 * k2);
      sub(k2)[sidx<R, LOGN, OP>(p, n1)] = y;
    }
  }

  // ---- phase B: the N-point transform of each sub-line ----
#pragma unroll 1
  for (int s = 0; s < R0; ++s) {
    Cx<R>* zs = sub(s);
    Cx<R> v[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) v[r] = zs[sidx<R, LOGN, OP>(p, b + r * T)];
    // every thread of the line has read its inputs before the first exchange writes
    line_sync<R, LOGN, OP>(a.lmap_tile != 0, p);
    fast_stages<R, LOGN, SIGN, OP>(v, zs, p, b, a.tw, a.lmap_tile != 0);
    // fast_stages ends after a barrier that follows the last exchange read:
    // the outputs X[s + R0 k1], k1 = b + r T, overwrite the sub-line
#pragma unroll
    for (int r = 0; r < 8; ++r) zs[sidx<R, LOGN, OP>(p, b + r * T)] = v[r];
  }
  __syncthreads();

  // ---- store: element k of line i is sub-line k mod R0 at k / R0 ----
  auto at = [&](int i, int k) { return sub(k % R0)[sidx<R, LOGN, OP>(i, k / R0)]; };
  auto eo = [&](int i) { return IO::kDD ? lexp[i] + a.emax_shift : 0; };
  if constexpr (OP == OP_C2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    constexpr int tot = TW * M;
    for (int e = tid; e < tot; e += NT) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { k = e % M; i = e / M; }
      if (i >= nvalid) continue;
      Cx<R> y = apply_scale(at(i, k), a);
      if (a.deriv == 2) {
        const int64_t idx = a.deriv_role == 0 ? (int64_t)k : a.deriv_role == 1 ? t0 + i : didx;
        y = mul_ik(y, idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
      }
      MC q;
      q.x = outr<R>(y.re, eo(i));
      q.y = outr<R>(y.im, eo(i));
      out[(int64_t)k * a.out_sa + (int64_t)i * a.out_st] = q;
    }
  } else if constexpr (OP == OP_R2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    constexpr int m = M / 2 + 1;
    constexpr int tot = TW * m;
    for (int e = tid; e < tot; e += NT) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % m; q = e / m; }
      const Cx<R> f = at(q, k);
      const Cx<R> g = conj(at(q, k == 0 ? 0 : M - k));
      Cx<R> A = f + g, B = mul_mi(f - g);
      A = apply_scale(mk(half(A.re), half(A.im)), a);
      B = apply_scale(mk(half(B.re), half(B.im)), a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (i0 < nvalid) {
        MC w;
        w.x = outr<R>(A.re, eo(q));
        w.y = outr<R>(A.im, eo(q));
        out[off + (int64_t)i0 * a.out_st] = w;
      }
      if (i1 < nvalid) {
        MC w;
        w.x = outr<R>(B.re, eo(q));
        w.y = outr<R>(B.im, eo(q));
        out[off + (int64_t)i1 * a.out_st] = w;
      }
    }
  } else {  // C2R: real outputs of lines 2q and 2q + 1
    MR* out = reinterpret_cast<MR*>(a.out) + ooff;
    constexpr int tot = TW * M;
    for (int e = tid; e < tot; e += NT) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { k = e % M; q = e / M; }
      const Cx<R> y = apply_scale(at(q, k), a);
      const int i0 = 2 * q, i1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (i0 < nvalid) out[off + (int64_t)i0 * a.out_st] = outr<R>(y.re, eo(q));
      if (i1 < nvalid) out[off + (int64_t)i1 * a.out_st] = outr<R>(y.im, eo(q));
    }
  }
}

template <typename R, int R0, int LOGN, int SIGN, int OP>
__global__ void __launch_bounds__(mr_threads<R>(LOGN)) mr_pass(const FastArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  mr_tile<R, R0, LOGN, SIGN, OP>(a, blockIdx.x, reinterpret_cast<Cx<R>*>(smem_raw));
}

// Launchers; grid == 0 only sets the shared-memory attribute.  Line lengths:
// R0 = 3 and 5 with N = 8 .. 512.
int fail_cuda(cudaError_t e, const char* what);

template <typename R, int R0, int LOGN, int SIGN, int OP>
static int launch_mr_one(const FastArgs& A, int64_t grid, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  const size_t smem = mr_smem<R>(R0, LOGN, OP);
  int rc = ensure_smem_attr(mr_pass<R, R0, LOGN, SIGN, OP>, (int)smem, configured, "cudaFuncSetAttribute(mr_pass)");
  if (rc || grid == 0) return rc;
  mr_pass<R, R0, LOGN, SIGN, OP><<<(unsigned)grid, mr_threads<R>(LOGN), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "mr_pass launch");
  return PFGB_OK;
}

template <typename R, int R0, int SIGN, int OP>
static int launch_mr_n(int logn, const FastArgs& A, int64_t grid, cudaStream_t s) {
  switch (logn) {
    case 3: return launch_mr_one<R, R0, 3, SIGN, OP>(A, grid, s);
    case 4: return launch_mr_one<R, R0, 4, SIGN, OP>(A, grid, s);
    case 5: return launch_mr_one<R, R0, 5, SIGN, OP>(A, grid, s);
    case 6: return launch_mr_one<R, R0, 6, SIGN, OP>(A, grid, s);
    case 7: return launch_mr_one<R, R0, 7, SIGN, OP>(A, grid, s);
    case 8: return launch_mr_one<R, R0, 8, SIGN, OP>(A, grid, s);
    case 9: return launch_mr_one<R, R0, 9, SIGN, OP>(A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

template <typename R, int R0, int OP>
static int launch_mr_r0(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign < 0 ? launch_mr_n<R, R0, -1, OP>(logn, A, grid, s) : launch_mr_n<R, R0, 1, OP>(logn, A, grid, s);
}

}  // namespace pfgb
