// Bluestein (chirp-z) register pass: lines of any length M <= 2048 for c2c,
// r2c and c2r, in FP32 or in double-float (doubles in and out, one exponent
// per complex line), any input / output layout; c2c lines take the fused
// spectral derivative (i k times the input or the output).
//
// With w[j] = exp(s i pi j^2 / M) (s the transform's sign),
//   X[k] = w[k] sum_n (x[n] w[n]) conj(w[k - n]),
// a cyclic convolution of length L = 2^LOGL >= 2M - 1 computed as
// c = IFFT_L(FFT_L(a) * B), a = x w zero-padded, B = FFT_L(conj(w) extended
// cyclically) / L (a table).  The two L-point transforms are the register
// stages of the power-of-two pass (fast_stages, forward then inverse): a
// thread holds the positions b + r L/8 of its line, which are both the input
// layout and the output layout of fast_stages, so the filter multiply sits
// between the two transforms in registers.  The outputs X[k] = w[k] c[k],
// k < M, go through shared memory to one store loop (c2c, the r2c split of
// two packed real lines, or the two real outputs of a c2r line).
#pragma once

#include "pfgb_fast.cuh"

namespace pfgb {

template <typename R>
__host__ __device__ constexpr int bs_threads(int logl) {
  return fast_threads<R>(logl, OP_C2C);
}
// 8 points a thread (the register stages' default), whatever the power-of-two
// pass uses for this length
template <typename R>
__host__ __device__ constexpr int bs_tw(int logl) {
  return (bs_threads<R>(logl) * 8) >> logl > 0 ? (bs_threads<R>(logl) * 8) >> logl : 1;
}
template <typename R>
__host__ __device__ constexpr size_t bs_smem(int logl) {
  return (size_t)bs_tw<R>(logl) * fast_pitch<R>(logl, OP_C2C) * sizeof(Cx<R>);
}

// x * w for a table entry w (Cx<R>: float (re, im) or dd (re.h, re.l, im.h, im.l))
template <typename R>
__device__ __forceinline__ Cx<R> bs_mul(Cx<R> x, const void* t, int j) {
  return x * ldg_tw<R>(t, j);
}

template <typename R, int LOGL, int OP>
__device__ __forceinline__ void bs_tile(const FastArgs& a, int64_t bid, Cx<R>* z) {
  using IO = FastIO<R>;
  using MR = typename IO::MR;
  using MC = typename IO::MC;
  constexpr int L = 1 << LOGL;
  constexpr int T = L / 8;
  constexpr int NT = bs_threads<R>(LOGL);
  constexpr int TW = bs_tw<R>(LOGL);
  constexpr bool packed = OP == OP_R2C || OP == OP_C2R;
  const int M = a.bs_m;

  const int tid = threadIdx.x;
  int p, b;
  if (a.lmap_tile) { p = tid % TW; b = tid / TW; } else { b = tid % T; p = tid / T; }
  const int lines = packed ? 2 * TW : TW;
  const TileOrigin o = tile_origin(a, (unsigned)bid, lines);
  const int64_t t0 = o.t0, ooff = o.ooff, ioff = o.ioff, didx = o.didx;
  const int nvalid = (int)min((int64_t)lines, a.nt - t0);
  const int ncl_valid = packed ? (nvalid + 1) / 2 : nvalid;
  const int64_t ssa = a.in_sa, sst = a.in_st;
  const int i0 = 2 * p, i1 = 2 * p + 1;

  // ---- load (positions pos = b + r T < M of the line; M <= L / 2 = 4 T,
  // so r < 4) ----
  MC ra[4], rb[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int pos = b + r * T;
    ra[r] = MC{0, 0};
    rb[r] = MC{0, 0};
    if (pos >= M) continue;
    if constexpr (OP == OP_C2C) {
      if (p < nvalid) ra[r] = reinterpret_cast<const MC*>(a.in)[ioff + (int64_t)pos * ssa + (int64_t)p * sst];
    } else if constexpr (OP == OP_R2C) {
      const MR* in = reinterpret_cast<const MR*>(a.in) + ioff + (int64_t)pos * ssa;
      ra[r].x = i0 < nvalid ? in[(int64_t)i0 * sst] : MR(0);
      ra[r].y = i1 < nvalid ? in[(int64_t)i1 * sst] : MR(0);
    } else {  // C2R: Hermitian extension, n_in = M / 2 + 1 inputs
      const int m = a.n_in;
      const int k = pos < m ? pos : M - pos;
      const MC* in = reinterpret_cast<const MC*>(a.in) + ioff + (int64_t)k * ssa;
      if (i0 < nvalid) ra[r] = in[(int64_t)i0 * sst];
      if (i1 < nvalid) rb[r] = in[(int64_t)i1 * sst];
    }
  }
  int emax = 0;
  __shared__ int lexp[TW];
  if constexpr (IO::kDD) {
    unsigned emx = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      emx = max(emx, max(max(dexp_u(ra[r].x), dexp_u(ra[r].y)), max(dexp_u(rb[r].x), dexp_u(rb[r].y))));
    emax = line_exponent<R, LOGL, OP_C2C>(emx, a, (unsigned)bid, t0, p, ncl_valid, a.lmap_tile != 0);
    if (b == 0) lexp[p] = emax;
  }
  Cx<R> v[8];
#pragma unroll
  for (int r = 4; r < 8; ++r) v[r] = mk(R(0), R(0));  // zero padding (not read by the first stage)
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int pos = b + r * T;
    Cx<R> x = mk(mkr<R>(ra[r].x, emax), mkr<R>(ra[r].y, emax));
    if constexpr (OP == OP_C2R) {
      const int m = a.n_in;
      const int k = pos < m ? pos : M - pos;
      Cx<R> B = mk(mkr<R>(rb[r].x, emax), mkr<R>(rb[r].y, emax));
      if (k == 0 || 2 * k == M) { x.im = R(0); B.im = R(0); }
      if (pos >= m) { x.im = -x.im; B.im = -B.im; }
      x = mk(x.re - B.im, x.im + B.re);  // A + i B
    }
    if constexpr (OP == OP_C2C) {
      if (a.deriv == 1) {  // fused spectral derivative on the input
        const int64_t idx = a.deriv_role == 0 ? (int64_t)pos : a.deriv_role == 1 ? t0 + p : didx;
        x = mul_ik(x, idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
      }
    }
    v[r] = pos < M ? bs_mul(x, a.bs_chirp, pos) : mk(R(0), R(0));
  }

  // ---- convolution: forward L-point transform (its inputs' upper half is
  // the zero padding), filter, inverse ----
  fast_stages<R, LOGL, -1, OP_C2C, 8, true>(v, z, p, b, a.tw, a.lmap_tile != 0);
#pragma unroll
  for (int r = 0; r < 8; ++r) v[r] = bs_mul(v[r], a.bs_filt, b + r * T);
  fast_stages<R, LOGL, 1, OP_C2C>(v, z, p, b, a.tw, a.lmap_tile != 0);

  // ---- X[k] = w[k] c[k], k < M <= 4 T, into the line's shared memory (the
  // inverse transform's outputs at r >= 4 are not used) ----
  // (fast_stages ends after a barrier that follows its last exchange read)
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int pos = b + r * T;
    if (pos < M) z[sidx<R, LOGL, OP_C2C>(p, pos)] = bs_mul(v[r], a.bs_chirp, pos);
  }
  __syncthreads();

  // ---- store ----
  auto at = [&](int i, int k) { return z[sidx<R, LOGL, OP_C2C>(i, k)]; };
  auto eo = [&](int i) { return IO::kDD ? lexp[i] + a.emax_shift : 0; };
  if constexpr (OP == OP_C2C) {
    MC* out = reinterpret_cast<MC*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += NT) {
      int i, k;
      if (a.out_tfast) { i = e % TW; k = e / TW; } else { i = (int)div31((unsigned)e, a.div_m); k = e - i * M; }
      if (i >= nvalid) continue;
      Cx<R> y = apply_scale(at(i, k), a);
      if (a.deriv == 2) {  // fused spectral derivative on the output
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
    const int m = a.n_out;  // M / 2 + 1
    const int tot = TW * m;
    for (int e = tid; e < tot; e += NT) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { q = (int)div31((unsigned)e, a.div_m); k = e - q * m; }
      const Cx<R> f = at(q, k);
      const Cx<R> g = conj(at(q, k == 0 ? 0 : M - k));
      Cx<R> A = f + g, B = mul_mi(f - g);
      A = apply_scale(mk(half(A.re), half(A.im)), a);
      B = apply_scale(mk(half(B.re), half(B.im)), a);
      const int j0 = 2 * q, j1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (j0 < nvalid) {
        MC w;
        w.x = outr<R>(A.re, eo(q));
        w.y = outr<R>(A.im, eo(q));
        out[off + (int64_t)j0 * a.out_st] = w;
      }
      if (j1 < nvalid) {
        MC w;
        w.x = outr<R>(B.re, eo(q));
        w.y = outr<R>(B.im, eo(q));
        out[off + (int64_t)j1 * a.out_st] = w;
      }
    }
  } else {  // C2R: real outputs of lines 2q and 2q + 1
    MR* out = reinterpret_cast<MR*>(a.out) + ooff;
    const int tot = TW * M;
    for (int e = tid; e < tot; e += NT) {
      int q, k;
      if (a.out_tfast) { q = e % TW; k = e / TW; } else { q = (int)div31((unsigned)e, a.div_m); k = e - q * M; }
      const Cx<R> y = apply_scale(at(q, k), a);
      const int j0 = 2 * q, j1 = 2 * q + 1;
      const int64_t off = (int64_t)k * a.out_sa;
      if (j0 < nvalid) out[off + (int64_t)j0 * a.out_st] = outr<R>(y.re, eo(q));
      if (j1 < nvalid) out[off + (int64_t)j1 * a.out_st] = outr<R>(y.im, eo(q));
    }
  }
}

// CTAs per SM the register allocation is sized for: two (64 registers for
// the 512-thread Float32 CTAs, 128 for the 256-thread double-float ones).
// Unbounded, the kernels take 80-100 (Float32) and 128-152 (dd) registers,
// so one CTA per SM was resident; at two the spills are 0-12 bytes up to
// L = 512 (Float32) and L = 2048 (dd), past which the bound is one.
template <typename R>
__host__ __device__ constexpr int bs_min_blocks(int logl) {
  return sizeof(R) == 4 ? (logl <= 9 ? 2 : 1) : (logl <= 11 ? 2 : 1);
}
template <typename R, int LOGL, int OP>
__global__ void __launch_bounds__(bs_threads<R>(LOGL), bs_min_blocks<R>(LOGL)) bs_pass(const FastArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  bs_tile<R, LOGL, OP>(a, blockIdx.x, reinterpret_cast<Cx<R>*>(smem_raw));
}

int fail_cuda(cudaError_t e, const char* what);

// grid == 0 only sets the shared-memory attribute
template <typename R, int LOGL, int OP>
static int launch_bs_one(const FastArgs& A, int64_t grid, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  const size_t smem = bs_smem<R>(LOGL);
  int rc = ensure_smem_attr(bs_pass<R, LOGL, OP>, (int)smem, configured, "cudaFuncSetAttribute(bs_pass)");
  if (rc || grid == 0) return rc;
  bs_pass<R, LOGL, OP><<<(unsigned)grid, bs_threads<R>(LOGL), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "bs_pass launch");
  return PFGB_OK;
}

template <typename R, int OP>
static int launch_bs_op(int logl, const FastArgs& A, int64_t grid, cudaStream_t s) {
  switch (logl) {
    case 4: return launch_bs_one<R, 4, OP>(A, grid, s);
    case 5: return launch_bs_one<R, 5, OP>(A, grid, s);
    case 6: return launch_bs_one<R, 6, OP>(A, grid, s);
    case 7: return launch_bs_one<R, 7, OP>(A, grid, s);
    case 8: return launch_bs_one<R, 8, OP>(A, grid, s);
    case 9: return launch_bs_one<R, 9, OP>(A, grid, s);
    case 10: return launch_bs_one<R, 10, OP>(A, grid, s);
    case 11: return launch_bs_one<R, 11, OP>(A, grid, s);
    case 12: return launch_bs_one<R, 12, OP>(A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

}  // namespace pfgb
