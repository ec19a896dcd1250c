// Kernel instantiations and launchers for the transform passes.
#include <cuda_runtime.h>

#include <string>

#include "pencilfft_gb300.h"
#include "pfgb_device.cuh"
#include "pfgb_fast.cuh"

namespace pfgb {

int fail_cuda(cudaError_t e, const char* what);

template <typename R>
static int launch_pass_t(const PassArgs& A, int64_t grid, int threads, size_t smem, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  int rc = ensure_smem_attr(pass_kernel<R>, 200 * 1024, configured, "cudaFuncSetAttribute(pass_kernel)");
  if (rc || grid == 0) return rc;
  pass_kernel<R><<<(unsigned)grid, threads, smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "pass_kernel launch");
  return PFGB_OK;
}

int launch_pass(int real_bytes, const PassArgs& A, int64_t grid, int threads, size_t smem,
                cudaStream_t s) {
  if (real_bytes == 8) return launch_pass_t<double>(A, grid, threads, smem, s);
  return launch_pass_t<float>(A, grid, threads, smem, s);
}

int launch_copy(int elt_bytes, const CopyArgs& C, cudaStream_t s) {
  if (C.total == 0) return PFGB_OK;
  int64_t blocks = (C.total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  switch (elt_bytes) {
    case 4: copy_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(C); break;
    case 8: copy_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(C); break;
    default: copy_kernel<double2><<<(unsigned)blocks, 256, 0, s>>>(C); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "copy_kernel launch");
  return PFGB_OK;
}

template <typename R, typename C>
__device__ __forceinline__ Cx<R> ldc(const void* p, int64_t i) {
  const C v = reinterpret_cast<const C*>(p)[i];
  return mk(v.x, v.y);
}
template <typename R, typename C>
__device__ __forceinline__ void stc(void* p, int64_t i, Cx<R> v) {
  C w;
  w.x = v.re;
  w.y = v.im;
  reinterpret_cast<C*>(p)[i] = w;
}

// One iteration point of an LPackMode map between its loads and its stores.
template <typename R>
struct LPoint {
  int64_t oo, k;
  bool ok, two;
  Cx<R> u, v;  // the loaded (R2R, chirp and filter maps: computed) values
};

// Output offset, axis index k and input offset of point e.
template <bool BIG>
__device__ __forceinline__ void lp_index(const LPackArgs& a, int64_t e, int64_t& io, int64_t& oo, int64_t& k,
                                         int64_t& c) {
  int64_t rem = e;
  io = oo = k = c = 0;
  for (int q = 0; q < a.nd; ++q) {
    int64_t idx;
    if constexpr (BIG) {
      idx = rem % a.ext[q];
      rem /= a.ext[q];
    } else {
      const unsigned qq = div31((unsigned)rem, a.dext[q]);
      idx = rem - (int64_t)qq * a.ext[q];
      rem = qq;
    }
    io += idx * a.ist[q];
    oo += idx * a.ost[q];
    if (q == a.qa) k = idx;
    if (q == a.qp) c = idx;
  }
}

// Load phase of point e: every read of the map (no stores).
template <typename R, typename C, bool BIG>
__device__ __forceinline__ void lp_load(const LPackArgs& a, int64_t e, LPoint<R>& p) {
  p.ok = e < a.total;
  if (!p.ok) return;
  int64_t io, c;
  lp_index<BIG>(a, e, io, p.oo, p.k, c);
  p.two = a.qp >= 0 && 2 * c + 1 < a.npair;
  const int64_t k = p.k;
  const Cx<R> zero = mk(R(0), R(0));
  switch (a.mode) {
    case LP_R2C_PACK: {
      const R* x = reinterpret_cast<const R*>(a.in);
      p.u = mk(x[io], p.two ? x[io + a.in_pst] : R(0));
      break;
    }
    case LP_R2C_SEP:
      p.u = ldc<R, C>(a.in, io);
      p.v = ldc<R, C>(a.in, io + ((k ? a.n - k : 0) - k) * a.ist_a);  // Z[n-k]
      break;
    case LP_C2R_HPACK:
      p.u = ldc<R, C>(a.in, io);
      p.v = p.two ? ldc<R, C>(a.in, io + a.in_pst) : zero;
      break;
    case LP_C2R_UNPACK: p.u = ldc<R, C>(a.in, io); break;
    case LP_R2R_PRE: {
      // point j of the extension from the line's points (r2r_pre, gathered)
      const int64_t j = k, n = a.n, m = a.m, base = io - j * a.ist_a;
      const bool two = p.two;
      auto get = [&](int64_t i) -> Cx<R> {
        const int64_t off = base + i * a.ist_a;
        if (a.packed) {
          const R* x = reinterpret_cast<const R*>(a.in);
          return mk(x[off], two ? x[off + a.in_pst] : R(0));
        }
        return ldc<R, C>(a.in, off);
      };
      Cx<R> z = zero;
      switch (a.kind) {
        case K_DHT: z = get(j); break;
        case K_REDFT00: z = get(j <= n - 1 ? j : m - j); break;
        case K_RODFT00:
          if (j >= 1 && j <= n) z = get(j - 1);
          else if (j >= n + 2) z = -get(m - 1 - j);
          break;
        case K_REDFT10: z = j < n ? get(j) : get(2 * n - 1 - j); break;
        case K_RODFT10: z = j < n ? get(j) : -get(2 * n - 1 - j); break;
        case K_REDFT11:
          z = j < n ? get(j) * ldc<R, C>(a.tab, 2 * j) : -(get(2 * n - 1 - j) * ldc<R, C>(a.tab, 2 * j));
          break;
        case K_RODFT11:
          z = (j < n ? get(j) : get(2 * n - 1 - j)) * ldc<R, C>(a.tab, 2 * j);
          break;
        case K_REDFT01:
          if (j < n) z = scal(get(j) * ldc<R, C>(a.tab, 2 * j), j == 0 ? R(0.5) : R(1));
          break;
        default:  // K_RODFT01
          if (j >= 1 && j <= n) z = scal(mul_i(get(j - 1) * ldc<R, C>(a.tab, 2 * j)), j == n ? R(0.5) : R(1));
          break;
      }
      p.u = z;
      break;
    }
    case LP_R2R_POST: {
      // output k from the extension's transform (r2r_post)
      const int64_t n = a.n, m = a.m, base = io - k * a.ist_a;
      auto Z = [&](int64_t q) { return ldc<R, C>(a.in, base + q * a.ist_a); };
      auto t = [&](int64_t q) { return ldc<R, C>(a.tab, q); };
      Cx<R> y;
      switch (a.kind) {
        case K_DHT: {
          const Cx<R> f = Z(k), g = Z(k == 0 ? 0 : m - k);
          y = scal((f + g) + mul_i(f - g), R(0.5));
          break;
        }
        case K_REDFT00: y = Z(k); break;
        case K_RODFT00: y = mul_i(Z(k + 1)); break;
        case K_REDFT10: y = t(2 * k) * Z(k); break;
        case K_RODFT10: y = mul_i(t(2 * (k + 1)) * Z(k + 1)); break;
        case K_REDFT11: y = t(2 * k + 1) * Z(k); break;
        case K_RODFT11: y = mul_i(t(2 * k + 1) * Z(k)); break;
        case K_REDFT01: y = Z(k) + Z(2 * n - 1 - k); break;
        default: y = Z(k) - Z(2 * n - 1 - k); break;  // K_RODFT01
      }
      p.u = y;
      break;
    }
    case LP_CHIRP_PRE: p.u = k < a.n ? ldc<R, C>(a.in, io) * ldc<R, C>(a.tab, k) : zero; break;
    default: p.u = ldc<R, C>(a.in, io) * ldc<R, C>(a.tab, k); break;  // LP_MUL, LP_CHIRP_POST
  }
}

// Store phase of a point.
template <typename R, typename C>
__device__ __forceinline__ void lp_store(const LPackArgs& a, const LPoint<R>& p) {
  if (!p.ok) return;
  const int64_t oo = p.oo, k = p.k;
  switch (a.mode) {
    case LP_R2C_SEP: {
      const Cx<R> u = p.u, v = p.v;
      stc<R, C>(a.out, oo, mk(R(0.5) * (u.re + v.re), R(0.5) * (u.im - v.im)));
      if (p.two) stc<R, C>(a.out, oo + a.out_pst, mk(R(0.5) * (u.im + v.im), R(0.5) * (v.re - u.re)));
      break;
    }
    case LP_C2R_HPACK: {
      Cx<R> x1 = p.u, x2 = p.v;
      const bool self = k == 0 || 2 * k == a.n;  // entries of a real DFT value
      if (self) {
        x1.im = R(0);
        x2.im = R(0);
      }
      stc<R, C>(a.out, oo, mk(x1.re - x2.im, x1.im + x2.re));
      if (!self) stc<R, C>(a.out, oo + (a.n - 2 * k) * a.ost_a, mk(x1.re + x2.im, x2.re - x1.im));  // Z[n-k]
      break;
    }
    case LP_C2R_UNPACK: {
      R* x = reinterpret_cast<R*>(a.out);
      x[oo] = p.u.re;
      if (p.two) x[oo + a.out_pst] = p.u.im;
      break;
    }
    case LP_R2R_POST:
      if (a.packed) {
        R* x = reinterpret_cast<R*>(a.out);
        x[oo] = p.u.re;
        if (p.two) x[oo + a.out_pst] = p.u.im;
      } else {
        stc<R, C>(a.out, oo, p.u);
      }
      break;
    default:  // LP_R2C_PACK, LP_R2R_PRE, LP_CHIRP_PRE, LP_MUL, LP_CHIRP_POST
      stc<R, C>(a.out, oo, p.u);
      break;
  }
}

// The element maps of LPackMode in the output's memory order, grid stride,
// U points per thread: the loads of all U points are issued before any of
// their stores (more bytes in flight per thread; no map reads what another
// point of it writes, and the in-place product reads each point before
// writing it).  Where both layouts share their order, consecutive threads
// touch consecutive elements on both sides, partner Z[n-k] included (a
// descending run when the line axis is the fastest).
template <typename R, typename C, bool BIG>
__global__ void __launch_bounds__(256) lpack_kernel(const LPackArgs a) {
  constexpr int U = sizeof(R) == 8 ? 2 : 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e0 < a.total; e0 += U * stride) {
    LPoint<R> p[U];
#pragma unroll
    for (int u = 0; u < U; ++u) lp_load<R, C, BIG>(a, e0 + u * stride, p[u]);
#pragma unroll
    for (int u = 0; u < U; ++u) lp_store<R, C>(a, p[u]);
  }
}

int launch_lpack(int real_bytes, const LPackArgs& L, cudaStream_t s) {
  if (L.total == 0) return PFGB_OK;
  int64_t blocks = (L.total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  const bool big = L.total >= (int64_t{1} << 31);
  if (real_bytes == 8) {
    if (big) lpack_kernel<double, double2, true><<<(unsigned)blocks, 256, 0, s>>>(L);
    else lpack_kernel<double, double2, false><<<(unsigned)blocks, 256, 0, s>>>(L);
  } else {
    if (big) lpack_kernel<float, float2, true><<<(unsigned)blocks, 256, 0, s>>>(L);
    else lpack_kernel<float, float2, false><<<(unsigned)blocks, 256, 0, s>>>(L);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "lpack_kernel launch");
  return PFGB_OK;
}

}  // namespace pfgb
