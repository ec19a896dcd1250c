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

// The element maps of LPackMode, one iteration point per thread (grid
// stride), in the output's memory order.  Where both layouts share it,
// consecutive threads touch consecutive elements on both sides, partner
// Z[n-k] included (a descending run when the line axis is the fastest).
template <typename R, typename C, bool BIG>
__global__ void __launch_bounds__(256) lpack_kernel(const LPackArgs a) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = e, io = 0, oo = 0, k = 0, c = 0;
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
    const bool two = a.qp >= 0 && 2 * c + 1 < a.npair;
    switch (a.mode) {
      case LP_R2C_PACK: {
        const R* x = reinterpret_cast<const R*>(a.in);
        C z;
        z.x = x[io];
        z.y = two ? x[io + a.in_pst] : R(0);
        reinterpret_cast<C*>(a.out)[oo] = z;
        break;
      }
      case LP_R2C_SEP: {
        const C* Z = reinterpret_cast<const C*>(a.in);
        C* X = reinterpret_cast<C*>(a.out);
        const C u = Z[io];
        const C v = Z[io + ((k ? a.n - k : 0) - k) * a.ist_a];  // Z[n-k]
        C x1, x2;
        x1.x = R(0.5) * (u.x + v.x);
        x1.y = R(0.5) * (u.y - v.y);
        X[oo] = x1;
        if (two) {
          x2.x = R(0.5) * (u.y + v.y);
          x2.y = R(0.5) * (v.x - u.x);
          X[oo + a.out_pst] = x2;
        }
        break;
      }
      case LP_C2R_HPACK: {
        const C* X = reinterpret_cast<const C*>(a.in);
        C* Z = reinterpret_cast<C*>(a.out);
        C x1 = X[io], x2;
        if (two) {
          x2 = X[io + a.in_pst];
        } else {
          x2.x = R(0);
          x2.y = R(0);
        }
        const bool self = k == 0 || 2 * k == a.n;  // entries of a real DFT value
        if (self) {
          x1.y = R(0);
          x2.y = R(0);
        }
        C z;
        z.x = x1.x - x2.y;
        z.y = x1.y + x2.x;
        Z[oo] = z;
        if (!self) {
          z.x = x1.x + x2.y;
          z.y = x2.x - x1.y;
          Z[oo + (a.n - 2 * k) * a.ost_a] = z;  // Z[n-k]
        }
        break;
      }
      case LP_C2R_UNPACK: {
        const C z = reinterpret_cast<const C*>(a.in)[io];
        R* x = reinterpret_cast<R*>(a.out);
        x[oo] = z.x;
        if (two) x[oo + a.out_pst] = z.y;
        break;
      }
      case LP_R2R_PRE: {
        // point j of the extension from the line's points (r2r_pre, gathered)
        const int64_t j = k, n = a.n, m = a.m, base = io - j * a.ist_a;
        auto get = [&](int64_t i) -> Cx<R> {
          const int64_t off = base + i * a.ist_a;
          if (a.packed) {
            const R* x = reinterpret_cast<const R*>(a.in);
            return mk(x[off], two ? x[off + a.in_pst] : R(0));
          }
          return ldc<R, C>(a.in, off);
        };
        Cx<R> z = mk(R(0), R(0));
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
        stc<R, C>(a.out, oo, z);
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
        if (a.packed) {
          R* x = reinterpret_cast<R*>(a.out);
          x[oo] = y.re;
          if (two) x[oo + a.out_pst] = y.im;
        } else {
          stc<R, C>(a.out, oo, y);
        }
        break;
      }
      case LP_CHIRP_PRE: {
        Cx<R> z = mk(R(0), R(0));
        if (k < a.n) z = ldc<R, C>(a.in, io) * ldc<R, C>(a.tab, k);
        stc<R, C>(a.out, oo, z);
        break;
      }
      default: {  // LP_MUL, LP_CHIRP_POST: product with the table entry of point k
        stc<R, C>(a.out, oo, ldc<R, C>(a.in, io) * ldc<R, C>(a.tab, k));
        break;
      }
    }
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
