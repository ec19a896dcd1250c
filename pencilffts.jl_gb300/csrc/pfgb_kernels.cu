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

// Largest biased exponent field over n doubles (atomicMax into *out, which
// the caller zeroes).  Sets the power-of-two scale of a run of dd passes.
__global__ void __launch_bounds__(256) emax_kernel(const unsigned long long* x, int64_t n, int* out) {
  int m = 0;
  // 16-byte vector loads from the first 16-byte boundary; the (at most two)
  // elements outside the vector range are read by thread 0 of block 0
  const int head = (int)((reinterpret_cast<uintptr_t>(x) & 15) != 0);
  const int64_t n2 = (n - head) / 2;
  const ulonglong2* x2 = reinterpret_cast<const ulonglong2*>(x + head);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2;
       i += (int64_t)gridDim.x * blockDim.x) {
    const ulonglong2 w = x2[i];
    m = max(m, max((int)((w.x >> 52) & 0x7FF), (int)((w.y >> 52) & 0x7FF)));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (head && n > 0) m = max(m, (int)((x[0] >> 52) & 0x7FF));
    if (head + 2 * n2 < n) m = max(m, (int)((x[n - 1] >> 52) & 0x7FF));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

int launch_emax(const void* x, int64_t n, int* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int), s);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemsetAsync(emax)");
  int64_t blocks = (n / 2 + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  emax_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(x), n, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "emax_kernel launch");
  return PFGB_OK;
}

}  // namespace pfgb
