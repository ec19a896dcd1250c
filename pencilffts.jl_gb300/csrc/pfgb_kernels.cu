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

}  // namespace pfgb
