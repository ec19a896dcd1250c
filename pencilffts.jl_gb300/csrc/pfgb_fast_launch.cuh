// Launchers of the register Stockham pass (fast_pass) and of its TMA-fed
// persistent form, as templates over the arithmetic type, the operation and
// the input / output mode (IOM: dd input bit 0, dd output bit 1); each variant
// is instantiated in its own translation unit
// (pfgb_fast_{f32,dd}_{c2c,r2c,c2r}[_iom].cu) so that they compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_fast.cuh"

namespace pfgb {

int fail_cuda(cudaError_t e, const char* what);

// grid == 0 only sets the kernel's shared-memory attribute (plan creation, so
// that recording a CUDA graph later only launches)
template <typename R, int LOGM, int SIGN, int OP, int IOM>
static int launch_fast_one(const FastArgs& A, int64_t grid, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  const size_t smem = fast_smem<R>(LOGM, OP);
  int rc = ensure_smem_attr(fast_pass<R, LOGM, SIGN, OP, IOM>, (int)smem, configured, "cudaFuncSetAttribute(fast_pass)");
  if (rc || grid == 0) return rc;
  fast_pass<R, LOGM, SIGN, OP, IOM><<<(unsigned)grid, fast_threads<R>(LOGM, OP), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "fast_pass launch");
  return PFGB_OK;
}

template <typename R, int SIGN, int OP, int IOM>
static int launch_fast_sign(int logm, const FastArgs& A, int64_t grid, cudaStream_t s) {
  switch (logm) {
    case 3: return launch_fast_one<R, 3, SIGN, OP, IOM>(A, grid, s);
    case 4: return launch_fast_one<R, 4, SIGN, OP, IOM>(A, grid, s);
    case 5: return launch_fast_one<R, 5, SIGN, OP, IOM>(A, grid, s);
    case 6: return launch_fast_one<R, 6, SIGN, OP, IOM>(A, grid, s);
    case 7: return launch_fast_one<R, 7, SIGN, OP, IOM>(A, grid, s);
    case 8: return launch_fast_one<R, 8, SIGN, OP, IOM>(A, grid, s);
    case 9: return launch_fast_one<R, 9, SIGN, OP, IOM>(A, grid, s);
    case 10: return launch_fast_one<R, 10, SIGN, OP, IOM>(A, grid, s);
    case 11: return launch_fast_one<R, 11, SIGN, OP, IOM>(A, grid, s);
    case 12: return launch_fast_one<R, 12, SIGN, OP, IOM>(A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

template <typename R, int OP, int IOM>
static int launch_fast_op(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign < 0 ? launch_fast_sign<R, -1, OP, IOM>(logm, A, grid, s)
                  : launch_fast_sign<R, 1, OP, IOM>(logm, A, grid, s);
}

// Operations that only run with the forward sign (REDFT00 / RODFT00 through
// their extensions, which are real-symmetric in the sign)
template <typename R, int OP, int IOM>
static int launch_fast_op_fwd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign < 0 ? launch_fast_sign<R, -1, OP, IOM>(logm, A, grid, s) : PFGB_ERR_UNSUPPORTED;
}
// Operations whose DFT runs with the backward sign only (REDFT01 / RODFT01
// through an inverse DFT)
template <typename R, int OP, int IOM>
static int launch_fast_op_bwd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign > 0 ? launch_fast_sign<R, 1, OP, IOM>(logm, A, grid, s) : PFGB_ERR_UNSUPPORTED;
}

// TMA-fed persistent form (c2r passes); A.total == 0 only configures it.
template <typename R, int LOGM, int SIGN, int IOM>
static int launch_tma_one(const FastArgs& A, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  static int max_grid[kMaxDevicesConfigured] = {};
  const size_t smem = tma_smem<R, LOGM>(OP_C2R);
  int rc = ensure_smem_attr(fast_pass_tma<R, LOGM, SIGN, IOM>, (int)smem, configured, "cudaFuncSetAttribute(fast_pass_tma)");
  if (rc) return rc;
  int dev = 0;
  cudaGetDevice(&dev);
  if (max_grid[dev] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fast_pass_tma<R, LOGM, SIGN, IOM>,
                                                                  fast_threads<R>(LOGM, OP_C2R), smem);
    if (e != cudaSuccess) return fail_cuda(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    max_grid[dev] = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (A.total == 0) return PFGB_OK;
  const int64_t grid = A.total < max_grid[dev] ? A.total : max_grid[dev];
  fast_pass_tma<R, LOGM, SIGN, IOM><<<(unsigned)grid, fast_threads<R>(LOGM, OP_C2R), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "fast_pass_tma launch");
  return PFGB_OK;
}

template <typename R, int SIGN, int IOM>
static int launch_tma_sign(int logm, const FastArgs& A, cudaStream_t s) {
  switch (logm) {
    case 3: return launch_tma_one<R, 3, SIGN, IOM>(A, s);
    case 4: return launch_tma_one<R, 4, SIGN, IOM>(A, s);
    case 5: return launch_tma_one<R, 5, SIGN, IOM>(A, s);
    case 6: return launch_tma_one<R, 6, SIGN, IOM>(A, s);
    case 7: return launch_tma_one<R, 7, SIGN, IOM>(A, s);
    case 8: return launch_tma_one<R, 8, SIGN, IOM>(A, s);
    case 9: return launch_tma_one<R, 9, SIGN, IOM>(A, s);
    case 10: return launch_tma_one<R, 10, SIGN, IOM>(A, s);
    case 11: return launch_tma_one<R, 11, SIGN, IOM>(A, s);
    case 12: return launch_tma_one<R, 12, SIGN, IOM>(A, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

}  // namespace pfgb
