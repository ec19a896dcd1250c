// Instantiations of the register Stockham pass for R = dd.
#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_fast.cuh"

namespace pfgb {

int fail_cuda(cudaError_t e, const char* what);

template <int LOGM, int SIGN>
static int launch_one(const FastArgs& A, int64_t grid, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  const size_t smem = fast_smem<dd>(LOGM);
  int rc = ensure_smem_attr(fast_pass<dd, LOGM, SIGN>, (int)smem, configured,
                            "cudaFuncSetAttribute(fast_pass)");
  if (rc || grid == 0) return rc;
  fast_pass<dd, LOGM, SIGN><<<(unsigned)grid, fast_threads<dd>(LOGM), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "fast_pass launch");
  return PFGB_OK;
}

template <int SIGN>
static int launch_sign(int logm, const FastArgs& A, int64_t grid, cudaStream_t s) {
  switch (logm) {
    case 3: return launch_one<3, SIGN>(A, grid, s);
    case 4: return launch_one<4, SIGN>(A, grid, s);
    case 5: return launch_one<5, SIGN>(A, grid, s);
    case 6: return launch_one<6, SIGN>(A, grid, s);
    case 7: return launch_one<7, SIGN>(A, grid, s);
    case 8: return launch_one<8, SIGN>(A, grid, s);
    case 9: return launch_one<9, SIGN>(A, grid, s);
    case 10: return launch_one<10, SIGN>(A, grid, s);
    case 11: return launch_one<11, SIGN>(A, grid, s);
    case 12: return launch_one<12, SIGN>(A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

template <int LOGM, int SIGN>
static int launch_tma_one(const FastArgs& A, cudaStream_t s) {
  static bool configured[kMaxDevicesConfigured] = {};
  static int max_grid[kMaxDevicesConfigured] = {};
  const size_t smem = tma_smem<dd, LOGM>(A.op);
  const size_t smem_max = tma_smem<dd, LOGM>(OP_C2R) > tma_smem<dd, LOGM>(OP_C2C)
                              ? tma_smem<dd, LOGM>(OP_C2R) : tma_smem<dd, LOGM>(OP_C2C);
  int rc = ensure_smem_attr(fast_pass_tma<dd, LOGM, SIGN>, (int)smem_max, configured,
                            "cudaFuncSetAttribute(fast_pass_tma)");
  if (rc) return rc;
  int dev = 0;
  cudaGetDevice(&dev);
  if (max_grid[dev] == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, fast_pass_tma<dd, LOGM, SIGN>, fast_threads<dd>(LOGM), smem_max);
    if (e != cudaSuccess) return fail_cuda(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    max_grid[dev] = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (A.total == 0) return PFGB_OK;
  const int64_t grid = A.total < max_grid[dev] ? A.total : max_grid[dev];
  fast_pass_tma<dd, LOGM, SIGN><<<(unsigned)grid, fast_threads<dd>(LOGM), smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "fast_pass_tma launch");
  return PFGB_OK;
}

template <int SIGN>
static int launch_tma_sign(int logm, const FastArgs& A, cudaStream_t s) {
  switch (logm) {
    case 3: return launch_tma_one<3, SIGN>(A, s);
    case 4: return launch_tma_one<4, SIGN>(A, s);
    case 5: return launch_tma_one<5, SIGN>(A, s);
    case 6: return launch_tma_one<6, SIGN>(A, s);
    case 7: return launch_tma_one<7, SIGN>(A, s);
    case 8: return launch_tma_one<8, SIGN>(A, s);
    case 9: return launch_tma_one<9, SIGN>(A, s);
    case 10: return launch_tma_one<10, SIGN>(A, s);
    case 11: return launch_tma_one<11, SIGN>(A, s);
    case 12: return launch_tma_one<12, SIGN>(A, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

// TMA-fed persistent form; A.total == 0 only configures the kernel.
int launch_fast_tma_dd(int logm, int sign, const FastArgs& A, cudaStream_t s) {
  return sign < 0 ? launch_tma_sign<-1>(logm, A, s) : launch_tma_sign<1>(logm, A, s);
}

int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign < 0 ? launch_sign<-1>(logm, A, grid, s) : launch_sign<1>(logm, A, grid, s);
}

}  // namespace pfgb
