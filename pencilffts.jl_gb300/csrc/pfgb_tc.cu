// Instantiations and launcher of the tensor-core split form (tc_pass) for
// Float32 c2c lines of 256, 512 and 1024 points.
#include <cuda_runtime.h>

#include <algorithm>

#include "pencilfft_gb300.h"
#include "pfgb_tc.cuh"

namespace pfgb {

int fail_cuda(cudaError_t e, const char* what);

template <int LN1, int LN2, int SIGN>
static int launch_tc_one(const FastArgs& A, cudaStream_t s) {
  using C = TcCfg<LN1, LN2>;
  static bool configured[kMaxDevicesConfigured] = {};
  static int max_grid[kMaxDevicesConfigured] = {};
  int rc = ensure_smem_attr(tc_pass<LN1, LN2, SIGN>, C::SMEM, configured, "cudaFuncSetAttribute(tc_pass)");
  if (rc) return rc;
  int dev = 0;
  cudaGetDevice(&dev);
  if (max_grid[dev] == 0) {
    // resident CTAs per SM from the SM's shared memory, registers and tensor
    // memory (the occupancy query, without a carveout preference, reported
    // one CTA where the launch fits two)
    cudaError_t e = cudaFuncSetAttribute(tc_pass<LN1, LN2, SIGN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute(carveout)");
    int sms = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, tc_pass<LN1, LN2, SIGN>);
    if (e != cudaSuccess) return fail_cuda(e, "cudaFuncGetAttributes(tc_pass)");
    const int regs = (fa.numRegs + 7) / 8 * 8;
    int per_sm = smem_sm / (C::SMEM + reserved);
    per_sm = std::min(per_sm, regs_sm / (regs * 256));
    per_sm = std::min(per_sm, 512 / C::TMEM_COLS);  // tensor memory: 512 columns per SM
    per_sm = std::min(per_sm, 2048 / 256);
    max_grid[dev] = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (A.total == 0) return PFGB_OK;
  const int64_t grid = A.total < max_grid[dev] ? A.total : max_grid[dev];
  tc_pass<LN1, LN2, SIGN><<<(unsigned)grid, 256, C::SMEM, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "tc_pass launch");
  return PFGB_OK;
}

template <int SIGN>
static int launch_tc_sign(int logm, const FastArgs& A, cudaStream_t s) {
  switch (logm) {
    case 8: return launch_tc_one<4, 4, SIGN>(A, s);
    case 9: return launch_tc_one<4, 5, SIGN>(A, s);
    case 10: return launch_tc_one<5, 5, SIGN>(A, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

// A.total == 0 only configures the kernel.
int launch_tc(int logm, int sign, const FastArgs& A, cudaStream_t s) {
  return sign < 0 ? launch_tc_sign<-1>(logm, A, s) : launch_tc_sign<1>(logm, A, s);
}

// Lines per tile of the tensor-core form for lines of 2^logm points (0: not
// available), and the split 2^logm = 2^ln1 * 2^ln2 it uses.
int tc_lines(int logm) {
  switch (logm) {
    case 8: return TcCfg<4, 4>::L;
    case 9: return TcCfg<4, 5>::L;
    case 10: return TcCfg<5, 5>::L;
    default: return 0;
  }
}
void tc_split_of(int logm, int& ln1, int& ln2) {
  ln1 = 4 + (logm >= 10 ? 1 : 0);
  ln2 = logm - ln1;
}

}  // namespace pfgb
