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

int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return sign < 0 ? launch_sign<-1>(logm, A, grid, s) : launch_sign<1>(logm, A, grid, s);
}

}  // namespace pfgb
