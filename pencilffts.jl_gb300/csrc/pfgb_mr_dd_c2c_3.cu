// Mixed-radix register pass (lines of 3 * 2^k points), double-float (dd) arithmetic for Float64 data, c2c lines.
#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_mr.cuh"

namespace pfgb {

int launch_mr_dd_c2c_3(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_mr_r0<dd, 3, OP_C2C>(logn, sign, A, grid, s);
}

int launch_mr_dd_c2c_5(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

// Entry point of the mixed-radix c2c passes of this type: dispatch on R0.
int launch_mr_dd_c2c(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  if (r0 == 3) return launch_mr_dd_c2c_3(logn, sign, A, grid, s);
  if (r0 == 5) return launch_mr_dd_c2c_5(logn, sign, A, grid, s);
  return PFGB_ERR_UNSUPPORTED;
}

}  // namespace pfgb
