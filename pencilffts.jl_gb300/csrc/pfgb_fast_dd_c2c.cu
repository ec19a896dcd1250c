// Register Stockham pass, double-float (dd) arithmetic for Float64 data, c2c lines.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_r2c(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2r(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

int launch_fast_dd_c2c(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_C2C>(logm, sign, A, grid, s);
}

// Entry point of the pass kernels of this type: dispatch on the operation.
int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  switch (A.op) {
    case OP_C2C: return launch_fast_dd_c2c(logm, sign, A, grid, s);
    case OP_R2C: return launch_fast_dd_r2c(logm, sign, A, grid, s);
    case OP_C2R: return launch_fast_dd_c2r(logm, sign, A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

}  // namespace pfgb
