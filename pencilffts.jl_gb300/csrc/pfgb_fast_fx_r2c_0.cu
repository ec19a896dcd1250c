// Register Stockham pass, block floating point (fx) arithmetic for Float64 data, r2c lines, double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_fx_r2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<fx, OP_R2C, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
