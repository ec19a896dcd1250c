// Register Stockham pass, block floating point (fx) arithmetic for Float64 data, c2c lines, fx input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_fx_c2c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<fx, OP_C2C, 1>(logm, sign, A, grid, s);
}

}  // namespace pfgb
