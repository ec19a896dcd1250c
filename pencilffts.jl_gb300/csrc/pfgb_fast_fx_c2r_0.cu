// Register Stockham pass, block floating point (fx) arithmetic for Float64 data, c2r lines, double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_fx_c2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<fx, OP_C2R, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
