// Register Stockham pass, double-float (dd) arithmetic for Float64 data, c2c lines, dd input, dd output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_c2c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_C2C, 3>(logm, sign, A, grid, s);
}

}  // namespace pfgb
