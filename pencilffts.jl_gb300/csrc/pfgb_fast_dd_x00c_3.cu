// Register Stockham pass, double-float (dd) arithmetic for Float64 data,
// REDFT00 / RODFT00 on complex lines through their extensions, dd input, dd output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_x00c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_X00C, 3>(logm, sign, A, grid, s);
}

}  // namespace pfgb
