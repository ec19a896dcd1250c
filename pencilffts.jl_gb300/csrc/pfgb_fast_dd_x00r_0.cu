// Register Stockham pass, double-float (dd) arithmetic for Float64 data,
// REDFT00 / RODFT00 on two real lines packed in one complex line, double
// input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_x00r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_X00R, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
