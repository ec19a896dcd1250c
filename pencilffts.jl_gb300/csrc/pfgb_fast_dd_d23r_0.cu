// Register Stockham pass, double-float (dd) arithmetic for Float64 data: REDFT10 / RODFT10 and
// REDFT01 / RODFT01 through one DFT of their length, two real lines packed in one complex line,
// double input and output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_d2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_D2R, 0>(logm, sign, A, grid, s);
}
int launch_fast_dd_d3r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_bwd<dd, OP_D3R, 0>(logm, sign, A, grid, s);
}
int launch_fast_dd_d4r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_D4R, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
