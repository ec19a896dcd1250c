// Register Stockham pass, double-float (dd) arithmetic for Float64 data: REDFT10 / RODFT10,
// REDFT01 / RODFT01 and DHT through one DFT of their length, REDFT11 / RODFT11 through one of twice it, complex lines, dd input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_d2c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_D2C, 1>(logm, sign, A, grid, s);
}
int launch_fast_dd_d3c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_bwd<dd, OP_D3C, 1>(logm, sign, A, grid, s);
}
int launch_fast_dd_d4c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<dd, OP_D4C, 1>(logm, sign, A, grid, s);
}

}  // namespace pfgb
