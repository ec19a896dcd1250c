// Register Stockham pass, Float32 arithmetic: REDFT10 / RODFT10 and REDFT01 / RODFT01 through
// one DFT of their length, on complex lines and on two real lines packed in one complex line.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_f32_d2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_D2C, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_d3c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_bwd<float, OP_D3C, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_d2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_D2R, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_d3r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_bwd<float, OP_D3R, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
