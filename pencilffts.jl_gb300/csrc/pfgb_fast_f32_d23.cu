// Register Stockham pass, Float32 arithmetic: REDFT10 / RODFT10, REDFT01 / RODFT01 and DHT
// through one DFT of their length, REDFT11 / RODFT11 through one of twice it, on complex lines and on two real lines packed in one complex line.
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
int launch_fast_f32_d4c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_D4C, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_d4r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_D4R, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
