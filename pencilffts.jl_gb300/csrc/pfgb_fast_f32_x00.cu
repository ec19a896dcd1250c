// Register Stockham pass, Float32 arithmetic: REDFT00 / RODFT00 through
// their extensions, on complex lines and on two real lines packed in one
// complex line; and the c2c pass whose input is a sum of spectral
// derivatives of several sources (fused divergence / curl); and the first
// pass of a line split in two (c2c with the split's twiddles on its outputs).
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_f32_x00c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_X00C, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_x00r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op_fwd<float, OP_X00R, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_csum_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<float, OP_CSUM, 0>(logm, sign, A, grid, s);
}
int launch_fast_f32_c2ct_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<float, OP_C2CT, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
