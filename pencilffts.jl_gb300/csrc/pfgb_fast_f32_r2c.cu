// Register Stockham pass, Float32 arithmetic, r2c lines.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_f32_r2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<float, OP_R2C, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
