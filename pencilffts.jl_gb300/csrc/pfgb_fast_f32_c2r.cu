// Register Stockham pass, Float32 arithmetic, c2r lines.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_f32_c2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<float, OP_C2R, 0>(logm, sign, A, grid, s);
}

// TMA-fed persistent form (c2r passes); A.total == 0 only configures it.
int launch_fast_tma_f32(int logm, int sign, const FastArgs& A, cudaStream_t s) {
  return sign < 0 ? launch_tma_sign<float, -1, 0>(logm, A, s) : launch_tma_sign<float, 1, 0>(logm, A, s);
}

}  // namespace pfgb
