// Register Stockham pass, double-float (dd) arithmetic for Float64 data, c2r lines, double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_c2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_C2R, 0>(logm, sign, A, grid, s);
}

// TMA-fed persistent form (c2r passes); A.total == 0 only configures it.
int launch_fast_tma_dd_1(int logm, int sign, const FastArgs& A, cudaStream_t s);
int launch_fast_tma_dd(int logm, int sign, const FastArgs& A, cudaStream_t s) {
  if (A.in_dd) return launch_fast_tma_dd_1(logm, sign, A, s);
  return sign < 0 ? launch_tma_sign<dd, -1, 0>(logm, A, s) : launch_tma_sign<dd, 1, 0>(logm, A, s);
}

}  // namespace pfgb
