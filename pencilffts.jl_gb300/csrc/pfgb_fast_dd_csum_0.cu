// Register Stockham pass, double-float (dd) arithmetic for Float64 data:
// c2c pass whose input is a sum of spectral derivatives of several sources
// (fused divergence / curl), double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_csum_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_CSUM, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
