// Register Stockham pass, double-float (dd) arithmetic for Float64 data: the
// first pass of a line split in two (c2c with the split's twiddles on its
// outputs), double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_c2ct_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_C2CT, 0>(logm, sign, A, grid, s);
}

}  // namespace pfgb
