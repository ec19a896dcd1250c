// Bluestein register pass (lines of any length up to 2048), double-float (dd) arithmetic for Float64 data, c2c lines.
#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_bs.cuh"

namespace pfgb {

int launch_bs_dd_c2c(int logl, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_bs_op<dd, OP_C2C>(logl, A, grid, s);
}

}  // namespace pfgb
