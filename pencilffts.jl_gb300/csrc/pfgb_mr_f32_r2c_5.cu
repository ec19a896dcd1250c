// Mixed-radix register pass (lines of 5 * 2^k points), Float32 arithmetic, r2c lines.
#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_mr.cuh"

namespace pfgb {

int launch_mr_f32_r2c_5(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_mr_r0<float, 5, OP_R2C>(logn, sign, A, grid, s);
}

}  // namespace pfgb
