// Mixed-radix register pass (lines of 3 * 2^k points), Float32 arithmetic, c2r lines.
#include <cuda_runtime.h>

#include "pencilfft_gb300.h"
#include "pfgb_mr.cuh"

namespace pfgb {

int launch_mr_f32_c2r_3(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_mr_r0<float, 3, OP_C2R>(logn, sign, A, grid, s);
}

int launch_mr_f32_c2r_5(int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

// Entry point of the mixed-radix c2r passes of this type: dispatch on R0.
int launch_mr_f32_c2r(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  if (r0 == 3) return launch_mr_f32_c2r_3(logn, sign, A, grid, s);
  if (r0 == 5) return launch_mr_f32_c2r_5(logn, sign, A, grid, s);
  return PFGB_ERR_UNSUPPORTED;
}

}  // namespace pfgb
