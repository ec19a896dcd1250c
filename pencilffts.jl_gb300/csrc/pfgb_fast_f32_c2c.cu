// Register Stockham pass, Float32 arithmetic, c2c lines.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_f32_r2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_c2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_x00c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_x00r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_csum_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_c2ct_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

int launch_fast_f32_c2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<float, OP_C2C, 0>(logm, sign, A, grid, s);
}

// Entry point of the pass kernels of this type: dispatch on the operation
// and on the input / output form.
int launch_fast_f32_d2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_d3c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_d2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_d3r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_d4c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_f32_d4r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

int launch_fast_f32(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  const int iom = 0;
  switch (A.op * 4 + iom) {
    case OP_C2C * 4 + 0: return launch_fast_f32_c2c_0(logm, sign, A, grid, s);
    case OP_R2C * 4 + 0: return launch_fast_f32_r2c_0(logm, sign, A, grid, s);
    case OP_C2R * 4 + 0: return launch_fast_f32_c2r_0(logm, sign, A, grid, s);
    case OP_X00C * 4 + 0: return launch_fast_f32_x00c_0(logm, sign, A, grid, s);
    case OP_X00R * 4 + 0: return launch_fast_f32_x00r_0(logm, sign, A, grid, s);
    case OP_CSUM * 4 + 0: return launch_fast_f32_csum_0(logm, sign, A, grid, s);
    case OP_C2CT * 4 + 0: return launch_fast_f32_c2ct_0(logm, sign, A, grid, s);
    case OP_D2C * 4 + 0: return launch_fast_f32_d2c_0(logm, sign, A, grid, s);
    case OP_D3C * 4 + 0: return launch_fast_f32_d3c_0(logm, sign, A, grid, s);
    case OP_D2R * 4 + 0: return launch_fast_f32_d2r_0(logm, sign, A, grid, s);
    case OP_D3R * 4 + 0: return launch_fast_f32_d3r_0(logm, sign, A, grid, s);
    case OP_D4C * 4 + 0: return launch_fast_f32_d4c_0(logm, sign, A, grid, s);
    case OP_D4R * 4 + 0: return launch_fast_f32_d4r_0(logm, sign, A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

}  // namespace pfgb
