// Register Stockham pass, double-float (dd) arithmetic for Float64 data, c2c lines, double input, double output.
#include "pfgb_fast_launch.cuh"

namespace pfgb {

int launch_fast_dd_c2c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_r2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_r2c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2r_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_x00c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_x00c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_x00c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_x00c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_x00r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_csum_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_csum_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_c2ct_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d3c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d2c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d3c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d2c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d3c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d2c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d3c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d4c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d4c_1(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d4c_2(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d4c_3(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d4r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d2r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd_d3r_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

int launch_fast_dd_c2c_0(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  return launch_fast_op<dd, OP_C2C, 0>(logm, sign, A, grid, s);
}

// Entry point of the pass kernels of this type: dispatch on the operation
// and on the input / output form.
int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s) {
  const int iom = (A.in_dd ? 1 : 0) | (A.out_dd ? 2 : 0);
  switch (A.op * 4 + iom) {
    case OP_C2C * 4 + 0: return launch_fast_dd_c2c_0(logm, sign, A, grid, s);
    case OP_C2C * 4 + 1: return launch_fast_dd_c2c_1(logm, sign, A, grid, s);
    case OP_C2C * 4 + 2: return launch_fast_dd_c2c_2(logm, sign, A, grid, s);
    case OP_C2C * 4 + 3: return launch_fast_dd_c2c_3(logm, sign, A, grid, s);
    case OP_R2C * 4 + 0: return launch_fast_dd_r2c_0(logm, sign, A, grid, s);
    case OP_R2C * 4 + 2: return launch_fast_dd_r2c_2(logm, sign, A, grid, s);
    case OP_C2R * 4 + 0: return launch_fast_dd_c2r_0(logm, sign, A, grid, s);
    case OP_C2R * 4 + 1: return launch_fast_dd_c2r_1(logm, sign, A, grid, s);
    case OP_X00C * 4 + 0: return launch_fast_dd_x00c_0(logm, sign, A, grid, s);
    case OP_X00C * 4 + 1: return launch_fast_dd_x00c_1(logm, sign, A, grid, s);
    case OP_X00C * 4 + 2: return launch_fast_dd_x00c_2(logm, sign, A, grid, s);
    case OP_X00C * 4 + 3: return launch_fast_dd_x00c_3(logm, sign, A, grid, s);
    case OP_X00R * 4 + 0: return launch_fast_dd_x00r_0(logm, sign, A, grid, s);
    case OP_CSUM * 4 + 0: return launch_fast_dd_csum_0(logm, sign, A, grid, s);
    case OP_CSUM * 4 + 2: return launch_fast_dd_csum_2(logm, sign, A, grid, s);
    case OP_C2CT * 4 + 0: return launch_fast_dd_c2ct_0(logm, sign, A, grid, s);
    case OP_D2C * 4 + 0: return launch_fast_dd_d2c_0(logm, sign, A, grid, s);
    case OP_D3C * 4 + 0: return launch_fast_dd_d3c_0(logm, sign, A, grid, s);
    case OP_D2C * 4 + 1: return launch_fast_dd_d2c_1(logm, sign, A, grid, s);
    case OP_D3C * 4 + 1: return launch_fast_dd_d3c_1(logm, sign, A, grid, s);
    case OP_D2C * 4 + 2: return launch_fast_dd_d2c_2(logm, sign, A, grid, s);
    case OP_D3C * 4 + 2: return launch_fast_dd_d3c_2(logm, sign, A, grid, s);
    case OP_D2C * 4 + 3: return launch_fast_dd_d2c_3(logm, sign, A, grid, s);
    case OP_D3C * 4 + 3: return launch_fast_dd_d3c_3(logm, sign, A, grid, s);
    case OP_D4C * 4 + 0: return launch_fast_dd_d4c_0(logm, sign, A, grid, s);
    case OP_D4C * 4 + 1: return launch_fast_dd_d4c_1(logm, sign, A, grid, s);
    case OP_D4C * 4 + 2: return launch_fast_dd_d4c_2(logm, sign, A, grid, s);
    case OP_D4C * 4 + 3: return launch_fast_dd_d4c_3(logm, sign, A, grid, s);
    case OP_D4R * 4 + 0: return launch_fast_dd_d4r_0(logm, sign, A, grid, s);
    case OP_D2R * 4 + 0: return launch_fast_dd_d2r_0(logm, sign, A, grid, s);
    case OP_D3R * 4 + 0: return launch_fast_dd_d3r_0(logm, sign, A, grid, s);
    default: return PFGB_ERR_UNSUPPORTED;
  }
}

}  // namespace pfgb
