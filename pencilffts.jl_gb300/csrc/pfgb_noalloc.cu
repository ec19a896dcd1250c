// pfgb_fft1d_noalloc: a batched 1D Float64 complex FFT that allocates no
// device memory.
//
// Some callers cannot call cudaMalloc: code that runs under a memory manager
// that owns the whole device budget up front (a pool allocator, a solver
// that reserves its working set at start-up and must not fragment it), code
// on a latency-critical path where cudaMalloc's implicit device
// synchronisation is not acceptable, or code inside a host callback from
// which CUDA allocation calls are not allowed.  pfgb_plan_create allocates
// twiddle tables, an exponent word and intermediate buffers, so those callers
// use this entry point instead: the caller passes the input and output
// arrays, and the only other device memory the kernels touch is the
// file-scope array below.
//
// Scratch: g_noalloc_scratch holds an exponent word and the double-float
// twiddle tables of every power-of-two length 32..4096 (8160 entries of 16
// bytes).  It is 130,816 bytes, resident on every GPU that loads the library
// until the process exits.  Each line is scaled by its own largest exponent
// (the kernel's per-line scaling), so lines of very different magnitude in
// one batch keep their full accuracy; the exponent word only collects the
// lines' exponents (atomicMax) and no result depends on it.  Every call
// shares the array and it keeps the last call's contents: the tables are
// written once per device and then only read, and the word is never cleared.
// Calls that overlap on the GPU (different streams, or different host
// threads) write the word concurrently; that race changes no result, but the
// library makes no other promise for overlapping calls: serialise them.
//
// Set-up: the first call on a device (with that device current) resolves the
// device address of the array with cudaGetSymbolAddress and fills the tables
// with cudaMemcpyToSymbol, which is a synchronous host-to-device copy; make
// that first call before any stream capture.  Later calls on the same device
// only launch kernels.  The set-up is cached per device index for the life of
// the process: a device reset (cudaDeviceReset) is not supported, since the
// cached address and tables would belong to the released context.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pencilfft_gb300.h"
#include "pfgb_fast.cuh"

namespace pfgb {

int fail_cuda(cudaError_t e, const char* what);
int fail_argument(const std::string& msg);
int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

namespace {

constexpr int kNoAllocMinLog = 5;   // 32 points
constexpr int kNoAllocMaxLog = 12;  // 4096 points
constexpr int kTableEntries = (1 << (kNoAllocMaxLog + 1)) - (1 << kNoAllocMinLog);  // 8160
constexpr int kHeaderFloats = 64;   // exponent word, padded to 256 bytes
constexpr int kScratchFloats = kHeaderFloats + 4 * kTableEntries;
constexpr int kMaxDevices = 64;

// [0]: exponent word (int, written, never read for results); from float 64 on: tables, the one of length M at
// entry offset M - 32, entries (re.hi, re.lo, im.hi, im.lo).
static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

struct DeviceState {
  bool ready = false;
  float* base = nullptr;  // device address of g_noalloc_scratch
};
DeviceState g_state[kMaxDevices];
std::mutex g_mutex;

int setup_device(int dev, float** base) {
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceState& st = g_state[dev];
  if (st.ready) {
    *base = st.base;
    return PFGB_OK;
  }
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  // double-float twiddles exp(-2 pi i m / M) for every supported M
  std::vector<float> tab(4 * (size_t)kTableEntries);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int lg = kNoAllocMinLog; lg <= kNoAllocMaxLog; ++lg) {
    const int M = 1 << lg;
    float* t = tab.data() + 4 * (size_t)(M - 32);
    for (int m = 0; m < M; ++m) {
      const long double a = 2.0L * pi * (long double)m / (long double)M;
      const long double c = cosl(a), s = -sinl(a);
      t[4 * m + 0] = (float)c;
      t[4 * m + 1] = (float)(c - (long double)(float)c);
      t[4 * m + 2] = (float)s;
      t[4 * m + 3] = (float)(s - (long double)(float)s);
    }
  }
  e = cudaMemcpyToSymbol(g_noalloc_scratch, tab.data(), tab.size() * sizeof(float),
                         kHeaderFloats * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpyToSymbol(g_noalloc_scratch)");
  st.base = static_cast<float*>(ptr);
  st.ready = true;
  *base = st.base;
  return PFGB_OK;
}

}  // namespace
}  // namespace pfgb

extern "C" int pfgb_fft1d_noalloc(int sign, int64_t n, int64_t howmany, void* out, const void* in,
                                  void* stream) {
  using namespace pfgb;
  if (!out || !in) return fail_argument("null array");
  if (sign != -1 && sign != 1) return fail_argument("sign must be -1 (FFT) or +1 (BFFT)");
  if (howmany < 1) return fail_argument("howmany must be at least 1");
  int lg = 0;
  while ((int64_t(1) << lg) < n && lg < 62) ++lg;
  if (n < (1 << kNoAllocMinLog) || n > (1 << kNoAllocMaxLog) || (int64_t(1) << lg) != n)
    return fail_argument("pfgb_fft1d_noalloc: n = " + std::to_string(n) +
                         " is outside its fixed scratch: n must be a power of two in [32, 4096]");
  if (in != out) {
    const char* a = static_cast<const char*>(in);
    const char* b = static_cast<const char*>(out);
    const int64_t bytes = n * howmany * 16;
    if (a < b + bytes && b < a + bytes) return fail_argument("input and output overlap partially");
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail_argument("device index beyond the supported 64");
  float* base = nullptr;
  int rc = setup_device(dev, &base);
  if (rc) return rc;
  int* emax = reinterpret_cast<int*>(base);
  const float* tw = base + kHeaderFloats + 4 * (size_t)(n - 32);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FastArgs A;
  std::memset(&A, 0, sizeof(A));
  A.in = in;
  A.out = out;
  A.tw = tw;
  A.op = OP_C2C;
  A.n_in = A.n_out = (int)n;
  A.lmap_tile = 0;      // lines are contiguous
  A.store_direct = 1;
  A.out_tfast = 0;
  A.scale_on = 0;
  A.in_dd = A.out_dd = 0;
  // each line scaled by its own largest exponent; no per-line record (te)
  A.self_scale = 1;
  A.te = nullptr;
  A.emax_ptr = emax;
  A.nouter = 0;
  A.nt = howmany;
  const int tw_lines = fast_tw<dd>(lg);
  A.ntiles = (howmany + tw_lines - 1) / tw_lines;
  if (A.ntiles >= (int64_t(1) << 31)) return fail_argument("howmany too large for one launch");
  A.div_tiles = make_div31(A.ntiles);
  A.in_sa = A.out_sa = 1;
  A.in_st = A.out_st = n;
  return launch_fast_dd(lg, sign, A, A.ntiles, s);
}
