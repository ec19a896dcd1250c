// Host side of the C ABI: plan construction, pass scheduling, device tables
// and execution.
//
// Reference behaviour restated here (paths within PencilFFTs.jl):
//   - plan construction and per-dimension 1D plans: src/plans.jl:241-320,
//     406-449, 523-553; global sizes and input type: src/global_params.jl:43-95
//   - transform descriptors (length_output, binv, scale_factor):
//     src/Transforms/{c2c,r2c,r2r,no_transform}.jl
//   - execution order (forward left to right, backward right to left, ldiv!
//     scaling): src/operations.jl:24-70, 154-257
//   - output memory order reversed when permute_dims: src/plans.jl:503-521
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "pencilfft_gb300.h"
#include "pfgb_device.cuh"
#include "pfgb_fast.cuh"
#include "pfgb_mr.cuh"
#include "pfgb_bs.cuh"
#include "pfgb_tc.cuh"
#include "pfgb_persist.h"

namespace pfgb {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int fail_argument(const std::string& msg) { return fail(PFGB_ERR_ARGUMENT, msg); }

int fail_cuda(cudaError_t e, const char* what) {
  return fail(PFGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define PFGB_CUDA(call)                                                         \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess)                                                      \
      return fail(PFGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// logical dimensions of a layout: transformed + extra, plus one for the
// second part of a line split in two (the two passes of a long line)
constexpr int kMaxD = PFGB_MAX_DIMS + PFGB_MAX_EXTRA + 1;
constexpr int kMaxLc = 8192;  // longest line held in shared memory

// ---------------------------------------------------------------------------
// Layout of an array: logical sizes and memory order.
// ---------------------------------------------------------------------------
struct Layout {
  int D = 0;
  int64_t size[kMaxD] = {};
  int perm[kMaxD] = {};  // perm[0] = fastest logical dim
  int64_t pitch0 = 0;    // allocated extent of the fastest dim (>= its size)
  int elt = 0;           // element bytes
  bool complex = false;

  int64_t stride(int d) const {
    int64_t s = 1;
    for (int q = 0; q < D; ++q) {
      if (perm[q] == d) return s;
      s *= (q == 0 ? pitch0 : size[perm[q]]);
    }
    return -1;
  }
  int64_t elems() const {
    int64_t s = pitch0;
    for (int q = 1; q < D; ++q) s *= size[perm[q]];
    return s;
  }
  int64_t bytes() const { return elems() * elt; }
  bool same_order(const Layout& o) const {
    if (D != o.D) return false;
    for (int q = 0; q < D; ++q)
      if (perm[q] != o.perm[q]) return false;
    return true;
  }
};

// ---------------------------------------------------------------------------
// One executable pass.
// ---------------------------------------------------------------------------
// PK_LPACK: an element map beside the c2c transform of a line longer than
// one pass takes (LPackMode lp_mode; lp_dim the pair dimension of packed
// real lines or -1)
enum PassKind { PK_TRANSFORM = 0, PK_COPY = 1, PK_LPACK = 2 };

struct Pass {
  PassKind pk = PK_TRANSFORM;
  int op = OP_C2C;
  int r2r_kind = 0;
  int sign = -1;
  int axis = 0;
  Layout lin, lout;
  // DFT geometry
  int M = 0, L = 0, nst = 0, rad[kMaxStages] = {};
  const void* tw = nullptr;
  const void* chirp = nullptr;
  const void* bfilt = nullptr;
  const void* r2rtw = nullptr;
  // register Stockham kernel for power-of-two lines (fast_pass) and its
  // operation (OP_C2C, OP_R2C, OP_C2R, or OP_X00C / OP_X00R for REDFT00 and
  // RODFT00 through their power-of-two extensions)
  bool fast = false;
  int fop = -1;
  // mixed-radix register pass (mr_pass) for lines of r0 * 2^logn points
  bool mr = false;
  int r0 = 0, logn = 0;
  const void* ftw2 = nullptr;  // its r0 * 2^logn-point twiddle table
  // Bluestein register pass (bs_pass) for other lines up to 2048 points:
  // convolution length 2^logl (ftw holds its twiddles), chirp and filter
  // tables; the generic kernel's geometry is kept (g_*) for executions it
  // must take (a fused derivative on this pass)
  // line split in two (lines longer than one register pass takes): both
  // passes carry `four`; the first (t4_dim >= 0) multiplies its outputs by
  // W_M^(n1 k2), n1 the index along dimension t4_dim, M = t4_M
  bool four = false;
  int t4_dim = -1;
  int64_t t4_M = 0;
  const void* t4_tab = nullptr;
  // REDFT10 / 01, RODFT10 / 01 on the register pass: w_k = exp(-i pi k / (2n))
  const void* d23_tab = nullptr;
  bool bs = false;
  int logl = 0;
  const void* bs_chirp = nullptr;
  const void* bs_filt = nullptr;
  int g_lines = 0, g_clines = 0, g_threads = 0;
  size_t g_smem = 0;
  // Float64 fast passes: dd-form input / output between consecutive dd passes,
  // and an exponent reduction over the input before the first pass of a run
  bool in_dd = false, out_dd = false, reduce_before = false;
  // run exponent without a reduction pass: the first pass of a run scales
  // each tile by itself (self_scale); the second maps each element to its
  // first-pass tile (te_rescale, te_sh / te_mul per role)
  bool self_scale = false, te_rescale = false;
  // the last pass of a double-float run that starts with an r2c pass: the
  // r2c split leaves out its factor 1/2, which this pass's output exponent
  // takes instead
  bool half_fold = false;
  int te_sh[2 + kMaxOuter] = {};
  unsigned te_mul[2 + kMaxOuter] = {};
  int logm = 0;
  const void* ftw = nullptr;     // its twiddle table (float or dd entries)
  const void* ftw_fx = nullptr;  // Float64 plans: fx entries with the pass's sign
  // kernel variant chosen by the planner's measurement (autotune): -1
  // default, 0 plain fast_pass, 1 TMA-fed persistent form (c2r passes)
  int variant = -1;
  // tensor-core split form (Float32 c2c, precision PFGB_PRECISION_TC_SPLIT)
  bool tc = false;
  const void* tcb = nullptr;  // DFT matrices, tf32 hi / lo in operand layout
  // launch geometry
  int lines = 1, clines = 1, bpl = 1, lp = 0, threads = 0;
  size_t smem = 0;
  bool zero_fill = false;
  int lp_mode = 0, lp_dim = -1;
  int64_t lp_n = 0, lp_m = 0;  // line length; extension / convolution length
  bool lp_packed = false;      // R2R maps: two real lines per packed line
  const void* lp_tab = nullptr;
  // buffer assignment: 0 = src, 1 = dst, 2 = scratch 1, 3 = scratch 2
  int bin = 0, bout = 1;
};

struct Direction {
  std::vector<Pass> passes;
};

// Spectral derivative fused into a plan execution: multiply the spectrum by
// i k along logical dimension `dim` (k = 2 pi f / length).  mode 2: on the
// output of the last forward pass; mode 1: on the input of the first backward
// pass.
struct Deriv {
  int mode = 0;
  int dim = -1;
  int64_t n = 0;  // physical length along dim
  int half = 0;   // 1 along the half-spectrum dimension of r2c / c2r plans
  double k0 = 0;
  // mode 3: the input of the first backward pass is sum_t i k_t src[t] over
  // nterm sources (k_t = tk0[t] f along logical dimension tdim[t])
  int nterm = 0;
  const void* tsrc[kMaxTerms] = {};
  int tdim[kMaxTerms] = {}, thalf[kMaxTerms] = {};
  int64_t tn[kMaxTerms] = {};
  double tk0[kMaxTerms] = {};
};

}  // namespace pfgb

struct pfgb_plan {
  pfgb_plan_desc desc;
  int N = 0, K = 0, D = 0;
  int rb = 8;  // real bytes
  int precision = 0;  // PFGB_PRECISION_*
  bool inplace = false;
  bool permute = true;
  int64_t dims_in[pfgb::kMaxD] = {}, dims_out[pfgb::kMaxD] = {};
  bool in_complex = false, out_complex = false;
  double scale = 1.0;
  pfgb::Layout in_layout, out_layout;  // user-visible input/output layouts
  int64_t inplace_bytes = 0;
  pfgb::Direction fwd, bwd;
  void* scratch[2] = {nullptr, nullptr};
  int64_t scratch_bytes[2] = {0, 0};
  std::vector<void*> allocations;
  std::map<std::string, void*> tables;
  int* emax_dev = nullptr;  // scale exponent of the current run of dd passes
  int* te_dev = nullptr;    // per-tile exponents of a run's first pass
  // Float64 plans in block floating point (PFGB_PRECISION_BLOCK_FLOAT): fast
  // passes in fx arithmetic (executions with a fused derivative use dd), and
  // the exponent words of
  // the lines passed between consecutive fast passes (pass i writes
  // te_fx[i & 1])
  bool fx = false;
  int* te_fx[2] = {nullptr, nullptr};
  int device = 0;
  bool query_only = false;  // plan analysed on the host only (no device memory)
  // opt-in per-launch timing: (direction, pass index, start, stop)
  bool timing = false;
  // test of the bounded waits' give-up path (pfgb_plan_set_wait_test)
  int wait_test = 0;
  bool force_tma = false;
  struct Rec {
    int dir, pass;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
};

namespace pfgb {

// ---------------------------------------------------------------------------
// Transform descriptors (reference src/Transforms/*.jl)
// ---------------------------------------------------------------------------
static bool r2r_kind_supported(int k) { return k >= PFGB_DHT && k <= PFGB_RODFT11; }

static int r2r_inverse(int k) {  // reference r2r.jl:103-131
  switch (k) {
    case PFGB_REDFT01: return PFGB_REDFT10;
    case PFGB_REDFT10: return PFGB_REDFT01;
    case PFGB_RODFT01: return PFGB_RODFT10;
    case PFGB_RODFT10: return PFGB_RODFT01;
    default: return k;
  }
}

static int64_t length_output(int kind, bool even, int64_t n) {  // r2c.jl:74-75
  if (kind == PFGB_RFFT) return n / 2 + 1;
  if (kind == PFGB_BRFFT) return 2 * n - 1 - (even ? 1 : 0);
  return n;
}

// Scale factor of a 1D transform evaluated on an input of length n
// (reference c2c.jl:71, r2c.jl:103-111, r2r.jl:96-101, no_transform.jl:26).
static double scale_1d(int kind, int r2r, bool even, int64_t n) {
  switch (kind) {
    case PFGB_FFT: case PFGB_BFFT: case PFGB_RFFT: return (double)n;
    case PFGB_BRFFT: return (double)length_output(kind, even, n);
    case PFGB_R2R:
      if (r2r == PFGB_REDFT00) return 2.0 * (double)(n - 1);
      if (r2r == PFGB_RODFT00) return 2.0 * (double)(n + 1);
      if (r2r == PFGB_DHT) return (double)n;
      return 2.0 * (double)n;
    default: return 1.0;
  }
}

// ---------------------------------------------------------------------------
// Host tables (long double), converted to the device real type.
// ---------------------------------------------------------------------------
typedef long double ld;
static const ld kPi = 3.141592653589793238462643383279502884L;

// exp(-i pi m / d), argument reduced exactly in integers.
static std::complex<ld> expi_pi(int64_t m, int64_t d) {
  const int64_t two_d = 2 * d;
  m %= two_d;
  if (m < 0) m += two_d;
  const ld ang = kPi * (ld)m / (ld)d;
  return std::complex<ld>(cosl(ang), -sinl(ang));
}

static void host_fft_pow2(std::vector<std::complex<ld>>& x, int sign) {
  const size_t n = x.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(x[i], x[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    for (size_t i = 0; i < n; i += len) {
      for (size_t k = 0; k < len / 2; ++k) {
        std::complex<ld> w = expi_pi(2 * (int64_t)k, (int64_t)len);  // exp(-2 pi i k/len)
        if (sign > 0) w = std::conj(w);
        std::complex<ld> u = x[i + k], v = x[i + k + len / 2] * w;
        x[i + k] = u + v;
        x[i + k + len / 2] = u - v;
      }
    }
  }
}

template <typename T>
static int upload_table(pfgb_plan* P, const std::string& key, const std::vector<std::complex<T>>& v,
                        const void** out) {
  if (P->query_only) {
    *out = nullptr;
    return PFGB_OK;
  }
  auto it = P->tables.find(key);
  if (it != P->tables.end()) {
    *out = it->second;
    return PFGB_OK;
  }
  void* d = nullptr;
  size_t bytes = v.size() * 2 * P->rb;
  PFGB_CUDA(cudaMalloc(&d, std::max<size_t>(bytes, 16)));
  if (P->rb == 8) {
    std::vector<double> h(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) { h[2 * i] = (double)v[i].real(); h[2 * i + 1] = (double)v[i].imag(); }
    PFGB_CUDA(cudaMemcpy(d, h.data(), bytes, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> h(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) { h[2 * i] = (float)v[i].real(); h[2 * i + 1] = (float)v[i].imag(); }
    PFGB_CUDA(cudaMemcpy(d, h.data(), bytes, cudaMemcpyHostToDevice));
  }
  P->tables[key] = d;
  *out = d;
  return PFGB_OK;
}

// Twiddles of the fast kernel: float (re, im) for Float32 plans, dd
// (re.hi, re.lo, im.hi, im.lo) for Float64 plans.
static int upload_fast_table(pfgb_plan* P, int M, const void** out) {
  if (P->query_only) {
    *out = nullptr;
    return PFGB_OK;
  }
  const std::string key = (P->rb == 8 ? "ftwdd" : "ftwf") + std::to_string(M);
  auto it = P->tables.find(key);
  if (it != P->tables.end()) {
    *out = it->second;
    return PFGB_OK;
  }
  std::vector<float> h;
  h.reserve((size_t)M * 4);
  for (int m = 0; m < M; ++m) {
    const std::complex<ld> w = expi_pi(2 * (int64_t)m, M);
    if (P->rb == 8) {
      for (ld c : {w.real(), w.imag()}) {
        const float hi = (float)c;
        const float lo = (float)(c - (ld)hi);
        h.push_back(hi);
        h.push_back(lo);
      }
    } else {
      h.push_back((float)w.real());
      h.push_back((float)w.imag());
    }
  }
  void* d = nullptr;
  PFGB_CUDA(cudaMalloc(&d, h.size() * sizeof(float)));
  PFGB_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  P->tables[key] = d;
  *out = d;
  return PFGB_OK;
}

// A complex table in the register kernels' format (float (re, im), or dd
// (re.hi, re.lo, im.hi, im.lo) for Float64 plans).
static int upload_fast_vec(pfgb_plan* P, const std::string& key, const std::vector<std::complex<ld>>& v,
                           const void** out) {
  if (P->query_only) {
    *out = nullptr;
    return PFGB_OK;
  }
  const std::string k = (P->rb == 8 ? "fvdd" : "fvf") + key;
  auto it = P->tables.find(k);
  if (it != P->tables.end()) {
    *out = it->second;
    return PFGB_OK;
  }
  std::vector<float> h;
  h.reserve(v.size() * 4);
  for (const auto& w : v) {
    if (P->rb == 8) {
      for (ld c : {w.real(), w.imag()}) {
        const float hi = (float)c;
        h.push_back(hi);
        h.push_back((float)(c - (ld)hi));
      }
    } else {
      h.push_back((float)w.real());
      h.push_back((float)w.imag());
    }
  }
  void* d = nullptr;
  PFGB_CUDA(cudaMalloc(&d, std::max<size_t>(h.size() * sizeof(float), 16)));
  PFGB_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  P->tables[k] = d;
  *out = d;
  return PFGB_OK;
}

// Bluestein tables of a length-M DFT of sign `sign` with convolution length
// L >= 2M - 1: chirp w[j] = exp(sign i pi j^2 / M) (j < M) and the filter
// spectrum FFT_L(b) / L of b[j] = conj(w[j]), b[L - j] = conj(w[j]).
// Host FFT in double of a power-of-two length over a twiddle table computed
// once (the filters of long Bluestein convolutions, up to 2^24 points, where
// the long double form above would take minutes).
static void host_fft_pow2_d(std::vector<std::complex<double>>& x, int sign) {
  const size_t n = x.size();
  std::vector<std::complex<double>> w(n / 2);
  for (size_t k = 0; k < n / 2; ++k) {
    const double ang = 2.0 * 3.141592653589793238 * (double)k / (double)n;
    w[k] = std::complex<double>(std::cos(ang), sign < 0 ? -std::sin(ang) : std::sin(ang));
  }
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(x[i], x[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const size_t step = n / len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; ++k) {
        const std::complex<double> u = x[i + k], v = x[i + k + len / 2] * w[k * step];
        x[i + k] = u + v;
        x[i + k + len / 2] = u - v;
      }
  }
}

// Tables of the long Bluestein form of an M-point c2c line of sign `sign`
// with convolution length L: the chirp w_j = exp(sign i pi j^2 / M) (j < M)
// and the filter spectrum DFT_L(b) / L of b_j = conj(w_j) at j and L - j.
static void bluestein_long_tables(int64_t M, int64_t L, int sign, std::vector<std::complex<double>>& w,
                                  std::vector<std::complex<double>>& bf) {
  w.assign(M, {0, 0});
  for (int64_t j = 0; j < M; ++j) {
    const int64_t r = (j * j) % (2 * M);  // j < 2^23: no overflow
    const double ang = 3.141592653589793238 * (double)r / (double)M;
    w[j] = std::complex<double>(std::cos(ang), sign < 0 ? -std::sin(ang) : std::sin(ang));
  }
  bf.assign(L, {0, 0});
  for (int64_t j = 0; j < M; ++j) bf[j] = std::conj(w[j]);
  for (int64_t j = 1; j < M; ++j) bf[L - j] = std::conj(w[j]);
  host_fft_pow2_d(bf, -1);
  for (auto& x : bf) x /= (double)L;
}

static void bluestein_tables(int M, int L, int sign, std::vector<std::complex<ld>>& w,
                             std::vector<std::complex<ld>>& bf) {
  w.assign(M, {0, 0});
  for (int j = 0; j < M; ++j) {
    const int64_t jj = ((int64_t)j * j) % (2 * (int64_t)M);
    w[j] = expi_pi(jj, M);  // exp(-i pi j^2 / M)
    if (sign > 0) w[j] = std::conj(w[j]);
  }
  bf.assign(L, {0, 0});
  for (int j = 0; j < M; ++j) bf[j] = std::conj(w[j]);
  for (int j = 1; j < M; ++j) bf[L - j] = std::conj(w[j]);
  host_fft_pow2(bf, -1);
  for (auto& x : bf) x /= (ld)L;
}

// Twiddles of the fast kernel in fx form: exp(sign 2 pi i m / M) as
// W = round(w 2^60) (clamped below 2^60) per part, stored as
// (4 * (W >> 31), W & (2^31 - 1)) for the real and imaginary parts.
static int upload_fast_table_fx(pfgb_plan* P, int M, int sign, const void** out) {
  if (P->query_only) {
    *out = nullptr;
    return PFGB_OK;
  }
  const std::string key = "ftwfx" + std::to_string(sign) + "_" + std::to_string(M);
  auto it = P->tables.find(key);
  if (it != P->tables.end()) {
    *out = it->second;
    return PFGB_OK;
  }
  std::vector<int32_t> h;
  h.reserve((size_t)M * 4);
  const ld two60 = std::ldexp((ld)1, 60);
  for (int m = 0; m < M; ++m) {
    const std::complex<ld> w = expi_pi(2 * (int64_t)m * (sign < 0 ? 1 : -1), M);
    for (ld c : {w.real(), w.imag()}) {
      long long W = (long long)std::llround(c * two60);
      if (W > (1ll << 60) - 1) W = (1ll << 60) - 1;
      if (W < -(1ll << 60)) W = -(1ll << 60);
      h.push_back((int32_t)(4 * (W >> 31)));
      h.push_back((int32_t)(W & 0x7FFFFFFFll));
    }
  }
  void* d = nullptr;
  PFGB_CUDA(cudaMalloc(&d, h.size() * sizeof(int32_t)));
  PFGB_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  P->tables[key] = d;
  *out = d;
  return PFGB_OK;
}

// Geometry of the tensor-core split form (pfgb_tc.cu)
int tc_lines(int logm);
void tc_split_of(int logm, int& ln1, int& ln2);

// DFT matrices of the tensor-core split form for lines of 2^logm points and
// one sign: for each distinct factor N of the split, the real form
// [[C, -S], [S, C]] of F_N[k][n] = exp(sign 2 pi i k n / N) (2N x 2N, rows
// (re/im, k), columns (re/im, n)) as a tf32 hi part (round to nearest) and
// the rounded remainder, each in the K-major operand layout of tc_pass.
static int upload_tc_table(pfgb_plan* P, int logm, int sign, const void** out) {
  if (P->query_only) {
    *out = nullptr;
    return PFGB_OK;
  }
  const std::string key = "tcb" + std::to_string(logm) + (sign < 0 ? "-" : "+");
  auto it = P->tables.find(key);
  if (it != P->tables.end()) {
    *out = it->second;
    return PFGB_OK;
  }
  auto tf32 = [](float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;  // nearest, ties away
    float r;
    std::memcpy(&r, &u, 4);
    return r;
  };
  int ln1 = 0, ln2 = 0;
  tc_split_of(logm, ln1, ln2);
  std::vector<float> blob;
  const int factors[2] = {1 << ln1, 1 << ln2};
  for (int f = 0; f < (ln1 == ln2 ? 1 : 2); ++f) {
    const int N = factors[f], K = 2 * N;
    std::vector<float> hi((size_t)K * K), lo((size_t)K * K);
    for (int row = 0; row < K; ++row)
      for (int col = 0; col < K; ++col) {
        const int c = row / N, k = row % N, c2 = col / N, m = col % N;
        const std::complex<ld> w = expi_pi(2 * (int64_t)k * m, N);  // exp(-2 pi i k m / N)
        const ld fr = w.real(), fi = sign < 0 ? w.imag() : -w.imag();
        const ld v = c == 0 ? (c2 == 0 ? fr : -fi) : (c2 == 0 ? fi : fr);
        const float h = tf32((float)v);
        const size_t at = (size_t)tc_off(row, col, K) / 4;
        hi[at] = h;
        lo[at] = tf32((float)(v - (ld)h));
      }
    blob.insert(blob.end(), hi.begin(), hi.end());
    blob.insert(blob.end(), lo.begin(), lo.end());
  }
  void* d = nullptr;
  PFGB_CUDA(cudaMalloc(&d, blob.size() * sizeof(float)));
  PFGB_CUDA(cudaMemcpy(d, blob.data(), blob.size() * sizeof(float), cudaMemcpyHostToDevice));
  P->tables[key] = d;
  *out = d;
  return PFGB_OK;
}

// Radix plan for a DFT length: returns false if a prime factor > 13 remains.
static bool factor_radices(int n, std::vector<int>& rad) {
  rad.clear();
  int e = 0;
  while (n % 2 == 0) { n /= 2; ++e; }
  static const int odd[] = {3, 5, 7, 11, 13};
  std::vector<int> odds;
  for (int p : odd)
    while (n % p == 0) { n /= p; odds.push_back(p); }
  if (n != 1) return false;
  if (e > 0) {
    const int s = (e + 3) / 4;
    for (int i = 0; i < s; ++i) {
      const int ei = e / s + (i < e % s ? 1 : 0);
      rad.push_back(1 << ei);
    }
  }
  for (int p : odds) rad.push_back(p);
  return true;
}

// ---------------------------------------------------------------------------
// Pass preparation: DFT geometry, tables, launch shape.
// ---------------------------------------------------------------------------
static int prepare_core(pfgb_plan* P, Pass& ps, int M) {
  ps.M = M;
  std::vector<int> rad;
  int Lc = M;
  if (!factor_radices(M, rad)) {
    int L = 1;
    while (L < 2 * M - 1) L <<= 1;
    ps.L = L;
    Lc = L;
    factor_radices(L, rad);
  }
  if (Lc > kMaxLc)
    return fail(PFGB_ERR_UNSUPPORTED, "transform length " + std::to_string(M) +
                                          " exceeds the longest supported line (core length " +
                                          std::to_string(Lc) + " > 8192)");
  ps.nst = (int)rad.size();
  for (int i = 0; i < ps.nst; ++i) ps.rad[i] = rad[i];
  // core twiddles exp(-2 pi i m / Lc)
  {
    std::vector<std::complex<ld>> t(Lc);
    for (int m = 0; m < Lc; ++m) t[m] = expi_pi(2 * (int64_t)m, Lc);
    int rc = upload_table(P, "tw" + std::to_string(Lc), t, &ps.tw);
    if (rc) return rc;
  }
  if (ps.L > 0) {
    const int L = ps.L;
    std::vector<std::complex<ld>> c(M), b(L, std::complex<ld>(0, 0));
    for (int j = 0; j < M; ++j) {
      const int64_t jj = ((int64_t)j * j) % (2 * (int64_t)M);
      c[j] = expi_pi(jj, M);  // exp(-i pi j^2 / M)
    }
    for (int j = 0; j < M; ++j) b[j] = std::conj(c[j]);
    for (int j = 1; j < M; ++j) b[L - j] = std::conj(c[j]);
    std::vector<std::complex<ld>> cs(M), bs(b);
    if (ps.sign > 0) {
      for (int j = 0; j < M; ++j) cs[j] = std::conj(c[j]);
      for (auto& v : bs) v = std::conj(v);
    } else {
      cs = c;
    }
    host_fft_pow2(bs, -1);
    for (auto& v : bs) v /= (ld)L;
    const std::string k = std::to_string(M) + (ps.sign > 0 ? "+" : "-");
    int rc = upload_table(P, "chirp" + k, cs, &ps.chirp);
    if (rc) return rc;
    rc = upload_table(P, "bfilt" + k, bs, &ps.bfilt);
    if (rc) return rc;
  }
  return PFGB_OK;
}

// The Bluestein register pass's form of a c2c / r2c / c2r pass of ps.M <= 2048
// points: convolution length 2^logl >= 2 M - 1, its twiddles, the chirp and
// filter tables, and the tile geometry.
static int bluestein_form(pfgb_plan* P, Pass& ps) {
  const int M = ps.M;
  int logl = 4;
  while ((1 << logl) < 2 * M - 1) ++logl;
  std::vector<std::complex<ld>> w, bf;
  bluestein_tables(M, 1 << logl, ps.sign, w, bf);
  const std::string key = std::to_string(M) + "/" + std::to_string(1 << logl) + (ps.sign > 0 ? "+" : "-");
  int rc = upload_fast_table(P, 1 << logl, &ps.ftw);
  if (!rc) rc = upload_fast_vec(P, "bsw" + key, w, &ps.bs_chirp);
  if (!rc) rc = upload_fast_vec(P, "bsf" + key, bf, &ps.bs_filt);
  if (rc) return rc;
  ps.mr = false;
  ps.fast = false;
  ps.bs = true;
  ps.fop = ps.op;
  ps.logl = logl;
  const bool pk = fast_packed(ps.op);
  ps.clines = P->rb == 8 ? bs_tw<dd>(logl) : bs_tw<float>(logl);
  ps.lines = pk ? 2 * ps.clines : ps.clines;
  ps.threads = P->rb == 8 ? bs_threads<dd>(logl) : bs_threads<float>(logl);
  ps.smem = P->rb == 8 ? bs_smem<dd>(logl) : bs_smem<float>(logl);
  return PFGB_OK;
}

static int prepare_pass(pfgb_plan* P, Pass& ps) {
  if (ps.pk == PK_COPY || ps.pk == PK_LPACK) {
    ps.threads = 256;
    if (ps.pk == PK_COPY || P->query_only) return PFGB_OK;
    const int md = ps.lp_mode;
    if (md == LP_R2R_PRE || md == LP_R2R_POST) {
      // exp(-i pi q / (4n)), q <= 4n + 1, in double (lines beyond one pass)
      const std::string key = "r2rd" + std::to_string(ps.lp_n);
      if (!P->tables.count(key)) {
        const int64_t n = ps.lp_n;
        std::vector<std::complex<double>> t(4 * (size_t)n + 2);
        for (int64_t q = 0; q < 4 * n + 2; ++q) {
          const double ang = 3.141592653589793238 * (double)(q % (8 * n)) / (4.0 * (double)n);
          t[q] = std::complex<double>(std::cos(ang), -std::sin(ang));
        }
        int rc = upload_table(P, key, t, &ps.lp_tab);
        if (rc) return rc;
      }
      ps.lp_tab = P->tables[key];
    } else if (md == LP_CHIRP_PRE || md == LP_MUL || md == LP_CHIRP_POST) {
      const std::string k = std::to_string(ps.lp_n) + (ps.sign > 0 ? "+" : "-");
      if (!P->tables.count("lchirp" + k)) {
        std::vector<std::complex<double>> w, bf;
        bluestein_long_tables(ps.lp_n, ps.lp_m, ps.sign, w, bf);
        const void* t = nullptr;
        int rc = upload_table(P, "lchirp" + k, w, &t);
        if (!rc) rc = upload_table(P, "lfilt" + k, bf, &t);
        if (rc) return rc;
      }
      ps.lp_tab = P->tables[(md == LP_MUL ? "lfilt" : "lchirp") + k];
    }
    return PFGB_OK;
  }
  const int a = ps.axis;
  const int64_t n_in = ps.lin.size[a], n_out = ps.lout.size[a];
  if (n_in > kMaxLc * 2 || n_out > kMaxLc * 2)
    return fail(PFGB_ERR_UNSUPPORTED, "line too long");
  int M = 0;
  switch (ps.op) {
    case OP_C2C: M = (int)n_in; break;
    case OP_R2C: M = (int)n_in; break;
    case OP_C2R: M = (int)n_out; break;
    default: {
      const int n = (int)n_in;
      switch (ps.r2r_kind) {
        case K_DHT: M = n; break;
        case K_REDFT00:
          if (n < 2) return fail(PFGB_ERR_ARGUMENT, "REDFT00 requires a length of at least 2");
          M = 2 * (n - 1);
          break;
        case K_RODFT00: M = 2 * (n + 1); break;
        default: M = 2 * n; break;
      }
      ps.sign = -1;
      if (ps.r2r_kind != K_DHT) {
        std::vector<std::complex<ld>> t(4 * (size_t)n + 2);
        for (int m = 0; m < 4 * n + 2; ++m) t[m] = expi_pi(m, 4 * (int64_t)n);
        int rc = upload_table(P, "r2r" + std::to_string(n), t, &ps.r2rtw);
        if (rc) return rc;
      }
      break;
    }
  }
  int rc = prepare_core(P, ps, M);
  if (rc) return rc;
  // power-of-two c2c / r2c / c2r lines, and REDFT00 / RODFT00 lines whose
  // extension has a power-of-two length (n = 2^k + 1, 2^k - 1), take the
  // register Stockham kernel; on Float64 plans it computes in dd unless
  // native FP64 was requested (block floating point plans keep the R2R kinds
  // on the generic kernel)
  const bool x00 = (ps.op == OP_R2R_C || ps.op == OP_R2R_R) &&
                   (ps.r2r_kind == K_REDFT00 || ps.r2r_kind == K_RODFT00) && !P->fx;
  // REDFT10 / RODFT10, REDFT01 / RODFT01 and DHT of a power-of-two length n
  // (8 <= n <= 4096) take the register pass through one n-point DFT
  {
    const int n = (int)n_in;
    const bool dht = ps.r2r_kind == K_DHT;
    // REDFT11 / RODFT11 of n points: one 2n-point DFT (4 <= n <= 2048)
    const bool d4 = ps.r2r_kind == K_REDFT11 || ps.r2r_kind == K_RODFT11;
    if ((ps.op == OP_R2R_C || ps.op == OP_R2R_R) && d4 && !P->fx && n >= 4 && n <= 2048 && (n & (n - 1)) == 0 &&
        !(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
      ps.fast = true;
      ps.fop = ps.op == OP_R2R_C ? OP_D4C : OP_D4R;
      ps.sign = -1;
      ps.logm = 0;
      while ((1 << ps.logm) < 2 * n) ++ps.logm;
      std::vector<std::complex<ld>> w(2 * (size_t)n);
      for (int j = 0; j < n; ++j) {
        w[j] = expi_pi(j, 2 * (int64_t)n);                   // c_j = exp(-i pi j / (2n))
        w[n + j] = expi_pi(2 * (int64_t)j + 1, 4 * (int64_t)n);  // d_j = exp(-i pi (2j+1) / (4n))
      }
      int rc2 = upload_fast_table(P, 2 * n, &ps.ftw);
      if (!rc2) rc2 = upload_fast_vec(P, "d4/" + std::to_string(n), w, &ps.d23_tab);
      if (rc2) return rc2;
      const bool packed = fast_packed(ps.fop);
      ps.clines = P->rb == 8 ? fast_tw<dd>(ps.logm, ps.fop) : fast_tw<float>(ps.logm, ps.fop);
      ps.lines = packed ? 2 * ps.clines : ps.clines;
      ps.threads = P->rb == 8 ? fast_threads<dd>(ps.logm, ps.fop) : fast_threads<float>(ps.logm, ps.fop);
      ps.smem = P->rb == 8 ? fast_smem<dd>(ps.logm, ps.fop) : fast_smem<float>(ps.logm, ps.fop);
      return PFGB_OK;
    }
    const bool d2 = ps.r2r_kind == K_REDFT10 || ps.r2r_kind == K_RODFT10 || dht;
    const bool d3 = ps.r2r_kind == K_REDFT01 || ps.r2r_kind == K_RODFT01;
    if ((ps.op == OP_R2R_C || ps.op == OP_R2R_R) && (d2 || d3) && !P->fx && n >= 8 && n <= 4096 &&
        (n & (n - 1)) == 0 && !(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
      ps.fast = true;
      const bool cplx = ps.op == OP_R2R_C;
      ps.fop = d2 ? (cplx ? OP_D2C : OP_D2R) : (cplx ? OP_D3C : OP_D3R);
      ps.sign = d2 ? -1 : 1;
      ps.logm = 0;
      while ((1 << ps.logm) < n) ++ps.logm;
      std::vector<std::complex<ld>> w(n);
      for (int k = 0; k < n; ++k)  // exp(-i pi k / (2n)); DHT: (1 + i) / 2
        w[k] = dht ? std::complex<ld>(0.5L, 0.5L) : expi_pi(k, 2 * (int64_t)n);
      int rc2 = upload_fast_table(P, n, &ps.ftw);
      if (!rc2) rc2 = upload_fast_vec(P, (dht ? "dht/" : "d23/") + std::to_string(n), w, &ps.d23_tab);
      if (rc2) return rc2;
      const bool packed = fast_packed(ps.fop);
      ps.clines = P->rb == 8 ? fast_tw<dd>(ps.logm, ps.fop) : fast_tw<float>(ps.logm, ps.fop);
      ps.lines = packed ? 2 * ps.clines : ps.clines;
      ps.threads = P->rb == 8 ? fast_threads<dd>(ps.logm, ps.fop) : fast_threads<float>(ps.logm, ps.fop);
      ps.smem = P->rb == 8 ? fast_smem<dd>(ps.logm, ps.fop) : fast_smem<float>(ps.logm, ps.fop);
      return PFGB_OK;
    }
  }
  if ((ps.op == OP_C2C || ps.op == OP_R2C || ps.op == OP_C2R || x00) && ps.L == 0 && M >= 8 &&
      M <= 4096 && (M & (M - 1)) == 0 &&
      !(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
    ps.fast = true;
    ps.fop = x00 ? (ps.op == OP_R2R_C ? OP_X00C : OP_X00R) : ps.t4_dim >= 0 ? OP_C2CT : ps.op;
    if (ps.t4_dim >= 0) {
      rc = upload_fast_table(P, (int)ps.t4_M, &ps.t4_tab);
      if (rc) return rc;
    }
    ps.logm = 0;
    while ((1 << ps.logm) < M) ++ps.logm;
    rc = upload_fast_table(P, M, &ps.ftw);
    if (!rc && P->fx) rc = upload_fast_table_fx(P, M, ps.sign, &ps.ftw_fx);
    if (rc) return rc;
    const bool packed = fast_packed(ps.fop);
    ps.clines = P->rb == 8 ? fast_tw<dd>(ps.logm, ps.fop) : fast_tw<float>(ps.logm, ps.fop);
    ps.lines = packed ? 2 * ps.clines : ps.clines;
    ps.threads = P->rb == 8 ? fast_threads<dd>(ps.logm, ps.fop) : fast_threads<float>(ps.logm, ps.fop);
    ps.smem = P->rb == 8 ? fast_smem<dd>(ps.logm, ps.fop) : fast_smem<float>(ps.logm, ps.fop);
    if (P->precision == PFGB_PRECISION_TC_SPLIT && ps.fop == OP_C2C && tc_lines(ps.logm) > 0) {
      ps.tc = true;
      ps.clines = ps.lines = tc_lines(ps.logm);
      rc = upload_tc_table(P, ps.logm, ps.sign, &ps.tcb);
      if (rc) return rc;
    }
    return PFGB_OK;
  }
  // lines of 3 * 2^k and 5 * 2^k points (8 <= 2^k <= 512) take the
  // mixed-radix register pass, in dd for Float64 data unless native FP64
  // was requested
  if ((ps.op == OP_C2C || ps.op == OP_R2C || ps.op == OP_C2R) && ps.L == 0 &&
      !(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
    for (int r0 : {3, 5}) {
      if (M % r0) continue;
      const int n = M / r0;
      if (n < 8 || n > 512 || (n & (n - 1))) continue;
      ps.mr = true;
      ps.fop = ps.op;
      ps.r0 = r0;
      ps.logn = 0;
      while ((1 << ps.logn) < n) ++ps.logn;
      rc = upload_fast_table(P, n, &ps.ftw);
      if (!rc) rc = upload_fast_table(P, M, &ps.ftw2);
      if (rc) return rc;
      const bool packed = fast_packed(ps.op);
      ps.clines = P->rb == 8 ? mr_tw<dd>(ps.logn) : mr_tw<float>(ps.logn);
      ps.lines = packed ? 2 * ps.clines : ps.clines;
      ps.threads = P->rb == 8 ? mr_threads<dd>(ps.logn) : mr_threads<float>(ps.logn);
      ps.smem = P->rb == 8 ? mr_smem<dd>(r0, ps.logn, ps.op) : mr_smem<float>(r0, ps.logn, ps.op);
      return PFGB_OK;
    }
  }
  const int Lc = ps.L > 0 ? ps.L : ps.M;
  int rmin = 64;
  for (int i = 0; i < ps.nst; ++i) rmin = std::min(rmin, ps.rad[i]);
  ps.bpl = std::max(1, Lc / rmin);  // a line of one point has no stage (identity)
  ps.lp = Lc;
  const bool packed = ps.op == OP_R2C || ps.op == OP_C2R || ps.op == OP_R2R_R;
  const size_t cbytes = 2 * (size_t)P->rb;
  // complex lines per CTA: bounded by 1024 threads and the shared-memory budget
  const size_t smem_budget = 96 * 1024;
  int cl_thr = std::max(1, 1024 / ps.bpl);
  int cl_smem = (int)std::max<size_t>(1, smem_budget / (Lc * cbytes));
  int target = 16;  // aim at 16 array lines per tile (coalescing of strided axes)
  int cl = std::min({cl_thr, cl_smem, packed ? target / 2 : target});
  // threads: at least the butterflies, at least 128 for the load/store loops
  if (cl < 1) cl = 1;
  ps.clines = cl;
  ps.lines = packed ? 2 * cl : cl;
  int th = cl * ps.bpl;
  th = std::max(th, 128);
  th = std::min(th, 1024);
  th = (th + 31) / 32 * 32;
  ps.threads = th;
  ps.smem = (size_t)cl * ps.lp * cbytes;
  if (ps.smem > 200 * 1024)
    return fail(PFGB_ERR_UNSUPPORTED, "line does not fit in shared memory");
  ps.zero_fill = ps.L > 0 || (ps.op == OP_R2R_C || ps.op == OP_R2R_R);
  // other c2c / r2c / c2r lines up to 2048 points take the Bluestein register
  // pass (double-float for Float64 data unless native FP64 was requested)
  if ((ps.op == OP_C2C || ps.op == OP_R2C || ps.op == OP_C2R) && M >= 2 && M <= 2048 &&
      !(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
    ps.g_lines = ps.lines;
    ps.g_clines = ps.clines;
    ps.g_threads = ps.threads;
    ps.g_smem = ps.smem;
    return bluestein_form(P, ps);
  }
  return PFGB_OK;
}

// Fills the kernel arguments of a transform pass for given buffers.
// Tile dimension of a pass (-1 for 1D): the contiguous dimension of the
// input when the axis is not, else the output's, else the next in the input.
static int tile_dim(const Pass& ps) {
  const int a = ps.axis;
  const bool a_fast_in = ps.lin.perm[0] == a;
  const bool a_fast_out = ps.lout.perm[0] == a;
  if (!a_fast_in) return ps.lin.perm[0];
  if (!a_fast_out) return ps.lout.perm[0];
  return ps.lin.D > 1 ? ps.lin.perm[1] : -1;
}

// Role of logical dimension dim in a pass: 0 the axis, 1 the tile dimension,
// 2 + o the o-th outer dimension (input memory order), -1 absent.
static int pass_role(const Pass& ps, int dim) {
  if (dim == ps.axis) return 0;
  const int t = tile_dim(ps);
  if (dim == t) return 1;
  int o = 0;
  for (int q = 0; q < ps.lin.D; ++q) {
    const int d = ps.lin.perm[q];
    if (d == ps.axis || d == t) continue;
    if (d == dim) return 2 + o;
    ++o;
  }
  return -1;
}

// Complex lines of a fast pass along its tile dimension (two real lines per
// complex line for r2c / c2r).
static int64_t complex_lines(const Pass& ps) {
  const int t = tile_dim(ps);
  const int64_t nt = t >= 0 ? ps.lin.size[t] : 1;
  return fast_packed(ps.fop) ? (nt + 1) / 2 : nt;
}

// Element -> first-pass line map of the second pass of a Float64 run: the
// first pass p1 numbers its complex lines (coordinate along its tile
// dimension t1, halved when packed) + ncl1 * (outer index in p1's input
// order); for each role of p2 (axis, tile dimension, outer dimensions in
// p2's input order) the coordinate contributes (c >> sh) * mul.  Returns the
// number of p1's complex lines.
static int64_t te_mapping(const Pass& p1, Pass& p2) {
  const int a1 = p1.axis, t1 = tile_dim(p1);
  const int sh1 = fast_packed(p1.fop) ? 1 : 0;
  const int64_t ncl1 = complex_lines(p1);
  int64_t mul1[kMaxD] = {};
  int64_t m = ncl1;
  for (int q = 0; q < p1.lin.D; ++q) {
    const int d = p1.lin.perm[q];
    if (d == a1 || d == t1) continue;
    mul1[d] = m;
    m *= p1.lin.size[d];
  }
  auto role = [&](int d, int& sh, unsigned& mul) {
    if (d >= 0 && d == t1) {
      sh = sh1;
      mul = 1;
    } else if (d < 0 || d == a1) {
      sh = 0;
      mul = 0;
    } else {
      sh = 0;
      mul = (unsigned)mul1[d];
    }
  };
  const int t2 = tile_dim(p2);
  role(p2.axis, p2.te_sh[0], p2.te_mul[0]);
  role(t2, p2.te_sh[1], p2.te_mul[1]);
  int o = 0;
  for (int q = 0; q < p2.lin.D && o < kMaxOuter; ++q) {
    const int d = p2.lin.perm[q];
    if (d == p2.axis || d == t2) continue;
    role(d, p2.te_sh[2 + o], p2.te_mul[2 + o]);
    ++o;
  }
  return m;
}

static int make_args(const pfgb_plan* P, const Pass& ps, const void* in, void* out, bool scale_on,
                     PassArgs& A, int64_t& grid, const Deriv* dv = nullptr) {
  std::memset(&A, 0, sizeof(A));
  A.in = in;
  A.out = out;
  A.tw = ps.tw;
  A.chirp = ps.chirp;
  A.bfilt = ps.bfilt;
  A.r2rtw = ps.r2rtw;
  A.op = ps.op;
  A.r2r_kind = ps.r2r_kind;
  A.sign = ps.sign;
  A.scale_on = scale_on ? 1 : 0;
  A.scale = scale_on ? 1.0 / P->scale : 1.0;
  const int a = ps.axis;
  A.n_in = (int)ps.lin.size[a];
  A.n_out = (int)ps.lout.size[a];
  A.M = ps.M;
  A.L = ps.L;
  A.nst = ps.nst;
  for (int i = 0; i < ps.nst; ++i) A.rad[i] = ps.rad[i];
  A.lines = ps.lines;
  A.clines = ps.clines;
  A.bpl = ps.bpl;
  A.lp = ps.lp;
  A.zero_fill = ps.zero_fill ? 1 : 0;
  // strides in elements of each side
  const int D = ps.lin.D;
  A.in_sa = ps.lin.stride(a);
  A.out_sa = ps.lout.stride(a);
  const bool a_fast_in = ps.lin.perm[0] == a;
  const bool a_fast_out = ps.lout.perm[0] == a;
  int t = -1;
  if (!a_fast_in) {
    t = ps.lin.perm[0];
    if (!a_fast_out && ps.lout.perm[0] != t)
      return fail(PFGB_ERR_UNSUPPORTED, "internal: incompatible pass layouts");
  } else if (!a_fast_out) {
    t = ps.lout.perm[0];
  } else if (D > 1) {
    t = ps.lin.perm[1];
  }
  if (t >= 0) {
    A.nt = ps.lin.size[t];
    A.in_st = ps.lin.stride(t);
    A.out_st = ps.lout.stride(t);
  } else {
    A.nt = 1;
    A.in_st = A.out_st = 0;
  }
  A.in_tfast = (t >= 0 && A.in_st == 1) ? 1 : 0;
  A.out_tfast = (t >= 0 && A.out_st == 1) ? 1 : 0;
  A.ntiles = (A.nt + ps.lines - 1) / ps.lines;
  int no = 0;
  int64_t nblocks = A.ntiles;
  for (int q = 0; q < D; ++q) {  // outer dims in input memory order
    const int d = ps.lin.perm[q];
    if (d == a || d == t) continue;
    if (no >= kMaxOuter) return fail(PFGB_ERR_UNSUPPORTED, "too many dimensions");
    A.osz[no] = ps.lin.size[d];
    A.in_so[no] = ps.lin.stride(d);
    A.out_so[no] = ps.lout.stride(d);
    nblocks *= ps.lin.size[d];
    ++no;
  }
  A.nouter = no;
  grid = nblocks;
  // role of logical dimension dim in this pass: 0 axis, 1 tile, 2 + o outer
  auto role_of = [&](int dim) {
    if (dim == a) return 0;
    if (dim == t) return 1;
    int o = 0;
    for (int q = 0; q < D; ++q) {
      const int d = ps.lin.perm[q];
      if (d == a || d == t) continue;
      if (d == dim) return 2 + o;
      ++o;
    }
    return -1;
  };
  if (dv && dv->mode == 3) {
    A.nterm = dv->nterm;
    for (int k = 0; k < dv->nterm; ++k) {
      const int role = role_of(dv->tdim[k]);
      if (role < 0) return fail(PFGB_ERR_ARGUMENT, "derivative dimension not found in the pass");
      A.tsrc[k] = dv->tsrc[k];
      A.trole[k] = role;
      A.thalf[k] = dv->thalf[k];
      A.tn[k] = dv->tn[k];
      A.tk0[k] = dv->tk0[k];
    }
  } else if (dv && dv->mode) {
    const int role = role_of(dv->dim);
    if (role < 0) return fail(PFGB_ERR_ARGUMENT, "derivative dimension not found in the pass");
    A.deriv = dv->mode;
    A.deriv_role = role;
    A.deriv_half = dv->half;
    A.deriv_n = dv->n;
    A.k0 = dv->k0;
  }
  return PFGB_OK;
}

// fxi: index of the pass in its direction for fx arithmetic (selects the
// exponent-word buffers), -1 for float / dd.
static int make_fast_args(const pfgb_plan* P, const Pass& ps, const void* in, void* out,
                          bool scale_on, FastArgs& F, int64_t& grid, const Deriv* dv = nullptr,
                          int fxi = -1) {
  PassArgs A;
  int rc = make_args(P, ps, in, out, scale_on, A, grid, dv);
  if (rc) return rc;
  std::memset(&F, 0, sizeof(F));
  F.in = in;
  F.out = out;
  F.tw = ps.ftw;
  F.tw2 = ps.ftw2;
  F.t4_tab = ps.t4_tab;
  F.t4_role = ps.t4_dim >= 0 ? pass_role(ps, ps.t4_dim) : 0;
  F.op = ps.fop;
  F.r2r_odd = (ps.r2r_kind == K_RODFT00 || ps.r2r_kind == K_RODFT10 || ps.r2r_kind == K_RODFT01 ||
               ps.r2r_kind == K_RODFT11) ? 1
              : ps.r2r_kind == K_DHT                                                             ? 2
                                                                                                 : 0;
  F.d23_tab = ps.d23_tab;
  F.n_in = A.n_in;
  F.n_out = A.n_out;
  F.lmap_tile = A.in_tfast;
  F.out_tfast = A.out_tfast;
  {  // float r2c: the split's two output lines in one 16-byte store (in the
     // c2c kernel the same branch cost registers and spills, so it is r2c only)
    bool v2 = P->rb == 4 && ps.op == OP_R2C && A.out_tfast && A.out_st == 1 &&
              A.out_sa % 2 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    for (int d = 0; d < A.nouter; ++d) v2 = v2 && A.out_so[d] % 2 == 0;
    F.vec2 = v2 ? 1 : 0;
  }
  F.store_direct = A.in_tfast ? A.out_tfast : (A.out_sa == 1 ? 1 : 0);
  F.in_dd = ps.in_dd ? 1 : 0;
  F.out_dd = ps.out_dd ? 1 : 0;
  F.emax_ptr = P->emax_dev;
  F.self_scale = ps.self_scale ? 1 : 0;
  F.te_rescale = ps.te_rescale ? 1 : 0;
  F.te = (ps.self_scale && ps.out_dd) || ps.te_rescale ? P->te_dev : nullptr;
  F.te_ncl = complex_lines(ps);
  for (int i = 0; i < 2 + kMaxOuter; ++i) {
    F.te_sh[i] = ps.te_sh[i];
    F.te_mul[i] = ps.te_mul[i];
  }
  F.scale_on = scale_on ? 1 : 0;
  const ld sc = 1.0L / (ld)P->scale;
  F.scale_h = (float)sc;
  F.scale_l = (float)(sc - (ld)F.scale_h);
  if (F.scale_on && P->rb == 8 && !ps.out_dd) {
    // a power-of-two normalisation of double outputs is an exponent offset
    int k = 0;
    const ld mant = frexpl(sc, &k);
    if (mant == 0.5L) {
      F.scale_on = 0;
      F.emax_shift = k - 1;
    } else if (fxi >= 0) {
      // fx: multiply by the significand, add the exponent at the conversion
      F.scale_fx = (long long)llroundl(mant * std::ldexp((ld)1, 60));
      F.emax_shift = k;
    }
  }
  if (ps.half_fold && fxi < 0) F.emax_shift -= 1;
  if (fxi >= 0) {
    F.tw = ps.ftw_fx;
    F.te_in = ps.in_dd ? P->te_fx[(fxi + 1) & 1] : nullptr;
    F.te_out = ps.out_dd ? P->te_fx[fxi & 1] : nullptr;
    F.self_scale = 0;
    F.te_rescale = 0;
    F.te = nullptr;
  }
  if (A.nterm > 0) {
    if (ps.fop != OP_C2C) return fail(PFGB_ERR_UNSUPPORTED, "internal: derivative sum on a non-c2c pass");
    F.op = OP_CSUM;
    F.nterm = A.nterm;
    for (int k = 0; k < A.nterm; ++k) {
      F.tsrc[k] = A.tsrc[k];
      F.trole[k] = A.trole[k];
      F.thalf[k] = A.thalf[k];
      F.tn[k] = A.tn[k];
      F.tk0_h[k] = (float)A.tk0[k];
      F.tk0_l[k] = (float)((ld)A.tk0[k] - (ld)F.tk0_h[k]);
    }
  }
  F.deriv = A.deriv;
  F.deriv_role = A.deriv_role;
  F.deriv_half = A.deriv_half;
  F.deriv_n = A.deriv_n;
  F.k0_h = (float)A.k0;
  F.k0_l = (float)((ld)A.k0 - (ld)F.k0_h);
  F.nouter = A.nouter;
  F.nt = A.nt;
  F.ntiles = A.ntiles;
  F.in_sa = A.in_sa;
  F.in_st = A.in_st;
  F.out_sa = A.out_sa;
  F.out_st = A.out_st;
  if (grid >= (int64_t{1} << 31)) return fail(PFGB_ERR_UNSUPPORTED, "too many tiles in one pass");
  F.div_tiles = make_div31(A.ntiles);
  for (int d = 0; d < A.nouter; ++d) {
    F.osz[d] = A.osz[d];
    F.in_so[d] = A.in_so[d];
    F.out_so[d] = A.out_so[d];
    F.div_osz[d] = make_div31(A.osz[d]);
  }
  return PFGB_OK;
}

static int make_copy_args(const Pass& ps, const void* in, void* out, CopyArgs& C) {
  std::memset(&C, 0, sizeof(C));
  C.in = in;
  C.out = out;
  const int D = ps.lout.D;
  C.nd = D;
  int64_t total = 1;
  for (int q = 0; q < D; ++q) {
    const int d = ps.lout.perm[q];
    C.osz[q] = ps.lout.size[d];
    C.ist[q] = ps.lin.stride(d);
    C.ost[q] = ps.lout.stride(d);
    total *= ps.lout.size[d];
  }
  C.total = total;
  return PFGB_OK;
}

// Iteration space of a PK_LPACK map: the output layout's memory order, the
// output's points along the axis (n, n / 2 + 1 on the half-spectrum side,
// or the extension / convolution length m), the pair dimension halved; on
// the side that holds both lines of a pair the pair coordinate c addresses
// line 2c, and line 2c + 1 is in_pst / out_pst further.
static int make_lpack_args(const Pass& ps, const void* in, void* out, LPackArgs& L) {
  std::memset(&L, 0, sizeof(L));
  L.in = in;
  L.out = out;
  const int md = ps.lp_mode;
  L.mode = md;
  L.n = ps.lp_n;
  L.m = ps.lp_m;
  L.kind = ps.r2r_kind;
  L.packed = ps.lp_packed ? 1 : 0;
  L.tab = ps.lp_tab;
  const int a = ps.axis, p = ps.lp_dim;
  // maps whose input is the user-side line (the output the packed line)
  const bool data_in = md == LP_R2C_PACK || md == LP_C2R_HPACK || md == LP_R2R_PRE || md == LP_CHIRP_PRE;
  const bool in_pairs = p >= 0 && data_in;
  const bool out_pairs = p >= 0 && !data_in;
  const Layout& O = ps.lout;
  const Layout& H = data_in ? ps.lout : ps.lin;  // one line per pair
  const Layout& F = data_in ? ps.lin : ps.lout;  // both lines
  int64_t ka = ps.lp_n;
  if (md == LP_R2C_SEP || md == LP_C2R_HPACK) ka = ps.lp_n / 2 + 1;
  if (md == LP_R2R_PRE || md == LP_CHIRP_PRE || md == LP_MUL) ka = ps.lp_m;
  if (O.D > kMaxOuter) return fail(PFGB_ERR_UNSUPPORTED, "too many dimensions");
  L.nd = O.D;
  L.qa = L.qp = -1;
  int64_t total = 1;
  for (int q = 0; q < O.D; ++q) {
    const int d = O.perm[q];
    L.ext[q] = d == a ? ka : H.size[d];
    L.ist[q] = ps.lin.stride(d) * (in_pairs && d == p ? 2 : 1);
    L.ost[q] = ps.lout.stride(d) * (out_pairs && d == p ? 2 : 1);
    if (d == a) L.qa = q;
    if (d == p) L.qp = q;
    total *= L.ext[q];
  }
  L.total = total;
  for (int q = 0; q < O.D; ++q) L.dext[q] = make_div31(L.ext[q] < (int64_t{1} << 31) ? L.ext[q] : 1);
  L.npair = p >= 0 ? F.size[p] : 1;
  L.ist_a = ps.lin.stride(a);
  L.ost_a = ps.lout.stride(a);
  L.in_pst = in_pairs ? ps.lin.stride(p) : 0;
  L.out_pst = out_pairs ? ps.lout.stride(p) : 0;
  return PFGB_OK;
}

// Launchers (pfgb_kernels.cu)
int launch_pass(int real_bytes, const PassArgs& A, int64_t grid, int threads, size_t smem,
                cudaStream_t s);
int launch_copy(int elt_bytes, const CopyArgs& C, cudaStream_t s);
int launch_lpack(int real_bytes, const LPackArgs& L, cudaStream_t s);
int launch_fast_f32(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_dd(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

// The register pass kernel of a plain (not TMA-fed, not tensor-core) launch.
static int launch_plain(const pfgb_plan* P, const Pass& ps, const FastArgs& F, int64_t grid, cudaStream_t s) {
  return P->rb == 8 ? launch_fast_dd(ps.logm, ps.sign, F, grid, s) : launch_fast_f32(ps.logm, ps.sign, F, grid, s);
}
int launch_fast_fx(int logm, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_fast_tma_f32(int logm, int sign, const FastArgs& A, cudaStream_t s);
int launch_tc(int logm, int sign, const FastArgs& A, cudaStream_t s);
int launch_fast_tma_dd(int logm, int sign, const FastArgs& A, cudaStream_t s);
int launch_mr_f32_c2c(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_mr_f32_r2c(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_mr_f32_c2r(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_mr_dd_c2c(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_mr_dd_r2c(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_mr_dd_c2r(int r0, int logn, int sign, const FastArgs& A, int64_t grid, cudaStream_t s);

int launch_bs_f32_c2c(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_bs_f32_r2c(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_bs_f32_c2r(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_bs_dd_c2c(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_bs_dd_r2c(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);
int launch_bs_dd_c2r(int logl, const FastArgs& A, int64_t grid, cudaStream_t s);

// Bluestein pass of a plan (grid == 0: configure only)
static int launch_bs(const pfgb_plan* P, const Pass& ps, const FastArgs& F, int64_t grid, cudaStream_t s) {
  const bool d = P->rb == 8;
  switch (ps.op) {
    case OP_C2C: return d ? launch_bs_dd_c2c(ps.logl, F, grid, s) : launch_bs_f32_c2c(ps.logl, F, grid, s);
    case OP_R2C: return d ? launch_bs_dd_r2c(ps.logl, F, grid, s) : launch_bs_f32_r2c(ps.logl, F, grid, s);
    case OP_C2R: return d ? launch_bs_dd_c2r(ps.logl, F, grid, s) : launch_bs_f32_c2r(ps.logl, F, grid, s);
    default: return fail(PFGB_ERR_UNSUPPORTED, "internal: Bluestein pass operation");
  }
}

// The generic-kernel form of a Bluestein pass (its own geometry)
static Pass generic_form(const Pass& ps) {
  Pass g = ps;
  g.bs = false;
  g.lines = ps.g_lines;
  g.clines = ps.g_clines;
  g.threads = ps.g_threads;
  g.smem = ps.g_smem;
  return g;
}

// mixed-radix pass of a plan (grid == 0: configure only); OP_CSUM runs the
// c2c kernel (its load sums the terms)
static int launch_mr(const pfgb_plan* P, const Pass& ps, const FastArgs& F, int64_t grid, cudaStream_t s) {
  const bool d = P->rb == 8;
  switch (F.op) {
    case OP_C2C: case OP_CSUM:
      return d ? launch_mr_dd_c2c(ps.r0, ps.logn, ps.sign, F, grid, s)
               : launch_mr_f32_c2c(ps.r0, ps.logn, ps.sign, F, grid, s);
    case OP_R2C:
      return d ? launch_mr_dd_r2c(ps.r0, ps.logn, ps.sign, F, grid, s)
               : launch_mr_f32_r2c(ps.r0, ps.logn, ps.sign, F, grid, s);
    case OP_C2R:
      return d ? launch_mr_dd_c2r(ps.r0, ps.logn, ps.sign, F, grid, s)
               : launch_mr_f32_c2r(ps.r0, ps.logn, ps.sign, F, grid, s);
    default:
      return fail(PFGB_ERR_UNSUPPORTED, "internal: mixed-radix pass operation");
  }
}

#ifndef PFGB_FAST_TMA
#define PFGB_FAST_TMA 0
#endif

// The TMA-fed persistent form needs contiguous input lines (stride 1 along
// the axis) whose byte length and start addresses are multiples of 16, and is
// written for c2r passes (each input element feeds two positions of the
// Hermitian extension, so reading the tile from shared memory halves the
// global loads).  Off by default: with three resident 256-thread CTAs per SM
// the plain kernel overlaps load and compute better (Float64 512^3 c2r pass
// 1.05 ms against 1.09 ms; the TMA form's two tile buffers allow two CTAs).
static bool tma_eligible(const pfgb_plan* P, const Pass& ps, const FastArgs& F) {
  const bool wanted = ps.variant == 1 || (ps.variant < 0 && (PFGB_FAST_TMA || P->force_tma));
  if (!wanted || !ps.fast || F.op != OP_C2R || F.lmap_tile || F.in_sa != 1) return false;
  const int esz = F.op == OP_R2C ? P->rb : 2 * P->rb;
  const int64_t line = (int64_t)(F.op == OP_C2R ? F.n_in : (1 << ps.logm)) * esz;
  if (line % 16) return false;
  if ((F.in_st * esz) % 16) return false;
  for (int d = 0; d < F.nouter; ++d)
    if ((F.in_so[d] * esz) % 16) return false;
  return (reinterpret_cast<uintptr_t>(F.in) & 15) == 0;
}

// ---------------------------------------------------------------------------
// Schedule: build the passes of one direction and assign buffers.
// ---------------------------------------------------------------------------
static Layout natural_layout(const pfgb_plan* P, const int64_t* sizes, bool complex, int64_t pitch0) {
  Layout L;
  L.D = P->D;
  for (int d = 0; d < P->N; ++d) L.size[d] = sizes[d];
  for (int e = 0; e < P->K; ++e) L.size[P->N + e] = P->desc.extra_dims[e];
  for (int q = 0; q < L.D; ++q) L.perm[q] = q;
  L.pitch0 = pitch0 > 0 ? pitch0 : L.size[L.perm[0]];
  L.complex = complex;
  L.elt = complex ? 2 * P->rb : P->rb;
  return L;
}

static Layout final_layout(const pfgb_plan* P, const int64_t* sizes, bool complex) {
  Layout L = natural_layout(P, sizes, complex, 0);
  if (P->permute) {
    for (int q = 0; q < P->N; ++q) L.perm[q] = P->N - 1 - q;
    L.pitch0 = L.size[L.perm[0]];
  }
  return L;
}

static bool layouts_differ(const pfgb_plan* P) { return P->permute && P->N >= 2; }

// In-place safety of a pass: every tile writes exactly the bytes it read.
static bool inplace_ok(const Pass& ps) {
  if (!ps.lin.same_order(ps.lout)) return false;
  const int a = ps.axis;
  for (int d = 0; d < ps.lin.D; ++d) {
    if (d == a) continue;
    if (ps.lin.stride(d) * ps.lin.elt != ps.lout.stride(d) * ps.lout.elt) return false;
  }
  if (ps.lin.perm[0] == a) {
    return ps.lin.pitch0 * ps.lin.elt == ps.lout.pitch0 * ps.lout.elt;
  }
  return ps.lin.elt == ps.lout.elt && ps.lin.size[a] == ps.lout.size[a];
}

// A line length one register pass takes: a power of two up to 4096 (fast
// pass; lengths below 8 through Bluestein), 3 * 2^k or 5 * 2^k with
// 8 <= 2^k <= 512 (mixed-radix pass), or any length up to 2048 (Bluestein).
static bool one_pass_length(int64_t n) {
  if (n < 2 || n > 4096) return false;
  if ((n & (n - 1)) == 0) return true;
  for (int r0 : {3, 5}) {
    const int64_t m = n / r0;
    if (n % r0 == 0 && m >= 8 && m <= 512 && (m & (m - 1)) == 0) return true;
  }
  return n <= 2048;
}

// Inserts dimension v right after (after = true) or before dimension a in a
// layout's memory order, a keeping m1 points and v taking m2 (a line of
// m1 * m2 points seen as two dimensions).  false if a is the fastest
// dimension and padded.
static bool split_layout(const Layout& L, int a, int v, int64_t m1, int64_t m2, bool after, Layout& out) {
  if (L.perm[0] == a && L.pitch0 != L.size[a]) return false;
  out = L;
  out.D = L.D + 1;
  out.size[a] = m1;
  out.size[v] = m2;
  int q = 0;
  for (int i = 0; i < L.D; ++i) {
    if (L.perm[i] == a) {
      if (after) { out.perm[q++] = a; out.perm[q++] = v; }
      else { out.perm[q++] = v; out.perm[q++] = a; }
    } else {
      out.perm[q++] = L.perm[i];
    }
  }
  out.pitch0 = out.size[out.perm[0]];
  if (L.perm[0] != a) out.pitch0 = L.pitch0;
  return true;
}

// Memory orders a transform pass can pair: its axis the fastest dimension on
// one side, or both sides with the same fastest dimension (the tile
// dimension of the pass kernels).
static bool orders_compatible(const Layout& lin, const Layout& lout, int a) {
  return lin.perm[0] == a || lout.perm[0] == a || lin.perm[0] == lout.perm[0];
}

// The sizes, element type and padding-free extent of `L` in the memory
// order of `order`.
static Layout reordered(const Layout& L, const Layout& order) {
  Layout r = L;
  for (int q = 0; q < L.D; ++q) r.perm[q] = order.perm[q];
  r.pitch0 = r.size[r.perm[0]];
  return r;
}

// The power-of-two factor M2 (8 <= M2 <= 4096) of the most balanced split
// M = M1 * M2 with M1 a one-pass length; 0 if none.
static int64_t split_factor(int64_t M) {
  if (M <= 4096 || M > (int64_t{1} << 24)) return 0;
  int64_t best_m2 = 0;
  double best = 1e9;
  for (int64_t m2 = 8; m2 <= 4096 && m2 < M; m2 *= 2) {
    if (M % m2 || !one_pass_length(M / m2)) continue;
    const double d = std::fabs(std::log2((double)(M / m2)) - std::log2((double)m2));
    if (d < best) { best = d; best_m2 = m2; }
  }
  return best_m2;
}

// How a c2c line of M points runs: one pass (register or generic kernel,
// LF_ONE), split in two passes (LF_SPLIT), or as a Bluestein convolution of
// a power-of-two length through split passes (LF_BLUESTEIN); LF_NONE beyond
// 2^23 points without a split.
enum LongForm { LF_NONE = -1, LF_ONE = 0, LF_SPLIT = 1, LF_BLUESTEIN = 2 };
static int64_t bluestein_length(int64_t M) {
  int64_t L = 1;
  while (L < 2 * M - 1) L <<= 1;
  return L;
}
static int long_c2c_form(int64_t M) {
  if (M <= 4096) return LF_ONE;
  if (split_factor(M)) return LF_SPLIT;
  std::vector<int> rad;
  if (M <= kMaxLc && factor_radices((int)M, rad)) return LF_ONE;  // the generic kernel's core
  return bluestein_length(M) <= (int64_t{1} << 24) ? LF_BLUESTEIN : LF_NONE;
}

// Long c2c lines (M > 4096): M = M1 * M2 with M2 = 2^k (8 <= 2^k <= 4096)
// and M1 a one-pass length, two passes: with n = n1 + M1 n2 and
// k = k2 + M2 k1, pass A transforms n2 (the layout's dimension a split as
// (n1 faster, n2)) and multiplies by W_M^(n1 k2); pass B transforms n1 and
// writes X[k2 + M2 k1] through the output layout split as (k2 faster, k1).
// Chooses the split with the most balanced M1, M2; false if none, or if the
// second pass's orders do not pair (an axis that is fastest on neither side
// of a pass that changes the memory order).
static bool split_long_pass(const Pass& ps, Pass& A, Pass& B) {
  if (ps.pk != PK_TRANSFORM || ps.op != OP_C2C) return false;
  const int a = ps.axis;
  const int64_t M = ps.lin.size[a];
  const int64_t m2 = split_factor(M);
  if (!m2) return false;
  const int64_t m1 = M / m2;
  const int v = ps.lin.D;  // the split's second dimension
  Layout lin_s, lout_s;
  if (!split_layout(ps.lin, a, v, m1, m2, true, lin_s)) return false;
  if (!split_layout(ps.lout, a, v, m1, m2, false, lout_s)) return false;
  if (!orders_compatible(lin_s, lout_s, a)) return false;
  A = ps;
  A.four = true;
  A.axis = v;
  A.lin = lin_s;
  A.lout = lin_s;  // the intermediate keeps the input's order (in place possible)
  A.t4_dim = a;
  A.t4_M = M;
  B = ps;
  B.four = true;
  B.axis = a;
  B.lin = lin_s;
  B.lout = lout_s;
  return true;
}

// Pair dimension of packed real lines along axis a: the slowest other
// dimension of even size, else the slowest of size >= 2 (-1: one line).
static int pair_dim(const Layout& R, int a) {
  for (int q = R.D - 1; q >= 0; --q)
    if (R.perm[q] != a && R.size[R.perm[q]] >= 2 && R.size[R.perm[q]] % 2 == 0) return R.perm[q];
  for (int q = R.D - 1; q >= 0; --q)
    if (R.perm[q] != a && R.size[R.perm[q]] >= 2) return R.perm[q];
  return -1;
}

// The packed complex lines of a long-line form: the sizes of `data` (axis a
// at m points, pair dimension p halved) in the memory order of `order`,
// complex elements of elt bytes, no padding.
static Layout packed_layout(const Layout& data, const Layout& order, int a, int64_t m, int p, int elt) {
  Layout z = order;
  for (int d = 0; d < z.D; ++d) z.size[d] = data.size[d];
  z.size[a] = m;
  if (p >= 0) z.size[p] = (data.size[p] + 1) / 2;
  z.complex = true;
  z.elt = elt;
  z.pitch0 = z.size[z.perm[0]];
  return z;
}

// Long r2c / c2r lines (n > 4096 real points whose n-point c2c line is
// split or runs as a Bluestein convolution): an element map that packs two
// real lines (neighbours along the pair dimension) into one complex line
// (r2c: z = x1 + i x2; c2r: Z = X1 + i X2 over the Hermitian extension of
// both half spectra), the n-point c2c transform of the packed lines, and an
// element map that separates the two spectra (r2c) or the real and imaginary
// parts (c2r).  The packed layouts take the memory order of the map beside
// them, so that a split c2c transform carries any re-layout; where its passes
// cannot (or for a Bluestein form) the c2c lines keep one order and the
// separating map re-lays out.
static bool expand_long_real(const Pass& ps, Pass& pre, Pass& c, Pass& post) {
  if (ps.pk != PK_TRANSFORM || (ps.op != OP_R2C && ps.op != OP_C2R)) return false;
  const int a = ps.axis;
  const bool r2c = ps.op == OP_R2C;
  const Layout& R = r2c ? ps.lin : ps.lout;  // real side
  const Layout& X = r2c ? ps.lout : ps.lin;  // complex side (half spectra)
  const int64_t n = R.size[a];
  const int form = long_c2c_form(n);
  if (n <= 4096 || R.D > kMaxOuter || (form != LF_SPLIT && form != LF_BLUESTEIN)) return false;
  const int p = pair_dim(R, a);
  const Layout z_real = packed_layout(R, R, a, n, p, X.elt), z_cplx = packed_layout(R, X, a, n, p, X.elt);
  c = ps;
  c.op = OP_C2C;
  c.sign = r2c ? -1 : 1;
  c.lin = r2c ? z_real : z_cplx;
  c.lout = r2c ? z_cplx : z_real;
  Pass A, B;
  if (form == LF_BLUESTEIN || !split_long_pass(c, A, B)) c.lout = c.lin;
  pre = ps;
  pre.pk = PK_LPACK;
  pre.lp_mode = r2c ? LP_R2C_PACK : LP_C2R_HPACK;
  pre.lp_dim = p;
  pre.lp_n = n;
  pre.lin = ps.lin;
  pre.lout = c.lin;
  post = pre;
  post.lp_mode = r2c ? LP_R2C_SEP : LP_C2R_UNPACK;
  post.lin = c.lout;
  post.lout = ps.lout;
  return true;
}

// Extension length of an R2R line of n points (the generic kernel's DFT).
static int64_t r2r_extension(int kind, int64_t n) {
  switch (kind) {
    case K_DHT: return n;
    case K_REDFT00: return 2 * (n - 1);
    case K_RODFT00: return 2 * (n + 1);
    default: return 2 * n;
  }
}

// R2R kinds and lengths with a register-pass form of their own (prepare_pass:
// REDFT00 / RODFT00 through a power-of-two extension, the D2 / D3 / DHT
// kinds of 2^k points, REDFT11 / RODFT11 of 2^k points up to 2048).
static bool r2r_register_form(const pfgb_plan* P, int kind, int64_t n) {
  if (P->fx || (P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) return false;
  auto pow2 = [](int64_t v) { return v > 0 && (v & (v - 1)) == 0; };
  switch (kind) {
    case K_REDFT00:
    case K_RODFT00: {
      const int64_t m = r2r_extension(kind, n);
      return pow2(m) && m >= 8 && m <= 4096;
    }
    case K_REDFT11:
    case K_RODFT11: return pow2(n) && n >= 4 && n <= 2048;
    default: return pow2(n) && n >= 8 && n <= 4096;
  }
}

// R2R lines through their extension (m points) as a c2c line: the extension
// gathered into packed complex lines (two real lines per complex line for
// real data: every kind has a real kernel), the m-point c2c transform, and
// the outputs read from it.  Taken where the extension is beyond the generic
// kernel's core (split or Bluestein c2c), and in Float64 plans for every line
// without a register form of its own whose extension is a one-pass length:
// the c2c pass then runs in double-float on a register kernel instead of the
// generic kernel's native FP64.
static bool expand_long_r2r(const pfgb_plan* P, const Pass& ps, Pass& pre, Pass& c, Pass& post) {
  if (ps.pk != PK_TRANSFORM || (ps.op != OP_R2R_C && ps.op != OP_R2R_R)) return false;
  const int a = ps.axis;
  const int64_t n = ps.lin.size[a];
  if (n < 2 || ps.lin.D > kMaxOuter) return false;
  const int64_t m = r2r_extension(ps.r2r_kind, n);
  std::vector<int> rad;
  const bool generic = m <= kMaxLc && (factor_radices((int)m, rad) || bluestein_length(m) <= kMaxLc);
  const int form = long_c2c_form(m);
  const bool dd_route = P->rb == 8 && !P->fx && !r2r_register_form(P, ps.r2r_kind, n) && one_pass_length(m);
  if (!dd_route && (generic || (form != LF_SPLIT && form != LF_BLUESTEIN))) return false;
  const bool real = ps.op == OP_R2R_R;
  const int p = real ? pair_dim(ps.lin, a) : -1;
  const int celt = real ? 2 * ps.lin.elt : ps.lin.elt;
  const Layout z = packed_layout(ps.lin, ps.lin, a, m, p, celt);
  c = ps;
  c.op = OP_C2C;
  c.sign = -1;
  c.r2r_kind = 0;
  c.lin = c.lout = z;
  pre = ps;
  pre.pk = PK_LPACK;
  pre.lp_mode = LP_R2R_PRE;
  pre.lp_dim = p;
  pre.lp_n = n;
  pre.lp_m = m;
  pre.lp_packed = real;
  pre.lin = ps.lin;
  pre.lout = z;
  post = pre;
  post.lp_mode = LP_R2R_POST;
  post.lin = z;
  post.lout = ps.lout;
  return true;
}

// c2c lines of M points without a split beyond the generic kernel's core:
// Bluestein with a power-of-two convolution length L >= 2M - 1 as element
// maps and two split L-point transforms, chirp product and zero padding,
// forward transform, product with the filter spectrum, inverse transform,
// chirp product and truncation (the output map re-lays out).
static bool expand_bluestein(const Pass& ps, std::vector<Pass>& out) {
  if (ps.pk != PK_TRANSFORM || ps.op != OP_C2C || ps.four) return false;
  const int a = ps.axis;
  const int64_t M = ps.lin.size[a];
  if (long_c2c_form(M) != LF_BLUESTEIN || ps.lin.D > kMaxOuter) return false;
  const int64_t L = bluestein_length(M);
  const Layout z = packed_layout(ps.lin, ps.lin, a, L, -1, ps.lin.elt);
  Pass m = ps;
  m.pk = PK_LPACK;
  m.lp_dim = -1;
  m.lp_n = M;
  m.lp_m = L;
  Pass pre = m, mul = m, post = m;
  pre.lp_mode = LP_CHIRP_PRE;
  pre.lout = z;
  mul.lp_mode = LP_MUL;
  mul.lin = mul.lout = z;
  post.lp_mode = LP_CHIRP_POST;
  post.lin = z;
  Pass f = ps, b = ps;
  f.lin = f.lout = b.lin = b.lout = z;
  f.sign = -1;
  b.sign = 1;
  out.push_back(pre);
  out.push_back(f);
  out.push_back(mul);
  out.push_back(b);
  out.push_back(post);
  return true;
}

struct Step {  // one transform of the reference's per-dimension loop
  int axis, op, r2r, sign;
};

static int build_direction(pfgb_plan* P, bool forward, Direction& dir, int64_t cap_src,
                           int64_t cap_dst, int64_t pitch_real) {
  const int N = P->N;
  const pfgb_plan_desc& d = P->desc;
  // Element type and sizes along the chain.
  int64_t sizes[kMaxD];
  bool cplx;
  std::vector<Step> steps;
  if (forward) {
    for (int n = 0; n < N; ++n) sizes[n] = P->dims_in[n];
    cplx = P->in_complex;
    for (int n = 0; n < N; ++n) {
      Step s{n, -1, 0, -1};
      switch (d.kind[n]) {
        case PFGB_FFT: s.op = OP_C2C; s.sign = -1; break;
        case PFGB_BFFT: s.op = OP_C2C; s.sign = 1; break;
        case PFGB_RFFT: s.op = OP_R2C; s.sign = -1; break;
        case PFGB_BRFFT: s.op = OP_C2R; s.sign = 1; break;
        case PFGB_R2R: s.op = OP_R2R_C; s.r2r = d.r2r_kind[n]; break;
        default: continue;
      }
      steps.push_back(s);
    }
  } else {
    for (int n = 0; n < N; ++n) sizes[n] = P->dims_out[n];
    cplx = P->out_complex;
    for (int n = N - 1; n >= 0; --n) {
      Step s{n, -1, 0, -1};
      switch (d.kind[n]) {  // binv (reference c2c.jl:58-61, r2c.jl:98-101, r2r.jl:103-131)
        case PFGB_FFT: s.op = OP_C2C; s.sign = 1; break;
        case PFGB_BFFT: s.op = OP_C2C; s.sign = -1; break;
        case PFGB_RFFT: s.op = OP_C2R; s.sign = 1; break;
        case PFGB_BRFFT: s.op = OP_R2C; s.sign = -1; break;
        case PFGB_R2R: s.op = OP_R2R_C; s.r2r = r2r_inverse(d.r2r_kind[n]); break;
        default: continue;
      }
      steps.push_back(s);
    }
  }
  const bool change = layouts_differ(P);
  // index of the step that performs the layout change
  int tx = -1;
  if (change) {
    for (size_t i = 0; i < steps.size(); ++i)
      if (steps[i].axis == 0 || steps[i].axis == N - 1) { tx = (int)i; break; }
  }
  std::vector<Pass> passes;
  auto mk_layout = [&](bool fin, const int64_t* sz, bool cx, int64_t pitch) {
    // "fin" = final (output-pencil) order in the forward direction
    if (fin) return final_layout(P, sz, cx);
    return natural_layout(P, sz, cx, pitch);
  };
  // In the forward direction the data starts in natural order and ends in the
  // final order; backward is the reverse.
  bool start_fin = !forward;
  bool end_fin = forward;
  if (!change) start_fin = end_fin = false;
  const int64_t pitch_start = forward ? pitch_real : 0;
  const int64_t pitch_end = forward ? 0 : pitch_real;
  Layout cur = mk_layout(start_fin, sizes, cplx, pitch_start);
  bool cur_fin = start_fin;
  if (change && tx < 0) {
    // no step can re-layout: a permuted copy first
    Pass c;
    c.pk = PK_COPY;
    c.lin = cur;
    c.lout = mk_layout(end_fin, sizes, cplx, 0);
    c.axis = -1;
    passes.push_back(c);
    cur = c.lout;
    cur_fin = end_fin;
  }
  for (size_t i = 0; i < steps.size(); ++i) {
    const Step& s = steps[i];
    Pass ps;
    ps.pk = PK_TRANSFORM;
    ps.axis = s.axis;
    ps.sign = s.sign;
    ps.r2r_kind = s.r2r;
    ps.op = s.op;
    if (s.op == OP_R2R_C && !cplx) ps.op = OP_R2R_R;
    ps.lin = cur;
    int64_t nsz[kMaxD];
    for (int q = 0; q < N; ++q) nsz[q] = sizes[q];
    bool ncx = cplx;
    if (s.op == OP_R2C) {
      nsz[s.axis] = sizes[s.axis] / 2 + 1;
      ncx = true;
    } else if (s.op == OP_C2R) {
      // output length: forward BRFFT uses even_output; backward RFFT^-1 restores dims_in
      nsz[s.axis] = forward ? length_output(PFGB_BRFFT, d.brfft_even[s.axis] != 0, sizes[s.axis])
                            : P->dims_in[s.axis];
      ncx = false;
    }
    const bool last = i + 1 == steps.size();
    const bool out_fin = ((int)i >= tx && tx >= 0) ? end_fin : cur_fin;
    const int64_t pitch = (last && !out_fin) ? pitch_end : 0;
    ps.lout = mk_layout(out_fin, nsz, ncx, pitch && !ncx ? pitch : 0);
    passes.push_back(ps);
    cur = ps.lout;
    cur_fin = out_fin;
    for (int q = 0; q < N; ++q) sizes[q] = nsz[q];
    cplx = ncx;
  }
  // lines longer than one register pass: real lines through a packed c2c
  // transform, c2c lines in two passes each
  if (!(P->rb == 8 && P->precision == PFGB_PRECISION_NATIVE)) {
    std::vector<Pass> ex;
    for (const Pass& ps : passes) {
      Pass pre, c, post;
      if (expand_long_real(ps, pre, c, post) || expand_long_r2r(P, ps, pre, c, post)) {
        ex.push_back(pre);
        ex.push_back(c);
        ex.push_back(post);
      } else {
        ex.push_back(ps);
      }
    }
    passes.swap(ex);
    ex.clear();
    for (const Pass& ps : passes)
      if (!expand_bluestein(ps, ex)) ex.push_back(ps);
    passes.swap(ex);
    std::vector<Pass> split;
    for (const Pass& ps : passes) {
      Pass A, B;
      if (split_long_pass(ps, A, B)) {
        split.push_back(A);
        split.push_back(B);
        continue;
      }
      // orders the split cannot pair: the two passes in the input's order,
      // then a copy into the output order
      Pass c = ps;
      if (ps.pk == PK_TRANSFORM && ps.op == OP_C2C) c.lout = reordered(ps.lout, ps.lin);
      if (!ps.lin.same_order(ps.lout) && split_long_pass(c, A, B)) {
        Pass cp;
        cp.pk = PK_COPY;
        cp.lin = c.lout;
        cp.lout = ps.lout;
        cp.axis = -1;
        split.push_back(A);
        split.push_back(B);
        split.push_back(cp);
      } else {
        split.push_back(ps);
      }
    }
    passes.swap(split);
  }
  for (const Pass& ps : passes)
    if (ps.pk == PK_TRANSFORM && !orders_compatible(ps.lin, ps.lout, ps.axis))
      return fail(PFGB_ERR_UNSUPPORTED, "internal: incompatible pass layouts");
  if (passes.empty()) {
    if (!P->inplace) {
      Pass c;
      c.pk = PK_COPY;
      c.lin = cur;
      c.lout = cur;
      c.axis = -1;
      passes.push_back(c);
    }
  }
  // Buffer assignment (brute force over {dst, s1, s2} for intermediates).
  const int m = (int)passes.size();
  if (m == 0) {
    dir.passes.clear();
    return PFGB_OK;
  }
  for (int attempt = 0; attempt < 2; ++attempt) {
    const int mm = (int)passes.size();
    int best_cost_ok = 0;
    int64_t best_cost = -1;
    std::vector<int> best;
    std::vector<int> asg(mm);
    // every assignment up to 12 passes; beyond (long lines in several
    // dimensions) the two scratch buffers alternate
    int64_t combos = 1;
    for (int i = 0; i < mm - 1 && mm <= 12; ++i) combos *= 3;
    for (int64_t c = 0; c < combos; ++c) {
      int64_t cc = c;
      for (int i = 0; i < mm - 1; ++i) {
        asg[i] = mm <= 12 ? 1 + (int)(cc % 3) : 2 + (i & 1);
        cc /= 3;
      }
      asg[mm - 1] = 1;
      bool ok = true;
      int64_t need[4] = {0, 0, 0, 0};
      int prev = P->inplace ? 1 : 0;  // in-place plans read the dst buffer
      for (int i = 0; i < mm && ok; ++i) {
        const int bi = prev, bo = asg[i];
        const Pass& ps = passes[i];
        const bool ip = ps.pk == PK_COPY ? ps.lin.same_order(ps.lout) && ps.lin.pitch0 == ps.lout.pitch0 && ps.lin.elt == ps.lout.elt
                        : ps.pk == PK_LPACK ? ps.lp_mode == LP_MUL  // the others read a pair's two
                                                                  // lines, Z[k] and Z[n-k], or change length
                                           : inplace_ok(ps);
        if (bi == bo && !ip) ok = false;
        need[bo] = std::max(need[bo], ps.lout.bytes());
        prev = bo;
      }
      if (!ok) continue;
      if (need[1] > cap_dst) continue;
      const int64_t cost = need[2] + need[3];
      if (best_cost < 0 || cost < best_cost) {
        best_cost = cost;
        best = asg;
        best_cost_ok = 1;
      }
    }
    if (best_cost_ok) {
      int prev = P->inplace ? 1 : 0;
      for (int i = 0; i < mm; ++i) {
        passes[i].bin = prev;
        passes[i].bout = best[i];
        prev = best[i];
        if (best[i] >= 2) {
          const int s = best[i] - 2;
          P->scratch_bytes[s] = std::max(P->scratch_bytes[s], passes[i].lout.bytes());
        }
      }
      dir.passes = passes;
      return PFGB_OK;
    }
    // infeasible: append an identity copy so the data can return to dst
    Pass c;
    c.pk = PK_COPY;
    c.lin = passes.back().lout;
    c.lout = passes.back().lout;
    c.axis = -1;
    passes.push_back(c);
  }
  (void)cap_src;
  return fail(PFGB_ERR_UNSUPPORTED, "internal: no buffer assignment for this plan");
}

static int execute(pfgb_plan* P, const Direction& dir, void* dst, const void* src,
                   cudaStream_t s, bool normalise, int dsign, const Deriv* dv = nullptr) {
  const int m = (int)dir.passes.size();
  if (m == 0) return dv && dv->mode ? fail(PFGB_ERR_UNSUPPORTED, "plan has no transform pass") : PFGB_OK;
  int last_tr = -1, first_tr = -1;
  for (int i = 0; i < m; ++i)
    if (dir.passes[i].pk == PK_TRANSFORM) {
      last_tr = i;
      if (first_tr < 0) first_tr = i;
    }
  const int dpass = dv && dv->mode ? (dv->mode == 2 ? last_tr : first_tr) : -1;
  if (dv && dv->mode == 3 && dpass != 0)
    return fail(PFGB_ERR_UNSUPPORTED, "a sum of derivatives needs the first backward pass to be a transform");
  // Float64 fast passes: fx, or dd for an execution with a fused derivative
  const bool fxrun = P->fx && !(dv && dv->mode);
  if (dv && dv->mode) {
    if (dpass < 0 || dir.passes[dpass].op != OP_C2C)
      return fail(PFGB_ERR_UNSUPPORTED, "the fused derivative needs a complex-to-complex pass at that end "
                                        "of the plan");
    if (dir.passes[dpass].four)
      return fail(PFGB_ERR_UNSUPPORTED, "the fused derivative is not available on a line split in two passes");
  }
  for (int i = 0; i < m; ++i) {
    const Pass& ps = dir.passes[i];
    auto buf = [&](int b) -> void* {
      switch (b) {
        case 0: return const_cast<void*>(src);
        case 1: return dst;
        default: return P->scratch[b - 2];
      }
    };
    const void* in = buf(ps.bin);
    void* out = buf(ps.bout);
    if (ps.pk == PK_COPY && in == out && ps.lin.same_order(ps.lout)) continue;
    if (ps.fast && ps.reduce_before) {
      // the run's exponent word collects the first pass's tile exponents
      PFGB_CUDA(cudaMemsetAsync(P->emax_dev, 0, sizeof(int), s));
    }
    pfgb_plan::Rec rec{dsign, i, nullptr, nullptr};
    if (P->timing) {
      PFGB_CUDA(cudaEventCreate(&rec.a));
      PFGB_CUDA(cudaEventCreate(&rec.b));
      PFGB_CUDA(cudaEventRecord(rec.a, s));
    }
    if (ps.pk == PK_COPY) {
      CopyArgs C;
      make_copy_args(ps, in, out, C);
      int rc = launch_copy(ps.lout.elt, C, s);
      if (rc) return rc;
    } else if (ps.pk == PK_LPACK) {
      LPackArgs L;
      int rc = make_lpack_args(ps, in, out, L);
      if (!rc) rc = launch_lpack(P->rb, L, s);
      if (rc) return rc;
    } else if (ps.fast) {
      FastArgs F;
      int64_t grid = 0;
      const bool fxp = fxrun && !ps.four;  // split lines run in double-float
      int rc = make_fast_args(P, ps, in, out, normalise && i == last_tr, F, grid, i == dpass ? dv : nullptr,
                              fxp ? i : -1);
      if (rc) return rc;
      if (fxp) {
        rc = launch_fast_fx(ps.logm, ps.sign, F, grid, s);
      } else if (ps.tc) {
        F.total = grid;
        F.err = P->emax_dev + 1;
        F.wait_test = P->wait_test;
        F.tcb = ps.tcb;
        rc = launch_tc(ps.logm, ps.sign, F, s);
      } else if (tma_eligible(P, ps, F)) {
        F.total = grid;
        F.err = P->emax_dev + 1;
        F.wait_test = P->wait_test;
        rc = P->rb == 8 ? launch_fast_tma_dd(ps.logm, ps.sign, F, s)
                        : launch_fast_tma_f32(ps.logm, ps.sign, F, s);
      } else {
        rc = launch_plain(P, ps, F, grid, s);
      }
      if (rc) return rc;
    } else if (ps.mr) {
      FastArgs F;
      int64_t grid = 0;
      int rc = make_fast_args(P, ps, in, out, normalise && i == last_tr, F, grid, i == dpass ? dv : nullptr);
      if (rc) return rc;
      rc = launch_mr(P, ps, F, grid, s);
      if (rc) return rc;
    } else if (ps.bs && ps.variant != 2 && !(i == dpass && dv && dv->mode == 3)) {
      FastArgs F;
      int64_t grid = 0;
      int rc = make_fast_args(P, ps, in, out, normalise && i == last_tr, F, grid, i == dpass ? dv : nullptr);
      if (rc) return rc;
      F.bs_m = ps.M;
      F.bs_chirp = ps.bs_chirp;
      F.bs_filt = ps.bs_filt;
      F.div_m = make_div31(ps.op == OP_R2C ? ps.M / 2 + 1 : ps.M);
      rc = launch_bs(P, ps, F, grid, s);
      if (rc) return rc;
    } else {
      // generic kernel (a Bluestein-eligible pass runs here with its generic
      // geometry when a fused sum of derivatives applies to it, or when the
      // planner measured this form faster)
      const Pass g = ps.bs ? generic_form(ps) : ps;
      PassArgs A;
      int64_t grid = 0;
      int rc = make_args(P, g, in, out, normalise && i == last_tr, A, grid, i == dpass ? dv : nullptr);
      if (rc) return rc;
      rc = launch_pass(P->rb, A, grid, g.threads, g.smem, s);
      if (rc) return rc;
    }
    if (P->timing) {
      PFGB_CUDA(cudaEventRecord(rec.b, s));
      P->recs.push_back(rec);
    }
  }
  return PFGB_OK;
}


// ---------------------------------------------------------------------------
// The passes of one execution as work items of the persistent batch kernel
// (pfgb_persist.h) instead of launches.  Float32 plans; each pass takes the
// tile form of its kernel: power-of-two lines of 8 .. 512 points the
// register tile, 3 * 2^k lines (2^k = 128 .. 512) the mixed-radix tile with
// the kernel's 512 threads, every other c2c / r2c / c2r line of 2 .. 1024
// points the Bluestein tile (tables added to the plan when the pass ran
// another kernel).  Other passes (copies, R2R, split lines, longer lines,
// sums of derivatives) have no tile form: PFGB_ERR_UNSUPPORTED.
// ---------------------------------------------------------------------------
static int persist_opc(int op, int sign) { return op == OP_C2C ? (sign < 0 ? 0 : 1) : op == OP_R2C ? 2 : 3; }

static int collect_persist(pfgb_plan* P, const Direction& dir, void* dst, const void* src, bool normalise,
                           const Deriv* dv, std::vector<PersistItem>& items) {
  if (P->rb != 4) return fail(PFGB_ERR_UNSUPPORTED, "persistent batch form: Float32 plans only");
  const int m = (int)dir.passes.size();
  int last_tr = -1, first_tr = -1;
  for (int i = 0; i < m; ++i)
    if (dir.passes[i].pk == PK_TRANSFORM) {
      last_tr = i;
      if (first_tr < 0) first_tr = i;
    }
  const int dpass = dv && dv->mode ? (dv->mode == 2 ? last_tr : first_tr) : -1;
  if (dv && dv->mode == 3) return fail(PFGB_ERR_UNSUPPORTED, "persistent batch form: no sums of derivatives");
  if (dv && dv->mode && (dpass < 0 || dir.passes[dpass].op != OP_C2C))
    return fail(PFGB_ERR_UNSUPPORTED, "the fused derivative needs a complex-to-complex pass at that end of the plan");
  for (int i = 0; i < m; ++i) {
    const Pass& ps = dir.passes[i];
    auto buf = [&](int b) -> void* {
      switch (b) {
        case 0: return const_cast<void*>(src);
        case 1: return dst;
        default: return P->scratch[b - 2];
      }
    };
    const void* in = buf(ps.bin);
    void* out = buf(ps.bout);
    if (ps.pk == PK_COPY && in == out && ps.lin.same_order(ps.lout)) continue;
    const bool cplx = ps.op == OP_C2C || ps.op == OP_R2C || ps.op == OP_C2R;
    Pass q = ps;
    int code = -1;
    if (ps.pk == PK_TRANSFORM && cplx) {
      if (ps.fast && !ps.tc && ps.fop == ps.op && ps.logm >= 3 && ps.logm <= 9) {
        code = persist_code(PK_FAST_TILE, persist_opc(ps.op, ps.sign), ps.logm);
      } else if (ps.mr && ps.r0 == 3 && ps.logn >= 7 && ps.logn <= 9) {
        q.clines = kPersistThreads / ((1 << ps.logn) / 8);
        q.lines = fast_packed(ps.op) ? 2 * q.clines : q.clines;
        code = persist_code(PK_MR_TILE, persist_opc(ps.op, ps.sign), ps.logn);
      } else if (!ps.fast && ps.M >= 2 && ps.M <= 1024) {
        if (!ps.bs) {
          int rc = bluestein_form(P, q);
          if (rc) return rc;
        }
        code = persist_code(PK_BS_TILE, persist_opc(ps.op, ps.sign), q.logl);
      }
    }
    if (code < 0 || persist_smem(code) == 0)
      return fail(PFGB_ERR_UNSUPPORTED, "persistent batch form: pass " + std::to_string(i) + " has no tile form");
    PersistItem it;
    std::memset(&it, 0, sizeof(it));
    int64_t grid = 0;
    int rc = make_fast_args(P, q, in, out, normalise && i == last_tr, it.F, grid, i == dpass ? dv : nullptr);
    if (rc) return rc;
    if (q.bs) {
      it.F.bs_m = q.M;
      it.F.bs_chirp = q.bs_chirp;
      it.F.bs_filt = q.bs_filt;
      it.F.div_m = make_div31(q.op == OP_R2C ? q.M / 2 + 1 : q.M);
    }
    it.code = code;
    it.ntiles = (int)grid;
    if (it.ntiles > 0) items.push_back(it);
  }
  return PFGB_OK;
}

}  // namespace pfgb

using namespace pfgb;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Batches (pfgb_batch_*): graph form and persistent form
// ---------------------------------------------------------------------------
struct pfgb_batch {
  cudaStream_t cap = nullptr;
  std::vector<cudaStream_t> side;  // branches of the recorded graph form
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int n = 0;
  int form = PFGB_BATCH_GRAPH;
  int device = 0;
  // persistent form: one device allocation holding the work list, the
  // per-launch counters and the control words
  void* dmem = nullptr;
  int* status = nullptr;
  int* polls = nullptr;
  int items = 0;
  int64_t tiles = 0;
  int grid = 0;
  size_t smem = 0;
  int64_t wave = 0;  // data per wave of the work list's order (bytes)
  double graph_ms = 0, persistent_ms = 0;
};

namespace pfgb {

// one transform of a batch
struct BatchOp {
  pfgb_plan* plan;
  int dir, norm;
  void* dst;
  const void* src;
  bool has_dv;
  Deriv dv;
};

static int run_op(const BatchOp& o, cudaStream_t s) {
  pfgb_plan* P = o.plan;
  const Deriv* d = o.has_dv ? &o.dv : nullptr;
  return o.dir >= 0 ? execute(P, P->fwd, o.dst, o.src, s, false, 1, d)
                    : execute(P, P->bwd, o.dst, o.src, s, o.norm != 0, -1, d);
}

// byte ranges read and written by an operation
struct ByteRange {
  const char* a;
  int64_t n;
};
static bool ranges_overlap(const ByteRange& x, const ByteRange& y) { return x.a < y.a + y.n && y.a < x.a + x.n; }
static void op_ranges(const BatchOp& o, ByteRange& rd, ByteRange& wr) {
  const pfgb_plan* P = o.plan;
  const bool f = o.dir >= 0;
  const int64_t bi = P->inplace ? P->inplace_bytes : (f ? P->in_layout.bytes() : P->out_layout.bytes());
  const int64_t bo = P->inplace ? P->inplace_bytes : (f ? P->out_layout.bytes() : P->in_layout.bytes());
  rd = {static_cast<const char*>(o.src), bi};
  wr = {static_cast<const char*>(o.dst), bo};
}
// operation j (earlier) must complete before operation i: the same plan
// (shared scratch), or i reads or writes what j wrote, or writes what j read
static bool op_depends(const std::vector<BatchOp>& ops, int i, int j) {
  if (ops[i].plan == ops[j].plan) return true;
  ByteRange ri, wi, rj, wj;
  op_ranges(ops[i], ri, wi);
  op_ranges(ops[j], rj, wj);
  return ranges_overlap(wj, ri) || ranges_overlap(wj, wi) || ranges_overlap(rj, wi);
}

static void release_graph(pfgb_batch* B) {
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  B->exec = nullptr;
  B->graph = nullptr;
}

static void release_batch(pfgb_batch* B) {
  release_graph(B);
  for (auto st : B->side) cudaStreamDestroy(st);
  if (B->cap) cudaStreamDestroy(B->cap);
  if (B->dmem) cudaFree(B->dmem);
  delete B;
}

// Graph form: the launches of every transform recorded into one CUDA graph
// with one branch per plan (the transforms of a plan share its scratch and
// stay in order on their branch); a transform also waits for every earlier
// one of another branch that it depends on (op_depends).
static int record_graph_form(pfgb_batch* B, const std::vector<BatchOp>& ops) {
  const int n = (int)ops.size();
  std::vector<cudaEvent_t> events;
  auto cleanup = [&](int rc) {
    for (auto ev : events) cudaEventDestroy(ev);
    return rc;
  };
  auto new_event = [&](cudaEvent_t* ev) {
    cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e == cudaSuccess) events.push_back(*ev);
    return e;
  };
  std::vector<int> branch(n);
  std::map<const pfgb_plan*, int> plan_branch;
  for (int i = 0; i < n; ++i) {
    auto it = plan_branch.find(ops[i].plan);
    if (it == plan_branch.end()) {
      cudaStream_t st = nullptr;
      cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
      if (e != cudaSuccess) return cleanup(fail(PFGB_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)));
      B->side.push_back(st);
      it = plan_branch.emplace(ops[i].plan, (int)B->side.size() - 1).first;
    }
    branch[i] = it->second;
  }
  cudaError_t e = cudaStreamBeginCapture(B->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cleanup(fail(PFGB_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e)));
  int rc = PFGB_OK;
  cudaEvent_t fork = nullptr;
  if ((e = new_event(&fork)) != cudaSuccess || (e = cudaEventRecord(fork, B->cap)) != cudaSuccess)
    rc = fail(PFGB_ERR_CUDA, std::string("batch fork event: ") + cudaGetErrorString(e));
  for (auto st : B->side)
    if (!rc && (e = cudaStreamWaitEvent(st, fork, 0)) != cudaSuccess)
      rc = fail(PFGB_ERR_CUDA, std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e));
  std::vector<cudaEvent_t> done(n, nullptr);
  for (int i = 0; i < n && !rc; ++i) {
    cudaStream_t st = B->side[branch[i]];
    for (int j = 0; j < i && !rc; ++j) {
      if (branch[j] == branch[i] || !op_depends(ops, i, j)) continue;
      if ((e = cudaStreamWaitEvent(st, done[j], 0)) != cudaSuccess)
        rc = fail(PFGB_ERR_CUDA, std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e));
    }
    if (rc) break;
    rc = run_op(ops[i], st);
    if (!rc && ((e = new_event(&done[i])) != cudaSuccess || (e = cudaEventRecord(done[i], st)) != cudaSuccess))
      rc = fail(PFGB_ERR_CUDA, std::string("batch event: ") + cudaGetErrorString(e));
  }
  // join every branch into the capturing stream
  for (auto st : B->side) {
    cudaEvent_t j = nullptr;
    if ((e = new_event(&j)) != cudaSuccess || (e = cudaEventRecord(j, st)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(B->cap, j, 0)) != cudaSuccess) {
      if (!rc) rc = fail(PFGB_ERR_CUDA, std::string("batch join: ") + cudaGetErrorString(e));
    }
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(B->cap, &g);
  B->graph = g;
  if (rc) return cleanup(rc);
  if (e != cudaSuccess) return cleanup(fail(PFGB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e)));
  e = cudaGraphInstantiate(&B->exec, B->graph, 0);
  if (e != cudaSuccess) return cleanup(fail(PFGB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)));
  return cleanup(PFGB_OK);
}

// default polls of a dependency wait of the persistent kernel (each poll an
// acquire load and a 64 ns sleep: of the order of a second in all)
constexpr int kPersistPolls = 1 << 21;

// Persistent form: the work list of every transform's passes (collect_persist),
// dependencies per pass, and a graph of one counter reset and one launch.
// Items are ordered by level + rank, level the pass's dependency depth and
// rank = (bytes read and written by the earlier transforms) / wave_bytes:
// along a dependency the level grows and the rank does not fall, so every
// item follows its dependencies, and the passes in flight at a time touch
// about one wave of data per level (kept in L2 between the passes of a
// transform) instead of every transform's (wave_bytes 0: level order).
static int record_persistent_form(pfgb_batch* B, const std::vector<BatchOp>& ops, int64_t wave_bytes) {
  const int n = (int)ops.size();
  std::vector<PersistItem> items;
  std::vector<std::vector<int>> deps;
  std::vector<int> first(n), last(n);
  for (int i = 0; i < n; ++i) {
    const BatchOp& o = ops[i];
    std::vector<PersistItem> mine;
    const Direction& dir = o.dir >= 0 ? o.plan->fwd : o.plan->bwd;
    int rc = collect_persist(o.plan, dir, o.dst, o.src, o.dir < 0 && o.norm != 0, o.has_dv ? &o.dv : nullptr, mine);
    if (rc) return rc;
    if (mine.empty()) return fail(PFGB_ERR_UNSUPPORTED, "persistent batch form: a transform without passes");
    first[i] = (int)items.size();
    for (size_t k = 0; k < mine.size(); ++k) {
      std::vector<int> d;
      if (k > 0) {
        d.push_back((int)items.size() - 1);
      } else {
        for (int j = 0; j < i; ++j)
          if (op_depends(ops, i, j)) d.push_back(last[j]);
      }
      items.push_back(mine[k]);
      deps.push_back(d);
    }
    last[i] = (int)items.size() - 1;
  }
  const int m = (int)items.size();
  std::vector<int64_t> key(m, 0);
  {
    std::vector<int64_t> rank(n, 0);
    int64_t cum = 0;
    for (int i = 0; i < n; ++i) {
      rank[i] = wave_bytes > 0 ? cum / wave_bytes : 0;
      ByteRange rd, wr;
      op_ranges(ops[i], rd, wr);
      cum += rd.n + wr.n;
    }
    std::vector<int64_t> level(m, 0);
    for (int i = 0; i < n; ++i)
      for (int x = first[i]; x <= last[i]; ++x) {
        for (int d : deps[x]) level[x] = std::max(level[x], level[d] + 1);
        key[x] = level[x] + rank[i];
      }
  }
  std::vector<int> order(m);
  for (int x = 0; x < m; ++x) order[x] = x;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  std::vector<int> pos(m);
  for (int x = 0; x < m; ++x) pos[order[x]] = x;
  std::vector<PersistItem> sorted(m);
  std::vector<int> dlist;
  std::vector<long long> tb(m + 1, 0);
  size_t smem = 0;
  for (int x = 0; x < m; ++x) {
    PersistItem it = items[order[x]];
    it.dep_begin = (int)dlist.size();
    for (int d : deps[order[x]]) dlist.push_back(pos[d]);
    it.dep_end = (int)dlist.size();
    sorted[x] = it;
    tb[x + 1] = tb[x] + it.ntiles;
    smem = std::max(smem, persist_smem(it.code));
  }
  int per_sm = 0;
  int rc = persist_blocks_per_sm(smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return fail(PFGB_ERR_UNSUPPORTED, "persistent batch form: tiles do not fit on an SM");
  int sms = 0;
  PFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, B->device));
  // device layout: items | tile_begin | deps | next, abort, done[m] | status, polls
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_items = 0;
  const size_t o_tb = o_items + al(sizeof(PersistItem) * m);
  const size_t o_deps = o_tb + al(sizeof(long long) * (m + 1));
  const size_t o_cnt = o_deps + al(sizeof(int) * std::max<size_t>(1, dlist.size()));
  const size_t cnt_bytes = 16 + sizeof(unsigned) * m;
  const size_t o_ctl = o_cnt + al(cnt_bytes);
  const size_t total = o_ctl + 256;
  PFGB_CUDA(cudaMalloc(&B->dmem, total));
  char* base = static_cast<char*>(B->dmem);
  PFGB_CUDA(cudaMemcpy(base + o_items, sorted.data(), sizeof(PersistItem) * m, cudaMemcpyHostToDevice));
  PFGB_CUDA(cudaMemcpy(base + o_tb, tb.data(), sizeof(long long) * (m + 1), cudaMemcpyHostToDevice));
  if (!dlist.empty())
    PFGB_CUDA(cudaMemcpy(base + o_deps, dlist.data(), sizeof(int) * dlist.size(), cudaMemcpyHostToDevice));
  const int ctl[2] = {0, kPersistPolls};
  PFGB_CUDA(cudaMemcpy(base + o_ctl, ctl, sizeof(ctl), cudaMemcpyHostToDevice));
  PersistArgs A;
  A.items = reinterpret_cast<const PersistItem*>(base + o_items);
  A.tile_begin = reinterpret_cast<const long long*>(base + o_tb);
  A.deps = reinterpret_cast<const int*>(base + o_deps);
  A.next = reinterpret_cast<unsigned long long*>(base + o_cnt);
  A.abort_flag = reinterpret_cast<unsigned*>(base + o_cnt + 8);
  A.done = reinterpret_cast<unsigned*>(base + o_cnt + 16);
  A.status = reinterpret_cast<int*>(base + o_ctl);
  A.polls = reinterpret_cast<const int*>(base + o_ctl + sizeof(int));
  A.n = m;
  A.total = tb[m];
  B->status = A.status;
  B->polls = reinterpret_cast<int*>(base + o_ctl + sizeof(int));
  B->items = m;
  B->tiles = tb[m];
  B->grid = (int)std::min<long long>(tb[m], (long long)per_sm * sms);
  B->smem = smem;
  cudaError_t e = cudaStreamBeginCapture(B->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(PFGB_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  e = cudaMemsetAsync(base + o_cnt, 0, cnt_bytes, B->cap);
  rc = e != cudaSuccess ? fail(PFGB_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e))
                        : launch_persist(A, smem, B->grid, B->cap);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(B->cap, &g);
  B->graph = g;
  if (rc) return rc;
  if (e != cudaSuccess) return fail(PFGB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&B->exec, B->graph, 0);
  if (e != cudaSuccess) return fail(PFGB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

// ms per launch of an instantiated form (2 untimed launches, then 5 timed)
static int time_form(pfgb_batch* B, double* ms) {
  cudaEvent_t a = nullptr, b = nullptr;
  PFGB_CUDA(cudaEventCreate(&a));
  cudaError_t e = cudaEventCreate(&b);
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaGraphLaunch(B->exec, B->cap);
  if (e == cudaSuccess) e = cudaEventRecord(a, B->cap);
  for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = cudaGraphLaunch(B->exec, B->cap);
  if (e == cudaSuccess) e = cudaEventRecord(b, B->cap);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (e != cudaSuccess) return fail(PFGB_ERR_CUDA, std::string("batch form timing: ") + cudaGetErrorString(e));
  *ms = t / 5.0;
  return PFGB_OK;
}

// Wave sizes of the persistent form: the default, and the candidates timed by
// PFGB_BATCH_MEASURE (0: level order)
constexpr int64_t kPersistWave = int64_t(32) << 20;
constexpr int64_t kPersistWaveCandidates[] = {int64_t(8) << 20, int64_t(32) << 20, int64_t(128) << 20, 0};


// the persistent form's resources, moved out of / into a batch
struct PersistForm {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* dmem = nullptr;
  int* status = nullptr;
  int* polls = nullptr;
  int items = 0, grid = 0;
  int64_t tiles = 0, wave = 0;
  size_t smem = 0;
};
static PersistForm take_persistent(pfgb_batch* B) {
  PersistForm f;
  f.graph = B->graph;
  f.exec = B->exec;
  f.dmem = B->dmem;
  f.status = B->status;
  f.polls = B->polls;
  f.items = B->items;
  f.grid = B->grid;
  f.tiles = B->tiles;
  f.wave = B->wave;
  f.smem = B->smem;
  B->graph = nullptr;
  B->exec = nullptr;
  B->dmem = nullptr;
  B->status = B->polls = nullptr;
  B->items = B->grid = 0;
  B->tiles = B->wave = 0;
  B->smem = 0;
  return f;
}
static void put_persistent(pfgb_batch* B, const PersistForm& f) {
  B->graph = f.graph;
  B->exec = f.exec;
  B->dmem = f.dmem;
  B->status = f.status;
  B->polls = f.polls;
  B->items = f.items;
  B->grid = f.grid;
  B->tiles = f.tiles;
  B->wave = f.wave;
  B->smem = f.smem;
}
static void free_persistent(PersistForm& f) {
  if (f.exec) cudaGraphExecDestroy(f.exec);
  if (f.graph) cudaGraphDestroy(f.graph);
  if (f.dmem) cudaFree(f.dmem);
  f = PersistForm();
}

static int batch_create(const std::vector<BatchOp>& ops, int form, pfgb_batch** out) {
  if (form < PFGB_BATCH_GRAPH || form > PFGB_BATCH_MEASURE) return fail(PFGB_ERR_ARGUMENT, "unknown batch form");
  for (const BatchOp& o : ops)
    if (o.plan->timing) return fail(PFGB_ERR_ARGUMENT, "disable plan timing before recording a batch");
  pfgb_batch* B = new pfgb_batch();
  B->n = (int)ops.size();
  cudaGetDevice(&B->device);
  cudaError_t e = cudaStreamCreateWithFlags(&B->cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    release_batch(B);
    return fail(PFGB_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  int rc = PFGB_OK;
  if (form == PFGB_BATCH_GRAPH) {
    rc = record_graph_form(B, ops);
    B->form = PFGB_BATCH_GRAPH;
  } else if (form != PFGB_BATCH_MEASURE) {
    B->wave = kPersistWave;
    rc = record_persistent_form(B, ops, B->wave);
    B->form = PFGB_BATCH_PERSISTENT;
    // AUTO: a pass without a tile form leaves the batch to the graph form
    if (form == PFGB_BATCH_AUTO && rc == PFGB_ERR_UNSUPPORTED) {
      PersistForm f = take_persistent(B);
      free_persistent(f);
      rc = record_graph_form(B, ops);
      B->form = PFGB_BATCH_GRAPH;
    }
  } else {
    // every wave size of the persistent form, then the graph form, timed on
    // the batch's own buffers; the fastest is kept
    PersistForm best;
    double best_ms = -1;
    for (int64_t w : kPersistWaveCandidates) {
      B->wave = w;
      rc = record_persistent_form(B, ops, w);
      double ms = 0;
      if (!rc) rc = time_form(B, &ms);
      PersistForm f = take_persistent(B);
      if (rc) {
        free_persistent(f);
        break;
      }
      if (best_ms < 0 || ms < best_ms) {
        free_persistent(best);
        best = f;
        best_ms = ms;
      } else {
        free_persistent(f);
      }
    }
    if (rc == PFGB_ERR_UNSUPPORTED && best_ms < 0) rc = PFGB_OK;  // graph form only
    if (!rc) rc = record_graph_form(B, ops);
    if (!rc) rc = time_form(B, &B->graph_ms);
    B->persistent_ms = best_ms > 0 ? best_ms : 0;
    B->form = PFGB_BATCH_GRAPH;
    if (!rc && best_ms >= 0 && best_ms <= B->graph_ms) {
      release_graph(B);
      put_persistent(B, best);
      B->form = PFGB_BATCH_PERSISTENT;
    } else {
      free_persistent(best);
    }
  }
  if (rc) {
    release_batch(B);
    return rc;
  }
  *out = B;
  return PFGB_OK;
}

}  // namespace pfgb

extern "C" {

const char* pfgb_version(void) { return "pencilfft_gb300 0.1.0 (sm_103a)"; }

int pfgb_last_error(char* buf, size_t n) {
  const std::string& e = g_last_error;
  if (buf && n > 0) {
    size_t k = std::min(n - 1, e.size());
    std::memcpy(buf, e.data(), k);
    buf[k] = 0;
  }
  return (int)e.size();
}

static int autotune_passes(pfgb_plan* P);

// ---------------------------------------------------------------------------
// Planner wisdom: the kernel choices of the planner measurement, kept for
// later plans of the same pass geometry on the same kind of device and
// exported / imported as a text file (the image of FFTW's wisdom, which the
// reference's FFTW planner accumulates under fftw_flags = FFTW.MEASURE).
// ---------------------------------------------------------------------------
static std::mutex g_wisdom_mutex;
static std::map<std::string, int> g_wisdom;
static int g_wisdom_hits = 0;
static const char* kWisdomHeader = "pencilfft_gb300 wisdom 1";

static std::string device_tag(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string n = prop.name;
  for (auto& c : n)
    if (c == ' ' || c == '|' || c == '\t') c = '_';
  return n + "_sm" + std::to_string(prop.major) + std::to_string(prop.minor) + "x" +
         std::to_string(prop.multiProcessorCount);
}

static std::string layout_tag(const Layout& L) {
  std::ostringstream o;
  for (int q = 0; q < L.D; ++q) o << L.size[L.perm[q]] << (q + 1 < L.D ? "," : "");
  o << "p" << L.pitch0 << "e" << L.elt;
  for (int q = 0; q < L.D; ++q) o << "/" << L.perm[q];
  return o.str();
}

// Key of one measured choice: what was measured, device, arithmetic and the
// pass geometry (operation, sign, length, both layouts, double-float form)
static std::string wisdom_key(const pfgb_plan* P, const Pass& ps, const char* what) {
  std::ostringstream o;
  o << what << "|" << device_tag(P->device) << "|rb" << P->rb << "|pr" << P->precision << "|op" << ps.op
    << "|s" << ps.sign << "|M" << ps.M << "|" << layout_tag(ps.lin) << "|" << layout_tag(ps.lout) << "|dd"
    << ps.in_dd << ps.out_dd;
  return o.str();
}

static bool wisdom_lookup(const std::string& key, int* variant) {
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  auto it = g_wisdom.find(key);
  if (it == g_wisdom.end()) return false;
  *variant = it->second;
  ++g_wisdom_hits;
  return true;
}

static void wisdom_store(const std::string& key, int variant) {
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  g_wisdom[key] = variant;
}

static int plan_build(const pfgb_plan_desc* desc, pfgb_plan** out, bool query_only) {
  g_last_error.clear();
  if (!desc || !out) return fail(PFGB_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  const pfgb_plan_desc& d = *desc;
  if (d.ndims < 1 || d.ndims > PFGB_MAX_DIMS)
    return fail(PFGB_ERR_ARGUMENT, "ndims must be in [1, " + std::to_string(PFGB_MAX_DIMS) + "]");
  if (d.n_extra < 0 || d.n_extra > PFGB_MAX_EXTRA)
    return fail(PFGB_ERR_ARGUMENT, "too many extra_dims");
  if (d.real_bytes != 4 && d.real_bytes != 8)
    return fail(PFGB_ERR_ARGUMENT, "real type must be Float32 (4) or Float64 (8)");
  if (d.precision_mode != PFGB_PRECISION_DEFAULT && d.precision_mode != PFGB_PRECISION_NATIVE &&
      d.precision_mode != PFGB_PRECISION_TC_SPLIT && d.precision_mode != PFGB_PRECISION_BLOCK_FLOAT)
    return fail(PFGB_ERR_ARGUMENT, "unknown precision mode");
  if (d.precision_mode == PFGB_PRECISION_TC_SPLIT && d.real_bytes != 4)
    return fail(PFGB_ERR_ARGUMENT, "the tensor-core split form applies to Float32 plans");
  if (d.precision_mode == PFGB_PRECISION_BLOCK_FLOAT && d.real_bytes != 8)
    return fail(PFGB_ERR_ARGUMENT, "the block floating point form applies to Float64 plans");
  for (int n = 0; n < d.ndims; ++n) {
    if (d.dims[n] < 1) return fail(PFGB_ERR_ARGUMENT, "dimensions must be positive");
    if (d.kind[n] < PFGB_FFT || d.kind[n] > PFGB_NOTRANSFORM)
      return fail(PFGB_ERR_ARGUMENT, "unknown transform kind");
    if (d.kind[n] == PFGB_R2R && !r2r_kind_supported(d.r2r_kind[n]))
      return fail(PFGB_ERR_ARGUMENT, "unsupported r2r transform kind: " + std::to_string(d.r2r_kind[n]));
  }
  for (int e = 0; e < d.n_extra; ++e)
    if (d.extra_dims[e] < 1) return fail(PFGB_ERR_ARGUMENT, "extra dimensions must be positive");
  // reference global_params.jl:57-60: no mix of in-place and out-of-place
  for (int n = 1; n < d.ndims; ++n)
    if ((d.inplace[n] != 0) != (d.inplace[0] != 0))
      return fail(PFGB_ERR_ARGUMENT, "cannot combine in-place and out-of-place transforms");

  pfgb_plan* P = new pfgb_plan();
  P->query_only = query_only;
  P->desc = d;
  P->N = d.ndims;
  P->K = d.n_extra;
  P->D = P->N + P->K;
  P->rb = d.real_bytes;
  P->precision = d.precision_mode;
  P->fx = d.real_bytes == 8 && d.precision_mode == PFGB_PRECISION_BLOCK_FLOAT;
  P->inplace = d.inplace[0] != 0;
  P->permute = d.permute_dims != 0;
  if (!query_only) cudaGetDevice(&P->device);
  // input element type (reference global_params.jl:81-95)
  bool in_cx = false, decided = false;
  for (int n = 0; n < P->N && !decided; ++n) {
    switch (d.kind[n]) {
      case PFGB_FFT: case PFGB_BFFT: case PFGB_BRFFT: in_cx = true; decided = true; break;
      case PFGB_RFFT: in_cx = false; decided = true; break;
      default: break;
    }
  }
  P->in_complex = in_cx;
  // walk the chain: sizes, element types (reference global_params.jl:50-62)
  bool cx = in_cx;
  double scale = 1.0;
  for (int n = 0; n < P->N; ++n) {
    const int k = d.kind[n];
    if ((k == PFGB_FFT || k == PFGB_BFFT || k == PFGB_BRFFT) && !cx) {
      delete P;
      return fail(PFGB_ERR_ARGUMENT, "invalid input data type for transform along dimension " +
                                         std::to_string(n + 1) + ": expected complex data");
    }
    if (k == PFGB_RFFT && cx) {
      delete P;
      return fail(PFGB_ERR_ARGUMENT, "invalid input data type for RFFT along dimension " +
                                         std::to_string(n + 1) + ": expected real data");
    }
    P->dims_in[n] = d.dims[n];
    P->dims_out[n] = length_output(k, d.brfft_even[n] != 0, d.dims[n]);
    if (P->dims_out[n] < 1) {
      delete P;
      return fail(PFGB_ERR_ARGUMENT, "empty output dimension");
    }
    if (k == PFGB_RFFT) cx = true;
    if (k == PFGB_BRFFT) cx = false;
    // backward scale of this dimension (reference plans.jl:540-546): binv of
    // the transform evaluated on the forward output length
    int kb = k, rb = d.r2r_kind[n];
    bool eb = false;
    if (k == PFGB_FFT) kb = PFGB_BFFT;
    else if (k == PFGB_BFFT) kb = PFGB_FFT;
    else if (k == PFGB_RFFT) { kb = PFGB_BRFFT; eb = d.dims[n] % 2 == 0; }
    else if (k == PFGB_BRFFT) kb = PFGB_RFFT;
    else if (k == PFGB_R2R) rb = r2r_inverse(d.r2r_kind[n]);
    scale *= scale_1d(kb, rb, eb, P->dims_out[n]);
  }
  P->out_complex = cx;
  P->scale = scale;
  // in-place RFFT! uses a padded real view (reference multiarrays_r2c.jl:69-79)
  int64_t pitch_real = 0;
  const bool inplace_rfft = P->inplace && d.kind[0] == PFGB_RFFT;
  const bool inplace_brfft = P->inplace && d.kind[P->N - 1] == PFGB_BRFFT;
  if (inplace_rfft) pitch_real = 2 * (d.dims[0] / 2 + 1);
  if (inplace_brfft) {
    delete P;
    return fail(PFGB_ERR_UNSUPPORTED, "in-place BRFFT! plans are not supported (the reference has no "
                                      "container for them either)");
  }
  P->in_layout = natural_layout(P, P->dims_in, in_cx, inplace_rfft ? pitch_real : 0);
  P->out_layout = final_layout(P, P->dims_out, cx);
  // capacity of the aliased in-place buffer: largest array along the chain
  if (P->inplace) {
    if (in_cx != cx && !inplace_rfft) {
      delete P;
      return fail(PFGB_ERR_UNSUPPORTED, "in-place plans need the same element type throughout");
    }
    P->inplace_bytes = std::max(P->in_layout.bytes(), P->out_layout.bytes());
  }
  const int64_t cap_dst_f = P->inplace ? P->inplace_bytes : P->out_layout.bytes();
  const int64_t cap_dst_b = P->inplace ? P->inplace_bytes : P->in_layout.bytes();
  int rc = build_direction(P, true, P->fwd, P->in_layout.bytes(), cap_dst_f, pitch_real);
  if (!rc) rc = build_direction(P, false, P->bwd, P->out_layout.bytes(), cap_dst_b, pitch_real);
  for (auto* dir : {&P->fwd, &P->bwd})
    for (auto& ps : dir->passes)
      if (!rc) rc = prepare_pass(P, ps);
  // Float64 runs of consecutive fast passes exchange data in dd (or fx) form
  int64_t te_tiles = 0, fx_lines = 0;
  if (!rc && P->rb == 8) {
    for (auto* dir : {&P->fwd, &P->bwd}) {
      auto& v = dir->passes;
      // passes that exchange dd-form data with their neighbours (packed real
      // R2R lines always read and write doubles)
      auto chains = [](const Pass& q) {
        return q.fast && q.fop != OP_X00R && q.fop != OP_D2R && q.fop != OP_D3R && q.fop != OP_D4R && !q.four;
      };
      for (size_t i = 0; i < v.size(); ++i) {
        if (!v[i].fast) continue;
        const bool prev = chains(v[i]) && i > 0 && chains(v[i - 1]);
        const bool next = chains(v[i]) && i + 1 < v.size() && chains(v[i + 1]);
        v[i].in_dd = prev;
        v[i].out_dd = next;
        v[i].reduce_before = !prev;
        v[i].self_scale = !prev;
      }
      // runs that start with an r2c pass: its split's factor 1/2 goes into
      // the output exponent of the run's last pass
      for (size_t i = 0; i < v.size(); ++i) {
        if (!v[i].fast || v[i].fop != OP_R2C || v[i].in_dd) continue;
        size_t j = i;
        while (v[j].out_dd) ++j;
        v[j].half_fold = true;
      }
      // element -> previous-pass line maps: the second pass of a dd run
      // (te_rescale) and every pass of an fx run with fx input
      for (size_t i = 0; i + 1 < v.size(); ++i)
        if (v[i].out_dd) {
          const int64_t n = te_mapping(v[i], v[i + 1]);
          if (v[i].self_scale) {
            v[i + 1].te_rescale = true;
            te_tiles = std::max(te_tiles, n);
          }
          fx_lines = std::max(fx_lines, n);
        }
    }
  }
  // set the shared-memory opt-in of every kernel the plan launches now, so that
  // executions recorded into a CUDA graph only launch
  if (!rc && !query_only) {
    for (auto* dir : {&P->fwd, &P->bwd}) {
      for (auto& ps : dir->passes) {
        if (rc || ps.pk != PK_TRANSFORM) continue;
        if (ps.fast) {
          FastArgs F;
          std::memset(&F, 0, sizeof(F));
          F.op = ps.fop;
          F.in_dd = ps.in_dd ? 1 : 0;  // selects the kernel variant
          F.out_dd = ps.out_dd ? 1 : 0;
          rc = P->rb == 8 ? launch_fast_dd(ps.logm, ps.sign, F, 0, nullptr)
                          : launch_fast_f32(ps.logm, ps.sign, F, 0, nullptr);
          if (!rc && P->fx && !ps.four) rc = launch_fast_fx(ps.logm, ps.sign, F, 0, nullptr);
          if (!rc && PFGB_FAST_TMA)
            rc = P->rb == 8 ? launch_fast_tma_dd(ps.logm, ps.sign, F, nullptr)
                            : launch_fast_tma_f32(ps.logm, ps.sign, F, nullptr);
          if (!rc && ps.tc) rc = launch_tc(ps.logm, ps.sign, F, nullptr);
        } else if (ps.mr) {
          FastArgs F;
          std::memset(&F, 0, sizeof(F));
          F.op = ps.fop;
          rc = launch_mr(P, ps, F, 0, nullptr);
        } else if (ps.bs) {
          FastArgs F;
          std::memset(&F, 0, sizeof(F));
          rc = launch_bs(P, ps, F, 0, nullptr);
          if (!rc) {
            PassArgs A;
            std::memset(&A, 0, sizeof(A));
            rc = launch_pass(P->rb, A, 0, 0, 0, nullptr);
          }
        } else {
          PassArgs A;
          std::memset(&A, 0, sizeof(A));
          rc = launch_pass(P->rb, A, 0, 0, 0, nullptr);
        }
      }
    }
  }
  if (!rc && !query_only && te_tiles > 0) {
    cudaError_t e = cudaMalloc(&P->te_dev, (size_t)te_tiles * sizeof(int));
    if (e != cudaSuccess) rc = fail(PFGB_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  for (int i = 0; i < 2 && !rc && !query_only && P->fx && fx_lines > 0; ++i) {
    cudaError_t e = cudaMalloc(&P->te_fx[i], (size_t)fx_lines * sizeof(int));
    if (e != cudaSuccess) rc = fail(PFGB_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  // exponent word (Float64 runs) and error word of the TMA-fed passes
  if (!rc && !query_only) {
    cudaError_t e = cudaMalloc(&P->emax_dev, 16);
    if (e != cudaSuccess) rc = fail(PFGB_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    else if ((e = cudaMemset(P->emax_dev, 0, 16)) != cudaSuccess)
      rc = fail(PFGB_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
  }
  if (!rc && !query_only) {
    for (int s = 0; s < 2; ++s) {
      if (P->scratch_bytes[s] > 0) {
        cudaError_t e = cudaMalloc(&P->scratch[s], P->scratch_bytes[s]);
        if (e != cudaSuccess) {
          rc = fail(PFGB_ERR_ALLOC, std::string("scratch allocation failed: ") + cudaGetErrorString(e));
          break;
        }
      }
    }
  }
  if (!rc && !query_only && d.autotune) rc = autotune_passes(P);
  if (rc) {
    pfgb_plan_destroy(P);
    return rc;
  }
  *out = P;
  return PFGB_OK;
}

int pfgb_plan_create(const pfgb_plan_desc* desc, pfgb_plan** out) {
  return plan_build(desc, out, false);
}

int pfgb_plan_query(const pfgb_plan_desc* desc, pfgb_plan_info* info) {
  if (!info) return fail(PFGB_ERR_ARGUMENT, "null argument");
  pfgb_plan* P = nullptr;
  int rc = plan_build(desc, &P, true);
  if (rc) return rc;
  rc = pfgb_plan_info_get(P, info);
  pfgb_plan_destroy(P);
  return rc;
}

static void clear_records(pfgb_plan* P) {
  for (auto& r : P->recs) {
    if (r.a) cudaEventDestroy(r.a);
    if (r.b) cudaEventDestroy(r.b);
  }
  P->recs.clear();
}

int pfgb_plan_set_timing(pfgb_plan* P, int on) {
  if (!P) return fail(PFGB_ERR_ARGUMENT, "null plan");
  clear_records(P);
  P->timing = on != 0 && !P->query_only;
  return PFGB_OK;
}

// Planner measurement (desc.autotune; the reference's FFTW.MEASURE planning
// flag): every pass with alternative kernels runs each of them on temporary
// buffers filled with normal numbers (bytes 0x3F), and the faster is kept.
// Alternatives today: c2r passes of Float32 and double-float plans, plain
// fast_pass or the TMA-fed persistent form (when the buffers satisfy its
// alignment); lines taken by the Bluestein register pass, that pass or the
// generic kernel (radix 2..16 stages in shared memory, or its own Bluestein
// for long lines).
static int autotune_passes(pfgb_plan* P) {
  const int e1023 = 1023;
  for (auto* dir : {&P->fwd, &P->bwd}) {
    for (auto& ps : dir->passes) {
      if (!ps.fast || ps.op != OP_C2R || ps.tc || P->fx) continue;  // fx passes have one kernel
      const std::string wkey = wisdom_key(P, ps, "c2r-tma");
      int wv = 0;
      if (wisdom_lookup(wkey, &wv)) {
        ps.variant = wv;
        continue;
      }
      void* bin = nullptr;
      void* bout = nullptr;
      const size_t nin = (size_t)ps.lin.bytes(), nout = (size_t)ps.lout.bytes();
      PFGB_CUDA(cudaMalloc(&bin, nin));
      cudaError_t e = cudaMalloc(&bout, nout);
      if (e != cudaSuccess) {
        cudaFree(bin);
        return fail(PFGB_ERR_ALLOC, std::string("cudaMalloc (autotune): ") + cudaGetErrorString(e));
      }
      cudaEvent_t ea = nullptr, eb = nullptr;
      int rc = PFGB_OK;
      float best[2] = {3.0e38f, 3.0e38f};
      if ((e = cudaMemset(bin, 0x3F, nin)) != cudaSuccess ||
          (e = cudaMemcpy(P->emax_dev, &e1023, sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
          (e = cudaEventCreate(&ea)) != cudaSuccess || (e = cudaEventCreate(&eb)) != cudaSuccess)
        rc = fail_cuda(e, "autotune set-up");
      for (int v = 0; v < 2 && !rc; ++v) {
        ps.variant = v;
        FastArgs F;
        int64_t grid = 0;
        rc = make_fast_args(P, ps, bin, bout, false, F, grid);
        if (rc || (v == 1 && !tma_eligible(P, ps, F))) break;
        for (int it = 0; it < 7 && !rc; ++it) {
          cudaEventRecord(ea, 0);
          if (v == 0) {
            rc = launch_plain(P, ps, F, grid, 0);
          } else {
            F.total = grid;
            F.err = P->emax_dev + 1;
            rc = P->rb == 8 ? launch_fast_tma_dd(ps.logm, ps.sign, F, 0) : launch_fast_tma_f32(ps.logm, ps.sign, F, 0);
          }
          cudaEventRecord(eb, 0);
          if ((e = cudaEventSynchronize(eb)) != cudaSuccess) rc = fail_cuda(e, "autotune launch");
          float ms = 0.f;
          cudaEventElapsedTime(&ms, ea, eb);
          if (it >= 2 && ms < best[v]) best[v] = ms;
        }
      }
      ps.variant = best[1] < best[0] ? 1 : 0;
      if (!rc) wisdom_store(wkey, ps.variant);
      if (ea) cudaEventDestroy(ea);
      if (eb) cudaEventDestroy(eb);
      cudaFree(bin);
      cudaFree(bout);
      if (rc) return rc;
    }
  }
  // Bluestein-eligible passes: the Bluestein register pass (variant -1)
  // against the generic kernel (variant 2) on the same buffers
  for (auto* dir : {&P->fwd, &P->bwd}) {
    for (auto& ps : dir->passes) {
      if (!ps.bs) continue;
      const std::string wkey = wisdom_key(P, ps, "bluestein-generic");
      int wv = 0;
      if (wisdom_lookup(wkey, &wv)) {
        ps.variant = wv;
        continue;
      }
      void* bin = nullptr;
      void* bout = nullptr;
      const size_t nin = (size_t)ps.lin.bytes(), nout = (size_t)ps.lout.bytes();
      PFGB_CUDA(cudaMalloc(&bin, nin));
      cudaError_t e = cudaMalloc(&bout, nout);
      if (e != cudaSuccess) {
        cudaFree(bin);
        return fail(PFGB_ERR_ALLOC, std::string("cudaMalloc (autotune): ") + cudaGetErrorString(e));
      }
      cudaEvent_t ea = nullptr, eb = nullptr;
      int rc = PFGB_OK;
      float best[2] = {3.0e38f, 3.0e38f};
      if ((e = cudaMemset(bin, 0x3F, nin)) != cudaSuccess || (e = cudaEventCreate(&ea)) != cudaSuccess ||
          (e = cudaEventCreate(&eb)) != cudaSuccess)
        rc = fail_cuda(e, "autotune set-up");
      for (int v = 0; v < 2 && !rc; ++v) {
        for (int it = 0; it < 7 && !rc; ++it) {
          int64_t grid = 0;
          cudaEventRecord(ea, 0);
          if (v == 0) {
            FastArgs F;
            rc = make_fast_args(P, ps, bin, bout, false, F, grid);
            F.bs_m = ps.M;
            F.bs_chirp = ps.bs_chirp;
            F.bs_filt = ps.bs_filt;
            F.div_m = make_div31(ps.op == OP_R2C ? ps.M / 2 + 1 : ps.M);
            if (!rc) rc = launch_bs(P, ps, F, grid, 0);
          } else {
            const Pass g = generic_form(ps);
            PassArgs A;
            rc = make_args(P, g, bin, bout, false, A, grid);
            if (!rc) rc = launch_pass(P->rb, A, grid, g.threads, g.smem, 0);
          }
          cudaEventRecord(eb, 0);
          if ((e = cudaEventSynchronize(eb)) != cudaSuccess) rc = fail_cuda(e, "autotune launch");
          float ms = 0.f;
          cudaEventElapsedTime(&ms, ea, eb);
          if (it >= 2 && ms < best[v]) best[v] = ms;
        }
      }
      ps.variant = best[1] < best[0] ? 2 : -1;
      if (!rc) wisdom_store(wkey, ps.variant);
      if (ea) cudaEventDestroy(ea);
      if (eb) cudaEventDestroy(eb);
      cudaFree(bin);
      cudaFree(bout);
      if (rc) return rc;
    }
  }
  PFGB_CUDA(cudaMemset(P->emax_dev, 0, 16));  // exponent and error words
  return PFGB_OK;
}

int pfgb_wisdom_export(const char* path) {
  if (!path) return fail(PFGB_ERR_ARGUMENT, "null path");
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  std::ofstream f(path);
  if (!f) return fail(PFGB_ERR_ARGUMENT, std::string("cannot write wisdom file ") + path);
  f << kWisdomHeader << "\n";
  for (const auto& kv : g_wisdom) f << kv.second << "\t" << kv.first << "\n";
  return f.good() ? PFGB_OK : fail(PFGB_ERR_ARGUMENT, std::string("error writing wisdom file ") + path);
}

int pfgb_wisdom_import(const char* path) {
  if (!path) return fail(PFGB_ERR_ARGUMENT, "null path");
  std::ifstream f(path);
  if (!f) return fail(PFGB_ERR_ARGUMENT, std::string("cannot read wisdom file ") + path);
  std::string line;
  if (!std::getline(f, line) || line != kWisdomHeader)
    return fail(PFGB_ERR_ARGUMENT, std::string("not a pencilfft_gb300 wisdom file: ") + path);
  std::map<std::string, int> got;
  int lineno = 1;
  while (std::getline(f, line)) {
    ++lineno;
    if (line.empty()) continue;
    const size_t tab = line.find('\t');
    char* end = nullptr;
    const long v = tab == std::string::npos ? 0 : std::strtol(line.c_str(), &end, 10);
    if (tab == std::string::npos || tab == 0 || end != line.c_str() + tab || v < -1 || v > 2 || tab + 1 >= line.size())
      return fail(PFGB_ERR_ARGUMENT, "malformed wisdom line " + std::to_string(lineno) + " in " + path);
    got[line.substr(tab + 1)] = (int)v;
  }
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  for (const auto& kv : got) g_wisdom[kv.first] = kv.second;
  return PFGB_OK;
}

int pfgb_wisdom_forget(void) {
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  g_wisdom.clear();
  g_wisdom_hits = 0;
  return PFGB_OK;
}

int pfgb_wisdom_stats(int32_t* entries, int32_t* hits) {
  if (!entries || !hits) return fail(PFGB_ERR_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lock(g_wisdom_mutex);
  *entries = (int32_t)g_wisdom.size();
  *hits = (int32_t)g_wisdom_hits;
  return PFGB_OK;
}

int pfgb_plan_set_wait_test(pfgb_plan* P, int polls, int tma) {
  if (!P) return fail(PFGB_ERR_ARGUMENT, "null plan");
  if (polls < 0) return fail(PFGB_ERR_ARGUMENT, "polls must be >= 0");
  P->wait_test = polls;
  P->force_tma = tma != 0;
  return PFGB_OK;
}

int pfgb_device_status(pfgb_plan* P, void* stream, int32_t* flags) {
  if (!P || !flags) return fail(PFGB_ERR_ARGUMENT, "null argument");
  *flags = 0;
  if (P->query_only || !P->emax_dev) return PFGB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int word = 0;
  PFGB_CUDA(cudaMemcpyAsync(&word, P->emax_dev + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  PFGB_CUDA(cudaStreamSynchronize(s));
  PFGB_CUDA(cudaMemsetAsync(P->emax_dev + 1, 0, sizeof(int), s));
  PFGB_CUDA(cudaStreamSynchronize(s));
  *flags = word;
  return PFGB_OK;
}

int pfgb_plan_get_timing(pfgb_plan* P, pfgb_pass_timing* out, int max, int* n) {
  if (!P || !n || (max > 0 && !out)) return fail(PFGB_ERR_ARGUMENT, "null argument");
  std::vector<pfgb_pass_timing> acc;
  auto entry = [&](int dir, int pass) -> pfgb_pass_timing& {
    for (auto& e : acc)
      if (e.direction == dir && e.pass == pass) return e;
    pfgb_pass_timing e;
    std::memset(&e, 0, sizeof(e));
    e.direction = dir;
    e.pass = pass;
    const Pass& ps = (dir > 0 ? P->fwd : P->bwd).passes[pass];
    e.axis = ps.axis;
    e.op = ps.pk == PK_COPY ? -1 : ps.op;  // PK_LPACK: the r2c / c2r it belongs to
    e.bytes_per_launch = ps.lin.bytes() + ps.lout.bytes();
    const char* kname = ps.pk == PK_COPY ? "copy_kernel"
                        : ps.pk == PK_LPACK ? (P->rb == 8 ? "lpack_kernel<double>" : "lpack_kernel<float>")
                        : ps.tc ? "tc_pass<tf32x3>"
                        : ps.variant == 1 ? (P->rb == 8 ? "fast_pass_tma<dd>" : "fast_pass_tma<float>")
                        : ps.fast ? (P->rb == 4 ? "fast_pass<float>" : P->fx ? "fast_pass<fx>" : "fast_pass<dd>")
                        : ps.mr ? (P->rb == 4 ? "mr_pass<float>" : "mr_pass<dd>")
                        : ps.bs && ps.variant != 2 ? (P->rb == 4 ? "bs_pass<float>" : "bs_pass<dd>")
                                  : (P->rb == 8 ? "pass_kernel<double>" : "pass_kernel<float>");
    std::snprintf(e.kernel, sizeof(e.kernel), "%s", kname);
    acc.push_back(e);
    return acc.back();
  };
  for (auto& r : P->recs) {
    PFGB_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.f;
    PFGB_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    pfgb_pass_timing& e = entry(r.dir, r.pass);
    e.launches += 1;
    e.total_ms += ms;
  }
  clear_records(P);
  *n = (int)acc.size();
  for (int i = 0; i < std::min(max, (int)acc.size()); ++i) out[i] = acc[i];
  return PFGB_OK;
}

int pfgb_plan_destroy(pfgb_plan* P) {
  if (!P) return PFGB_OK;
  clear_records(P);
  for (int s = 0; s < 2; ++s)
    if (P->scratch[s]) cudaFree(P->scratch[s]);
  for (auto& kv : P->tables) cudaFree(kv.second);
  if (P->emax_dev) cudaFree(P->emax_dev);
  if (P->te_dev) cudaFree(P->te_dev);
  for (int i = 0; i < 2; ++i)
    if (P->te_fx[i]) cudaFree(P->te_fx[i]);
  delete P;
  return PFGB_OK;
}

int pfgb_plan_info_get(const pfgb_plan* P, pfgb_plan_info* info) {
  if (!P || !info) return fail(PFGB_ERR_ARGUMENT, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->ndims = P->N;
  for (int n = 0; n < P->N; ++n) {
    info->dims_in[n] = P->dims_in[n];
    info->dims_out[n] = P->dims_out[n];
  }
  for (int q = 0; q < P->N; ++q) info->perm_out[q] = P->out_layout.perm[q];
  info->eltype_in_complex = P->in_complex;
  info->eltype_out_complex = P->out_complex;
  info->real_bytes = P->rb;
  info->inplace = P->inplace;
  info->scale_factor = P->scale;
  info->input_bytes = P->in_layout.bytes();
  info->output_bytes = P->out_layout.bytes();
  info->inplace_bytes = P->inplace_bytes;
  info->scratch_bytes = P->scratch_bytes[0] + P->scratch_bytes[1];
  info->n_passes_forward = (int)P->fwd.passes.size();
  info->n_passes_backward = (int)P->bwd.passes.size();
  return PFGB_OK;
}

static int check_buffers(pfgb_plan* P, void* dst, const void* src, bool forward) {
  if (!P) return fail(PFGB_ERR_ARGUMENT, "null plan");
  if (!dst || !src) return fail(PFGB_ERR_ARGUMENT, "null array");
  if (P->inplace) {
    // reference operations.jl:98-108
    if (dst != src) return fail(PFGB_ERR_ARGUMENT, "input and output arrays for in-place plan must be the same");
  } else {
    // reference operations.jl:87-96 (Base.mightalias)
    const int64_t bi = forward ? P->in_layout.bytes() : P->out_layout.bytes();
    const int64_t bo = forward ? P->out_layout.bytes() : P->in_layout.bytes();
    const char* s = (const char*)src;
    const char* t = (const char*)dst;
    if (s < t + bo && t < s + bi) return fail(PFGB_ERR_ARGUMENT, "out-of-place plan applied to aliased data");
  }
  return PFGB_OK;
}

int pfgb_forward(pfgb_plan* P, void* dst, const void* src, void* stream) {
  int rc = check_buffers(P, dst, src, true);
  if (rc) return rc;
  return execute(P, P->fwd, dst, src, (cudaStream_t)stream, false, 1);
}

int pfgb_backward(pfgb_plan* P, void* dst, const void* src, void* stream, int normalise) {
  int rc = check_buffers(P, dst, src, false);
  if (rc) return rc;
  return execute(P, P->bwd, dst, src, (cudaStream_t)stream, normalise != 0, -1);
}

static int make_deriv(const pfgb_plan* P, int mode, int dim, double length, Deriv& dv);

int pfgb_batch_create(pfgb_plan* const* plans, const int* direction, const int* normalise,
                      void* const* dst, const void* const* src, int n, pfgb_batch** out) {
  g_last_error.clear();
  if (!out || n < 1 || !plans || !direction || !dst || !src)
    return fail(PFGB_ERR_ARGUMENT, "invalid batch description");
  *out = nullptr;
  std::vector<BatchOp> ops(n);
  for (int i = 0; i < n; ++i) {
    if (!plans[i]) return fail(PFGB_ERR_ARGUMENT, "null plan in batch");
    int rc = check_buffers(plans[i], dst[i], src[i], direction[i] >= 0);
    if (rc) return rc;
    ops[i] = BatchOp{plans[i], direction[i], normalise ? normalise[i] : 0, dst[i], src[i], false, Deriv()};
  }
  return batch_create(ops, PFGB_BATCH_GRAPH, out);
}

int pfgb_batch_create_ex(const pfgb_batch_op* desc, int n, int form, pfgb_batch** out) {
  g_last_error.clear();
  if (!out || n < 1 || !desc) return fail(PFGB_ERR_ARGUMENT, "invalid batch description");
  *out = nullptr;
  std::vector<BatchOp> ops(n);
  for (int i = 0; i < n; ++i) {
    const pfgb_batch_op& d = desc[i];
    if (!d.plan) return fail(PFGB_ERR_ARGUMENT, "null plan in batch");
    int rc = check_buffers(d.plan, d.dst, d.src, d.direction >= 0);
    if (rc) return rc;
    ops[i] = BatchOp{d.plan, d.direction, d.normalise, d.dst, d.src, false, Deriv()};
    if (d.deriv_dim >= 0) {
      rc = make_deriv(d.plan, d.direction >= 0 ? 2 : 1, d.deriv_dim, d.deriv_length, ops[i].dv);
      if (rc) return rc;
      ops[i].has_dv = true;
    }
  }
  return batch_create(ops, form, out);
}

int pfgb_batch_get_info(pfgb_batch* B, pfgb_batch_info* info) {
  if (!B || !info) return fail(PFGB_ERR_ARGUMENT, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->form = B->form;
  info->transforms = B->n;
  info->items = B->items;
  info->tiles = B->tiles;
  info->grid = B->grid;
  info->smem = (int64_t)B->smem;
  info->graph_ms = B->graph_ms;
  info->persistent_ms = B->persistent_ms;
  info->wave_bytes = B->form == PFGB_BATCH_PERSISTENT ? B->wave : 0;
  return PFGB_OK;
}

int pfgb_batch_launch(pfgb_batch* B, void* stream) {
  if (!B) return fail(PFGB_ERR_ARGUMENT, "null batch");
  cudaError_t e = cudaGraphLaunch(B->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(PFGB_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

int pfgb_batch_status(pfgb_batch* B, void* stream, int32_t* flags) {
  if (!B || !flags) return fail(PFGB_ERR_ARGUMENT, "null argument");
  *flags = 0;
  if (!B->status) return PFGB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int word = 0;
  PFGB_CUDA(cudaMemcpyAsync(&word, B->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  PFGB_CUDA(cudaStreamSynchronize(s));
  PFGB_CUDA(cudaMemsetAsync(B->status, 0, sizeof(int), s));
  PFGB_CUDA(cudaStreamSynchronize(s));
  *flags = word;
  return PFGB_OK;
}

int pfgb_batch_set_wait_test(pfgb_batch* B, int polls) {
  if (!B) return fail(PFGB_ERR_ARGUMENT, "null batch");
  if (!B->polls) return fail(PFGB_ERR_ARGUMENT, "the batch is not in the persistent form");
  const int v = polls > 0 ? polls : kPersistPolls;
  PFGB_CUDA(cudaMemcpy(B->polls, &v, sizeof(int), cudaMemcpyHostToDevice));
  return PFGB_OK;
}

int pfgb_batch_destroy(pfgb_batch* B) {
  if (!B) return PFGB_OK;
  release_batch(B);
  return PFGB_OK;
}

static int make_deriv(const pfgb_plan* P, int mode, int dim, double length, Deriv& dv) {
  if (dim < 0 || dim >= P->N) return fail(PFGB_ERR_ARGUMENT, "derivative dimension out of range");
  if (!(length > 0)) return fail(PFGB_ERR_ARGUMENT, "domain length must be positive");
  const int k = P->desc.kind[dim];
  if (k == PFGB_R2R || k == PFGB_NOTRANSFORM)
    return fail(PFGB_ERR_ARGUMENT, "a spectral derivative needs an FFT, BFFT, RFFT or BRFFT dimension");
  dv.mode = mode;
  dv.dim = dim;
  dv.half = (k == PFGB_RFFT || k == PFGB_BRFFT) ? 1 : 0;
  dv.n = k == PFGB_BRFFT ? P->dims_out[dim] : P->dims_in[dim];
  dv.k0 = 2.0 * 3.14159265358979323846264338327950288 / length;
  return PFGB_OK;
}

int pfgb_forward_deriv(pfgb_plan* P, void* dst, const void* src, void* stream, int dim, double length) {
  int rc = check_buffers(P, dst, src, true);
  if (rc) return rc;
  Deriv dv;
  rc = make_deriv(P, 2, dim, length, dv);
  if (rc) return rc;
  return execute(P, P->fwd, dst, src, (cudaStream_t)stream, false, 1, &dv);
}

int pfgb_backward_deriv(pfgb_plan* P, void* dst, const void* src, void* stream, int normalise, int dim,
                        double length) {
  int rc = check_buffers(P, dst, src, false);
  if (rc) return rc;
  Deriv dv;
  rc = make_deriv(P, 1, dim, length, dv);
  if (rc) return rc;
  return execute(P, P->bwd, dst, src, (cudaStream_t)stream, normalise != 0, -1, &dv);
}

int pfgb_backward_deriv_sum(pfgb_plan* P, void* dst, const void* const* src, int nterm, const int* dim,
                            const double* coef, const double* length, void* stream, int normalise) {
  if (!P) return fail(PFGB_ERR_ARGUMENT, "null plan");
  if (nterm < 1 || nterm > kMaxTerms)
    return fail(PFGB_ERR_ARGUMENT, "a sum of derivatives takes 1 to " + std::to_string(kMaxTerms) + " terms");
  if (!src || !dim || !coef || !length) return fail(PFGB_ERR_ARGUMENT, "null argument");
  if (P->inplace) return fail(PFGB_ERR_ARGUMENT, "a sum of derivatives needs an out-of-place plan");
  Deriv dv;
  dv.mode = 3;
  dv.nterm = nterm;
  for (int k = 0; k < nterm; ++k) {
    int rc = check_buffers(P, dst, src[k], false);
    if (rc) return rc;
    Deriv one;
    rc = make_deriv(P, 1, dim[k], length[k], one);
    if (rc) return rc;
    dv.tsrc[k] = src[k];
    dv.tdim[k] = one.dim;
    dv.thalf[k] = one.half;
    dv.tn[k] = one.n;
    dv.tk0[k] = coef[k] * one.k0;
  }
  return execute(P, P->bwd, dst, src[0], (cudaStream_t)stream, normalise != 0, -1, &dv);
}

int pfgb_execute_many(pfgb_plan* P, int direction, int normalise, void* const* dst,
                      const void* const* src, int n, void* stream) {
  if (!P) return fail(PFGB_ERR_ARGUMENT, "null plan");
  if (n < 0 || (n > 0 && (!dst || !src))) return fail(PFGB_ERR_ARGUMENT, "invalid collection");
  for (int i = 0; i < n; ++i) {
    int rc = direction >= 0 ? pfgb_forward(P, dst[i], src[i], stream)
                            : pfgb_backward(P, dst[i], src[i], stream, normalise);
    if (rc) return rc;
  }
  return PFGB_OK;
}

}  // extern "C"
