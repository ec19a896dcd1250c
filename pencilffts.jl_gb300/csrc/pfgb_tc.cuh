// Tensor-core split form of the Float32 complex-to-complex pass.
//
// A line of M = N1 * N2 points (N1, N2 in {16, 32}) is transformed as two
// small dense DFT-matrix products on the tensor cores (tcgen05.mma,
// kind::tf32, accumulators in tensor memory), with the twiddles applied on
// the CUDA cores between them (four-step factorisation, n = N2 n1 + n2,
// k = k1 + N1 k2, w = exp(sign 2 pi i / M)):
//   stage 1:  Y[k1, n2]      = sum_n1 F_N1[k1, n1] x[N2 n1 + n2]
//   twiddle:  Y[k1, n2]     *= w^(n2 k1)
//   stage 2:  X[k1 + N1 k2]  = sum_n2 F_N2[k2, n2] Y[k1, n2]
// Each product runs in real form: rows of A are (line, n) pairs holding
// [re(n) | im(n)], B is the 2N x 2N matrix [[C, -S], [S, C]] of F_N, and
// D = A B^T lands in tensor memory with [re(k) | im(k)] per row.  Every
// float operand is split into a tf32 hi part and the remainder lo, both
// rounded to nearest; the product keeps hi*hi + hi*lo + lo*hi with FP32
// accumulation (3xTF32, about 22 significant bits).  The tensor cores
// accumulate with truncation, so the two small products go first and the
// large one last: its 2N/8 instructions are then the only additions at the
// full magnitude of the result.
//
// Operands sit in shared memory in the K-major, non-swizzled canonical
// layout: core matrices of 8 rows x 16 bytes (4 tf32), 128 bytes each,
// adjacent along K at 128 bytes (LBO) and along M/N at (K/4)*128 bytes
// (SBO).  Rows are ordered (n2, line) in stage 1 and (k1, line) in stage 2,
// so that a warp's global accesses cover whole 32-byte sectors in both the
// axis-contiguous and the strided layouts and the transposed stage-2 writes
// of a warp fill one core matrix (32 distinct banks).
//
// CTAs of 256 threads (two per SM), persistent over the tiles of the pass:
// the DFT matrices (hi / lo) and the twiddle table are copied into shared
// memory once, and a tile's inputs are loaded into registers while the
// previous tile's second product runs.  Thread 0 issues the MMAs, commits
// them to an mbarrier and alone polls it (bounded: error word, then the
// tensor memory is released); the other warps wait at the CTA barrier, which
// costs no issue slots.
#pragma once

#include "pfgb_fast.cuh"

namespace pfgb {

template <int LN1, int LN2>
struct TcCfg {
  static constexpr int N1 = 1 << LN1, N2 = 1 << LN2, M = N1 * N2;
  static constexpr int L = 128 / (N1 < N2 ? N1 : N2);  // lines per tile
  static constexpr int R1 = L * N2, R2 = L * N1;       // rows of the two products: 128 or 256
  static constexpr int P1 = 256 / R1, P2 = 256 / R2;   // threads per row
  static constexpr int K1 = 2 * N1, K2 = 2 * N2;       // K (= N) of the two products
  static constexpr int ABYTES = (R1 * K1 > R2 * K2 ? R1 * K1 : R2 * K2) * 4;  // hi or lo
  static constexpr int B1BYTES = K1 * K1 * 4;
  static constexpr int B2BYTES = N1 == N2 ? 0 : K2 * K2 * 4;
  static constexpr int BBYTES = 2 * (B1BYTES + B2BYTES);  // hi and lo of each distinct matrix
  static constexpr int TWBYTES = M * 8;
  static constexpr int SMEM = 2 * ABYTES + BBYTES + TWBYTES + 64;
  static constexpr int C1 = (R1 / 128) * K1, C2 = (R2 / 128) * K2;
  static constexpr int TMEM_COLS = C1 > C2 ? C1 : C2;  // 32 or 64 columns
};

// byte offset of element (row, k) in a K-major operand with K columns
__host__ __device__ constexpr int tc_off(int row, int k, int K) {
  return (row >> 3) * (K >> 2) * 128 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// instruction descriptor: D f32, A and B tf32, both K-major, M x N
__host__ __device__ constexpr unsigned tc_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

#if defined(__CUDACC__)
// shared-memory matrix descriptor (no swizzle): start, LBO, SBO (bytes)
__device__ __forceinline__ unsigned long long tc_sdesc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tc_alloc(unsigned* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(unsigned dtmem, unsigned long long adesc, unsigned long long bdesc,
                                       unsigned idesc, unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// x rounded to tf32 (10 explicit significand bits), to nearest with ties
// away from zero, as two integer operations on the bit pattern (finite x)
__device__ __forceinline__ float tf32_rn(float x) {
#ifdef PFGB_TC_CVT
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
#else
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
#endif
}

// Two 32-lane x N-column loads from tensor memory and the wait for them in
// one statement, so that no use of the registers can be scheduled before
// the wait.
template <int N>
__device__ __forceinline__ void tc_ld2(unsigned ta, unsigned tb, float (&a)[N], float (&b)[N]);
template <>
__device__ __forceinline__ void tc_ld2<8>(unsigned ta, unsigned tb, float (&a)[8], float (&b)[8]) {
  unsigned ra[8], rb[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%16];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%17];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(ra[0]),"=r"(ra[1]),"=r"(ra[2]),"=r"(ra[3]),"=r"(ra[4]),"=r"(ra[5]),"=r"(ra[6]),"=r"(ra[7]), "=r"(rb[0]),"=r"(rb[1]),"=r"(rb[2]),"=r"(rb[3]),"=r"(rb[4]),"=r"(rb[5]),"=r"(rb[6]),"=r"(rb[7])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = __uint_as_float(ra[i]);
    b[i] = __uint_as_float(rb[i]);
  }
}
template <>
__device__ __forceinline__ void tc_ld2<16>(unsigned ta, unsigned tb, float (&a)[16], float (&b)[16]) {
  unsigned ra[16], rb[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(ra[0]),"=r"(ra[1]),"=r"(ra[2]),"=r"(ra[3]),"=r"(ra[4]),"=r"(ra[5]),"=r"(ra[6]),"=r"(ra[7]),"=r"(ra[8]),"=r"(ra[9]),"=r"(ra[10]),"=r"(ra[11]),"=r"(ra[12]),"=r"(ra[13]),"=r"(ra[14]),"=r"(ra[15]), "=r"(rb[0]),"=r"(rb[1]),"=r"(rb[2]),"=r"(rb[3]),"=r"(rb[4]),"=r"(rb[5]),"=r"(rb[6]),"=r"(rb[7]),"=r"(rb[8]),"=r"(rb[9]),"=r"(rb[10]),"=r"(rb[11]),"=r"(rb[12]),"=r"(rb[13]),"=r"(rb[14]),"=r"(rb[15])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    a[i] = __uint_as_float(ra[i]);
    b[i] = __uint_as_float(rb[i]);
  }
}
template <>
__device__ __forceinline__ void tc_ld2<32>(unsigned ta, unsigned tb, float (&a)[32], float (&b)[32]) {
  unsigned ra[32], rb[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(ra[0]),"=r"(ra[1]),"=r"(ra[2]),"=r"(ra[3]),"=r"(ra[4]),"=r"(ra[5]),"=r"(ra[6]),"=r"(ra[7]),"=r"(ra[8]),"=r"(ra[9]),"=r"(ra[10]),"=r"(ra[11]),"=r"(ra[12]),"=r"(ra[13]),"=r"(ra[14]),"=r"(ra[15]),"=r"(ra[16]),"=r"(ra[17]),"=r"(ra[18]),"=r"(ra[19]),"=r"(ra[20]),"=r"(ra[21]),"=r"(ra[22]),"=r"(ra[23]),"=r"(ra[24]),"=r"(ra[25]),"=r"(ra[26]),"=r"(ra[27]),"=r"(ra[28]),"=r"(ra[29]),"=r"(ra[30]),"=r"(ra[31]), "=r"(rb[0]),"=r"(rb[1]),"=r"(rb[2]),"=r"(rb[3]),"=r"(rb[4]),"=r"(rb[5]),"=r"(rb[6]),"=r"(rb[7]),"=r"(rb[8]),"=r"(rb[9]),"=r"(rb[10]),"=r"(rb[11]),"=r"(rb[12]),"=r"(rb[13]),"=r"(rb[14]),"=r"(rb[15]),"=r"(rb[16]),"=r"(rb[17]),"=r"(rb[18]),"=r"(rb[19]),"=r"(rb[20]),"=r"(rb[21]),"=r"(rb[22]),"=r"(rb[23]),"=r"(rb[24]),"=r"(rb[25]),"=r"(rb[26]),"=r"(rb[27]),"=r"(rb[28]),"=r"(rb[29]),"=r"(rb[30]),"=r"(rb[31])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    a[i] = __uint_as_float(ra[i]);
    b[i] = __uint_as_float(rb[i]);
  }
}

template <int LN1, int LN2, int SIGN>
__global__ void __launch_bounds__(256, 2) tc_pass(const FastArgs a) {
  using C = TcCfg<LN1, LN2>;
  constexpr int N1 = C::N1, N2 = C::N2, M = C::M, L = C::L;
  constexpr int NP1 = N1 / C::P1;  // n1 (stage-1 K) and k1 values per thread
  constexpr int NP2 = N2 / C::P2;  // k2 values per thread
  constexpr unsigned SBO1 = (C::K1 / 4) * 128, SBO2 = (C::K2 / 4) * 128;
  constexpr unsigned ID1 = tc_idesc(128, C::K1), ID2 = tc_idesc(128, C::K2);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* Ahi = smem_raw;
  unsigned char* Alo = smem_raw + C::ABYTES;
  unsigned char* Bs = smem_raw + 2 * C::ABYTES;
  float2* tws = reinterpret_cast<float2*>(Bs + C::BBYTES);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(Bs + C::BBYTES + C::TWBYTES);
  unsigned* tslot = reinterpret_cast<unsigned*>(bar + 1);
  int* sfail = reinterpret_cast<int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5;

  {  // constants: DFT matrices (already in operand layout) and twiddles
    const float4* src = reinterpret_cast<const float4*>(a.tcb);
    float4* dst = reinterpret_cast<float4*>(Bs);
    for (int i = tid; i < C::BBYTES / 16; i += 256) dst[i] = src[i];
    const float2* tw = reinterpret_cast<const float2*>(a.tw);
    for (int i = tid; i < M; i += 256) {
      float2 w = tw[i];
      if (SIGN > 0) w.y = -w.y;
      tws[i] = w;
    }
  }
  // never signalled: the give-up test's wait (FastArgs::wait_test)
  unsigned long long* dead = bar + 2;
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(dead, 1);
    *sfail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tc_alloc(tslot, C::TMEM_COLS);
    tc_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tslot;
  const unsigned lanes = (unsigned)((warp & 3) * 32) << 16;  // this warp's TMEM lane quarter

  // operand descriptors at the operands' first byte; an MMA adds its byte
  // offset / 16 to the start-address field (addresses stay below 2^18)
  const unsigned sA[2] = {smem_u32(Ahi), smem_u32(Alo)};
  const unsigned sB1[2] = {smem_u32(Bs), smem_u32(Bs + C::B1BYTES)};
  const unsigned sB2[2] = {C::B2BYTES ? smem_u32(Bs + 2 * C::B1BYTES) : sB1[0],
                           C::B2BYTES ? smem_u32(Bs + 2 * C::B1BYTES + C::B2BYTES) : sB1[1]};
  const unsigned long long dA1[2] = {tc_sdesc(sA[0], 128, SBO1), tc_sdesc(sA[1], 128, SBO1)};
  const unsigned long long dA2[2] = {tc_sdesc(sA[0], 128, SBO2), tc_sdesc(sA[1], 128, SBO2)};
  const unsigned long long dB1[2] = {tc_sdesc(sB1[0], 128, SBO1), tc_sdesc(sB1[1], 128, SBO1)};
  const unsigned long long dB2[2] = {tc_sdesc(sB2[0], 128, SBO2), tc_sdesc(sB2[1], 128, SBO2)};

  // thread roles: stage-1 row r1 = n2 L + line (part q1 of the row's n1 / k1
  // range), stage-2 row r2 = k1 L + line (part q2 of the row's k2 range)
  const int r1 = tid % C::R1, q1 = tid / C::R1;
  const int n2 = r1 / L, line1 = r1 % L;
  const int r2 = tid % C::R2, q2 = tid / C::R2;
  const int k1o = r2 / L, line2 = r2 % L;
  const float2 zero2 = make_float2(0.f, 0.f);
  unsigned phase = 0;

  // inputs x[line][N2 n1 + n2] of a tile, n1 in this thread's range; the
  // next tile's are loaded while the current tile's second product runs
  float2 x[NP1];
  TileOrigin onext;
  int nvnext = 0;
  auto load_tile = [&](int64_t b) {
    onext = tile_origin(a, (unsigned)b, L);
    nvnext = (int)min((int64_t)L, a.nt - onext.t0);
    const float2* in = reinterpret_cast<const float2*>(a.in) + onext.ioff + (int64_t)line1 * a.in_st;
#pragma unroll
    for (int j = 0; j < NP1; ++j) {
      const int n1 = q1 * NP1 + j;
      x[j] = line1 < nvnext ? in[(int64_t)(n1 * N2 + n2) * a.in_sa] : zero2;
    }
  };
  if ((int64_t)blockIdx.x < a.total) load_tile(blockIdx.x);

  for (int64_t bid = blockIdx.x; bid < a.total; bid += gridDim.x) {
    const TileOrigin o = onext;
    const int nvalid = nvnext;

    // ---- stage-1 operand ----
    {
      if (a.deriv == 1) {
#pragma unroll
        for (int j = 0; j < NP1; ++j) {
          const int64_t idx = a.deriv_role == 0 ? (int64_t)((q1 * NP1 + j) * N2 + n2)
                              : a.deriv_role == 1 ? o.t0 + line1 : o.didx;
          const Cx<float> y = mul_ik(mk(x[j].x, x[j].y), idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
          x[j] = make_float2(y.re, y.im);
        }
      }
#pragma unroll
      for (int j = 0; j < NP1; j += 4) {
        const int n1 = q1 * NP1 + j;
        float4 hr, hi;
        hr.x = tf32_rn(x[j].x); hr.y = tf32_rn(x[j + 1].x); hr.z = tf32_rn(x[j + 2].x); hr.w = tf32_rn(x[j + 3].x);
        hi.x = tf32_rn(x[j].y); hi.y = tf32_rn(x[j + 1].y); hi.z = tf32_rn(x[j + 2].y); hi.w = tf32_rn(x[j + 3].y);
        const float4 lr = make_float4(tf32_rn(x[j].x - hr.x), tf32_rn(x[j + 1].x - hr.y),
                                      tf32_rn(x[j + 2].x - hr.z), tf32_rn(x[j + 3].x - hr.w));
        const float4 li = make_float4(tf32_rn(x[j].y - hi.x), tf32_rn(x[j + 1].y - hi.y),
                                      tf32_rn(x[j + 2].y - hi.z), tf32_rn(x[j + 3].y - hi.w));
        *reinterpret_cast<float4*>(Ahi + tc_off(r1, n1, C::K1)) = hr;
        *reinterpret_cast<float4*>(Alo + tc_off(r1, n1, C::K1)) = lr;
        *reinterpret_cast<float4*>(Ahi + tc_off(r1, N1 + n1, C::K1)) = hi;
        *reinterpret_cast<float4*>(Alo + tc_off(r1, N1 + n1, C::K1)) = li;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int b = 0; b < C::R1 / 128; ++b)
#pragma unroll
        for (int pr = 0; pr < 3; ++pr)  // hi*lo, lo*hi, then hi*hi
#pragma unroll
          for (int kk = 0; kk < C::K1 / 8; ++kk)
            tc_mma(tmem + b * C::K1, dA1[pr == 1] + ((b * 16 * SBO1 + kk * 256) >> 4),
                   dB1[pr == 0] + ((kk * 256) >> 4), ID1, (pr | kk) ? 1u : 0u);
      tc_commit(bar);
      const bool ok = a.wait_test > 0 ? mbar_wait_bounded(dead, 0, a.wait_test) : mbar_wait_bounded(bar, phase);
      if (!ok) *sfail = 1;
      tc_fence_before();
    }
    phase ^= 1;
    __syncthreads();
    if (*sfail) break;  // the product may still run: no tensor-memory read
    tc_fence_after();

    // ---- twiddles, stage-2 operand: rows (k1, line), K = [re(n2) | im(n2)] ----
    {
      float yr[NP1], yi[NP1];
      const unsigned col = (unsigned)((r1 >> 7) * C::K1 + q1 * NP1);
      tc_ld2<NP1>(tmem + lanes + col, tmem + lanes + col + N1, yr, yi);
#pragma unroll
      for (int j = 0; j < NP1; ++j) {
        const int k1 = q1 * NP1 + j;
        const float2 w = tws[(n2 * k1) & (M - 1)];
        const float re = yr[j] * w.x - yi[j] * w.y;
        const float im = yr[j] * w.y + yi[j] * w.x;
        const int row = k1 * L + line1;
        const float hr = tf32_rn(re), hi = tf32_rn(im);
        *reinterpret_cast<float*>(Ahi + tc_off(row, n2, C::K2)) = hr;
        *reinterpret_cast<float*>(Alo + tc_off(row, n2, C::K2)) = tf32_rn(re - hr);
        *reinterpret_cast<float*>(Ahi + tc_off(row, N2 + n2, C::K2)) = hi;
        *reinterpret_cast<float*>(Alo + tc_off(row, N2 + n2, C::K2)) = tf32_rn(im - hi);
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int b = 0; b < C::R2 / 128; ++b)
#pragma unroll
        for (int pr = 0; pr < 3; ++pr)
#pragma unroll
          for (int kk = 0; kk < C::K2 / 8; ++kk)
            tc_mma(tmem + b * C::K2, dA2[pr == 1] + ((b * 16 * SBO2 + kk * 256) >> 4),
                   dB2[pr == 0] + ((kk * 256) >> 4), ID2, (pr | kk) ? 1u : 0u);
      tc_commit(bar);
    }
    if (bid + gridDim.x < a.total) load_tile(bid + gridDim.x);
    if (tid == 0) {
      if (!mbar_wait_bounded(bar, phase)) *sfail = 1;
      tc_fence_before();
    }
    phase ^= 1;
    __syncthreads();
    if (*sfail) break;
    tc_fence_after();

    // ---- output X[line][k1 + N1 k2] ----
    {
      float zr[NP2], zi[NP2];
      const unsigned col = (unsigned)((r2 >> 7) * C::K2 + q2 * NP2);
      tc_ld2<NP2>(tmem + lanes + col, tmem + lanes + col + N2, zr, zi);
      if (line2 < nvalid) {
        float2* out = reinterpret_cast<float2*>(a.out) + o.ooff + (int64_t)line2 * a.out_st;
#pragma unroll
        for (int j = 0; j < NP2; ++j) {
          const int pos = k1o + N1 * (q2 * NP2 + j);
          Cx<float> y = mk(zr[j], zi[j]);
          if (a.scale_on) y = mk(y.re * a.scale_h, y.im * a.scale_h);
          if (a.deriv == 2) {
            const int64_t idx = a.deriv_role == 0 ? (int64_t)pos : a.deriv_role == 1 ? o.t0 + line2 : o.didx;
            y = mul_ik(y, idx, a.deriv_half, a.deriv_n, a.k0_h, a.k0_l);
          }
          out[(int64_t)pos * a.out_sa] = make_float2(y.re, y.im);
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    if (*sfail) break;
  }
  if (tid == 0 && *sfail) {
    atomicOr(a.err, 2);
    // the product whose wait gave up (committed with parity phase ^ 1) may
    // still write tensor memory: wait for it once more, bounded, before the
    // memory is released; bit 4 if it still has not completed
    if (!mbar_wait_bounded(bar, phase ^ 1)) atomicOr(a.err, 4);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, C::TMEM_COLS);
  }
}
#endif

}  // namespace pfgb
