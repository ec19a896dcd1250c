// Persistent batch kernel (Float32): a work list of the tiles of many passes
// in one launch.  The scheduling and dependency rules are described in
// pfgb_persist.h; the tiles are the ones of the per-pass kernels
// (fast_tile, mr_tile, bs_tile), run here with 512 threads and a register
// allocation sized for two CTAs per SM.
#include "pfgb_persist.h"

#include <algorithm>

#include "pencilfft_gb300.h"
#include "pfgb_bs.cuh"
#include "pfgb_mr.cuh"

namespace pfgb {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_volatile_u32(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}

// Each tile form is its own (not inlined) function, so that each gets the
// register allocation of its own code rather than one over all of them.  The
// arguments are read in place from the work list, which the kernel never
// writes: a restrict pointer lets the compiler keep field loads out of the
// tile's loops (no store of the tile can alias them).
template <int L, int SIGN, int OP>
__device__ __noinline__ void run_fast(const FastArgs* __restrict__ ap, long long t, Cx<float>* z) {
  const FastArgs& a = *ap;
  fast_tile<float, L, SIGN, OP, 0>(a, t, z, a.in, -1, a.in_sa, a.in_st);
}
template <int L, int SIGN, int OP>
__device__ __noinline__ void run_mr(const FastArgs* __restrict__ ap, long long t, Cx<float>* z) {
  mr_tile<float, 3, L, SIGN, OP, kPersistThreads>(*ap, t, z);
}
template <int L, int OP>
__device__ __noinline__ void run_bs(const FastArgs* __restrict__ ap, long long t, Cx<float>* z) {
  bs_tile<float, L, OP>(*ap, t, z);
}

// One tile of the item whose arguments are `a`; the switch covers every
// (form, operation, length) combination the host may put in the list.
// Power-of-two lines stop at 512 points: the 16-point tiles of longer
// Float32 lines need all 64 registers of their own kernel and spill here.
__device__ __forceinline__ void persist_run(int code, const FastArgs* a, long long t, Cx<float>* z) {
  switch (code) {
#define PF_FAST(L)                                                                        \
  case persist_code(PK_FAST_TILE, 0, L): run_fast<L, -1, OP_C2C>(a, t, z); break; \
  case persist_code(PK_FAST_TILE, 1, L): run_fast<L, 1, OP_C2C>(a, t, z); break;  \
  case persist_code(PK_FAST_TILE, 2, L): run_fast<L, -1, OP_R2C>(a, t, z); break; \
  case persist_code(PK_FAST_TILE, 3, L): run_fast<L, 1, OP_C2R>(a, t, z); break;
    PF_FAST(3) PF_FAST(4) PF_FAST(5) PF_FAST(6) PF_FAST(7) PF_FAST(8) PF_FAST(9)
#undef PF_FAST
#define PF_MR(L)                                                                        \
  case persist_code(PK_MR_TILE, 0, L): run_mr<L, -1, OP_C2C>(a, t, z); break; \
  case persist_code(PK_MR_TILE, 1, L): run_mr<L, 1, OP_C2C>(a, t, z); break;  \
  case persist_code(PK_MR_TILE, 2, L): run_mr<L, -1, OP_R2C>(a, t, z); break; \
  case persist_code(PK_MR_TILE, 3, L): run_mr<L, 1, OP_C2R>(a, t, z); break;
    PF_MR(7) PF_MR(8) PF_MR(9)
#undef PF_MR
#define PF_BS(L)                                                 \
  case persist_code(PK_BS_TILE, 0, L):                          \
  case persist_code(PK_BS_TILE, 1, L): run_bs<L, OP_C2C>(a, t, z); break; \
  case persist_code(PK_BS_TILE, 2, L): run_bs<L, OP_R2C>(a, t, z); break; \
  case persist_code(PK_BS_TILE, 3, L): run_bs<L, OP_C2R>(a, t, z); break;
    PF_BS(4) PF_BS(5) PF_BS(6) PF_BS(7) PF_BS(8) PF_BS(9) PF_BS(10) PF_BS(11)
#undef PF_BS
    default: break;
  }
}

// Tiles a CTA claims with one atomic (consecutive numbers).
constexpr int kPersistChunk = 8;

// Thread 0 schedules.  While its CTA finishes a tile it picks the next tile
// number without blocking (claiming a chunk when the last one is used up;
// numbers only grow, so a forward cursor maps them to items) and posts it in
// the other of two slots, so that one barrier ends a tile and starts the
// next.  The CTA's completed tiles of an item are published in one release
// (fence, then one add) when the CTA moves to another item or leaves, always
// before it waits for the new item's dependencies: no CTA waits while
// holding unpublished completions, and the smallest unpublished tile number
// never waits (its dependencies carry smaller numbers).  A new item's
// dependencies are checked once per CTA.
__global__ void __launch_bounds__(kPersistThreads, 2) persist_batch(const PersistArgs pa) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_item[2], s_new[2], s_code, s_ok;
  __shared__ long long s_tile[2];
  Cx<float>* z = reinterpret_cast<Cx<float>*>(smem_raw);
  // thread 0's state, in shared memory so that no thread holds it in
  // registers across the tiles: chunk [c_next, c_end), first tile number of
  // the current item and of the next one, item of the running tiles and its
  // completed, unpublished tiles
  struct Sched {
    long long c_next, c_end, cb, nb;
    int cur, run_item;
    unsigned pend;
  };
  __shared__ Sched st;
  auto publish = [&]() {
    if (st.run_item >= 0 && st.pend > 0) {
      __threadfence();
      atomicAdd(pa.done + st.run_item, st.pend);
    }
    st.pend = 0;
  };
  // next tile into slot q (no wait: at most the claim's atomic)
  auto next_tile = [&](int q) {
    if (st.c_next >= st.c_end) {
      st.c_next = st.c_end = 0;
      if (ld_volatile_u32(pa.abort_flag) == 0) {
        const long long g = (long long)atomicAdd(pa.next, (unsigned long long)kPersistChunk);
        if (g < pa.total) {
          st.c_next = g;
          st.c_end = min(g + kPersistChunk, pa.total);
        }
      }
    }
    int item = -1;
    long long tile = 0;
    if (st.c_next < st.c_end) {
      const long long t = st.c_next++;
      while (st.nb <= t) {
        ++st.cur;
        st.cb = st.nb;
        st.nb = pa.tile_begin[st.cur + 1];
      }
      item = st.cur;
      tile = t - st.cb;
    }
    s_item[q] = item;
    s_tile[q] = tile;
    s_new[q] = item >= 0 && item != st.run_item;
  };
  // publish the running item's completions, then wait (bounded) until every
  // dependency of `item` has completed; false if a wait gave up
  auto enter_item = [&](int item) {
    publish();
    st.run_item = item;
    const int polls = *pa.polls;
    const int d0 = pa.items[item].dep_begin, d1 = pa.items[item].dep_end;
    for (int d = d0; d < d1; ++d) {
      const int j = pa.deps[d];
      const unsigned need = (unsigned)pa.items[j].ntiles;
      int k = 0;
      while (ld_acquire_u32(pa.done + j) < need) {
        if (++k > polls || ld_volatile_u32(pa.abort_flag)) {
          atomicOr(pa.status, kPersistWaitBit);
          atomicExch(pa.abort_flag, 1u);
          return false;
        }
        __nanosleep(64);
      }
    }
    return true;
  };
  if (threadIdx.x == 0) {
    st.c_next = st.c_end = st.cb = 0;
    st.nb = pa.tile_begin[1];
    st.cur = 0;
    st.run_item = -1;
    st.pend = 0;
    next_tile(0);
  }
  __syncthreads();
  for (int it = 0;; ++it) {
    const int q = it & 1;
    if (s_item[q] < 0) {
      if (threadIdx.x == 0) publish();
      return;
    }
    if (s_new[q]) {
      // (the slots are only read here; a failed wait is reported in s_ok,
      // written before the barrier and read after it)
      if (threadIdx.x == 0) {
        s_ok = enter_item(s_item[q]) ? 1 : 0;
        if (s_ok) s_code = pa.items[s_item[q]].code;
      }
      __syncthreads();
      if (!s_ok) return;
    }
    persist_run(s_code, &pa.items[s_item[q]].F, s_tile[q], z);
    if (threadIdx.x == 0) next_tile(q ^ 1);
    // every thread's stores of the tile precede its completion count, and
    // the next tile's slot is posted
    __syncthreads();
    if (threadIdx.x == 0) ++st.pend;
  }
}

size_t persist_smem(int code) {
  const int lg = code % 16, opc = (code / 16) % 4, kind = code / 64;
  const int op = opc < 2 ? OP_C2C : opc == 2 ? OP_R2C : OP_C2R;
  switch (kind) {
    case PK_FAST_TILE:
      return lg >= 3 && lg <= 9 ? fast_smem<float>(lg, op) : 0;
    case PK_MR_TILE: {
      if (lg < 7 || lg > 9) return 0;
      const int T = (1 << lg) / 8;
      return (size_t)3 * (kPersistThreads / T) * fast_pitch<float>(lg, op) * sizeof(Cx<float>);
    }
    case PK_BS_TILE:
      return lg >= 4 && lg <= 11 ? bs_smem<float>(lg) : 0;
    default:
      return 0;
  }
}

static size_t persist_smem_max() {
  size_t m = 0;
  for (int kind = 0; kind < 3; ++kind)
    for (int opc = 0; opc < 4; ++opc)
      for (int lg = 0; lg < 16; ++lg) m = std::max(m, persist_smem(persist_code(kind, opc, lg)));
  return m;
}

static int persist_attr() {
  static bool configured[kMaxDevicesConfigured] = {};
  return ensure_smem_attr(persist_batch, (int)persist_smem_max(), configured,
                          "cudaFuncSetAttribute(persist_batch)");
}

int persist_blocks_per_sm(size_t smem, int* per_sm) {
  int rc = persist_attr();
  if (rc) return rc;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, persist_batch, kPersistThreads, smem);
  if (e != cudaSuccess) return fail_cuda(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(persist_batch)");
  return PFGB_OK;
}

int launch_persist(const PersistArgs& A, size_t smem, int grid, cudaStream_t s) {
  int rc = persist_attr();
  if (rc || grid <= 0) return rc;
  persist_batch<<<(unsigned)grid, kPersistThreads, smem, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "persist_batch launch");
  return PFGB_OK;
}

}  // namespace pfgb
