// Persistent form of a batch of Float32 transforms: one kernel launch walks a
// device work list holding every tile of every pass of every transform of the
// batch.
//
// Items are the passes (one FastArgs each, with the tile form that runs them
// and their tile count), sorted by dependency level: a pass depends on the
// previous pass of its transform, and the first pass of a transform on the
// last pass of every earlier transform that shares its plan (scratch) or whose
// buffers overlap its own.  Tiles are numbered item after item; a CTA takes
// the next tile number from a global counter, and before running it waits
// until every tile of the item's dependencies has completed (per-item
// completion counters).  The tiles an item waits for carry smaller numbers
// and were therefore taken earlier by running CTAs, whose own waits are for
// smaller numbers still: the smallest unfinished tile never waits, so the
// kernel progresses whether or not all of its CTAs are resident.  Every wait
// is bounded: after `polls` polls the CTA records bit 8 in the batch's status
// word, raises the launch's abort flag (every CTA then stops taking tiles)
// and leaves.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pfgb_fast.cuh"

namespace pfgb {

constexpr int kPersistThreads = 512;
constexpr int kPersistWaitBit = 8;

// tile forms of the persistent kernel: the power-of-two register tile
// (fast_tile, lines of 8 .. 512 points), the mixed-radix tile for 3 * 2^k
// points (2^k = 128 .. 512, 512 threads) and the Bluestein tile (convolution
// lengths 16 .. 2048)
enum PersistKind : int { PK_FAST_TILE = 0, PK_MR_TILE = 1, PK_BS_TILE = 2 };
// opc: 0 c2c forward (sign -1), 1 c2c backward (+1), 2 r2c, 3 c2r; lg: log2 of
// the line (fast), of its power-of-two factor (mixed radix) or of the
// convolution length (Bluestein)
__host__ __device__ constexpr int persist_code(int kind, int opc, int lg) { return (kind * 4 + opc) * 16 + lg; }

struct PersistItem {
  FastArgs F;
  int code;
  int ntiles;
  int dep_begin, dep_end;  // deps[dep_begin .. dep_end): items that must complete first
};

struct PersistArgs {
  const PersistItem* items;
  const long long* tile_begin;  // n + 1 prefix sums of the items' tiles
  const int* deps;
  unsigned long long* next;  // next tile number (zeroed before each launch)
  unsigned* abort_flag;      // set when a wait gives up (zeroed before each launch)
  unsigned* done;            // completed tiles per item (zeroed before each launch)
  int* status;               // sticky status word (bit 8), cleared by the host
  const int* polls;          // polls of a dependency wait
  int n;
  long long total;
};

// dynamic shared memory of a tile form; 0 when the form is not built
size_t persist_smem(int code);
// resident CTAs per SM of the persistent kernel with `smem` bytes
int persist_blocks_per_sm(size_t smem, int* per_sm);
int launch_persist(const PersistArgs& A, size_t smem, int grid, cudaStream_t s);

}  // namespace pfgb
