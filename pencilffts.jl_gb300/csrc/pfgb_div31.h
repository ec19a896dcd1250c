// Division by a run-time constant d (1 <= d < 2^31) of numerators n < 2^31
// by a multiply and a shift (Granlund & Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994, theorem 4.2 with N = 31):
// l = ceil(log2 d), s = 31 + l, m = ceil(2^s / d) < 2^32; then
// floor(n / d) = (n * m) >> s for every 0 <= n < 2^31, and n * m < 2^63.
// Plain C++ so that the host-side test compiles it without nvcc.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PFGB_DIV_HD __host__ __device__ __forceinline__
#else
#define PFGB_DIV_HD inline
#endif

namespace pfgb {

struct Div31 {
  unsigned long long m;
  int s;
};

inline Div31 make_div31(int64_t d) {
  int l = 0;
  while ((int64_t{1} << l) < d) ++l;
  const int s = 31 + l;  // <= 62
  const unsigned long long p = 1ull << s;
  return Div31{(p + (unsigned long long)d - 1) / (unsigned long long)d, s};
}

PFGB_DIV_HD unsigned div31(unsigned n, Div31 d) { return (unsigned)((n * d.m) >> d.s); }

}  // namespace pfgb
