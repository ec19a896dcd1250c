"""The fast pass decodes tile indices with the multiply-and-shift division of
pfgb_div31.h; check it against integer division on the host (boundary
numerators for every divisor below 70000, powers of two +-3 up to 2^31, and
random divisors), compiled with g++ from the same header."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "pencilffts.jl_gb300" / "csrc"

DRIVER = r"""
#include <cstdio>
#include <random>
#include "pfgb_div31.h"
using namespace pfgb;
int main() {
  std::mt19937_64 g(7);
  long bad = 0;
  auto test = [&](int64_t d, int nrand) {
    const Div31 q = make_div31(d);
    if (q.m >= (1ull << 32)) ++bad;
    const unsigned top = 0x7fffffffu;
    unsigned fixed[] = {0u, 1u, (unsigned)(d - 1), (unsigned)d, (unsigned)(d + 1) & top, top, top - 1};
    for (unsigned n : fixed) if (div31(n, q) != n / d) ++bad;
    for (int k = 0; k < nrand; ++k) {
      const unsigned n = (unsigned)(g() & top);
      if (div31(n, q) != n / d) ++bad;
      const unsigned long long e = (unsigned long long)(n / d) * d + d - 1;  // last numerator of n's quotient
      if (e <= top && div31((unsigned)e, q) != (unsigned)e / d) ++bad;
    }
  };
  for (int64_t d = 1; d < 70000; ++d) test(d, 40);
  for (int l = 1; l <= 31; ++l)
    for (int64_t o = -3; o <= 3; ++o) {
      const int64_t d = (int64_t{1} << l) + o;
      if (d >= 1 && d < (int64_t{1} << 31)) test(d, 2000);
    }
  for (int k = 0; k < 5000; ++k) test(1 + (int64_t)(g() % 0x7ffffffe), 200);
  std::printf("%ld\n", bad);
  return bad != 0;
}
"""


def test_div31_matches_integer_division(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "div31.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "div31"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "0", r.stdout + r.stderr
