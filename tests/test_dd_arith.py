"""Double-float (dd) arithmetic of the Float64 fast passes (pfgb_dd.cuh), the
sums and products compiled for the host with g++ from the same header and
checked against long double:

* two_sum is error-free: s + e equals a + b exactly;
* dd sums and products of normalised operands are within 2^-44 of the
  operands' magnitude (the lazy low parts are not renormalised);
* a 512-point radix-2 FFT in dd (twiddles as hi + lo float pairs) against a
  long double FFT: relative L2 error below 2^-45."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "pencilffts.jl_gb300" / "csrc"

DRIVER = r"""
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>
#include "pfgb_dd.cuh"
using namespace pfgb;
typedef long double ld;

static dd split(ld x) { const float h = (float)x; return dd(h, (float)(x - (ld)h)); }
static ld val(dd a) { return (ld)a.h + (ld)a.l; }

int main() {
  std::mt19937_64 g(5);
  std::normal_distribution<double> un(0.0, 1.0);
  long bad = 0;
  double worst_add = 0, worst_mul = 0;
  for (int k = 0; k < 300000; ++k) {
    const float a = (float)(un(g) * std::ldexp(1.0, (int)(g() % 40) - 20));
    const float b = (float)(un(g) * std::ldexp(1.0, (int)(g() % 40) - 20));
    float s, e;
    two_sum(a, b, s, e);
    if ((ld)s + (ld)e != (ld)a + (ld)b) ++bad;
    const ld x = (ld)un(g), y = (ld)un(g) * (k % 3 == 0 ? 1e-3L : 1.0L);
    const dd X = split(x), Y = split(y);
    const ld mag = fabsl(x) + fabsl(y);
    worst_add = std::max(worst_add, (double)(fabsl(val(X + Y) - (val(X) + val(Y))) / mag));
    worst_add = std::max(worst_add, (double)(fabsl(val(X - Y) - (val(X) - val(Y))) / mag));
    worst_mul = std::max(worst_mul, (double)(fabsl(val(X * Y) - val(X) * val(Y)) / fabsl(val(X) * val(Y))));
  }
  if (!(worst_add < std::ldexp(1.0, -44)) || !(worst_mul < std::ldexp(1.0, -44))) ++bad;
  // 512-point radix-2 FFT in dd against long double
  const int M = 512;
  double worst_fft = 0;
  for (int trial = 0; trial < 10; ++trial) {
    std::vector<dd> vr(M), vi(M);
    std::vector<std::complex<ld>> ref(M);
    for (int i = 0; i < M; ++i) {
      const double xr = un(g), xi = un(g);
      vr[i] = split((ld)xr);
      vi[i] = split((ld)xi);
      ref[i] = {val(vr[i]), val(vi[i])};
    }
    for (int i = 1, j = 0; i < M; ++i) {
      int bit = M >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) { std::swap(vr[i], vr[j]); std::swap(vi[i], vi[j]); std::swap(ref[i], ref[j]); }
    }
    for (int len = 2; len <= M; len <<= 1)
      for (int i0 = 0; i0 < M; i0 += len)
        for (int j = 0; j < len / 2; ++j) {
          const ld ang = -2.0L * 3.14159265358979323846264338327950288L * j / len;
          const dd wr = split(cosl(ang)), wi = split(sinl(ang));
          const int q = i0 + j + len / 2;
          const dd br = vr[q] * wr - vi[q] * wi, bi = vr[q] * wi + vi[q] * wr;
          const dd ar = vr[i0 + j], ai = vi[i0 + j];
          vr[i0 + j] = ar + br; vi[i0 + j] = ai + bi;
          vr[q] = ar - br; vi[q] = ai - bi;
          const std::complex<ld> w(cosl(ang), sinl(ang));
          const std::complex<ld> u = ref[i0 + j], b = ref[q] * w;
          ref[i0 + j] = u + b;
          ref[q] = u - b;
        }
    ld num = 0, den = 0;
    for (int i = 0; i < M; ++i) {
      num += std::norm(std::complex<ld>(val(vr[i]), val(vi[i])) - ref[i]);
      den += std::norm(ref[i]);
    }
    worst_fft = std::max(worst_fft, (double)sqrtl(num / den));
  }
  if (!(worst_fft < std::ldexp(1.0, -45))) ++bad;
  std::printf("%ld %.3e %.3e %.3e\n", bad, worst_add, worst_mul, worst_fft);
  return bad != 0;
}
"""


def test_dd_arithmetic(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "dd.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "dd"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.split()[0] == "0", r.stdout + r.stderr
