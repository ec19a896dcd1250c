"""Block floating point (fx) arithmetic of the Float64 fast passes
(pfgb_fx.cuh), checked on the host against exact integer and long double
arithmetic, compiled with g++ from the same header:

* product with a constant and with a twiddle of the kernel's table layout,
  against round(a W / 2^60) in 128-bit integers: at most 4 and 7 units off
  over the whole operand range |a| < 2^61 (the dropped low products lie in
  [0, 4) units, their mean is in the rounding constant);
* double -> fx (d2fx): within half a unit of the line's scale;
* fx -> double (fx2d): correctly rounded up to ties (half an ulp), zero below
  the double range and infinity above it;
* a 512-point radix-2 FFT in fx against a long double FFT: relative L2 error
  below 2^-46 (the passes' headroom for 512-point lines is 50 bits)."""
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
#include "pfgb_fx.cuh"
using namespace pfgb;
typedef __int128 i128;
typedef long double ld;

static fx_tw table_entry(ld wr, ld wi) {  // as the plan uploads it
  auto part = [](ld c, int& h4, int& l) {
    long long W = llroundl(c * ldexpl(1.0L, 60));
    if (W > (1ll << 60) - 1) W = (1ll << 60) - 1;
    if (W < -(1ll << 60)) W = -(1ll << 60);
    h4 = (int)(4 * (W >> 31));
    l = (int)(W & 0x7FFFFFFFll);
  };
  fx_tw t;
  part(wr, t.rh4, t.rl);
  part(wi, t.ih4, t.il);
  return t;
}
static long long W_of(int h4, int l) { return (long long)(h4 / 4) * (1ll << 31) + l; }
static long long round_div60(i128 x) {  // round(x / 2^60)
  const i128 d = (i128)1 << 60;
  i128 q = x >= 0 ? (x + d / 2) / d : -((-x + d / 2) / d);
  return (long long)q;
}

int main() {
  std::mt19937_64 g(11);
  const long long lim = (1ll << 61) - 1;
  std::uniform_int_distribution<long long> ua(-lim, lim);
  std::uniform_real_distribution<double> uc(-1.0, 1.0);
  long bad = 0;
  long long worst_mul = 0, worst_tw = 0;
  // products with constants
  const double consts[] = {0.70710678118654752440, 0.92387953251128675613, 0.38268343236508977173, 1.0, -1.0, 0.0};
  for (int k = 0; k < 400000; ++k) {
    const long long a = k % 7 == 0 ? (k & 8 ? lim : -lim) : ua(g);
    const double c = k < 6 * 1000 ? consts[k % 6] : uc(g);
    const fx C(c);
    const long long got = (fx(a) * C).v;
    const long long ex = round_div60((i128)a * C.v);
    const long long err = got > ex ? got - ex : ex - got;
    if (err > worst_mul) worst_mul = err;
  }
  if (worst_mul > 4) ++bad;
  // products with twiddles
  for (int k = 0; k < 400000; ++k) {
    const ld ang = (ld)uc(g) * 3.14159265358979323846L;
    const fx_tw t = k % 97 == 0 ? table_entry(1.0L, 0.0L) : table_entry(cosl(ang), sinl(ang));
    const long long ar = k % 5 == 0 ? (k & 2 ? lim : -lim) : ua(g), ai = k % 3 == 0 ? (k & 4 ? lim : -lim) : ua(g);
    fx re(ar), im(ai);
    fx_twiddle(re, im, t);
    const long long Wr = W_of(t.rh4, t.rl), Wi = W_of(t.ih4, t.il);
    const long long er = round_div60((i128)ar * Wr - (i128)ai * Wi);
    const long long ei = round_div60((i128)ar * Wi + (i128)ai * Wr);
    const long long e1 = re.v > er ? re.v - er : er - re.v, e2 = im.v > ei ? im.v - ei : ei - im.v;
    if (e1 > worst_tw) worst_tw = e1;
    if (e2 > worst_tw) worst_tw = e2;
  }
  if (worst_tw > 7) ++bad;
  // double -> fx within half a unit of the scale 2^(eb - 1022 - H)
  std::normal_distribution<double> un(0.0, 1.0);
  for (int k = 0; k < 200000; ++k) {
    const int H = 44 + k % 9;
    const double x = un(g) * std::ldexp(1.0, (int)(g() % 2000) - 1000);
    const int eb = (int)((fx_dbits(x) >> 52) & 0x7FF) + (int)(g() % 4);  // line exponent >= x's
    if (eb > 2046) continue;
    const long long v = d2fx(x, eb + 53 - H);
    const ld S = ldexpl(1.0L, eb - 1022 - H);
    if (fabsl((ld)v * S - (ld)x) > 0.5L * S) ++bad;
  }
  // fx -> double: correct to half an ulp, zero / infinity outside the range
  for (int k = 0; k < 200000; ++k) {
    const long long v = ua(g) >> (g() % 60);
    const int s = (int)(g() % 2300) - 1150;
    const double d = fx2d(v, s);
    const ld ex = ldexpl((ld)v, s);
    if (v == 0) { if (d != 0.0) ++bad; continue; }
    if (fabsl(ex) >= 0x1p1024L) { if (!std::isinf(d) || (d > 0) != (v > 0)) ++bad; continue; }
    if (fabsl(ex) < 0x1p-1022L) { if (d != 0.0 && !(fabsl((ld)d - ex) <= ldexpl(fabsl(ex), -52))) ++bad; continue; }
    if (!(fabsl((ld)d - ex) <= ldexpl(fabsl(ex), -53))) ++bad;
  }
  // 512-point radix-2 FFT in fx (input scaled to the pass headroom) against
  // a long double FFT of the same doubles
  const int LOGM = 9, M = 1 << LOGM, H = fx_head(LOGM, false);
  double worst_fft = 0;
  for (int trial = 0; trial < 20; ++trial) {
    std::vector<double> xr(M), xi(M);
    unsigned emax = 0;
    for (int i = 0; i < M; ++i) {
      xr[i] = un(g) * (trial % 2 ? 1e-200 : 3.0);
      xi[i] = un(g) * (trial % 2 ? 1e-200 : 3.0);
      emax = std::max(emax, (unsigned)((fx_dbits(xr[i]) >> 52) & 0x7FF));
      emax = std::max(emax, (unsigned)((fx_dbits(xi[i]) >> 52) & 0x7FF));
    }
    std::vector<fx> vr(M), vi(M);
    std::vector<std::complex<ld>> ref(M);
    for (int i = 0; i < M; ++i) {
      vr[i] = fx(d2fx(xr[i], (int)emax + 53 - H));
      vi[i] = fx(d2fx(xi[i], (int)emax + 53 - H));
      ref[i] = {(ld)xr[i], (ld)xi[i]};
    }
    // bit reversal, then radix-2 butterflies with table twiddles exp(-2 pi i j / len)
    for (int i = 1, j = 0; i < M; ++i) {
      int bit = M >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) { std::swap(vr[i], vr[j]); std::swap(vi[i], vi[j]); std::swap(ref[i], ref[j]); }
    }
    for (int len = 2; len <= M; len <<= 1) {
      for (int i0 = 0; i0 < M; i0 += len)
        for (int j = 0; j < len / 2; ++j) {
          const ld ang = -2.0L * 3.14159265358979323846264338327950288L * j / len;
          const fx_tw t = table_entry(cosl(ang), sinl(ang));
          fx br = vr[i0 + j + len / 2], bi = vi[i0 + j + len / 2];
          fx_twiddle(br, bi, t);
          const fx ar = vr[i0 + j], ai = vi[i0 + j];
          vr[i0 + j] = ar + br; vi[i0 + j] = ai + bi;
          vr[i0 + j + len / 2] = ar - br; vi[i0 + j + len / 2] = ai - bi;
          const std::complex<ld> w(cosl(ang), sinl(ang));
          const std::complex<ld> u = ref[i0 + j], b = ref[i0 + j + len / 2] * w;
          ref[i0 + j] = u + b;
          ref[i0 + j + len / 2] = u - b;
        }
    }
    ld num = 0, den = 0;
    const int S = (int)emax - 1022 - H;
    for (int i = 0; i < M; ++i) {
      const std::complex<ld> got((ld)fx2d(vr[i].v, S), (ld)fx2d(vi[i].v, S));
      num += std::norm(got - ref[i]);
      den += std::norm(ref[i]);
    }
    const double e = (double)sqrtl(num / den);
    if (e > worst_fft) worst_fft = e;
  }
  if (!(worst_fft < std::ldexp(1.0, -46))) ++bad;
  std::printf("%ld %lld %lld %.3e\n", bad, worst_mul, worst_tw, worst_fft);
  return bad != 0;
}
"""


def test_fx_arithmetic(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "fx.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "fx"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.split()[0] == "0", r.stdout + r.stderr
