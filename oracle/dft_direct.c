/*
 * Direct O(n^2) evaluation of FFTW's published 1D transform definitions in
 * long double.  TEST INFRASTRUCTURE ONLY: the tests use it to pin the scipy
 * based oracle (oracle/pencilfft_oracle.py) on small sizes; the product path
 * never links it.
 *
 * The reference (PencilFFTs.jl) delegates every 1D transform to FFTW 3.3
 * (src/Transforms/c2c.jl:53-56, r2c.jl:83-96, r2r.jl:92-93).  The formulas
 * below are FFTW's documented definitions of those transforms (all
 * unnormalised); the angle arguments are reduced exactly in integers before
 * the trigonometric call.
 */
#include <math.h>
#include <stdint.h>

typedef long double ld;
static const ld PI_L = 3.141592653589793238462643383279502884L;

/* cos and sin of pi * m / d with m reduced modulo 2d. */
static void cs_pi(int64_t m, int64_t d, ld *c, ld *s) {
  int64_t two_d = 2 * d;
  m %= two_d;
  if (m < 0) m += two_d;
  ld a = PI_L * (ld)m / (ld)d;
  *c = cosl(a);
  *s = sinl(a);
}

/* Complex DFT, sign -1 (FFT) or +1 (BFFT), interleaved re/im. */
void pfo_dft(int64_t n, int sign, const double *in, double *out) {
  for (int64_t k = 0; k < n; ++k) {
    ld re = 0, im = 0;
    for (int64_t j = 0; j < n; ++j) {
      ld c, s;
      cs_pi(2 * ((j * k) % n), n, &c, &s); /* angle 2 pi jk / n */
      s = sign < 0 ? -s : s;
      ld xr = in[2 * j], xi = in[2 * j + 1];
      re += xr * c - xi * s;
      im += xr * s + xi * c;
    }
    out[2 * k] = (double)re;
    out[2 * k + 1] = (double)im;
  }
}

/* r2c: n reals -> n/2+1 complex (sign -1). */
void pfo_rfft(int64_t n, const double *in, double *out) {
  for (int64_t k = 0; k <= n / 2; ++k) {
    ld re = 0, im = 0;
    for (int64_t j = 0; j < n; ++j) {
      ld c, s;
      cs_pi(2 * ((j * k) % n), n, &c, &s);
      re += in[j] * c;
      im -= in[j] * s;
    }
    out[2 * k] = (double)re;
    out[2 * k + 1] = (double)im;
  }
}

/* c2r: n/2+1 complex -> n reals (sign +1, unnormalised).  Uses the Hermitian
 * extension of the input; the imaginary parts of the DC term and, for even n,
 * of the Nyquist term do not contribute. */
void pfo_brfft(int64_t n, const double *in, double *out) {
  int64_t m = n / 2 + 1;
  for (int64_t j = 0; j < n; ++j) {
    ld acc = in[0];
    for (int64_t k = 1; k < m; ++k) {
      ld c, s;
      cs_pi(2 * ((j * k) % n), n, &c, &s);
      ld xr = in[2 * k], xi = in[2 * k + 1];
      ld term = xr * c - xi * s; /* Re(X_k e^{+i theta}) */
      if (2 * k == n)
        acc += xr * c; /* Nyquist: real part only, appears once */
      else
        acc += 2 * term;
    }
    out[j] = (double)acc;
  }
}

/* Real-to-real transforms, FFTW kind codes (fftw3.h). */
enum { K_DHT = 2, K_REDFT00 = 3, K_REDFT01 = 4, K_REDFT10 = 5, K_REDFT11 = 6,
       K_RODFT00 = 7, K_RODFT01 = 8, K_RODFT10 = 9, K_RODFT11 = 10 };

int pfo_r2r(int kind, int64_t n, const double *x, double *y) {
  for (int64_t k = 0; k < n; ++k) {
    ld acc = 0, c, s;
    switch (kind) {
      case K_DHT:
        for (int64_t j = 0; j < n; ++j) {
          cs_pi(2 * ((j * k) % n), n, &c, &s);
          acc += x[j] * (c + s);
        }
        break;
      case K_REDFT00: /* X0 + (-1)^k X_{n-1} + 2 sum_{j=1}^{n-2} X_j cos(pi jk/(n-1)) */
        if (n < 2) return -1;
        acc = x[0] + ((k & 1) ? -x[n - 1] : x[n - 1]);
        for (int64_t j = 1; j < n - 1; ++j) {
          cs_pi(j * k, n - 1, &c, &s);
          acc += 2 * x[j] * c;
        }
        break;
      case K_REDFT10: /* 2 sum X_j cos(pi (2j+1) k / (2n)) */
        for (int64_t j = 0; j < n; ++j) {
          cs_pi((2 * j + 1) * k, 2 * n, &c, &s);
          acc += 2 * x[j] * c;
        }
        break;
      case K_REDFT01: /* X0 + 2 sum_{j>=1} X_j cos(pi j (2k+1) / (2n)) */
        acc = x[0];
        for (int64_t j = 1; j < n; ++j) {
          cs_pi(j * (2 * k + 1), 2 * n, &c, &s);
          acc += 2 * x[j] * c;
        }
        break;
      case K_REDFT11: /* 2 sum X_j cos(pi (2j+1)(2k+1) / (4n)) */
        for (int64_t j = 0; j < n; ++j) {
          cs_pi((2 * j + 1) * (2 * k + 1), 4 * n, &c, &s);
          acc += 2 * x[j] * c;
        }
        break;
      case K_RODFT00: /* 2 sum X_j sin(pi (j+1)(k+1) / (n+1)) */
        for (int64_t j = 0; j < n; ++j) {
          cs_pi((j + 1) * (k + 1), n + 1, &c, &s);
          acc += 2 * x[j] * s;
        }
        break;
      case K_RODFT10: /* 2 sum X_j sin(pi (2j+1)(k+1) / (2n)) */
        for (int64_t j = 0; j < n; ++j) {
          cs_pi((2 * j + 1) * (k + 1), 2 * n, &c, &s);
          acc += 2 * x[j] * s;
        }
        break;
      case K_RODFT01: /* (-1)^k X_{n-1} + 2 sum_{j=0}^{n-2} X_j sin(pi (j+1)(2k+1) / (2n)) */
        acc = (k & 1) ? -x[n - 1] : x[n - 1];
        for (int64_t j = 0; j < n - 1; ++j) {
          cs_pi((j + 1) * (2 * k + 1), 2 * n, &c, &s);
          acc += 2 * x[j] * s;
        }
        break;
      case K_RODFT11: /* 2 sum X_j sin(pi (2j+1)(2k+1) / (4n)) */
        for (int64_t j = 0; j < n; ++j) {
          cs_pi((2 * j + 1) * (2 * k + 1), 4 * n, &c, &s);
          acc += 2 * x[j] * s;
        }
        break;
      default:
        return -2;
    }
    y[k] = (double)acc;
  }
  return 0;
}
