"""Generates the known-answer fixtures in this folder from closed-form
expressions taken from the reference's own tests (no FFT is evaluated here).

* brfft_single_mode_{16,17}.npz -- reference test/brfft.jl:17-45: a spectrum
  with the single mode uc[2,4,3] = 1+2im (1-based) on (12,13,9) transformed by
  BRFFT((12,13,16|17)); the expected real field is
  2 Re[(1+2i) exp(2 pi i (x/12 + 3y/13 + 2z/Nz))].
* taylor_green_16_8_16.npz -- reference test/taylor_green.jl:26-76: the
  Taylor-Green field on (16,8,16) over [0,4pi) x [0,2pi)^2 with u0=3, k0=2,
  its exact RFFT coefficients and its exact vorticity.
* rfft_known_answer_{42,41}.npz -- reference test/rfft.jl:213-231: x[1]=1, x[2]=2,
  zeros elsewhere; after an RFFT round trip x[1:3] == [1, 2, 0].

Run: python tests/golden/make_golden.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def brfft_single_mode(nz):
    dims_coef = (12, 13, 9)
    uc = np.zeros(dims_coef, dtype=np.complex128)
    uc[1, 3, 2] = 1 + 2j
    x = np.arange(12)[:, None, None]
    y = np.arange(13)[None, :, None]
    z = np.arange(nz)[None, None, :]
    phase = 2 * np.pi * (x / 12 + 3 * y / 13 + 2 * z / nz)
    ur = 2 * np.real((1 + 2j) * np.exp(1j * phase))
    np.savez_compressed(os.path.join(HERE, f"brfft_single_mode_{nz}.npz"), uc=uc, ur=ur)


def taylor_green():
    dims = (16, 8, 16)
    L = (4 * np.pi, 2 * np.pi, 2 * np.pi)
    u0, k0 = 3.0, 2.0
    x, y, z = (np.arange(n) * (l / n) for n, l in zip(dims, L))
    X, Y, Zc = np.meshgrid(x, y, z, indexing="ij")
    u = np.stack([u0 * np.sin(k0 * X) * np.cos(k0 * Y) * np.cos(k0 * Zc),
                  -u0 * np.cos(k0 * X) * np.sin(k0 * Y) * np.cos(k0 * Zc),
                  np.zeros(dims)])
    w = np.stack([-u0 * k0 * np.cos(k0 * X) * np.sin(k0 * Y) * np.sin(k0 * Zc),
                  -u0 * k0 * np.sin(k0 * X) * np.cos(k0 * Y) * np.sin(k0 * Zc),
                  2 * u0 * k0 * np.sin(k0 * X) * np.sin(k0 * Y) * np.cos(k0 * Zc)])
    # exact RFFT coefficients: sin(2x) on 16 points over 4pi is mode 4, cos(2y)
    # on 8 points over 2pi is mode 2 (and 6), cos(2z) on 16 points is mode 2 (14)
    uF = np.zeros((3, 9, 8, 16), dtype=np.complex128)
    for ky in (2, 6):
        for kz in (2, 14):
            uF[0, 4, ky, kz] = u0 * (-8j) * 4 * 8          # sin -> -i N/2
            # u2 = -u0 cos(2x) sin(2y) cos(2z): cos -> N/2, sin -> -i N/2 (+i at N-k)
            s = -4j if ky == 2 else 4j
            uF[1, 4, ky, kz] = -u0 * 8 * s * 8
    np.savez_compressed(os.path.join(HERE, "taylor_green_16_8_16.npz"), u=u, w=w, uF=uF,
             L=np.array(L), u0=u0, k0=k0)


def rfft_known():
    # Julia's x[1], x[2] are the first two entries along dimension 1
    for dims in ((42, 24, 16), (41, 23, 15)):
        np.savez_compressed(os.path.join(HERE, f"rfft_known_answer_{dims[0]}.npz"),
                            dims=np.array(dims), nonzero=np.array([[0, 0, 0], [1, 0, 0]]),
                            values=np.array([1.0, 2.0]), expect_first3=np.array([1.0, 2.0, 0.0]))


if __name__ == "__main__":
    brfft_single_mode(16)
    brfft_single_mode(17)
    taylor_green()
    rfft_known()
    print("golden fixtures written to", HERE)
