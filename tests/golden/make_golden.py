"""Generate the committed golden vectors in this directory.

fft2_golden.npz: seeded random complex 2-D arrays and their transforms computed
by numpy.fft (an independent library), for the sign convention of the
reference's fourn.f call sites: solp_fft_tdma1.f:35 (isign=-1, the forward
transform numpy.fft.fft2 computes) and solp_fft_tdma3.f:36 (isign=+1,
unnormalised, i.e. numpy.fft.ifft2 times the element count).

Run: python tests/golden/make_golden.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    for n1, n2 in ((4, 4), (8, 4), (16, 32), (32, 16), (64, 8)):
        x = rng.normal(size=(n2, n1)) + 1j * rng.normal(size=(n2, n1))
        out[f"x_{n1}_{n2}"] = x
        out[f"fwd_{n1}_{n2}"] = np.fft.fft2(x)
        out[f"inv_{n1}_{n2}"] = np.fft.ifft2(x) * (n1 * n2)
    np.savez_compressed(os.path.join(HERE, "fft2_golden.npz"), **out)


if __name__ == "__main__":
    main()
