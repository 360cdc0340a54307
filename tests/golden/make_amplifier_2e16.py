"""Oracle reference for the 2^16-point fibre amplifier (CPU only, about 4 minutes)::

    python tests/golden/make_amplifier_2e16.py

The input is the 1 ps (FWHM), 100 W Gaussian at 1030 nm with a 2 ps^2 linear chirp
(pyofsschanged_gb300.amplifier builds it); the fibre is 3 m with saturable gain,
Raman and self-steepening; ARK4IP at local error 1e-6 by the FP64 oracle (a bit-exact
restatement of the reference's ARK4IP).  A full complex128 output would take 1 MB, so
the file keeps every 64th time sample and every 64th spectral bin of the output, its
Simpson energy and peak power, and the attempt and evaluation counts.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import gnlse_oracle as go  # noqa: E402
from pyofsschanged_gb300.amplifier import FIBRE, LAMBDA_NM, N, amplifier_input  # noqa: E402
from pyofsschanged_gb300.amplifier import LENGTH_KM as LENGTH  # noqa: E402

STRIDE = 64


def main():
    d, a0 = amplifier_input()
    grid = go.Grid(bit_width=100.0, samples_per_bit=N, centre_nu=299792.458 / LAMBDA_NM)
    p = go.Propagator(grid, LENGTH, **FIBRE)
    t0 = time.time()
    out, info = p.adaptive(a0.copy(), 1e-6)
    spec = go.fft(out)
    np.savez_compressed(os.path.join(HERE, "amplifier_2e16.npz"), stride=STRIDE,
                        out_samples=out[::STRIDE], spec_samples=spec[::STRIDE],
                        energy=go.energy(out, d.t), peak=np.max(np.abs(out) ** 2),
                        attempts=info["attempts"], evals=p.evals, wall_s=time.time() - t0)
    print(info["attempts"], p.evals, go.energy(out, d.t), time.time() - t0)


if __name__ == "__main__":
    main()
