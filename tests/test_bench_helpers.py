"""Host-side helpers of bench.py (no GPU)."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402


def test_spectral_power_db_error():
    rng = np.random.default_rng(5)
    t = np.linspace(-5, 5, 1024, endpoint=False)
    ref = np.exp(-t ** 2) * np.exp(1j * 0.3 * t ** 2)
    assert bench.spectral_power_db_error(ref, ref) == 0.0
    # a uniform 1% amplitude error is a 20 log10(1.01) dB power error everywhere
    assert abs(bench.spectral_power_db_error(1.01 * ref, ref) - 20 * np.log10(1.01)) < 1e-12
    # noise far below the -40 dB band does not count
    noisy = ref + 1e-9 * (rng.standard_normal(1024) + 1j * rng.standard_normal(1024))
    assert bench.spectral_power_db_error(noisy, ref) < 1e-3
