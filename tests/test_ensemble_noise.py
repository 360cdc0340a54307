"""One-photon-per-mode noise and the ensemble inputs (no reference counterpart; checked
against the oracle's restatement from the literature)."""

import math

import numpy as np

from oracle import gnlse_oracle as go
from pyofsschanged_gb300.domain import Domain, lambda_to_nu
from pyofsschanged_gb300.ensemble import DT, one_photon_noise, sc_ensemble


def _grid(d):
    return go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)


def test_noise_holds_one_photon_per_mode():
    for n in (4096, 8192, 16384):
        d = Domain(bit_width=DT * n, samples_per_bit=n, centre_nu=lambda_to_nu(835.0))
        a = one_photon_noise(d, np.random.default_rng(11))
        g = _grid(d)
        # photon number of every bin is 1: |A_k|^2 T = h nu_k (pyofss normalisation)
        spec = np.abs(go.fft(a)) ** 2 * d.window_t / (go.PLANCK_W_PS2 * go.fftshift(g.nu))
        np.testing.assert_allclose(spec, 1.0, rtol=1e-12)
        assert abs(go.photon_number(a, g) - n) <= 1e-9 * n
        # the same field as the oracle's restatement, bin for bin
        b = go.one_photon_noise(g, np.random.default_rng(11))
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * np.abs(b).max())


def test_noise_phases_are_the_seeded_uniform_draws():
    n = 4096
    d = Domain(bit_width=DT * n, samples_per_bit=n, centre_nu=lambda_to_nu(835.0))
    a = one_photon_noise(d, np.random.default_rng(3))
    phi = np.random.default_rng(3).uniform(0.0, 2.0 * math.pi, n)
    got = np.angle(go.fft(a)) % (2.0 * math.pi)
    diff = np.angle(np.exp(1j * (got - phi)))
    assert np.max(np.abs(diff)) < 1e-9


def test_ensemble_members_are_seeded_and_noise_is_added():
    m1, d1, f1 = sc_ensemble(12)
    m2, d2, f2 = sc_ensemble(12)
    for a, b in zip(f1, f2):
        np.testing.assert_array_equal(a, b)
    _, _, clean = sc_ensemble(12, noise=False)
    for m, a, c in zip(m1, f1, clean):
        d = d1[m.n]
        noise = a - c
        # the difference is exactly the member's own seeded one-photon field
        np.testing.assert_allclose(noise, one_photon_noise(d, np.random.default_rng(m.seed)),
                                   rtol=0, atol=1e-9 * np.abs(noise).max())
        assert abs(go.photon_number(noise, _grid(d)) - m.n) <= 1e-6 * m.n
        assert 4096 <= m.n <= 16384 and 5e-5 <= m.length <= 20e-5
        assert 2e3 <= m.peak_power <= 15e3 and 0.030 <= m.fwhm <= 0.120
