"""Field helpers with the pyofss conventions (pyofss/field.py:43-172).

pyofss's ``fft`` maps the temporal field to the spectrum with the physics sign
convention (sum with e^{+i w t}, scaled by 1/N) and ``ifft`` maps back; the
shift helpers are named the other way round from numpy's.  These are host
utilities for preparing inputs and reading results; the propagation itself
runs in the CUDA engine.
"""

import numpy as np


def fft(a_t):
    """Temporal -> spectral: (1/N) sum_n a_n e^{+2 pi i k n / N}."""
    return np.fft.ifft(a_t)


def ifft(a_nu):
    """Spectral -> temporal: sum_k A_k e^{-2 pi i k n / N}."""
    return np.fft.fft(a_nu)


def fftshift(a):
    """Consecutive order -> FFT order."""
    return np.fft.ifftshift(a)


def ifftshift(a):
    """FFT order -> consecutive order."""
    return np.fft.fftshift(a)


def temporal_power(a_t, normalise=False):
    p = np.abs(a_t) ** 2
    return p / np.max(p) if normalise else p


def spectral_power(a_t, normalise=False):
    p = np.abs(fft(a_t)) ** 2
    if normalise:
        p = p / np.max(p)
    return ifftshift(p)


def phase(a_t, unwrap=True):
    return np.unwrap(np.angle(a_t)) if unwrap else np.angle(a_t)


def simpson_weights(n):
    """Uniform-grid weights (units of dt) of scipy's even-N composite Simpson."""
    w = np.empty(n)
    w[0] = 1.0 / 3.0
    w[1:n - 2:2] = 4.0 / 3.0
    w[2:n - 2:2] = 2.0 / 3.0
    w[n - 2] = 1.0
    w[n - 3] -= 1.0 / 12.0
    w[n - 1] = 5.0 / 12.0
    return w


def energy(a_t, t):
    """Pulse energy in nJ (Simpson rule over t in ps, power in W)."""
    dt = t[1] - t[0]
    return float(np.sum(simpson_weights(len(a_t)) * np.abs(a_t) ** 2) * dt * 1e-3)


def spectral_phase(a_t, domain, gdd, centre_omega=None):
    """The field with the quadratic spectral phase exp(i gdd/2 (w - w0)^2) applied: a
    linear chirp of group-delay dispersion ``gdd`` (ps^2), the phase propagation through
    a length z of a fibre with beta_2 z = gdd acquires in the dispersion operator
    i sum_n beta_n (w - w0)^n / n! (pyofss/modules/linearity.py:162-186)."""
    w0 = domain.centre_omega if centre_omega is None else centre_omega
    dw = fftshift(np.asarray(domain.omega) - w0)
    return ifft(np.exp(0.5j * gdd * dw * dw) * fft(np.asarray(a_t, complex)))
