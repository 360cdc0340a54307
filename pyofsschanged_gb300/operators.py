"""Host-side construction of the fibre operator tables handed to the engine.

These are the tables pyofss builds once per domain:

* dispersion: ``sum_n beta_n (w - w0)^n / n!`` in FFT order and the loss
  ``alpha`` (``Linearity.default_linearity``, pyofss/modules/linearity.py:162-186);
* nonlinearity: ``gamma (1 + omega s)`` with s = 1/w0 (self_steepening=True) or
  the shock time given; the Raman response spectrum ``fft(h_R) * window_t``
  for the Blow-Wood (nonlinearity.py:53-69) or Hollenbeck-Cantrell
  (nonlinearity.py:72-100) model (``Nonlinearity.__call__``, nonlinearity.py:160-185);
* saturable gain: ``ln(10^(gain_dB/10))``, ``E_sat``, the fibre length and the
  Lorentzian profile ``1 / (1 + 4 (nu - nu0)^2 / dnu^2)`` with
  ``dnu = c bandwidth / lamb0^2`` in FFT order (``Amplifier``, amplifier.py:57-158).
"""

import math

import numpy as np
from scipy.integrate import simpson
from scipy.special import factorial

from .domain import LIGHT_SPEED, lambda_to_nu
from .field import fft, fftshift


class UnknownRamanResponseError(ValueError):
    pass


def dispersion_table(domain, beta, centre_omega=None):
    w0 = domain.centre_omega if centre_omega is None else centre_omega
    dw = domain.omega - w0
    terms = np.zeros(domain.total_samples)
    if beta is not None:
        for n, b in enumerate(beta):
            terms = terms + b * np.power(dw, n) / factorial(n)
    return fftshift(terms)


def raman_blowwood(domain, tau_1=12.2e-3, tau_2=32.0e-3):
    """h_R(t) = (tau1^2 + tau2^2)/(tau1 tau2^2) e^{-t/tau2} sin(t/tau1), t from 0."""
    t = domain.t - domain.t.min()
    amp = (tau_2 ** 2 + tau_1 ** 2) / (tau_1 * tau_2 ** 2)
    return amp * (np.exp(-t / tau_2) * np.sin(t / tau_1))


# Hollenbeck & Cantrell, JOSA B 19, 2886 (2002), Table 1: component positions
# (cm^-1), peak intensities, Gaussian FWHM (cm^-1), Lorentzian FWHM (cm^-1).
_HC_MODES = np.array([
    [56.25, 1.00, 52.10, 17.37], [100.00, 11.40, 110.42, 38.81], [231.25, 36.67, 175.00, 58.33],
    [362.50, 67.67, 162.50, 54.17], [463.00, 74.00, 135.33, 45.11], [497.00, 4.50, 24.50, 8.17],
    [611.50, 6.80, 41.50, 13.83], [691.67, 4.60, 155.00, 51.67], [793.67, 4.20, 59.50, 19.83],
    [835.50, 4.50, 64.30, 21.43], [930.00, 2.70, 150.00, 50.00], [1080.00, 3.10, 91.00, 30.33],
    [1215.00, 3.00, 160.00, 53.33]])


def raman_hollenbeck(domain):
    """Multiple-vibrational-mode silica response normalised to unit integral."""
    c = 299792458.0
    t = domain.t - domain.t.min()
    h = np.zeros_like(t)
    for cp, ai, gf, lf in _HC_MODES:
        h += (ai * np.exp(-np.pi * 1e-10 * c * lf * t)
              * np.exp(-((np.pi * 1e-10 * c * gf) ** 2) * (t ** 2) / 4.0)
              * np.sin(2 * np.pi * 1e-10 * c * cp * t))
    return h / simpson(h, x=domain.t)


def raman_spectrum(domain, use_all, tau_1=12.2e-3, tau_2=32.0e-3):
    """fft(h_R) * window_t (FFT order), or None when the Raman term is off."""
    if use_all is False or use_all is None:
        return None
    key = "blowwood" if use_all is True else str(use_all).lower()
    if key == "blowwood":
        h = raman_blowwood(domain, tau_1, tau_2)
    elif key == "hollenbeck":
        h = raman_hollenbeck(domain)
    else:
        raise UnknownRamanResponseError(
            'Use False, True or a sting from the list ["blowwood", "hollenbeck"]')
    return fft(h) * domain.window_t


def shock_factor(domain, self_steepening):
    if self_steepening is False or self_steepening is None:
        return 0.0
    if self_steepening is True:
        return 1.0 / domain.centre_omega
    return float(self_steepening)


def gain_profile(domain, lamb0=None, bandwidth=None):
    if bandwidth is not None and lamb0 is not None:
        delta = LIGHT_SPEED * bandwidth / (lamb0 * lamb0)
        prof = 1.0 / (1.0 + 4.0 * (((domain.nu - lambda_to_nu(lamb0)) ** 2) / (delta ** 2)))
    else:
        prof = np.ones(domain.total_samples)
    return fftshift(prof)


class GridTables:
    """All per-grid arrays and scalars of one (domain, fibre model) pair."""

    def __init__(self, domain, beta=None, alpha=None, gamma=0.0, self_steepening=False,
                 use_all=False, tau_1=12.2e-3, tau_2=32.0e-3, f_R=0.18, centre_omega=None,
                 small_signal_gain=None, E_sat=None, length=1.0, lamb0=None, bandwidth=None,
                 cluster=0):
        self.domain = domain
        self.n = domain.total_samples
        self.dt = float(domain.dt)
        self.window_t = float(domain.window_t)
        self.beta_w = np.ascontiguousarray(dispersion_table(domain, beta, centre_omega), float)
        self.alpha = 0.0 if alpha is None else float(alpha)
        self.gamma = 0.0 if gamma is None else float(gamma)
        s = shock_factor(domain, self_steepening)
        omega = fftshift(domain.omega - domain.centre_omega)
        self.ss_w = np.ascontiguousarray(1.0 + omega * s, float) if s != 0.0 else None
        hr = raman_spectrum(domain, use_all, tau_1, tau_2)
        self.f_R = float(f_R) if hr is not None else 0.0
        self.hR_re = None if hr is None else np.ascontiguousarray(hr.real, float)
        self.hR_im = None if hr is None else np.ascontiguousarray(hr.imag, float)
        self.nu = np.ascontiguousarray(fftshift(domain.nu), float)
        self.gain_on = small_signal_gain is not None and E_sat is not None
        self.gain_log = math.log(math.pow(10.0, 0.1 * small_signal_gain)) if self.gain_on else 0.0
        self.E_sat = float(E_sat) if self.gain_on else 0.0
        self.gain_length = float(length)
        self.gain_profile = (np.ascontiguousarray(gain_profile(domain, lamb0, bandwidth), float)
                             if self.gain_on else None)
        self.cluster = int(cluster)
