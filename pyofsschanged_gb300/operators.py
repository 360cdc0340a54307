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
  ``dnu = c bandwidth / lamb0^2`` in FFT order (``Amplifier``, amplifier.py:57-158);
* the Yb two-level gain (``Amplifier2LevelModel``, amplifier.py:178-379): the
  per-frequency gain and inversion tables and the pump constants;
* the legacy Raman term ``rs_factor d|A|^2/dt`` (``raman_scattering`` without
  ``use_all``, nonlinearity.py:236-248), as an equivalent response table.
"""

import importlib.util
import math
import os

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


def read_cross_section_table(path):
    """(wavelength m, sigma_12 m^2, sigma_21 m^2) columns of a Yb cross-section table
    such as pyofss/data/CrossSectionDataExp.txt.  As ``Amplifier2LevelModel`` reads it
    (pandas ``read_csv`` with its default header inference, amplifier.py:238-242), the
    first line names the columns and is not data."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    tab = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])
    return tab[:, 0], tab[:, 1], tab[:, 2]


def _reference_cross_section_file():
    spec = importlib.util.find_spec("pyofss")
    if spec is None or not spec.submodule_search_locations:
        return None
    for root in spec.submodule_search_locations:
        path = os.path.join(root, "data", "CrossSectionDataExp.txt")
        if os.path.exists(path):
            return path
    return None


class Amplifier2LevelModel:
    """Yb two-level rate-equation gain (pyofss/modules/amplifier.py:178-379).

    ``Pp`` (W), ``N`` (Yb density, 1e25 m^-3) and ``Rr`` (repetition rate, THz) as in
    the reference.  ``cross_sections`` gives the signal cross sections: a path to a
    table in the reference's format, ``(wavelength_m, sigma_12, sigma_21)`` columns, or
    ``(sigma_12, sigma_21)`` already on the domain (natural order, m^2).  By default the
    table of an importable pyofss installation is used.  The engine evaluates
    ``factor`` (amplifier.py:366-379) on the GPU; ``Pp`` holds the pump power reached
    by the last propagation.
    """

    h_p = 6.62e-34          # amplifier.py:201-218
    T = 850.0e-6
    a = 3.0e-6
    b = 60.0e-6
    NA = 0.13
    lamb_p = 976.0
    sigma12_p = 2.5e-24
    sigma21_p = 2.44e-24

    def __init__(self, name="amplifier2LevelModel", Pp=None, N=None, Rr=None, cross_sections=None):
        if Pp is None or N is None or Rr is None:
            raise ValueError("Amplifier2LevelModel needs Pp, N and Rr")
        self.name = name
        self.Pp_0 = float(Pp)
        self.Pp = self.Pp_0
        self.N = N * 1e25 * np.pi * self.a ** 2
        self.Tr = 1.0 / Rr
        self.cross_sections = cross_sections
        self.domain = None

    def _sigma_s(self, domain):
        cs = self.cross_sections
        if cs is None:
            cs = _reference_cross_section_file()
            if cs is None:
                raise FileNotFoundError(
                    "Amplifier2LevelModel needs the Yb cross sections: pass cross_sections= "
                    "(a table path, (wavelength_m, sigma_12, sigma_21) or (sigma_12, sigma_21) on the domain)")
        if isinstance(cs, (str, os.PathLike)):
            cs = read_cross_section_table(cs)
        if len(cs) == 2:
            s12, s21 = (np.asarray(x, float) for x in cs)
            if s12.shape != (domain.total_samples,) or s21.shape != s12.shape:
                raise ValueError("on-grid cross sections must have one value per sample")
            return s12, s21
        from scipy.interpolate import InterpolatedUnivariateSpline as IUS
        lam, c12, c21 = (np.asarray(x, float) for x in cs)
        s12 = IUS(lam * 1e9, c12 * 1e27, ext=1)(domain.Lambda) * 1e-27
        s21 = IUS(lam * 1e9, c21 * 1e27, ext=1)(domain.Lambda) * 1e-27
        return s12, s21

    def set_domain(self, domain):
        """Tables on ``domain`` (amplifier.py:247-344), in the engine's form: FFT order,
        signal gain alpha_s N and eta_s (1/m), and the inversion weights that turn
        |n fft(x)|^2 into Ps / Psat_s terms (Ps = spectral power * n dt / Tr)."""
        a = self.a
        s12, s21 = self._sigma_s(domain)
        self.sigma12_s, self.sigma21_s = s12, s21
        V = (2.0 * np.pi / domain.Lambda) * a * self.NA * 1e9
        omega_s = a * (0.616 + 1.66 / pow(V, 1.5) + 0.987 / pow(V, 6.0))
        rho_s = (1.0 - np.exp(-2.0 * a ** 2 / (omega_s * omega_s))) / (np.pi * a ** 2)
        rho_p = (a ** 2) / (self.b ** 2) / (np.pi * a ** 2)
        with np.errstate(divide="ignore", invalid="ignore"):
            psat_s = (self.h_p * domain.nu * 1e12) / (self.T * (s12 + s21) * rho_s)
            ratio_s = s12 / (s12 + s21)
            w_ratio = ratio_s / psat_s
            w_sat = 1.0 / psat_s
        scale = domain.dt / (domain.total_samples * self.Tr)
        # terms the reference drops as NaN (zero cross sections) weigh nothing
        self.w_ratio = np.ascontiguousarray(fftshift(np.nan_to_num(w_ratio, nan=0.0) * scale), float)
        self.w_sat = np.ascontiguousarray(fftshift(np.nan_to_num(w_sat, nan=0.0) * scale), float)
        self.alpha_s_N = np.ascontiguousarray(fftshift((s12 + s21) * rho_s * self.N), float)
        self.eta_s = np.ascontiguousarray(fftshift(s12 * rho_s * self.N), float)
        sp = self.sigma12_p + self.sigma21_p
        self.Psat_p = (self.h_p * lambda_to_nu(self.lamb_p) * 1e12) / (self.T * sp * rho_p)
        self.ratio_p = self.sigma12_p / sp
        self.alpha_p_N = sp * rho_p * self.N
        self.eta_p = self.sigma12_p * rho_p * self.N
        self.domain = domain
        return self


class GridTables:
    """All per-grid arrays and scalars of one (domain, fibre model) pair."""

    def __init__(self, domain, beta=None, alpha=None, gamma=0.0, self_steepening=False,
                 use_all=False, tau_1=12.2e-3, tau_2=32.0e-3, f_R=0.18, centre_omega=None,
                 small_signal_gain=None, E_sat=None, length=1.0, lamb0=None, bandwidth=None,
                 use_Yb_model=False, Pp_0=None, N=None, Rr=None, yb_cross_sections=None,
                 raman_scattering=False, rs_factor=3e-3, cluster=0):
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
        if raman_scattering and not use_all:
            # The legacy term (default_f_with_rs, nonlinearity.py:236-248):
            # i gamma (|x|^2 + rs ifft(i omega fft(|x|^2))) x.  The engine evaluates
            # i gamma' ((1 - f_R)|x|^2 + f_R ifft(hR/n ... )) x with hR = fft(h_R) window_t;
            # hR = i rs omega, f_R = 1/2 and gamma' = 2 gamma give the same term (the
            # factors 1/2 and 2 are exact in floating point).
            if s != 0.0:
                raise NotImplementedError(
                    "raman_scattering with self_steepening: the reference adds that self-steepening "
                    "term without the factor i gamma (nonlinearity.py:250-256); not on the CUDA path")
            hr = 1j * float(rs_factor) * omega
            self.f_R = 0.5
            self.gamma = 2.0 * self.gamma
        self.hR_re = None if hr is None else np.ascontiguousarray(hr.real, float)
        self.hR_im = None if hr is None else np.ascontiguousarray(hr.imag, float)
        self.nu = np.ascontiguousarray(fftshift(domain.nu), float)
        # fibre.py:97-103: the Yb model replaces the saturable amplifier
        self.yb = (Amplifier2LevelModel(Pp=Pp_0, N=N, Rr=Rr, cross_sections=yb_cross_sections)
                   .set_domain(domain) if use_Yb_model else None)
        self.gain_on = small_signal_gain is not None and E_sat is not None and not use_Yb_model
        self.gain_log = math.log(math.pow(10.0, 0.1 * small_signal_gain)) if self.gain_on else 0.0
        self.E_sat = float(E_sat) if self.gain_on else 0.0
        self.gain_length = float(length)
        self.gain_profile = (np.ascontiguousarray(gain_profile(domain, lamb0, bandwidth), float)
                             if self.gain_on else None)
        self.cluster = int(cluster)
