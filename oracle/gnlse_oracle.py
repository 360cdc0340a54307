"""FP64 CPU restatement of the pyofss GNLSE propagation path (the oracle).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this module, and only as the
checker or the timed CPU baseline.  The product package never calls it.

It restates, operation by operation and in complex128, the reference's
time-domain formulation of:

* the FFT convention of ``pyofss/field.py:109-158``: pyofss ``fft`` is
  scipy ``ifft`` (sum with e^{+i w t}, scaled by 1/N) and pyofss ``ifft`` is
  scipy ``fft``; ``fftshift``/``ifftshift`` are swapped likewise;
* ``Domain.__init__`` (``pyofss/domain.py:171-243``);
* ``Sech.generate``/``Sech.__call__`` (``pyofss/modules/sech.py:111-113,124-168``)
  and ``Gaussian`` (``pyofss/modules/gaussian.py:118,132-170``);
* ``Linearity.default_linearity``/``default_exp_f[_cached]``
  (``pyofss/modules/linearity.py:162-186,241-272``);
* ``Nonlinearity.__call__``, ``default_f_all``, ``default_f``,
  ``default_f_with_ss``, the legacy ``rs_factor`` terms (``default_f_with_rs``,
  ``default_f_with_ss_and_rs`` and their exponential forms) and the Blow-Wood /
  Hollenbeck Raman responses
  (``pyofss/modules/nonlinearity.py:53-100,160-207,213-270``);
* ``Amplifier.factor`` with the Lorentzian gain profile
  (``pyofss/modules/amplifier.py:110-158``) and Simpson energy
  (``pyofss/field.py:161-172``);
* the Yb two-level gain ``Amplifier2LevelModel`` (``pyofss/modules/amplifier.py:178-379``);
* ``Solver.rk4ip`` (``pyofss/modules/solver.py:339-354``) and the split-step methods
  ``ss_simple``, ``ss_symmetric``, ``ss_reduced``, ``ss_agrawal``, ``ss_sym_midpoint``,
  ``ss_sym_rk4`` (``solver.py:101-106,256-337``);
* ``Stepper.standard_stepper`` / ``adaptive_stepper`` / ``relative_local_error``
  (``pyofss/modules/stepper.py:164-221,231-376``).

Parity of this restatement with the unmodified reference is pinned by
``tests/test_oracle_vs_reference.py`` (run where the reference tree exists) and
by the committed fixtures in ``tests/golden/`` made by
``tests/golden/make_golden.py`` from the reference itself.
"""

import math

import numpy as np
import scipy.fftpack as _fftpack
import scipy.integrate as _integrate
import scipy.linalg as _linalg
from scipy.special import factorial as _factorial

LIGHT_SPEED_NM_PS = 1.0e-3 * 299792458.0  # scipy.constants.c in nm/ps (domain.py:160)
PLANCK_W_PS2 = 6.62607015e-34 * 1.0e24  # J s -> W ps^2


# ----------------------------------------------------------------------------
# FFT convention (field.py:109-158)
# ----------------------------------------------------------------------------
def fft(a_t):
    """pyofss ``fft``: temporal -> spectral, (1/N) sum a_n e^{+2 pi i k n / N}."""
    return _fftpack.ifft(a_t)


def ifft(a_nu):
    """pyofss ``ifft``: spectral -> temporal, sum A_k e^{-2 pi i k n / N}."""
    return _fftpack.fft(a_nu)


def fftshift(a):
    """pyofss ``fftshift``: consecutive order -> FFT order (scipy ``ifftshift``)."""
    return _fftpack.ifftshift(a)


def ifftshift(a):
    """pyofss ``ifftshift``: FFT order -> consecutive order (scipy ``fftshift``)."""
    return _fftpack.fftshift(a)


def temporal_power(a_t):
    return np.abs(a_t) ** 2


def spectral_power(a_t):
    """field.py:60-75 (unnormalised)."""
    return ifftshift(np.abs(fft(a_t)) ** 2)


def energy(a_t, t):
    """Simpson energy in nJ (field.py:161-172): simpson(|A|^2, t * 1e-3)."""
    return _integrate.simpson(temporal_power(a_t), x=t * 1e-3)


def simpson_weights(n):
    """Uniform-grid weights (in units of dt) reproducing scipy's even-N Simpson.

    scipy integrates points 0..n-2 with composite Simpson (1,4,2,...,4,1)/3 and
    adds Cartwright's correction for the last interval, which for uniform
    spacing is (5/12) y[n-1] + (2/3) y[n-2] - (1/12) y[n-3].
    """
    if n % 2 != 0 or n < 4:
        raise ValueError("even n >= 4 expected")
    w = np.empty(n)
    w[0] = 1.0 / 3.0
    w[1:n - 2:2] = 4.0 / 3.0
    w[2:n - 2:2] = 2.0 / 3.0
    w[n - 2] = 1.0 / 3.0 + 2.0 / 3.0
    w[n - 3] -= 1.0 / 12.0
    w[n - 1] = 5.0 / 12.0
    return w


# ----------------------------------------------------------------------------
# Grid (domain.py:171-243)
# ----------------------------------------------------------------------------
def lambda_to_nu(lam_nm):
    return LIGHT_SPEED_NM_PS / lam_nm


class Grid:
    """Restatement of ``Domain``: t, nu, omega, Lambda and their steps."""

    def __init__(self, total_bits=1, samples_per_bit=512, bit_width=100.0, centre_nu=193.1):
        self.total_bits = total_bits
        self.samples_per_bit = samples_per_bit
        self.bit_width = bit_width
        self.centre_nu = centre_nu
        self.total_samples = total_bits * samples_per_bit
        self.window_t = total_bits * bit_width
        self.centre_omega = 2.0 * math.pi * centre_nu
        self.centre_lambda = LIGHT_SPEED_NM_PS / centre_nu
        self.t, self.dt = np.linspace(-self.window_t / 2.0, self.window_t / 2.0,
                                      self.total_samples, False, True)
        self.window_nu = 1.0 / self.dt
        nu_min = centre_nu - 0.5 * self.window_nu
        self.nu, self.dnu = np.linspace(nu_min, nu_min + self.window_nu,
                                        self.total_samples, False, True)
        self.omega = 2.0 * math.pi * self.nu
        self.domega = 2.0 * math.pi * self.dnu
        self.Lambda = LIGHT_SPEED_NM_PS / self.nu


# ----------------------------------------------------------------------------
# Pulses (sech.py, gaussian.py)
# ----------------------------------------------------------------------------
def sech_width(width, using_fwhm):
    """FWHM -> half width at 1/e (sech.py:111-113)."""
    return width * (0.5 / math.log(1.0 + math.sqrt(2.0))) if using_fwhm else width


def gaussian_width(width, using_fwhm, m=1):
    """FWHM -> half width at 1/e (gaussian.py:118)."""
    return width * (0.5 / np.power(math.log(2.0), 1.0 / (2 * m))) if using_fwhm else width


def sech_field(t, window_t, peak_power, width, position=0.0, offset_nu=0.0, C=0.0,
               initial_phase=0.0):
    """``Sech.__call__`` added to a zero field (sech.py:124-146); width is HWIeM."""
    t_norm = (t - position * window_t) / width
    time = t_norm * t_norm
    phase = initial_phase
    phase = phase - (2.0 * np.pi * offset_nu * t + 0.5 * C * time)
    magnitude = np.sqrt(peak_power) / np.cosh(t_norm)
    return np.zeros(t.shape, complex) + magnitude * np.exp(1j * phase)


def gaussian_field(t, window_t, peak_power, width, position=0.0, offset_nu=0.0, m=1, C=0.0,
                   initial_phase=0.0):
    """``Gaussian.__call__`` added to a zero field (gaussian.py:132-153)."""
    t_norm = (t - position * window_t) / width
    # gaussian.py imports power from numpy.lib.scimath, which promotes a base
    # with negative entries to complex
    time = np.power(t_norm.astype(complex) if np.any(t_norm < 0) else t_norm, 2 * m)
    phase = initial_phase
    phase = phase - (2.0 * np.pi * offset_nu * t + 0.5 * C * time)
    magnitude = np.sqrt(peak_power) * np.exp(-0.5 * time)
    return np.zeros(t.shape, complex) + magnitude * np.exp(1j * phase)


# ----------------------------------------------------------------------------
# Operators
# ----------------------------------------------------------------------------
def dispersion_terms(grid, beta, centre_omega=None):
    """sum_n beta_n (w - w0)^n / n! in FFT order (linearity.py:167-181)."""
    w0 = grid.centre_omega if centre_omega is None else centre_omega
    d_omega = grid.omega - w0
    terms = 0.0
    for n, b in enumerate(beta):
        terms = terms + b * np.power(d_omega, n) / _factorial(n)
    return fftshift(terms)


def linear_factor(grid, beta=None, alpha=None, centre_omega=None):
    """``Linearity.default_linearity`` (linearity.py:162-186)."""
    if beta is None:
        factor = 0.0
    else:
        factor = 1j * dispersion_terms(grid, beta, centre_omega)
    if alpha is not None:
        factor = factor - 0.5 * alpha
    return factor


def raman_blowwood(grid, tau_1=12.2e-3, tau_2=32.0e-3):
    """Blow-Wood h_R(t), t from zero at index 0 (nonlinearity.py:53-69)."""
    t = grid.t - grid.t.min()
    h = (tau_2 ** 2 + tau_1 ** 2) / (tau_1 * tau_2 ** 2)
    return h * (np.exp(-t / tau_2) * np.sin(t / tau_1))


_HOLLENBECK = (
    (56.25, 100.00, 231.25, 362.50, 463.00, 497.00, 611.50, 691.67, 793.67, 835.50, 930.00,
     1080.00, 1215.00),
    (1.00, 11.40, 36.67, 67.67, 74.00, 4.50, 6.80, 4.60, 4.20, 4.50, 2.70, 3.10, 3.00),
    (52.10, 110.42, 175.00, 162.50, 135.33, 24.50, 41.50, 155.00, 59.50, 64.30, 150.00, 91.00,
     160.00),
    (17.37, 38.81, 58.33, 54.17, 45.11, 8.17, 13.83, 51.67, 19.83, 21.43, 50.00, 30.33, 53.33),
)


def raman_hollenbeck(grid):
    """Hollenbeck-Cantrell 13-mode response, unit integral (nonlinearity.py:72-100).

    The mode table (centre positions, amplitudes, Gaussian and Lorentzian
    widths in cm^-1) is the published one of Hollenbeck & Cantrell, JOSA B 19,
    2886 (2002), Table 1.
    """
    cp, ai, gf, lf = _HOLLENBECK
    c = 299792458.0
    t = grid.t - grid.t.min()
    h = np.zeros_like(t)
    for i in range(13):
        h += (ai[i] * np.exp(-np.pi * 1e-10 * c * lf[i] * t)
              * np.exp(-((np.pi * 1e-10 * c * gf[i]) ** 2) * (t ** 2) / 4.0)
              * np.sin(2 * np.pi * 1e-10 * c * cp[i] * t))
    norm = _integrate.simpson(h, x=grid.t)
    return h / norm


class Nonlinear:
    """``Nonlinearity`` for the default single-channel model (nonlinearity.py:103-207)."""

    def __init__(self, grid, gamma, self_steepening=False, use_all=False, tau_1=12.2e-3,
                 tau_2=32.0e-3, f_R=0.18, raman_scattering=False, rs_factor=3e-3):
        self.gamma = gamma
        self.f_R = f_R
        self.use_all = use_all
        self.rs_on = bool(raman_scattering)
        self.rs_factor = rs_factor
        self.omega = fftshift(grid.omega - grid.centre_omega)
        if self_steepening is False:
            self.ss_factor = 0.0
        elif self_steepening is True:
            self.ss_factor = 1.0 / grid.centre_omega
        else:
            self.ss_factor = float(self_steepening)
        if use_all is False:
            self.h_R = 0.0
        elif use_all is True or str(use_all).lower() == "blowwood":
            self.h_R = fft(raman_blowwood(grid, tau_1, tau_2))
        elif str(use_all).lower() == "hollenbeck":
            self.h_R = fft(raman_hollenbeck(grid))
        else:
            raise ValueError("use_all must be False, True, 'blowwood' or 'hollenbeck'")
        self.h_R = self.h_R * grid.window_t
        self.factor = 0.0 if gamma is None else 1j * gamma
        self.ss_on = bool(self_steepening)

    def __call__(self, A):
        if self.use_all:
            # default_f_all (nonlinearity.py:201-207)
            term_spm = np.abs(A) ** 2
            convolution = ifft(self.h_R * fft(term_spm))
            p = fft(A * (1.0 - self.f_R) * term_spm + self.f_R * A * convolution)
            return ifft(self.factor * (1.0 + self.omega * self.ss_factor) * p)
        if self.rs_on:
            # default_f_with_rs / default_f_with_ss_and_rs (nonlinearity.py:236-256); the
            # latter adds its self-steepening term without the factor i gamma
            term_spm = np.abs(A) ** 2
            term_rs = self.rs_factor * ifft(1j * self.omega * fft(term_spm))
            out = self.factor * (term_spm + term_rs) * A
            if self.ss_on:
                out = out + self.ss_factor * ifft(self.omega * fft(term_spm * A))
            return out
        if self.ss_on:
            # default_f_with_ss (nonlinearity.py:209-214)
            term_spm = np.abs(A) ** 2 * A
            term_ss = self.ss_factor * ifft(self.omega * fft(term_spm))
            return self.factor * (term_spm + term_ss)
        # default_f (nonlinearity.py:266-267)
        return self.factor * np.abs(A) ** 2 * A

    def exp_non(self, A, h, B):
        """Exponential nonlinear step of the split-step methods."""
        if self.use_all:
            # default_exp_f_all (nonlinearity.py:209-221)
            term_spm = np.abs(A) ** 2
            convolution = ifft(self.h_R * fft(term_spm))
            term_all = (1.0 - self.f_R) * term_spm + self.f_R * convolution
            with np.errstate(divide="ignore", invalid="ignore"):
                inv_b = np.where(np.abs(B) > 1e-15, self.ss_factor / B, 0.0)
            term_ss_all = inv_b * ifft(self.omega * fft(term_all * A))
            return np.exp(h * self.factor * (term_all + term_ss_all)) * B
        if self.rs_on:
            # default_exp_f_with_rs / default_exp_f_with_ss_and_rs (nonlinearity.py:243-264)
            term_spm = np.abs(A) ** 2
            term_rs = self.rs_factor * ifft(1j * self.omega * fft(term_spm))
            if self.ss_on:
                term_ss = (self.ss_factor / B) * ifft(self.omega * fft(term_spm * A))
                return np.exp(h * self.factor * (term_spm + term_ss + term_rs)) * B
            return np.exp(h * self.factor * (term_spm + term_rs)) * B
        if self.ss_on:
            # default_exp_f_with_ss (nonlinearity.py:230-234)
            term_spm = np.abs(A) ** 2
            term_ss = (self.ss_factor / B) * ifft(self.omega * fft(term_spm * A))
            return np.exp(h * self.factor * (term_spm + term_ss)) * B
        # default_exp_f (nonlinearity.py:269-270)
        return np.exp(h * self.factor * np.abs(A) ** 2) * B


class Gain:
    """``Amplifier`` simple saturable gain with Lorentzian profile (amplifier.py:42-158)."""

    def __init__(self, grid, gain_db, E_sat, length, lamb0=None, bandwidth=None):
        self.grid = grid
        self.length = length
        self.E_sat = E_sat
        self.gain_log = math.log(math.pow(10.0, 0.1 * gain_db))
        if bandwidth is not None and lamb0 is not None:
            delta = LIGHT_SPEED_NM_PS * bandwidth / (lamb0 * lamb0)
            prof = 1.0 / (1.0 + 4.0 * (((grid.nu - lambda_to_nu(lamb0)) ** 2) / (delta ** 2)))
        else:
            prof = np.ones(grid.total_samples)
        self.profile = fftshift(prof)

    def factor(self, A, h):
        g0 = (self.gain_log * h) / (2.0 * self.length)
        E = energy(A, self.grid.t)
        return g0 / (1.0 + E / self.E_sat) * self.profile


def yb_cross_sections(grid, path):
    """``Amplifier2LevelModel.interpolate_sigma_s`` (amplifier.py:234-245).

    The table (wavelength m, sigma_12 m^2, sigma_21 m^2, comma separated) is read as
    pandas does with its default header inference: the first line names the columns
    and is not data.  Cubic interpolating splines in (nm, 1e27 sigma), zero outside
    the table, evaluated at the grid's wavelengths (natural order).
    """
    from scipy.interpolate import InterpolatedUnivariateSpline as IUS
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    tab = np.array([[float(x) for x in ln.split(",")] for ln in lines[1:]])
    s12 = IUS(tab[:, 0] * 1e9, tab[:, 1] * 1e27, ext=1)(grid.Lambda) * 1e-27
    s21 = IUS(tab[:, 0] * 1e9, tab[:, 2] * 1e27, ext=1)(grid.Lambda) * 1e-27
    return s12, s21


class YbGain:
    """``Amplifier2LevelModel`` (amplifier.py:178-344): Yb two-level rate-equation gain.

    ``sigma12_s``/``sigma21_s`` are the signal cross sections on the grid (natural
    order, m^2).  Each ``factor`` call sets the inversion from the argument's
    spectral power and advances the pump power (``update_Pp``), as the reference
    does on every linear-operator call.
    """

    H_P = 6.62e-34            # amplifier.py:201-211
    T_LIFE = 850.0e-6         # s
    A_CORE = 3.0e-6           # m
    B_CLAD = 60.0e-6          # m
    NA = 0.13
    LAMBDA_P = 976.0          # nm
    SIGMA12_P = 2.5e-24       # m^2 (amplifier.py:217-218)
    SIGMA21_P = 2.44e-24

    def __init__(self, grid, Pp_0, N, Rr, sigma12_s, sigma21_s):
        a = self.A_CORE
        self.grid = grid
        self.N = N * 1e25 * np.pi * a ** 2
        self.Pp = Pp_0
        self.Tr = 1.0 / Rr
        s12, s21 = np.asarray(sigma12_s, float), np.asarray(sigma21_s, float)
        # rho_s, rho_p (amplifier.py:255-273)
        V = (2.0 * np.pi / grid.Lambda) * a * self.NA * 1e9
        omega_s = a * (0.616 + 1.66 / pow(V, 1.5) + 0.987 / pow(V, 6.0))
        gamma_s = 1.0 - np.exp(-2.0 * a ** 2 / (omega_s * omega_s))
        rho_s = gamma_s / (np.pi * a ** 2)
        rho_p = (a ** 2) / (self.B_CLAD ** 2) / (np.pi * a ** 2)
        with np.errstate(divide="ignore", invalid="ignore"):
            # Psat, eta, alpha, ratio (amplifier.py:275-344)
            self.Psat_s = (self.H_P * grid.nu * 1e12) / (self.T_LIFE * (s12 + s21) * rho_s)
            self.ratio_s = s12 / (s12 + s21)
        sp = self.SIGMA12_P + self.SIGMA21_P
        self.Psat_p = (self.H_P * lambda_to_nu(self.LAMBDA_P) * 1e12) / (self.T_LIFE * sp * rho_p)
        self.eta_s = s12 * rho_s * self.N
        self.eta_p = self.SIGMA12_P * rho_p * self.N
        self.alpha_s = (s12 + s21) * rho_s
        self.alpha_p = sp * rho_p
        self.ratio_p = self.SIGMA12_P / sp

    def calculate_N2(self, Ps):
        """amplifier.py:346-353; terms that are NaN (zero cross sections) are left out."""
        with np.errstate(divide="ignore", invalid="ignore"):
            x = self.ratio_s * Ps / self.Psat_s
            y = Ps / self.Psat_s
        num = self.ratio_p * self.Pp / self.Psat_p + np.sum(x[~np.isnan(x)])
        den = 1 + self.Pp / self.Psat_p + np.sum(y[~np.isnan(y)])
        return (num / den) * self.N

    def factor(self, A, h):
        """amplifier.py:366-379: the spectral power (natural order, like the tables)
        scaled to the average power at the repetition rate; the gain exponent is
        returned in FFT order."""
        N2 = self.calculate_N2(spectral_power(A) * len(A) * self.grid.dt / self.Tr)
        g_s = self.alpha_s * N2 - self.eta_s
        g_p = self.alpha_p * N2 - self.eta_p
        self.Pp = self.Pp * np.exp(g_p * h * 1e3)
        return fftshift(g_s * h * 1e3 / 2)


# ----------------------------------------------------------------------------
# Propagation
# ----------------------------------------------------------------------------
class StepperError(Exception):
    pass


class SmallStepSizeError(StepperError):
    pass


class SuitableStepSizeError(StepperError):
    pass


class MaximumStepsAllocatedError(StepperError):
    pass


# ----------------------------------------------------------------------------
# Explicit solvers and the fixed-step mesh on a generic ODE dA/dz = f(A, z)
# ----------------------------------------------------------------------------
def euler_step(A, z, h, f):
    """``Solver.euler`` (solver.py:93-98)."""
    k0 = h * f(A, z)
    return A + k0


def midpoint_step(A, z, h, f):
    """``Solver.midpoint`` (solver.py:100-106)."""
    k0 = h * f(A, z)
    k1 = h * f(A + 0.5 * k0, z + 0.5 * h)
    return A + k1


def rk4_step(A, z, h, f):
    """``Solver.rk4`` (solver.py:108-116)."""
    k0 = h * f(A, z)
    k1 = h * f(A + 0.5 * k0, z + 0.5 * h)
    k2 = h * f(A + 0.5 * k1, z + 0.5 * h)
    k3 = h * f(A + k2, z + h)
    return A + (k0 + 2.0 * (k1 + k2) + k3) / 6.0


def fixed_steps(step, A, f, length, total_steps):
    """``Stepper.standard_stepper``'s mesh (stepper.py:164-201): h = length / steps and
    z from ``linspace(0, length, steps + 1)``, one step from each z but the last."""
    h = length / total_steps
    for z in np.linspace(0.0, length, total_steps + 1)[:-1]:
        A = step(A, z, h, f)
    return A


class Propagator:
    """RK4IP / ARK4IP propagation through one fibre, restated from the reference.

    ``linear``, ``n`` and ``rk4ip`` follow ``Fibre.linear/n`` and
    ``Solver.rk4ip``; ``standard`` and ``adaptive`` follow the two stepper
    drivers including their trace-storage rules.
    """

    TOTAL_ATTEMPTS = 1000      # stepper.py:129
    STEPS_MAX = 100000         # stepper.py:130
    STEP_SIZE_MIN = 1e-37      # stepper.py:131
    SAFETY, MAX_FACTOR, MIN_FACTOR = 0.9, 10.0, 0.2  # stepper.py:133-135
    ETA = 5                    # solver.py:71
    # Solver.errors (solver.py:57-70): the order used by the adaptive driver per method
    ERRORS = {"rk4ip": 5, "ss_simple": 2, "ss_symmetric": 3, "ss_reduced": 2, "ss_agrawal": 3,
              "ss_sym_midpoint": 3, "ss_sym_rk4": 5}

    def __init__(self, grid, length, beta=None, alpha=None, gamma=0.0, self_steepening=False,
                 use_all=False, tau_1=12.2e-3, tau_2=32.0e-3, f_R=0.18, centre_omega=None,
                 raman_scattering=False, rs_factor=3e-3,
                 small_signal_gain=None, E_sat=None, lamb0=None, bandwidth=None,
                 use_Yb_model=False, Pp_0=None, N=None, Rr=None, yb_cross_sections=None):
        self.grid = grid
        self.length = length
        self.factor = linear_factor(grid, beta, alpha, centre_omega)
        self.nl = Nonlinear(grid, gamma, self_steepening, use_all, tau_1, tau_2, f_R,
                            raman_scattering, rs_factor)
        self.gain = None
        if use_Yb_model:  # fibre.py:97-103: the Yb model replaces the saturable amplifier
            s12, s21 = yb_cross_sections
            self.gain = YbGain(grid, Pp_0, N, Rr, s12, s21)
        elif small_signal_gain is not None and E_sat is not None:
            self.gain = Gain(grid, small_signal_gain, E_sat, length, lamb0, bandwidth)
        self.fft_count = 0
        self.evals = 0

    def linear(self, A, h):
        """``Linearity.default_exp_f`` (linearity.py:241-256)."""
        hf = self.factor * h
        if self.gain is None:
            return ifft(np.exp(hf) * fft(A))
        amp = self.gain.factor(A, h)
        return ifft(np.multiply(np.exp(amp), np.exp(hf) * fft(A)))

    def n(self, A):
        return self.nl(A)

    def rk4ip(self, A, h):
        """``Solver.rk4ip`` (solver.py:339-354)."""
        self.evals += 1
        hh = 0.5 * h
        A_I = self.linear(A, hh)
        k0 = self.linear(h * self.n(A), hh)
        k1 = h * self.n(A_I + 0.5 * k0)
        k2 = h * self.n(A_I + 0.5 * k1)
        k3 = h * self.n(self.linear(A_I + k2, hh))
        return (k3 / 6.0) + self.linear(A_I + (k0 + 2.0 * (k1 + k2)) / 6.0, hh)

    @staticmethod
    def rk4(A, h, f):
        """``Solver.rk4`` (solver.py:109-116) for an autonomous f (``rk4_step``)."""
        return rk4_step(A, 0.0, h, lambda x, z: f(x))

    def ss_symmetric(self, A, h):
        """``Solver.ss_symmetric`` (solver.py:267-275): linear half step, exponential
        nonlinear step evaluated with the unpropagated field, linear half step."""
        self.evals += 1
        A_L = self.linear(A, 0.5 * h)
        A_N = self.nl.exp_non(A, h, A_L)
        return self.linear(A_N, 0.5 * h)

    def ss_simple(self, A, h):
        """``Solver.ss_simple`` (solver.py:256-265): exponential nonlinear step with the
        field itself, then a full linear step."""
        self.evals += 1
        A_N = self.nl.exp_non(A, h, A)
        return self.linear(A_N, h)

    def ss_reduced(self, A, h):
        """``Solver.ss_reduced`` (solver.py:277-287): linear half step, exponential
        nonlinear step with the propagated field, linear half step."""
        self.evals += 1
        A_L = self.linear(A, 0.5 * h)
        A_N = self.nl.exp_non(A_L, h, A_L)
        return self.linear(A_N, 0.5 * h)

    def ss_agrawal(self, A, h):
        """``Solver.ss_agrawal`` (solver.py:290-320): iterated symmetric split step with the
        nonlinear exponent averaged over the step's ends, N(Y)/Y taken as 0 where
        |Y| <= 1e-5."""
        self.evals += 1

        def ratio(Y):
            with np.errstate(divide="ignore", invalid="ignore"):
                return np.where(np.abs(Y) > 1.0e-5, self.n(Y) / Y, 0.0)

        A_L = self.linear(A, 0.5 * h)
        r_A = ratio(A)
        A_N1 = np.exp(0.5 * h * (ratio(A) + r_A)) * A_L
        Y_1 = self.linear(A_N1, 0.5 * h)
        A_N2 = np.exp(0.5 * h * (ratio(Y_1) + r_A)) * A_L
        return self.linear(A_N2, 0.5 * h)

    def ss_sym_midpoint(self, A, h):
        """``Solver.ss_sym_midpoint`` (solver.py:323-328) with ``Solver.midpoint``
        (solver.py:101-106) on the nonlinear term."""
        self.evals += 1
        A_L = self.linear(A, 0.5 * h)
        A_N = midpoint_step(A_L, 0.0, h, lambda x, z: self.n(x))
        return self.linear(A_N, 0.5 * h)

    def ss_sym_rk4(self, A, h):
        """``Solver.ss_sym_rk4`` (solver.py:330-337): linear half step, classical RK4 on
        the nonlinear term, linear half step."""
        self.evals += 1
        A_L = self.linear(A, 0.5 * h)
        A_N = self.rk4(A_L, h, self.n)
        return self.linear(A_N, 0.5 * h)

    # -- fixed step (stepper.py:164-221) --------------------------------------
    def standard(self, A, total_steps, traces=1, method="rk4ip"):
        h = self.length / total_steps
        zs = np.linspace(0.0, self.length, total_steps + 1)
        storage_step = int(total_steps / traces)
        trace_z, trace_A = [], []
        step = self.step_function(method)
        for i, z in enumerate(zs[:-1]):
            A = step(A, h)
            if traces != 1 and i % storage_step == 0:
                trace_z.append(z + h)
                trace_A.append(A)
        return A, dict(trace_z=trace_z, trace_A=trace_A, h=h, steps=total_steps)

    # -- adaptive (stepper.py:231-376) ----------------------------------------
    @staticmethod
    def relative_local_error(A_fine, A_coarse):
        if np.isnan(A_fine).any() or np.isinf(A_fine).any():
            return 1.0
        norm_fine = _linalg.norm(A_fine)
        if norm_fine != 0.0:
            return _linalg.norm(A_fine - A_coarse) / norm_fine
        return _linalg.norm(A_fine - A_coarse)

    def initial_step(self, total_steps, traces):
        h = self.length / traces if traces > total_steps else self.length / total_steps
        return 1e-6 if h > 1e-6 else h

    def step_function(self, method):
        return {"rk4ip": self.rk4ip, "ss_sym_rk4": self.ss_sym_rk4, "ss_symmetric": self.ss_symmetric,
                "ss_simple": self.ss_simple, "ss_reduced": self.ss_reduced,
                "ss_sym_midpoint": self.ss_sym_midpoint, "ss_agrawal": self.ss_agrawal}[method]

    def adaptive(self, A, local_error=1e-6, total_steps=100, traces=1, max_attempts=None,
                 replay=None, method="rk4ip"):
        """Step doubling with local extrapolation.

        ``max_attempts`` bounds the total number of attempts (a CPU-time cap used
        for sampling; the run then returns with ``finished=False``).  ``replay``
        is a list of accepted step sizes to follow instead of the controller.
        """
        z = 0.0
        h = self.initial_step(total_steps, traces)
        step_storage = self.length / traces
        z_ignore = step_storage
        step = self.step_function(method)
        eta = self.ERRORS[method]  # stepper.py:143
        f_eta = np.power(2, eta - 1.0)
        f_alpha = f_eta / (f_eta - 1.0)
        f_beta = 1.0 / (f_eta - 1.0)
        trace_z, trace_A, steps = [], [], []
        if traces != 1:
            trace_z.append(z)
            trace_A.append(A)
        attempts = rejected = 0
        if replay is not None:
            for h_acc in replay:
                A_half = step(A, 0.5 * h_acc)
                A_fine = step(A_half, 0.5 * h_acc)
                A_coarse = step(A, h_acc)
                A = f_alpha * A_fine - f_beta * A_coarse
                z += h_acc
                steps.append((z, h_acc))
            return A, dict(z=z, steps=steps, attempts=len(replay), rejected=0,
                           trace_z=trace_z, trace_A=trace_A, finished=True)
        for _s in range(1, self.STEPS_MAX):
            if (z + h) > self.length:
                h = self.length - z
            for _ta in range(0, self.TOTAL_ATTEMPTS):
                if max_attempts is not None and attempts >= max_attempts:
                    return A, dict(z=z, steps=steps, attempts=attempts, rejected=rejected,
                                   trace_z=trace_z, trace_A=trace_A, finished=False, h=h)
                attempts += 1
                h_half = 0.5 * h
                A_half = step(A, h_half)
                A_fine = step(A_half, h_half)
                A_coarse = step(A, h)
                delta = self.relative_local_error(A_fine, A_coarse)
                h_temp = h
                if delta > 0.0:
                    error_ratio = local_error / delta
                    factor = self.SAFETY * np.power(error_ratio, 1.0 / eta)
                    h = h_temp * min(self.MAX_FACTOR, max(self.MIN_FACTOR, factor))
                else:
                    h = h_temp * self.MAX_FACTOR
                if delta < 2.0 * local_error:
                    z += h_temp
                    A = f_alpha * A_fine - f_beta * A_coarse
                    steps.append((z, h_temp))
                    if z > z_ignore:
                        trace_z.append(z)
                        trace_A.append(A)
                        z_ignore += step_storage
                    break
                rejected += 1
                if h < self.STEP_SIZE_MIN:
                    raise SmallStepSizeError("Step size is extremely small")
            else:
                raise SuitableStepSizeError("Failed to set suitable step-size")
            if z >= self.length:
                return A, dict(z=z, steps=steps, attempts=attempts, rejected=rejected,
                               trace_z=trace_z, trace_A=trace_A, finished=True, h=h)
        raise MaximumStepsAllocatedError("Failed to complete with maximum steps allocated")


# ----------------------------------------------------------------------------
# Items with no reference counterpart (parity unpinned; restated from the
# literature and used as the CPU check of the GPU implementations).
# ----------------------------------------------------------------------------
def one_photon_noise(grid, rng):
    """One photon per spectral mode with uniform random phase, temporal field.

    A spectral bin k holding one photon of energy h nu_k over the window T has
    |A_k|^2 T = h nu_k in the pyofss normalisation (energy = T sum |A_k|^2), so
    A_k = sqrt(h nu_k / T) e^{i phi_k}, phi_k ~ U[0, 2 pi).
    """
    nu = fftshift(grid.nu)
    amp = np.sqrt(PLANCK_W_PS2 * nu / grid.window_t)
    phi = rng.uniform(0.0, 2.0 * np.pi, grid.total_samples)
    return ifft(amp * np.exp(1j * phi))


def photon_number(a_t, grid):
    """sum_k |A_k|^2 T / (h nu_k) in FFT order (conserved by the lossless GNLSE)."""
    spec = np.abs(fft(a_t)) ** 2
    nu = fftshift(grid.nu)
    return float(np.sum(spec * grid.window_t / (PLANCK_W_PS2 * nu)))


def coherence_g12(spectra):
    """|g12| over an ensemble of spectra (rows): |<A_i* A_j>_{i!=j}| / <|A|^2>.

    Uses sum_{i!=j} A_i* A_j = |sum A_i|^2 - sum |A_i|^2 (O(n) in the members).
    """
    s = np.sum(spectra, axis=0)
    p = np.sum(np.abs(spectra) ** 2, axis=0)
    n = spectra.shape[0]
    num = np.abs(np.abs(s) ** 2 - p) / (n * (n - 1))
    den = p / n
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(den > 0, num / den, 0.0)
