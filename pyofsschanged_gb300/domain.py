"""Time / frequency grid with the pyofss ``Domain`` interface.

Same constructor, attributes and range checks as ``pyofss.domain.Domain``
(pyofss/domain.py:142-299): ``t`` spans [-T/2, T/2) with ``T = total_bits *
bit_width``; ``nu`` spans [centre_nu - 1/(2 dt), centre_nu + 1/(2 dt)) in
consecutive order; ``omega = 2 pi nu``; ``Lambda = c / nu`` with c in nm/ps.
The grid is host data: the engine receives the tables built from it.
"""

import math

import numpy as np

LIGHT_SPEED = 1.0e-3 * 299792458.0  # nm / ps


class DomainError(Exception):
    pass


class OutOfRangeError(DomainError):
    pass


class NotIntegerError(DomainError):
    pass


def nu_to_omega(nu):
    return 2.0 * math.pi * nu


def nu_to_lambda(nu):
    return LIGHT_SPEED / nu


def omega_to_nu(omega):
    return omega / (2.0 * math.pi)


def omega_to_lambda(omega):
    return 2.0 * math.pi * LIGHT_SPEED / omega


def lambda_to_nu(lam):
    return LIGHT_SPEED / lam


def lambda_to_omega(lam):
    return 2.0 * math.pi * LIGHT_SPEED / lam


def dnu_to_dlambda(dnu, nu):
    return LIGHT_SPEED * dnu / (nu * nu)


def dlambda_to_dnu(dlam, lam):
    return LIGHT_SPEED * dlam / (lam * lam)


class Domain:
    vacuum_light_speed = LIGHT_SPEED

    def __init__(self, total_bits=1, samples_per_bit=512, bit_width=100.0, centre_nu=193.1,
                 channels=1):
        checks = [
            (0 < total_bits < 4096, "total_bits is out of range. Must be in (0, 4096)"),
            (0 < samples_per_bit < 262144, "samples_per_bit is out of range. Must be in (0, 262144)"),
            (0.01 < bit_width < 10000.0, "bit_width is out of range. Must be in (0.01, 10000.0)"),
            (140.0 < centre_nu < 600.0, "centre_nu is out of range. Must be in (140.0, 600.0)"),
            (0 < channels < 3, "channels is out of range. Must be in (0, 3)"),
        ]
        for ok, msg in checks:
            if not ok:
                raise OutOfRangeError(msg)
        for v, name in ((total_bits, "total_bits"), (samples_per_bit, "samples_per_bit"),
                        (channels, "channels")):
            if int(v) != v:
                raise NotIntegerError(f"{name} must be an integer")
        self.total_bits = total_bits
        self.samples_per_bit = samples_per_bit
        self.bit_width = bit_width
        self.centre_nu = centre_nu
        self.channels = channels
        self.total_samples = total_bits * samples_per_bit
        self.window_t = total_bits * bit_width
        self.centre_omega = 2.0 * math.pi * centre_nu
        self.centre_lambda = LIGHT_SPEED / centre_nu
        self.t, self.dt = np.linspace(-self.window_t / 2.0, self.window_t / 2.0,
                                      self.total_samples, False, True)
        self.window_nu = 1.0 / self.dt
        nu_lo = centre_nu - 0.5 * self.window_nu
        self.nu, self.dnu = np.linspace(nu_lo, nu_lo + self.window_nu, self.total_samples,
                                        False, True)
        self.omega = 2.0 * math.pi * self.nu
        self.domega = 2.0 * math.pi * self.dnu
        self.window_omega = 2.0 * math.pi * self.window_nu
        self.Lambda = LIGHT_SPEED / self.nu
        self.dlambda = LIGHT_SPEED * self.dnu / (centre_nu ** 2)
        self.window_lambda = LIGHT_SPEED * self.window_nu / (centre_nu ** 2)

    def __eq__(self, other):
        return (isinstance(other, Domain) and other.total_bits == self.total_bits
                and other.samples_per_bit == self.samples_per_bit
                and other.bit_width == self.bit_width and other.centre_nu == self.centre_nu
                and other.channels == self.channels)

    def __hash__(self):
        return hash((self.total_bits, self.samples_per_bit, self.bit_width, self.centre_nu,
                     self.channels))

    def __str__(self):
        return (f"Domain:\n\ttotal_bits = {self.total_bits:d}\n\tsamples_per_bit = "
                f"{self.samples_per_bit:d}\n\tbit_width = {self.bit_width:.4f} ps\n\t"
                f"centre_nu = {self.centre_nu:.4f} THz\n\ttotal_samples = "
                f"{self.total_samples:d}\n\twindow_t = {self.window_t:.4f} ps\n\tdt = "
                f"{self.dt:.4f} ps\n\twindow_nu = {self.window_nu:.4f} THz")
