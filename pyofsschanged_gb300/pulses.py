"""Input pulse generators with the pyofss ``Sech`` / ``Gaussian`` interface.

``Sech`` follows pyofss/modules/sech.py:44-168 and ``Gaussian`` follows
pyofss/modules/gaussian.py:44-170: the width is a half width at 1/e of the
maximum unless ``using_fwhm`` converts it (sech: 0.5/ln(1+sqrt 2); Gaussian:
0.5/ln(2)^(1/2m)); the phase is initial_phase - 2 pi offset_nu t - C/2 (t/T0)^(2m).
Calling a pulse module adds the pulse to the field, as a pyofss module does.
"""

import math

import numpy as np


class PulseError(Exception):
    pass


class OutOfRangeError(PulseError):
    pass


class NotIntegerError(PulseError):
    pass


class _Pulse:
    offset_range = 200.0

    def _check(self, position, width, peak_power, offset_nu, C, initial_phase, channel):
        if not (-0.5 <= position <= 0.5):
            raise OutOfRangeError("position is out of range. Must be in [-0.5, 0.5]")
        if not (1e-3 < width < 1e3):
            raise OutOfRangeError("width is out of range. Must be in (1e-3, 1e3)")
        if not (0.0 <= peak_power < 1e9):
            raise OutOfRangeError("peak_power is out of range. Must be in [0.0, 1e9)")
        r = self.offset_range
        if not (-r < offset_nu < r):
            raise OutOfRangeError(f"offset_nu is out of range. Must be in ({-r}, {r})")
        if not (-1e3 < C < 1e3):
            raise OutOfRangeError("C is out of range. Must be in (-1e3, 1e3)")
        if not (0.0 <= initial_phase < 2.0 * math.pi):
            raise OutOfRangeError("initial_phase is out of range. Must be in [0.0, 2.0 * pi)")
        if not (0 <= channel < 2):
            raise OutOfRangeError("channel is out of range. Must be in [0, 2)")
        if int(channel) != channel:
            raise NotIntegerError("channel must be an integer")

    def _profile(self, t_norm):
        raise NotImplementedError

    def _field(self, t, t_span):
        t_norm = (t - self.position * t_span) / self.width
        shape, time = self._profile(t_norm)
        ph = self.initial_phase - (2.0 * math.pi * self.offset_nu * t + 0.5 * self.C * time)
        return shape * np.exp(1j * ph)

    def __call__(self, domain, field):
        add = self._field(domain.t, domain.window_t)
        if domain.channels > 1:
            field[self.channel] += add
        else:
            field += add
        self.field = field
        return field

    def generate(self, t):
        if len(t) < 8:
            raise OutOfRangeError("Require temporal array with at least 8 values")
        return self._field(t, t[-1] - t[0] + (t[1] - t[0]))


class Sech(_Pulse):
    def __init__(self, name="sech", position=0.0, width=10.0, peak_power=1e-3, offset_nu=0.0,
                 m=0, C=0.0, initial_phase=0.0, channel=0, using_fwhm=False):
        self._check(position, width, peak_power, offset_nu, C, initial_phase, channel)
        self.name, self.position, self.width = name, position, width
        self.peak_power, self.offset_nu, self.C = peak_power, offset_nu, C
        self.initial_phase, self.channel, self.fwhm, self.field = initial_phase, channel, None, None
        if using_fwhm:
            self.fwhm = width
            self.width = width * (0.5 / math.log(1.0 + math.sqrt(2.0)))

    def calculate_fwhm(self):
        return self.fwhm if self.fwhm is not None else self.width * 2.0 * math.log(1.0 + math.sqrt(2.0))

    def _profile(self, t_norm):
        return math.sqrt(self.peak_power) / np.cosh(t_norm), t_norm * t_norm


class Gaussian(_Pulse):
    offset_range = 300.0

    def __init__(self, name="gaussian", position=0.0, width=10.0, peak_power=1e-3, offset_nu=0.0,
                 m=1, C=0.0, initial_phase=0.0, channel=0, using_fwhm=False):
        self._check(position, width, peak_power, offset_nu, C, initial_phase, channel)
        if not (0 < m < 50):
            raise OutOfRangeError("m is out of range. Must be in (0, 50)")
        if int(m) != m:
            raise NotIntegerError("m must be an integer")
        self.name, self.position, self.width, self.m = name, position, width, m
        self.peak_power, self.offset_nu, self.C = peak_power, offset_nu, C
        self.initial_phase, self.channel, self.fwhm, self.field = initial_phase, channel, None, None
        if using_fwhm:
            self.fwhm = width
            self.width = width * (0.5 / np.power(math.log(2.0), 1.0 / (2 * m)))

    def calculate_fwhm(self):
        if self.fwhm is not None:
            return self.fwhm
        return self.width * 2.0 * math.pow(math.log(2.0), 1.0 / (2 * self.m))

    def _profile(self, t_norm):
        # numpy.lib.scimath.power semantics, as in the reference: a grid with
        # negative entries is promoted to complex before raising to 2m.
        base = t_norm.astype(complex) if np.any(t_norm < 0) else t_norm
        time = np.power(base, 2 * self.m)
        return math.sqrt(self.peak_power) * np.exp(-0.5 * time), time
