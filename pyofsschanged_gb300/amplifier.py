"""The large-grid fibre amplifier workload: 2^16 points, saturable gain, 3 m.

2^16 points over a 100 ps window centred at 1030 nm; the input is a 1 ps (FWHM)
Gaussian of 100 W peak power with a linear chirp of 2 ps^2 group-delay dispersion
(applied as a quadratic spectral phase, field.spectral_phase); the fibre is 3 m with
saturable gain g0 = 3 /m (39.09 dB small-signal gain over the length), E_sat = 5 nJ and
a 40 nm FWHM Lorentzian gain bandwidth (pyofss/modules/amplifier.py:110-158), beta_2 =
0.025 ps^2/m, beta_3 = 5e-5 ps^3/m, gamma = 0.005 /W/m, Blow-Wood Raman and
self-steepening, in the reference's units (km, ps^k/km, 1/(W km)).
"""

import numpy as np

from .domain import Domain
from .field import spectral_phase
from .pulses import Gaussian

LAMBDA_NM = 1030.0
N = 65536
LENGTH_KM = 3e-3
FIBRE = dict(beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0, self_steepening=True, use_all="blowwood",
             small_signal_gain=39.09, E_sat=5.0, lamb0=LAMBDA_NM, bandwidth=40.0)


def amplifier_input():
    """(Domain, chirped input field) of the workload."""
    d = Domain(bit_width=100.0, samples_per_bit=N, centre_nu=299792.458 / LAMBDA_NM)
    a0 = Gaussian(peak_power=100.0, width=1.0, using_fwhm=True)(d, np.zeros(N, complex))
    return d, spectral_phase(a0, d, 2.0)
