"""GB300-native GNLSE propagation engine with the pyofss System/Fibre/Domain API.

The propagation path (RK4IP / ARK4IP through a fibre with dispersion, loss,
SPM, self-steepening, Raman and saturable gain) runs as fused CUDA kernels for
sm_103a in ``libgnlse.so``, reached through the C ABI in ``include/gnlse.h``.
Everything in this package around it is host glue: grids, pulses, operator
tables, the module protocol and the batched-ensemble driver.
"""

from .domain import (Domain, dlambda_to_dnu, dnu_to_dlambda, lambda_to_nu, lambda_to_omega,
                     nu_to_lambda, nu_to_omega, omega_to_lambda, omega_to_nu)
from .engine import Instance, Plan
from .fibre import (Fibre, MaximumStepsAllocatedError, SmallStepSizeError, StepperError,
                    SuitableStepSizeError)
from .field import energy, fft, fftshift, ifft, ifftshift, spectral_power, temporal_power
from .operators import GridTables
from .pulses import Gaussian, Sech
from .system import System, field_load, field_save

__all__ = [
    "Domain", "System", "Fibre", "Sech", "Gaussian", "Plan", "Instance", "GridTables",
    "fft", "ifft", "fftshift", "ifftshift", "temporal_power", "spectral_power", "energy",
    "lambda_to_nu", "nu_to_lambda", "nu_to_omega", "omega_to_nu", "lambda_to_omega",
    "omega_to_lambda", "dnu_to_dlambda", "dlambda_to_dnu", "field_save", "field_load",
    "StepperError", "SmallStepSizeError", "SuitableStepSizeError", "MaximumStepsAllocatedError",
]
