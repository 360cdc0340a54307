"""Host helpers around the propagation path (CPU, no GPU): the chirp applied to the 2^16
amplifier input, the ensemble coherence sums, the common-frequency spectra of a ragged
ensemble, and the stepper exception classes raised by ``Fibre``."""

import math
import sys
import types

import numpy as np
import pytest

from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, Gaussian
from pyofsschanged_gb300 import ensemble as ens
from pyofsschanged_gb300 import fibre as fib
from pyofsschanged_gb300.amplifier import amplifier_input
from pyofsschanged_gb300.field import spectral_phase


def test_spectral_phase_is_the_reference_dispersion_step():
    """exp(i gdd/2 (w - w0)^2) in the spectral domain is the linear step of a fibre with
    beta_2 L = gdd (Linearity.default_linearity / default_exp_f, linearity.py:162-186,
    241-256, restated by the oracle)."""
    d = Domain(bit_width=40.0, samples_per_bit=1024, centre_nu=299792.458 / 1030.0)
    a0 = Gaussian(peak_power=10.0, width=1.0, using_fwhm=True)(d, np.zeros(1024, complex))
    beta2, length = 25.0, 0.012  # ps^2/km, km
    grid = go.Grid(bit_width=40.0, samples_per_bit=1024, centre_nu=299792.458 / 1030.0)
    want = go.Propagator(grid, length, beta=[0.0, 0.0, beta2]).linear(a0, length)
    got = spectral_phase(a0, d, beta2 * length)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.abs(want).max())


def test_spectral_phase_composes_and_keeps_energy():
    d = Domain(bit_width=40.0, samples_per_bit=2048, centre_nu=193.1)
    rng = np.random.default_rng(3)
    a = rng.standard_normal(2048) + 1j * rng.standard_normal(2048)
    b = spectral_phase(spectral_phase(a, d, 0.7), d, -0.2)
    np.testing.assert_allclose(b, spectral_phase(a, d, 0.5), rtol=0, atol=1e-12 * np.abs(a).max())
    np.testing.assert_allclose(np.sum(np.abs(b) ** 2), np.sum(np.abs(a) ** 2), rtol=1e-12)
    np.testing.assert_allclose(spectral_phase(a, d, 0.0), a, rtol=0, atol=1e-13 * np.abs(a).max())


def test_amplifier_input_is_the_chirped_gaussian():
    """1 ps FWHM Gaussian, 100 W, 2 ps^2 of group-delay dispersion: the field stays
    Gaussian with 1/e half width T1 = T0 sqrt(1 + (gdd / T0^2)^2) and peak P0 T0 / T1."""
    d, a = amplifier_input()
    assert len(a) == 65536
    t0 = 1.0 / (2.0 * math.sqrt(math.log(2.0)))
    t1 = t0 * math.sqrt(1.0 + (2.0 / t0 ** 2) ** 2)
    p = np.abs(a) ** 2
    np.testing.assert_allclose(p.max(), 100.0 * t0 / t1, rtol=1e-6)
    # energy P0 T0 sqrt(pi) is unchanged by the phase (pJ)
    np.testing.assert_allclose(np.sum(p) * d.dt, 100.0 * t0 * math.sqrt(math.pi), rtol=1e-9)
    half = np.flatnonzero(p >= 0.5 * p.max())
    fwhm = (half[-1] - half[0]) * d.dt
    np.testing.assert_allclose(fwhm, 2.0 * math.sqrt(math.log(2.0)) * t1, rtol=2e-3)


def _pair_average(spectra):
    n = spectra.shape[0]
    acc = np.zeros(spectra.shape[1], complex)
    for i in range(n):
        for j in range(n):
            if i != j:
                acc += np.conj(spectra[i]) * spectra[j]
    return np.abs(acc / (n * (n - 1))) / np.mean(np.abs(spectra) ** 2, axis=0)


def test_coherence_g12_is_the_pair_average():
    rng = np.random.default_rng(7)
    base = rng.standard_normal(33) + 1j * rng.standard_normal(33)
    spectra = base + 0.4 * (rng.standard_normal((7, 33)) + 1j * rng.standard_normal((7, 33)))
    np.testing.assert_allclose(ens.coherence_g12(spectra), _pair_average(spectra), rtol=1e-12)
    # identical members are fully coherent; an all-zero bin reports 0
    same = np.repeat(base[None, :], 5, axis=0)
    same[:, 4] = 0.0
    g = ens.coherence_g12(same)
    np.testing.assert_allclose(np.delete(g, 4), 1.0, rtol=1e-12)
    assert g[4] == 0.0


def test_coherence_partial_sums_over_shards():
    """The shards' sums (one of them empty) give the whole ensemble's |g12|."""
    rng = np.random.default_rng(11)
    spectra = rng.standard_normal((9, 17)) + 1j * rng.standard_normal((9, 17))
    parts = [ens.coherence_partial(spectra[:4]), ens.coherence_partial(spectra[4:4], n_bins=17),
             ens.coherence_partial(spectra[4:])]
    s = sum(p[0] for p in parts)
    pw = sum(p[1] for p in parts)
    n = sum(p[2] for p in parts)
    assert n == 9 and parts[1][2] == 0
    np.testing.assert_allclose(ens.coherence_from_sums(s, pw, n), ens.coherence_g12(spectra), rtol=1e-12)
    with pytest.raises(ValueError):
        ens.coherence_partial(spectra[:0])


def test_common_spectra_compare_grids_bin_by_bin():
    """A pulse inside both windows of two grids with a common dt has the same spectrum on
    the coarse grid's frequency points (every second point of the finer spectrum)."""
    dt = 12.5 / 8192
    fields = []
    for n in (4096, 8192):
        d = Domain(bit_width=n * dt, samples_per_bit=n, centre_nu=299792.458 / 835.0)
        fields.append(Gaussian(peak_power=1.0e3, width=0.05, using_fwhm=True)(d, np.zeros(n, complex)))
    sp = ens.common_spectra(fields, sizes_min=4096)
    assert sp.shape == (2, 4096)
    np.testing.assert_allclose(sp[1], sp[0], rtol=0, atol=1e-9 * np.abs(sp[0]).max())
    # the time origin at index 0: a pulse centred at t = 0 has a real, even spectrum
    np.testing.assert_allclose(sp[0].imag, 0.0, atol=1e-12 * np.abs(sp[0]).max())
    # and the two grids' members are mutually coherent bin by bin
    np.testing.assert_allclose(ens.coherence_g12(sp)[np.abs(sp[0]) > 1e-3 * np.abs(sp[0]).max()], 1.0,
                               rtol=1e-9)


def test_stepper_exceptions_derive_from_pyofss_classes(monkeypatch):
    """With pyofss's stepper module loaded, Fibre's stepper errors are also instances of
    pyofss's own classes (pyofss/modules/stepper.py:33-47), so either except clause
    catches them; without it they are this package's classes."""
    monkeypatch.delitem(sys.modules, "pyofss.modules.stepper", raising=False)
    assert fib.stepper_exception(fib.SmallStepSizeError) is fib.SmallStepSizeError

    ref = types.ModuleType("pyofss.modules.stepper")

    class StepperError(Exception):
        pass

    class SmallStepSizeError(StepperError):
        pass

    ref.StepperError, ref.SmallStepSizeError = StepperError, SmallStepSizeError
    monkeypatch.setitem(sys.modules, "pyofss.modules.stepper", ref)
    cls = fib.stepper_exception(fib.SmallStepSizeError)
    assert issubclass(cls, fib.SmallStepSizeError) and issubclass(cls, SmallStepSizeError)
    assert fib.stepper_exception(fib.SmallStepSizeError) is cls  # one class per pair
    with pytest.raises(SmallStepSizeError, match="extremely small"):
        fib.raise_for_status(fib.nat.GNLSE_SMALL_STEP)
    # a name pyofss does not define stays this package's class
    assert fib.stepper_exception(fib.MaximumStepsAllocatedError) is fib.MaximumStepsAllocatedError
