"""The large-grid fibre amplifier on the engine against the FP64 oracle.

2^16 points over a 100 ps window at 1030 nm; a 1 ps (FWHM) Gaussian of 100 W peak power
with a linear chirp of 2 ps^2 group-delay dispersion (field.spectral_phase); 3 m of fibre
with saturable gain (39.09 dB small-signal gain, E_sat = 5 nJ, 40 nm Lorentzian gain
bandwidth, the reference's Amplifier, pyofss/modules/amplifier.py:110-158, applied in
every linear-operator call as in linearity.py:241-256), beta_2 = 0.025 ps^2/m,
beta_3 = 5e-5 ps^3/m, gamma = 0.005 /W/m, Blow-Wood Raman and self-steepening.

The fp64 and df plans run it on a 16-CTA cluster of 4096-point slices (a non-portable
cluster: 16 SMs exchange through distributed shared memory), the mixed plan on an
8-CTA cluster of 8192-point complex64 slices.  A fixed-step segment and the full
adaptive run are checked against the oracle; the benchmark times the full run.
"""

import os

import numpy as np
import pytest

from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import GridTables, Instance, Plan
from pyofsschanged_gb300.amplifier import FIBRE, LAMBDA_NM, LENGTH_KM, N, amplifier_input
from pyofsschanged_gb300.pulses import Gaussian

pytestmark = pytest.mark.gpu

LENGTH = LENGTH_KM


def test_chirp_is_a_spectral_phase():
    d, a = amplifier_input()
    _, a0 = d, Gaussian(peak_power=100.0, width=1.0, using_fwhm=True)(d, np.zeros(N, complex))
    # same spectrum magnitude, broadened in time, the phase 2 ps^2 / 2 dw^2 around w0
    np.testing.assert_allclose(np.abs(go.fft(a)), np.abs(go.fft(a0)), rtol=0, atol=1e-12 * np.abs(go.fft(a0)).max())
    assert np.abs(a).max() ** 2 < 0.5 * 100.0


@pytest.mark.parametrize("precision,cluster,tol", [("fp64", 16, 1e-9), ("df", 16, 1e-9), ("mixed", 8, 1e-4)])
def test_fixed_step_segment_matches_oracle(cuda_ready, precision, cluster, tol):
    """The first 3 cm of the amplifier (its small-signal gain per length: 39.09 dB x 1/100
    over 3 cm) in 20 fixed RK4IP steps, against the oracle."""
    d, a0 = amplifier_input()
    steps, seg = 20, LENGTH / 100.0
    fibre = dict(FIBRE, small_signal_gain=FIBRE["small_signal_gain"] / 100.0)
    grid = go.Grid(bit_width=100.0, samples_per_bit=N, centre_nu=299792.458 / LAMBDA_NM)
    want, _ = go.Propagator(grid, seg, **fibre).standard(a0.copy(), steps)
    g = GridTables(d, length=seg, cluster=cluster, **fibre)
    plan = Plan([g], [Instance(0, method="rk4ip", length=seg, total_steps=steps)], precision=precision)
    assert plan.class_times()[0][1] == cluster
    f = plan.pack([a0])
    plan.propagate(f)
    st = plan.stats()[0]
    got = plan.unpack(f)[0].cpu().numpy().astype(complex)
    assert st["status"] == 0 and st["evals"] == steps
    err = np.linalg.norm(go.fft(got) - go.fft(want)) / np.linalg.norm(go.fft(want))
    assert err <= tol, err
    assert st["energy_out"] > st["energy_in"]


@pytest.mark.parametrize("precision,cluster,tol", [("fp64", 16, 1e-9), ("df", 16, 1e-9), ("mixed", 8, 1e-4)])
def test_full_amplifier_matches_oracle(cuda_ready, precision, cluster, tol):
    """The whole 3 m adaptive run (ARK4IP 1e-6) against the oracle's output
    (tests/golden/make_amplifier_2e16.py keeps every 64th time sample and spectral bin):
    fp64 and df take the oracle's 1489 attempts and match it within 1e-9."""
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "amplifier_2e16.npz"))
    stride = int(ref["stride"])
    d, a0 = amplifier_input()
    g = GridTables(d, length=LENGTH, cluster=cluster, **FIBRE)
    plan = Plan([g], [Instance(0, method="ark4ip", length=LENGTH, local_error=1e-6)], precision=precision)
    f = plan.pack([a0])
    plan.propagate(f)
    st = plan.stats()[0]
    got = plan.unpack(f)[0].cpu().numpy().astype(complex)
    assert st["status"] == 0
    if precision != "mixed":
        assert st["attempts"] == int(ref["attempts"]) and st["evals"] == int(ref["evals"])
    for mine, want in ((got[::stride], ref["out_samples"]), (go.fft(got)[::stride], ref["spec_samples"])):
        err = np.linalg.norm(mine - want) / np.linalg.norm(want)
        assert err <= tol, err
    assert st["energy_out"] == pytest.approx(float(ref["energy"]), rel=max(10 * tol, 1e-9))
