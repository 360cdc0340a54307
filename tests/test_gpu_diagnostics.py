"""The engine's FP64 energy and photon-number diagnostics (gnlse_stats energy_* /
photons_*), through the C ABI.

Both are Parseval sums over the spectral state, E = T sum_k |A_k|^2 (nJ) and
N_ph = T sum_k |A_k|^2 / (h nu_k) (no reference counterpart; pyofss computes energy by
Simpson's rule in time, pyofss/field.py:161-172).  Checked against numpy on the input
and on the oracle's output, and as conservation laws: without loss, gain or Raman the
GNLSE conserves energy, and with Raman and self-steepening it conserves the photon
number but not the energy."""

import numpy as np
import pytest

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, GridTables, Instance, Plan

pytestmark = pytest.mark.gpu


def parseval(a, d, nu):
    s = np.abs(go.fft(a)) ** 2
    return d.window_t * s.sum() * 1e-3, d.window_t * np.sum(s / (go.PLANCK_W_PS2 * nu))


def run(name, precision):
    case = gc.load(name)
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    method = fk.pop("method")
    steps = fk.pop("total_steps", 100)
    fk.pop("traces", None)
    tol = fk.pop("local_error", 1e-6)
    g = GridTables(d, **fk)
    plan = Plan([g], [Instance(0, method=method, length=fk["length"], local_error=tol,
                               total_steps=steps)], precision=precision)
    f = plan.pack([case["A0"]])
    plan.propagate(f)
    return case, d, g, plan.stats()[0], plan.unpack(f)[0].cpu().numpy().astype(complex)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
@pytest.mark.parametrize("name", ["soliton_n2_1024", "sc_blowwood_ark4ip_1024", "gain_ark4ip_1024"])
def test_diagnostics_match_numpy(cuda_ready, name, precision, tol):
    case, d, g, st, out = run(name, precision)
    assert st["status"] == 0
    e_in, n_in = parseval(case["A0"], d, g.nu)
    e_out, n_out = parseval(out, d, g.nu)
    assert abs(st["energy_in"] - e_in) <= tol * e_in
    assert abs(st["photons_in"] - n_in) <= tol * n_in
    assert abs(st["energy_out"] - e_out) <= tol * e_out
    assert abs(st["photons_out"] - n_out) <= tol * n_out
    # against the reference's output: a relative spectral error eps changes these
    # quadratic sums by at most 2 eps + eps^2 (eps <= 1e-9 in fp64, <= 1e-4 mixed)
    e_ref, n_ref = parseval(case["A_out"], d, g.nu)
    rt = 2.1e-9 if precision == "fp64" else 2.1e-4
    assert abs(st["energy_out"] - e_ref) <= rt * e_ref
    assert abs(st["photons_out"] - n_ref) <= rt * n_ref


def test_conservation_laws(cuda_ready):
    # SPM + dispersion, lossless: energy and photon number conserved up to the fixed-step
    # RK4IP truncation error (the reference's own output drifts by 6e-8 on this case)
    _, _, _, st, _ = run("soliton_n2_1024", "fp64")
    assert abs(st["energy_out"] / st["energy_in"] - 1.0) < 1e-6
    assert abs(st["photons_out"] / st["photons_in"] - 1.0) < 1e-6
    # Raman + self-steepening: the photon number is conserved (2e-9 in the reference's
    # output) while the energy is not
    _, _, _, st, _ = run("sc_blowwood_ark4ip_1024", "fp64")
    assert abs(st["photons_out"] / st["photons_in"] - 1.0) < 1e-7
    assert abs(st["energy_out"] / st["energy_in"] - 1.0) > 1e-3
    # saturable gain: both grow
    _, _, _, st, _ = run("gain_ark4ip_1024", "fp64")
    assert st["energy_out"] > 1.01 * st["energy_in"] and st["photons_out"] > 1.01 * st["photons_in"]
