"""Pin the FP64 oracle restatement against the golden vectors of the reference.

The fixtures in tests/golden/ were produced by running the unmodified pyofss
reference (tests/golden/make_golden.py).  The oracle must reproduce the
reference's output field, its step sequence and its trace positions.
"""

import os

import numpy as np
import pytest

import golden_cases as gc
from oracle import gnlse_oracle as go

FAST = [n for n in gc.names() if n != "sc_cfg_8192"]


def run_oracle(case):
    prm = case["params"]
    grid = go.Grid(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    method = fk.pop("method")
    steps = fk.pop("total_steps", 100)
    traces = fk.pop("traces", 1)
    tol = fk.pop("local_error", 1e-6)
    p = go.Propagator(grid, **fk)
    if method.startswith("a"):  # the stepper's adaptive methods (stepper.py:111-116)
        out, info = p.adaptive(case["A0"].copy(), tol, steps, traces, method=method[1:])
    else:
        out, info = p.standard(case["A0"].copy(), steps, traces, method=method)
    return p, out, info



def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", FAST)
def test_oracle_matches_reference_output(name):
    case = gc.load(name)
    p, out, info = run_oracle(case)
    assert rel_l2(out, case["A_out"]) <= 1e-12
    assert p.evals == gc.expected_evals(case)
    np.testing.assert_allclose(info["trace_z"], case["trace_z"], rtol=1e-13, atol=0)
    peaks = [np.max(np.abs(a) ** 2) for a in info["trace_A"]]
    np.testing.assert_allclose(peaks, case["trace_peak"], rtol=1e-10)


@pytest.mark.parametrize("name", FAST)
def test_oracle_pulse_generation(name):
    case = gc.load(name)
    prm = case["params"]
    grid = go.Grid(**gc.domain_kwargs(prm))
    pulse = dict(prm["pulse"])
    kind = pulse.pop("kind")
    fwhm = pulse.pop("using_fwhm", False)
    if kind == "sech":
        pulse["width"] = go.sech_width(pulse["width"], fwhm)
        a0 = go.sech_field(grid.t, grid.window_t, **pulse)
    else:
        pulse["width"] = go.gaussian_width(pulse["width"], fwhm)
        a0 = go.gaussian_field(grid.t, grid.window_t, **pulse)
    np.testing.assert_array_equal(a0, case["A0"])


def test_soliton_known_answer():
    """pyofss/tests/test_solver.py:278-284: RK4IP soliton peak power 4 after pi/2."""
    case = gc.load("soliton_test_solver_2048")
    _, out, _ = run_oracle(case)
    np.testing.assert_almost_equal(np.max(np.abs(out) ** 2), 4.0, 5)


def test_second_order_soliton_analytic():
    """Analytic N=2 soliton (examples/second_order_soliton/soliton.py:30-46) after two periods."""
    case = gc.load("soliton_n2_1024")
    grid = go.Grid(**gc.domain_kwargs(case["params"]))
    xi = np.pi  # z = pi/20 km = pi * L_D with L_D = T0^2/|b2| = 0.05 km
    tau = grid.t
    num = 4.0 * np.exp(0.5j * xi) * (np.cosh(3 * tau) + 3.0 * np.exp(4j * xi) * np.cosh(tau))
    den = np.cosh(4 * tau) + 4.0 * np.cosh(2 * tau) + 3.0 * np.cos(4 * xi)
    p_true = 20.0 * np.abs(num / den) ** 2
    p_num = np.abs(case["A_out"]) ** 2
    assert np.max(np.abs(p_num - p_true)) / np.max(p_true) < 1e-3


def test_simpson_weights_match_scipy():
    from scipy.integrate import simpson
    rng = np.random.default_rng(3)
    for n in (8, 64, 1024):
        y = rng.random(n)
        x = np.linspace(-1.0, 1.0, n, endpoint=False)
        dx = x[1] - x[0]
        assert abs(np.sum(go.simpson_weights(n) * y) * dx - simpson(y, x=x)) < 1e-13


@pytest.mark.skipif(os.environ.get("GNLSE_SLOW") != "1", reason="70 s CPU run; set GNLSE_SLOW=1")
def test_oracle_sc_cfg_8192():
    case = gc.load("sc_cfg_8192")
    p, out, _ = run_oracle(case)
    assert rel_l2(out, case["A_out"]) <= 1e-10
    assert p.evals == gc.expected_evals(case)


YB = [n for n in FAST if n.startswith("yb_")]


@pytest.mark.parametrize("name", YB)
def test_oracle_yb_pump_power(name):
    """Amplifier2LevelModel advances the pump power on every linear-operator call
    (amplifier.py:360-379); the oracle ends with the reference's pump power."""
    case = gc.load(name)
    p, _, _ = run_oracle(case)
    assert p.gain.Pp == pytest.approx(float(case["yb_pump_out"]), rel=1e-12)


@pytest.mark.parametrize("name", YB)
def test_oracle_yb_cross_sections(name):
    """interpolate_sigma_s (amplifier.py:234-245) restated on the reference's own table."""
    from oracle import ref_shim
    path = os.path.join(ref_shim.REFERENCE_ROOT, "pyofss", "data", "CrossSectionDataExp.txt")
    if not os.path.exists(path):
        pytest.skip("reference data table absent")
    case = gc.load(name)
    grid = go.Grid(**gc.domain_kwargs(case["params"]))
    s12, s21 = go.yb_cross_sections(grid, path)
    np.testing.assert_allclose(s12, case["yb_sigma12_s"], rtol=1e-13, atol=1e-40)
    np.testing.assert_allclose(s21, case["yb_sigma21_s"], rtol=1e-13, atol=1e-40)


@pytest.mark.parametrize("step,steps,want", [
    ("euler_step", 50, 0.72152686293820223), ("euler_step", 500, 0.71717199224362427),
    ("midpoint_step", 50, 0.71663952968427402), ("midpoint_step", 500, 0.71669512731047913),
    ("rk4_step", 50, 0.71669567757603803), ("rk4_step", 500, 0.71669567807363854)])
def test_explicit_solvers_match_reference_golden_values(step, steps, want):
    """pyofss/tests/test_solver.py:99-150 (CheckCoreRoutines): dA/dz = 3 exp(-4z) - 2A,
    A(0) = 1, to z = 0.5 with the fixed-step stepper; the reference asserts these values
    bit for bit, and so does this test (they pin the RK stage arithmetic and the z mesh
    that the split steps ss_sym_rk4 / ss_sym_midpoint use)."""
    def simple(A, z):
        return 3.0 * np.exp(-4.0 * z) - 2.0 * A

    got = go.fixed_steps(getattr(go, step), 1.0, simple, 0.5, steps)
    assert got == want
