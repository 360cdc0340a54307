"""Generate golden input/output vectors by running the unmodified pyofss reference.

Run from the repository root in an environment that has the reference tree
(``PYOFSS_REFERENCE``, default: a ``reference`` directory beside the repository root)::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [case ...]

Each case writes ``tests/golden/<case>.npz`` holding the seeded input field,
the reference output field, the accepted (z, h) step sequence, every call (z, h)
of the step method (``rk4ip_calls``: Solver.rk4ip, or the split step of an adaptive
split-step run), the trace z values and peak powers, the FFT count and a JSON string
with every parameter
needed to rebuild the run without the reference.  The tests compare the
oracle restatement and the CUDA engine against these files; they never need
the reference itself.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_shim  # noqa: E402

BETA_SC = [0.0, 0.0, -11.830, 8.1038e-2, -9.5205e-5, 2.0737e-7, -5.3943e-10, 1.3486e-12,
           -2.5495e-15, 3.0524e-18, -1.7140e-21]  # ps^k/km at 835 nm (x1e3 of the /m values)

CASES = {
    # Second-order soliton: P0 = |b2|/(g T0^2) = 20 W, amplitude 2 sqrt(P0); two soliton
    # periods z = 2 (pi/2) T0^2/|b2| = pi/20 km; 1000 fixed steps, 50 traces.
    "soliton_n2_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="rk4ip",
                   total_steps=1000, traces=50)),
    # pyofss/tests/test_solver.py:190-284 (RK4IP soliton, peak power 4 after pi/2).
    "soliton_test_solver_2048": dict(
        domain=dict(bit_width=200.0, samples_per_bit=2048, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=4.0, width=1.0),
        fibre=dict(length=0.5 * np.pi, beta=[0.0, 0.0, -1.0], gamma=1.0, method="rk4ip",
                   total_steps=1000, traces=1)),
    "spm_loss_fixed_2048": dict(
        domain=dict(bit_width=40.0, samples_per_bit=2048, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=10.0, width=1.0, C=0.5),
        fibre=dict(length=0.05, beta=[0.0, 0.0, -5.0, 0.3], alpha=2.0, gamma=2.0,
                   method="rk4ip", total_steps=200, traces=10)),
    "sc_blowwood_ark4ip_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=1.0e4, width=0.050, using_fwhm=True),
        fibre=dict(length=1.0e-5, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ark4ip", local_error=1e-6, traces=5)),
    "sc_hollenbeck_ark4ip_2048": dict(
        domain=dict(bit_width=12.5, samples_per_bit=2048, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=8.0e3, width=0.040, using_fwhm=True),
        fibre=dict(length=1.5e-5, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="hollenbeck", method="ark4ip", local_error=1e-6, traces=1)),
    "ss_only_ark4ip_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=1.0e-5, beta=BETA_SC[:4], gamma=110.0, self_steepening=True,
                   method="ark4ip", local_error=1e-6, traces=1)),
    "sc_blowwood_fixed_4096": dict(
        domain=dict(bit_width=12.5, samples_per_bit=4096, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=1.0e4, width=0.050, using_fwhm=True),
        fibre=dict(length=1.0e-5, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", method="rk4ip", total_steps=300, traces=1)),
    "gain_ark4ip_1024": dict(
        domain=dict(bit_width=100.0, samples_per_bit=1024, lambda_nm=1030.0),
        pulse=dict(kind="gaussian", peak_power=100.0, width=1.0, using_fwhm=True),
        fibre=dict(length=3.0e-5, beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0,
                   self_steepening=True, use_all="blowwood", small_signal_gain=39.09,
                   E_sat=5.0, lamb0=1030.0, bandwidth=40.0, method="ark4ip",
                   local_error=1e-6, traces=1)),
    "gain_fixed_2048": dict(
        domain=dict(bit_width=100.0, samples_per_bit=2048, lambda_nm=1030.0),
        pulse=dict(kind="gaussian", peak_power=100.0, width=1.0, using_fwhm=True, C=-3.0),
        fibre=dict(length=2.0e-4, beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0,
                   self_steepening=True, use_all="blowwood", small_signal_gain=39.09,
                   E_sat=0.05, lamb0=1030.0, bandwidth=40.0, method="rk4ip",
                   total_steps=100, traces=1)),
    # The single 2^13-point supercontinuum run: 50 fs FWHM sech, 10 kW, 15 cm, ARK4IP 1e-6.
    "sc_cfg_8192": dict(
        domain=dict(bit_width=12.5, samples_per_bit=8192, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=1.0e4, width=0.050, using_fwhm=True),
        fibre=dict(length=15.0e-5, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ark4ip", local_error=1e-6, traces=1)),
    # Symmetric split step with a classical RK4 nonlinear step (solver.py:330-337):
    # the N=2 soliton and a Raman + self-steepening supercontinuum, fixed step.
    "ss_sym_rk4_soliton_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="ss_sym_rk4",
                   total_steps=800, traces=8)),
    "ss_sym_rk4_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ss_sym_rk4", total_steps=400, traces=1)),
    # Symmetric split step with the exponential nonlinear step (solver.py:267-275):
    # SPM only, and Raman without self-steepening (with self-steepening the reference's
    # exponent divides by the propagated field and overflows in the pulse wings).
    "ss_symmetric_soliton_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="ss_symmetric",
                   total_steps=1000, traces=10)),
    "ss_symmetric_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=False,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ss_symmetric", total_steps=800, traces=1)),
    # Yb two-level gain (Amplifier2LevelModel, amplifier.py:178-344): 1 ps Gaussian at
    # 1030 nm through a pumped Yb fibre; the fixture also keeps the reference's cross
    # sections interpolated on the grid and its pump power after the propagation.
    "yb_ark4ip_1024": dict(
        domain=dict(bit_width=100.0, samples_per_bit=1024, lambda_nm=1030.0),
        pulse=dict(kind="gaussian", peak_power=100.0, width=1.0, using_fwhm=True),
        fibre=dict(length=5.0e-4, beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0,
                   self_steepening=True, use_all="blowwood", use_Yb_model=True, Pp_0=2.0,
                   N=2.0, Rr=1.0e-5, method="ark4ip", local_error=1e-6, traces=1)),
    "yb_fixed_2048": dict(
        domain=dict(bit_width=100.0, samples_per_bit=2048, lambda_nm=1030.0),
        pulse=dict(kind="gaussian", peak_power=100.0, width=1.0, using_fwhm=True, C=-3.0),
        fibre=dict(length=3.0e-4, beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0,
                   use_Yb_model=True, Pp_0=5.0, N=5.0, Rr=1.0e-5, method="rk4ip",
                   total_steps=200, traces=4)),
    # The legacy Raman term rs_factor d|A|^2/dt (raman_scattering=True without use_all,
    # nonlinearity.py:236-248): adaptive RK4IP and the exponential split step.
    "rs_ark4ip_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=1.0e-5, beta=BETA_SC, gamma=110.0, raman_scattering=True,
                   rs_factor=3.0e-3, method="ark4ip", local_error=1e-6, traces=1)),
    "rs_ss_symmetric_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, raman_scattering=True,
                   rs_factor=3.0e-3, method="ss_symmetric", total_steps=800, traces=1)),
    # Simple and reduced split steps (solver.py:256-287): SPM soliton and Raman.
    "ss_simple_soliton_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="ss_simple",
                   total_steps=2000, traces=10)),
    "ss_reduced_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=False,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ss_reduced", total_steps=800, traces=1)),
    # Adaptive split steps (the stepper's leading-A methods with Solver.errors' orders,
    # stepper.py:111-116,143): symmetric (order 3) and symmetric with RK4 (order 5).
    "ass_symmetric_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=False,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ass_symmetric", local_error=1e-6, traces=1)),
    "ass_sym_rk4_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ass_sym_rk4", local_error=1e-6, traces=1)),
    # Symmetric split step with the midpoint method on the nonlinear term
    # (solver.py:323-328): Raman + self-steepening supercontinuum and the N=2 soliton.
    "ss_sym_midpoint_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=True,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ss_sym_midpoint", total_steps=800, traces=1)),
    "ss_sym_midpoint_soliton_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="ss_sym_midpoint",
                   total_steps=1000, traces=5)),
    # Agrawal's iterated split step (solver.py:290-320): the N=2 soliton and a Raman
    # supercontinuum without self-steepening.
    "ss_agrawal_soliton_1024": dict(
        domain=dict(bit_width=32.0, samples_per_bit=1024, centre_nu=193.1),
        pulse=dict(kind="sech", peak_power=80.0, width=1.0),
        fibre=dict(length=np.pi / 20, beta=[0.0, 0.0, -20.0], gamma=1.0, method="ss_agrawal",
                   total_steps=1000, traces=1)),
    "ss_agrawal_sc_1024": dict(
        domain=dict(bit_width=12.5, samples_per_bit=1024, lambda_nm=835.0),
        pulse=dict(kind="sech", peak_power=5.0e3, width=0.050, using_fwhm=True),
        fibre=dict(length=5.0e-6, beta=BETA_SC, gamma=110.0, self_steepening=False,
                   use_all="blowwood", f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3,
                   method="ss_agrawal", total_steps=800, traces=1)),
}

SLOW = {"sc_cfg_8192"}


def build_domain(ref, d):
    d = dict(d)
    if "lambda_nm" in d:
        d["centre_nu"] = ref.domain.lambda_to_nu(d.pop("lambda_nm"))
    return ref.Domain(**d), d


def build_input(ref, domain, p):
    p = dict(p)
    kind = p.pop("kind")
    cls = ref.Sech if kind == "sech" else ref.Gaussian
    field = np.zeros(domain.total_samples, complex)
    return cls(**p)(domain, field)


def run_case(name, spec):
    ref = ref_shim.load()
    domain, dom_params = build_domain(ref, spec["domain"])
    A0 = build_input(ref, domain, spec["pulse"])
    method = spec["fibre"]["method"].lower()
    adaptive = method.startswith("a")
    # the step method whose calls are logged: rk4ip, or the adaptive split step's method
    logged = method[1:] if adaptive and method != "ark4ip" else "rk4ip"
    with ref_shim.StepLog(logged) as log:
        fib = ref_shim.make_fibre(**spec["fibre"])
        t0 = time.time()
        A_out = fib(domain, A0.copy())
        wall = time.time() - t0
    st = fib.stepper.storage
    steps = np.array(st.step_sizes if adaptive else [], float).reshape(-1, 2)
    calls = np.array(log.calls, float).reshape(-1, 2)
    trace_z = np.array(st.z, float)
    trace_peak = np.array([np.max(np.abs(a) ** 2) for a in st.As], float)
    params = dict(domain=dom_params, pulse=spec["pulse"], fibre=spec["fibre"])
    out = dict(A0=A0, A_out=A_out, rk4ip_calls=calls, step_sizes=steps, trace_z=trace_z,
               trace_peak=trace_peak, fft_total=np.int64(st.fft_total),
               wall_s=np.float64(wall), params=np.array(json.dumps(params)))
    if spec["fibre"].get("use_Yb_model"):
        amp = fib.amplifier
        out.update(yb_pump_out=np.float64(amp.Pp), yb_sigma12_s=np.asarray(amp.sigma12_s, float),
                   yb_sigma21_s=np.asarray(amp.sigma21_s, float))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: {wall:.2f} s, {len(calls)} step calls, fft {st.fft_total}, "
          f"peak_out {np.max(np.abs(A_out) ** 2):.6g}", flush=True)


def main(argv):
    names = argv or [n for n in CASES if n not in SLOW]
    if argv == ["all"]:
        names = list(CASES)
    for n in names:
        run_case(n, CASES[n])


if __name__ == "__main__":
    main(sys.argv[1:])
