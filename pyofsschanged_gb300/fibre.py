"""``Fibre`` module with CUDA RK4IP / ARK4IP methods (drop-in for pyofss's Fibre).

Constructor arguments are those of ``pyofss.modules.fibre.Fibre``
(pyofss/modules/fibre.py:74-134); calling the module with ``(domain, field)``
propagates the field through the fibre and returns it, as
``Fibre.__call__`` does (fibre.py:136-148).  ``method`` selects the engine
path: ``"cuda_rk4ip"`` / ``"rk4ip"`` (fixed step, ``total_steps`` steps),
``"cuda_ark4ip"`` / ``"ark4ip"`` (adaptive step doubling with tolerance
``local_error``), or the split-step methods ``"ss_sym_rk4"``, ``"ss_symmetric"``,
``"ss_simple"``, ``"ss_reduced"``, ``"ss_sym_midpoint"`` and ``"ss_agrawal"``
(pyofss/modules/solver.py:256-337) with the fixed-step driver, or, "a"-prefixed
(``"ass_symmetric"`` ...), with the adaptive one.  ``precision`` selects ``"mixed"``
(default: complex64 transforms with a double-float propagation state), ``"df"``
(double-float throughout), ``"fp32"`` (complex64 throughout) or ``"fp64"``
(complex128 throughout).  The stepper exceptions of
pyofss/modules/stepper.py:33-47 are raised with the same names.

The saturable amplifier and the Yb two-level gain (``use_Yb_model``; its cross
sections from ``yb_cross_sections`` or an importable pyofss installation, its pump
power after the run in ``fibre.amplifier.Pp``) run with the RK4IP methods, and the
legacy ``raman_scattering`` rs_factor term without self-steepening with every method.
Models outside the CUDA path (WDM two-channel, the rs_factor term with self-steepening,
the Er gain profile, ASE noise) raise ``NotImplementedError``.
"""

import sys

import numpy as np
import torch

from . import _native as nat
from .characteristics import trace_characteristics
from .engine import METHODS, Instance, Plan
from .operators import GridTables


class StepperError(Exception):
    pass


class SmallStepSizeError(StepperError):
    pass


class SuitableStepSizeError(StepperError):
    pass


class MaximumStepsAllocatedError(StepperError):
    pass


_STATUS_EXC = {
    nat.GNLSE_SMALL_STEP: (SmallStepSizeError, "Step size is extremely small"),
    nat.GNLSE_SUITABLE_STEP: (SuitableStepSizeError, "Failed to set suitable step-size"),
    nat.GNLSE_MAX_STEPS: (MaximumStepsAllocatedError,
                          "Failed to complete with maximum steps allocated"),
}


_BOTH = {}


def stepper_exception(cls):
    """The class to raise for one of the stepper exceptions above.

    When pyofss's own stepper module (pyofss/modules/stepper.py:33-47) is loaded in
    this process, a caller may catch pyofss's classes; the class returned then derives
    from both this module's class and pyofss's class of the same name, so an
    ``except`` clause written against either catches it.  Otherwise it is ``cls``.
    """
    ref = sys.modules.get("pyofss.modules.stepper")
    rc = getattr(ref, cls.__name__, None) if ref is not None else None
    if not (isinstance(rc, type) and issubclass(rc, Exception)) or issubclass(cls, rc):
        return cls
    key = (cls, rc)
    if key not in _BOTH:
        _BOTH[key] = type(cls.__name__, (cls, rc), {"__module__": __name__})
    return _BOTH[key]


def raise_for_status(status):
    if status in _STATUS_EXC:
        cls, msg = _STATUS_EXC[status]
        raise stepper_exception(cls)(msg)
    if status != nat.GNLSE_OK:
        raise nat.GnlseError(status, "propagation")


def trace_steps(log, length, traces):
    """The accepted steps (z, h) the adaptive stepper keeps in Storage.step_sizes: those
    with z > z_ignore, z_ignore advancing by length / traces (stepper.py:339-345)."""
    out, step = [], length / traces
    z_ignore = step
    for z, h in log:
        if z > z_ignore:
            out.append((float(z), float(h)))
            z_ignore += step
    return out


CHARACT_LISTS = ("energy_list", "max_power_list", "peaks_list", "duration_list", "spec_width_list",
                 "l_nl_list", "l_d_list")


class Storage:
    """Trace store with the fields pyofss's Storage exposes (storage.py:140-165), including
    the per-trace characteristics of ``update_characts`` (storage.py:195-209)."""

    def __init__(self):
        self.z = []
        self.As = []
        self.step_sizes = []
        self.fft_total = 0
        self.domain = None
        for k in CHARACT_LISTS:
            setattr(self, k, [])

    def __call__(self, domain):
        self.domain = domain

    def reset_array(self):
        self.z, self.As = [], []

    def reset_characts(self):
        for k in CHARACT_LISTS:
            setattr(self, k, [])

    def get_df(self, type="complex", z_curr=0):
        """storage.py:250-268 for type 'complex' (needs pandas, like the reference)."""
        import pandas as pd
        if type != "complex":
            raise NotImplementedError("only the complex-field dataframe is produced")
        arr_z = np.array(self.z) * 10 ** 6 + z_curr  # mm
        index = pd.MultiIndex.from_product([arr_z], names=["z [mm]"])
        return pd.DataFrame(self.As, index=index)


class _StepperView:
    def __init__(self, method, traces, local_error, total_steps, length):
        self.method = method
        self.adaptive = method.startswith("a")
        self.traces = traces
        self.local_error = local_error
        self.total_steps = total_steps
        self.length = length
        self.storage = Storage()
        self.stats = None


class Fibre:
    def __init__(self, name="fibre", length=1.0, alpha=None, beta=None, gamma=0.0, sim_type=None,
                 traces=1, local_error=1.0e-6, method="cuda_ark4ip", total_steps=100,
                 self_steepening=False, raman_scattering=False, rs_factor=0.003, use_all=False,
                 centre_omega=None, tau_1=12.2e-3, tau_2=32.0e-3, f_R=0.18,
                 small_signal_gain=None, E_sat=None, P_sat=None, Tr=None, lamb0=None,
                 bandwidth=None, use_Er_profile=False, use_Er_noise=False, use_Yb_model=False,
                 Pp_0=None, N=None, Rr=None, dir=None, save_represent="power", cycle=None,
                 downsampling=None, precision="mixed", cluster=0, yb_cross_sections=None):
        m = method.lower()
        if m.startswith("cuda_"):
            m = m[5:]
        if m not in METHODS:
            raise NotImplementedError(
                f"method {method!r}: the CUDA engine runs {' / '.join(METHODS)}")
        if sim_type not in (None, "default"):
            raise NotImplementedError("sim_type='wdm' is not on the CUDA path")
        if raman_scattering and not use_all and self_steepening:
            raise NotImplementedError("the legacy rs_factor Raman term with self-steepening is not on "
                                      "the CUDA path")
        if use_Er_profile or use_Er_noise:
            raise NotImplementedError("the Er gain profile and ASE noise are not on the CUDA path")
        if small_signal_gain is not None and E_sat is None and P_sat is not None:
            if Tr is None:
                raise Exception("Repetition rate is not defined.")
            E_sat = P_sat * Tr
        gain = use_Yb_model or (small_signal_gain is not None and E_sat is not None)
        if gain and m.startswith(("ss_", "ass_")):
            raise NotImplementedError("the split-step methods run without gain on the CUDA path")
        if self_steepening and m.lstrip("a") in ("ss_symmetric", "ss_simple", "ss_reduced"):
            # the reference's exponential step divides by the field (nonlinearity.py:230-234)
            raise NotImplementedError(f"{m} with self-steepening is not on the CUDA path")
        self.name = name
        self.length = length
        self.alpha, self.beta, self.gamma = alpha, beta, gamma
        self.self_steepening, self.use_all = self_steepening, use_all
        self.tau_1, self.tau_2, self.f_R = tau_1, tau_2, f_R
        self.raman_scattering, self.rs_factor = raman_scattering, rs_factor
        self.centre_omega = centre_omega
        self.small_signal_gain, self.E_sat = small_signal_gain, E_sat
        self.lamb0, self.bandwidth = lamb0, bandwidth
        self.use_Yb_model, self.Pp_0, self.N, self.Rr = use_Yb_model, Pp_0, N, Rr
        self.yb_cross_sections = yb_cross_sections
        self.amplifier = None
        self.method = m
        self.precision = precision
        self.cluster = cluster
        self.cycle = cycle
        self.domain = None
        self._plan = None
        self.stepper = _StepperView(m, traces, local_error, total_steps, length)

    def _build(self, domain):
        g = GridTables(domain, beta=self.beta, alpha=self.alpha, gamma=self.gamma,
                       self_steepening=self.self_steepening, use_all=self.use_all,
                       tau_1=self.tau_1, tau_2=self.tau_2, f_R=self.f_R,
                       raman_scattering=self.raman_scattering, rs_factor=self.rs_factor,
                       centre_omega=self.centre_omega, small_signal_gain=self.small_signal_gain,
                       E_sat=self.E_sat, length=self.length, lamb0=self.lamb0,
                       bandwidth=self.bandwidth, use_Yb_model=self.use_Yb_model, Pp_0=self.Pp_0,
                       N=self.N, Rr=self.Rr, yb_cross_sections=self.yb_cross_sections,
                       cluster=self.cluster)
        self.amplifier = g.yb
        st = self.stepper
        inst = Instance(0, method=st.method, length=self.length, local_error=st.local_error,
                        total_steps=st.total_steps, traces=st.traces)
        self._plan = Plan([g], [inst], precision=self.precision)
        if st.adaptive:  # every accepted step, up to the stepper's steps_max (stepper.py:130)
            self._plan.set_step_log(0, 100000)
        self.domain = domain
        st.storage(domain)

    def _run(self, field):
        """Propagate one field through the engine: (output field, stats, trace z values,
        trace fields as a [k, n] device tensor)."""
        plan = self._plan
        flat = plan.pack([np.asarray(field)])
        plan.propagate(flat)
        stats = plan.stats()
        torch.cuda.current_stream(plan.device).synchronize()
        z, As = plan.instance_traces(0, stats, device=True)
        return plan.unpack(flat)[0].cpu().numpy().astype(complex), stats[0], z, As

    def _step_sizes(self, st):
        """Storage.step_sizes (stepper.py:339-345): (z, h) of the accepted steps that stored
        a trace, from the engine's log of every accepted step."""
        return trace_steps(self._plan.step_log(0, [st]), self.length, self.stepper.traces)

    def __call__(self, domain, field):
        if self.domain != domain or self._plan is None:
            self._build(domain)
        out, st, z, As = self._run(field)
        self.stepper.stats = st
        if self.amplifier is not None:  # Amplifier2LevelModel.Pp after update_Pp calls
            self.amplifier.Pp = st["pump_w"]
        storage = self.stepper.storage
        storage.reset_array()
        storage.reset_characts()
        storage.z = list(z)
        storage.As = [a.astype(complex) for a in As.cpu().numpy()]
        if len(z):
            beta2 = self.beta[2] if self.beta is not None and len(self.beta) > 2 else None
            ch = trace_characteristics(As, domain, self.gamma, beta2)
            for k in CHARACT_LISTS:
                setattr(storage, k, ch[k])
        storage.step_sizes = self._step_sizes(st) if self.stepper.adaptive else []
        storage.fft_total = int(st["evals"]) * 16
        raise_for_status(st["status"])
        return out
