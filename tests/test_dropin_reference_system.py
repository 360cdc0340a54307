"""This package's Fibre inside the reference's own System (pyofss/system.py:220-243).

The reference tree is present only on a development host without a GPU, and the GPU
host does not have it, so no single run has both.  This CPU test therefore runs the
unmodified reference System, Domain and Sech (imported through oracle/ref_shim.py)
with this package's Fibre, whose engine call ``Fibre._run`` is replaced by the FP64
oracle.  It checks the module protocol the reference's System relies on: ``name``,
``__call__(domain, field) -> field``, the ``fields`` dictionary, the
``update_result_df`` type checks (the CUDA Fibre is not pyofss's ``Fibre`` class, so
System skips its dataframe hooks), the trace storage of ``fibre.stepper.storage``, and
stepper exceptions that a pyofss caller catches with pyofss's own classes
(pyofss/modules/stepper.py:33-47).  The engine behind ``_run`` is checked against the
same golden cases by the GPU parity tests.
"""

import importlib

import numpy as np
import pytest
import torch

import golden_cases as gc
from oracle import gnlse_oracle as go
from oracle import ref_shim
from pyofsschanged_gb300 import _native as nat
from pyofsschanged_gb300 import fibre as cf

pytestmark = pytest.mark.skipif(not ref_shim.available(), reason="reference tree absent")


class OracleEngineFibre(cf.Fibre):
    """The CUDA Fibre with its device plan replaced by the FP64 oracle (test double)."""

    status = nat.GNLSE_OK

    def _build(self, domain):
        self.domain = domain
        self._plan = "oracle"
        self.stepper.storage(domain)

    def _run(self, field):
        d = self.domain
        grid = go.Grid(total_bits=d.total_bits, samples_per_bit=d.samples_per_bit,
                       bit_width=d.bit_width, centre_nu=d.centre_nu)
        p = go.Propagator(grid, self.length, beta=self.beta, gamma=self.gamma,
                          self_steepening=self.self_steepening, use_all=self.use_all,
                          tau_1=self.tau_1, tau_2=self.tau_2, f_R=self.f_R)
        st = self.stepper
        out, info = p.adaptive(np.array(field, complex), st.local_error, st.total_steps, st.traces)
        stats = {"status": self.status, "evals": p.evals, "pump_w": 0.0}
        tr = np.array(info["trace_A"]).reshape(-1, grid.total_samples)
        self._oracle_steps = info["steps"]
        return out, stats, np.array(info["trace_z"]), torch.as_tensor(tr)

    def _step_sizes(self, st):
        return cf.trace_steps(self._oracle_steps, self.length, self.stepper.traces)


def _reference_system(case, fibre):
    ref = ref_shim.load()
    system_mod = importlib.import_module("pyofss.system")
    prm = case["params"]
    dom = ref.Domain(**gc.domain_kwargs(prm))
    pulse = prm["pulse"]
    sys_ = system_mod.System(dom)
    sys_.add(ref.Sech(peak_power=pulse["peak_power"], width=pulse["width"],
                      using_fwhm=pulse["using_fwhm"]))
    sys_.add(fibre)
    return ref, sys_


def _fibre(cls, case):
    fk = gc.fibre_kwargs(case["params"])
    return cls(name="fibre", length=fk["length"], beta=fk["beta"], gamma=fk["gamma"],
               self_steepening=fk["self_steepening"], use_all=fk["use_all"], f_R=fk["f_R"],
               tau_1=fk["tau_1"], tau_2=fk["tau_2"], traces=fk["traces"],
               local_error=fk["local_error"], method="cuda_ark4ip")


def test_cuda_fibre_runs_in_reference_system():
    case = gc.load("sc_blowwood_ark4ip_1024")
    fib = _fibre(OracleEngineFibre, case)
    _, sys_ = _reference_system(case, fib)
    sys_.run()
    np.testing.assert_array_equal(sys_.fields["sech"], case["A0"])
    out = sys_.fields["fibre"]
    assert out.dtype == complex and out.shape == case["A0"].shape
    err = np.linalg.norm(go.fft(out) - go.fft(case["A_out"])) / np.linalg.norm(go.fft(case["A_out"]))
    assert err <= 1e-12
    # System.update_result_df skips modules that are not pyofss's Fibre / OpenclFibre
    assert sys_.df_results is None
    storage = fib.stepper.storage
    np.testing.assert_allclose(storage.z, case["trace_z"], rtol=1e-14, atol=0)
    # Storage.step_sizes by the reference's rule (z > z_ignore) from the log of every step
    np.testing.assert_allclose(np.array(storage.step_sizes), case["step_sizes"], rtol=1e-13, atol=0)
    assert len(storage.As) == len(storage.energy_list) == len(case["trace_z"])


def test_stepper_errors_are_pyofss_classes():
    case = gc.load("sc_blowwood_ark4ip_1024")

    class Failing(OracleEngineFibre):
        status = nat.GNLSE_SMALL_STEP

    ref, sys_ = _reference_system(case, _fibre(Failing, case))
    with pytest.raises(ref.stepper.SmallStepSizeError) as ei:
        sys_.run()
    assert isinstance(ei.value, cf.SmallStepSizeError)
    assert isinstance(ei.value, ref.stepper.StepperError)
    assert str(ei.value) == "Step size is extremely small"
