"""The drop-in module path: System + Sech + Fibre(method='cuda_ark4ip'/'cuda_rk4ip')."""

import numpy as np
import pytest

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import (Domain, Fibre, Gaussian, Sech, SmallStepSizeError, System)

pytestmark = pytest.mark.gpu


def spec_err(a, b):
    return float(np.linalg.norm(go.fft(a) - go.fft(b)) / np.linalg.norm(go.fft(b)))


@pytest.mark.parametrize("name,precision,tol", [
    ("sc_blowwood_ark4ip_1024", "fp64", 1e-9), ("sc_blowwood_ark4ip_1024", "mixed", 1e-4),
    ("gain_ark4ip_1024", "mixed", 1e-4), ("soliton_n2_1024", "fp64", 1e-9)])
def test_system_with_cuda_fibre(cuda_ready, name, precision, tol):
    case = gc.load(name)
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    p = dict(prm["pulse"])
    cls = Sech if p.pop("kind") == "sech" else Gaussian
    fk = gc.fibre_kwargs(prm)
    fk["method"] = "cuda_" + fk["method"]
    sys_ = System(d)
    sys_.add(cls(**p))
    sys_.add(Fibre(precision=precision, **fk))
    sys_.run()
    out = sys_.fields["fibre"]
    assert spec_err(out, case["A_out"]) <= tol
    st = sys_["fibre"].stepper
    # mixed plans estimate the local error from complex64 stages, so accepted
    # step sizes (and trace positions) follow FP64 only to ~1e-4 relative
    np.testing.assert_allclose(st.storage.z, case["trace_z"], rtol=1e-9 if precision == "fp64" else 2e-3)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-4)])
def test_yb_fibre_in_system(cuda_ready, precision, tol):
    """Fibre(use_Yb_model=True) in a System: output and pump power as the reference's."""
    case = gc.load("yb_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    p = dict(prm["pulse"])
    p.pop("kind")
    fk = gc.fibre_kwargs(prm)
    fk["method"] = "cuda_" + fk["method"]
    sys_ = System(d)
    sys_.add(Gaussian(**p))
    sys_.add(Fibre(precision=precision, **fk))
    sys_.run()
    assert spec_err(sys_.fields["fibre"], case["A_out"]) <= tol
    assert sys_["fibre"].amplifier.Pp == pytest.approx(float(case["yb_pump_out"]),
                                                      rel=1e-9 if precision == "fp64" else 1e-5)


def test_fibre_raises_reference_exception(cuda_ready):
    d = Domain(bit_width=12.5, samples_per_bit=1024, centre_nu=359.0)
    a = Sech(peak_power=100.0, width=0.1)(d, np.zeros(1024, complex))
    a[5] = np.inf
    fib = Fibre(length=1e-5, beta=[0, 0, -10.0], gamma=100.0, method="cuda_ark4ip")
    with pytest.raises(SmallStepSizeError):
        fib(d, a)
