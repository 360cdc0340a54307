"""Trace characteristics (Storage lists) against the reference's own field.py rules.

Runs where the reference tree exists (it is read through oracle/ref_shim.py as
the checker); elsewhere the comparison is skipped.
"""

import numpy as np
import pytest
import torch

import golden_cases as gc
from oracle import ref_shim
from pyofsschanged_gb300 import Domain
from pyofsschanged_gb300.characteristics import trace_characteristics

pytestmark = pytest.mark.skipif(not ref_shim.available(), reason="reference tree absent")


@pytest.mark.parametrize("name", ["soliton_n2_1024", "sc_blowwood_ark4ip_1024", "gain_fixed_2048",
                                  "sc_hollenbeck_ark4ip_2048"])
def test_characteristics_match_reference(name):
    ref = ref_shim.load()
    f = ref.field
    case = gc.load(name)
    prm = case["params"]
    dom = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    gamma, beta = fk.get("gamma", 0.0), fk.get("beta")
    beta2 = beta[2] if beta is not None and len(beta) > 2 else None
    fields = np.stack([case["A0"], case["A_out"]])
    got = trace_characteristics(torch.as_tensor(fields), dom, gamma, beta2)
    for j, A in enumerate(fields):
        P = f.temporal_power(A)
        assert got["energy_list"][j] == pytest.approx(f.energy(A, dom.t), rel=1e-12)
        assert got["max_power_list"][j] == pytest.approx(np.amax(P), rel=1e-12)
        np.testing.assert_array_equal(got["peaks_list"][j], f.get_peaks(P))
        dur = f.get_duration(P, dom.dt)
        assert got["duration_list"][j] == pytest.approx(dur, rel=1e-12)
        assert got["spec_width_list"][j] == pytest.approx(
            f.get_duration_spec(f.spectral_power(A), dom.dnu), rel=1e-12)
        if gamma:
            assert got["l_nl_list"][j] == pytest.approx(1.0 / (gamma * np.amax(P)), rel=1e-12)
        if beta2:
            assert got["l_d_list"][j] == pytest.approx(dur ** 2 / abs(beta2), rel=1e-12)
