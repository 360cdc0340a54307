"""The plain (unfused, one library call per reference op) GPU path against the golden vectors."""

import numpy as np
import pytest
import torch

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, GridTables
from pyofsschanged_gb300.plain import PlainRK4IP

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["soliton_n2_1024", "sc_blowwood_ark4ip_1024", "gain_fixed_2048",
                                  "gain_ark4ip_1024"])
def test_plain_fp64_matches_reference(cuda_ready, name):
    case = gc.load(name)
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    method = fk.pop("method")
    steps = fk.pop("total_steps", 100)
    fk.pop("traces", None)
    tol = fk.pop("local_error", 1e-6)
    p = PlainRK4IP(GridTables(d, **fk), fk["length"])
    a0 = torch.as_tensor(case["A0"]).cuda()
    if method == "ark4ip":
        out, attempts, done = p.adaptive(a0, tol)
        assert done and 3 * attempts == len(case["rk4ip_calls"])
    else:
        out = p.fixed(a0, steps)
    out = out.cpu().numpy()
    err = np.linalg.norm(go.fft(out) - go.fft(case["A_out"])) / np.linalg.norm(go.fft(case["A_out"]))
    assert err <= 1e-9
