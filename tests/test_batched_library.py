"""The batched library comparator (pyofsschanged_gb300/batched_library.py) on the CPU
against the FP64 oracle: three fields of one grid in one batch, each with its own
fibre length, must follow the oracle's ARK4IP step sequences."""

import numpy as np
import torch

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, GridTables
from pyofsschanged_gb300.batched_library import BatchedARK4IP


def test_batched_ark4ip_matches_oracle_per_member():
    case = gc.load("sc_blowwood_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    for k in ("method", "traces", "local_error", "total_steps"):
        fk.pop(k, None)
    length = fk["length"]
    g = GridTables(d, **fk)
    fields = [case["A0"], 0.8 * case["A0"], np.roll(case["A0"], 7)]
    lengths = [length, 0.6 * length, 1.3 * length]
    b = BatchedARK4IP(g, device="cpu")
    out, attempts, _ = b.propagate(torch.as_tensor(np.array(fields)), lengths, 1e-6)
    grid = go.Grid(**gc.domain_kwargs(prm))
    kw = {k: v for k, v in fk.items() if k != "length"}
    for j, (a0, L) in enumerate(zip(fields, lengths)):
        want, info = go.Propagator(grid, L, **kw).adaptive(a0.copy(), 1e-6)
        got = out[j].numpy()
        assert int(attempts[j]) == info["attempts"]
        err = np.linalg.norm(go.fft(got) - go.fft(want)) / np.linalg.norm(go.fft(want))
        assert err <= 1e-10, (j, err)
    # the first member is the reference's own golden run
    err = np.linalg.norm(out[0].numpy() - case["A_out"]) / np.linalg.norm(case["A_out"])
    assert err <= 1e-10
