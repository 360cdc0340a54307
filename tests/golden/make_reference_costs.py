"""Per-attempt cost of the unmodified reference against the oracle port, on one core.

Run from the repository root where the reference tree is present (CPU only)::

    OMP_NUM_THREADS=1 PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_reference_costs.py

The CPU baseline of the benchmark times the oracle (a bit-exact numpy restatement of the
reference's ARK4IP) because the reference cannot run where the GPU is.  This script shows
that the port costs what the reference costs: it runs the same three ensemble members
(the first on each grid size, 1 cm of the ensemble fibre, ARK4IP 1e-6, as in
tests/golden/make_ensemble_members.py) through the reference's own ``Fibre`` (imported by
oracle/ref_shim.py) and through the oracle, each alone on one core, and records both
wall times per attempt and the agreement of the outputs.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import gnlse_oracle as go  # noqa: E402
from oracle import ref_shim  # noqa: E402
from pyofsschanged_gb300.ensemble import FIBRE_835, sc_ensemble  # noqa: E402

LENGTH_KM = 1.0e-5
REPEATS = 2


def main():
    ref = ref_shim.load()
    members, domains, fields = sc_ensemble(256)
    seen, rows = set(), []
    for i, m in enumerate(members):
        if m.n in seen:
            continue
        seen.add(m.n)
        d = domains[m.n]
        rd = ref.Domain(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
        t_ref, t_port = [], []
        for _ in range(REPEATS):
            fib = ref_shim.make_fibre(length=LENGTH_KM, method="ark4ip", local_error=1e-6, traces=1,
                                      **FIBRE_835)
            t0 = time.perf_counter()
            out_ref = fib(rd, fields[i].copy())
            t_ref.append(time.perf_counter() - t0)
            grid = go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
            p = go.Propagator(grid, LENGTH_KM, **FIBRE_835)
            t0 = time.perf_counter()
            out_port, info = p.adaptive(fields[i].copy(), 1e-6)
            t_port.append(time.perf_counter() - t0)
        err = float(np.linalg.norm(go.fft(out_port) - go.fft(out_ref)) / np.linalg.norm(go.fft(out_ref)))
        rows.append({"member": i, "n": m.n, "attempts": info["attempts"],
                     "ref_s_per_attempt": min(t_ref) / info["attempts"],
                     "port_s_per_attempt": min(t_port) / info["attempts"],
                     "port_over_ref": min(t_port) / min(t_ref), "output_spectral_rel_diff": err})
        print(rows[-1], flush=True)
    with open(os.path.join(HERE, "reference_costs.json"), "w") as f:
        json.dump({"length_km": LENGTH_KM, "local_error": 1e-6, "cores": 1,
                   "machine": "development host (x86_64), one core per run, best of %d" % REPEATS,
                   "results": rows}, f, indent=1)


if __name__ == "__main__":
    main()
