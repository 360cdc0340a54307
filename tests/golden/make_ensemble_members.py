"""Oracle outputs for three members of the benchmark's noise ensemble (one per grid size).

Run from the repository root (CPU only, a few minutes)::

    python tests/golden/make_ensemble_members.py

The members are the first member of each grid size (2^12, 2^13, 2^14 points) of the
seeded 256-member ensemble (``pyofsschanged_gb300.ensemble.sc_ensemble``, default seed),
with their sech pulse and one-photon-per-mode noise, propagated over a shortened 1 cm
of the ensemble's fibre with ARK4IP at local error 1e-6 by the FP64 oracle (a bit-exact
restatement of the reference's ARK4IP); the 2^12-point member also over its full
length (a complete ensemble member solve).  The inputs are regenerated from the seed by the
test; the file keeps each input's checksum, the output field, the attempt and evaluation
counts and the accepted step sequence.
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import gnlse_oracle as go  # noqa: E402
from pyofsschanged_gb300.ensemble import FIBRE_835, sc_ensemble  # noqa: E402

LENGTH_KM = 1.0e-5
TOL = 1e-6


def selected(members):
    out, seen = [], set()
    for i, m in enumerate(members):
        if m.n not in seen:
            seen.add(m.n)
            out.append(i)
    return sorted(out, key=lambda i: members[i].n)


def main():
    members, domains, fields = sc_ensemble(256)
    res = {}
    meta = []
    runs = [(i, LENGTH_KM, f"{members[i].n}_1cm") for i in selected(members)]
    first = runs[0][0]
    runs.append((first, members[first].length, f"{members[first].n}_full"))
    for i, length, tag in runs:
        m = members[i]
        d = domains[m.n]
        grid = go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
        p = go.Propagator(grid, length, **FIBRE_835)
        t0 = time.time()
        out, info = p.adaptive(fields[i].copy(), TOL)
        a0 = fields[i]
        res[f"out_{tag}"] = out
        res[f"steps_{tag}"] = np.array(info["steps"])
        meta.append({"tag": tag, "member": i, "n": m.n, "length_km": length,
                     "attempts": info["attempts"], "evals": p.evals,
                     "input_abs_sum": float(np.abs(a0).sum()),
                     "input_first": [float(a0[0].real), float(a0[0].imag)],
                     "wall_s": round(time.time() - t0, 1)})
        print(meta[-1], flush=True)
    res["meta"] = json.dumps({"local_error": TOL, "runs": meta})
    np.savez_compressed(os.path.join(HERE, "ensemble_members.npz"), **res)


if __name__ == "__main__":
    main()
