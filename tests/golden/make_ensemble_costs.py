"""Per-member cost of the benchmark ensemble under the FP64 oracle.

Runs the oracle restatement of pyofss's ARK4IP (complex128) over every member
of ``pyofsschanged_gb300.ensemble.sc_ensemble()`` and records, per member,
the attempts / accepted / rejected steps and RK4IP evaluations, plus the output
energy and peak power.  The CPU baseline of bench.py extrapolates its bounded
per-attempt timing samples to full solves with these counts.

    python tests/golden/make_ensemble_costs.py [-j WORKERS] [--members N]

Writes tests/golden/ensemble_costs.json.
"""

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _solve(args):
    i, n_members = args
    import numpy as np
    from oracle import gnlse_oracle as go
    from pyofsschanged_gb300.ensemble import FIBRE_835, sc_ensemble
    members, domains, fields = sc_ensemble(n_members)
    m = members[i]
    d = domains[m.n]
    grid = go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
    p = go.Propagator(grid, m.length, **FIBRE_835)
    t0 = time.time()
    out, info = p.adaptive(fields[i].copy(), 1e-6)
    return dict(member=i, n=m.n, length_km=m.length, peak_power=m.peak_power, fwhm_ps=m.fwhm,
                attempts=info["attempts"], rejected=info["rejected"],
                accepted=len(info["steps"]), evals=p.evals, wall_s=time.time() - t0,
                energy_out_nj=float(go.energy(out, grid.t)),
                peak_out_w=float(np.max(np.abs(out) ** 2)))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", "--jobs", type=int, default=max(1, (os.cpu_count() or 2) - 2))
    ap.add_argument("--members", type=int, default=256)
    a = ap.parse_args(argv)
    ctx = mp.get_context("spawn")
    res = []
    with ctx.Pool(a.jobs) as pool:
        for r in pool.imap_unordered(_solve, [(i, a.members) for i in range(a.members)]):
            res.append(r)
            print(f"member {r['member']:3d} n={r['n']:5d} attempts={r['attempts']:6d} "
                  f"{r['wall_s']:.1f}s", flush=True)
    res.sort(key=lambda r: r["member"])
    out = dict(members=a.members, local_error=1e-6, source="oracle (FP64 restatement of pyofss ARK4IP)",
               results=res)
    with open(os.path.join(HERE, "ensemble_costs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
