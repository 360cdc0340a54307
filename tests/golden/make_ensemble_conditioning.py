"""Conditioning of the benchmark ensemble members under the FP64 oracle.

For the first members of ``pyofsschanged_gb300.ensemble.sc_ensemble()`` this
propagates, with the oracle restatement of pyofss's ARK4IP (complex128), the
seeded input field and the same field rounded to complex64, and records the
relative spectral L2 difference of the two outputs.  That difference is the
error any evaluation with complex64 inputs or intermediates inherits from the
dynamics alone (modulation instability amplifies the one-photon noise and
roundoff alike), to be read beside bench.py's ``accuracy_vs_fp64``.

    python tests/golden/make_ensemble_conditioning.py [-j WORKERS] [--count K]

Writes tests/golden/ensemble_conditioning.json.
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


def _solve(i):
    import numpy as np
    from oracle import gnlse_oracle as go
    from pyofsschanged_gb300.ensemble import FIBRE_835, sc_ensemble
    members, domains, fields = sc_ensemble(256)
    m = members[i]
    d = domains[m.n]
    grid = go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
    t0 = time.time()
    a = fields[i].copy()
    out, info = go.Propagator(grid, m.length, **FIBRE_835).adaptive(a.copy(), 1e-6)
    a32 = a.astype(np.complex64).astype(np.complex128)
    out32, info32 = go.Propagator(grid, m.length, **FIBRE_835).adaptive(a32, 1e-6)
    s, s32 = go.fft(out), go.fft(out32)
    return dict(member=i, n=m.n, length_km=m.length, peak_power=m.peak_power, fwhm_ps=m.fwhm,
                input_rel_change=float(np.linalg.norm(a32 - a) / np.linalg.norm(a)),
                output_spectral_rel_change=float(np.linalg.norm(s32 - s) / np.linalg.norm(s)),
                attempts=info["attempts"], attempts_c64_input=info32["attempts"],
                wall_s=time.time() - t0)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", "--jobs", type=int, default=max(1, (os.cpu_count() or 2) - 2))
    ap.add_argument("--count", type=int, default=12)
    a = ap.parse_args(argv)
    ctx = mp.get_context("spawn")
    res = []
    with ctx.Pool(a.jobs) as pool:
        for r in pool.imap_unordered(_solve, range(a.count)):
            res.append(r)
            print(f"member {r['member']:3d} n={r['n']:5d} out change {r['output_spectral_rel_change']:.3e} "
                  f"{r['wall_s']:.1f}s", flush=True)
    res.sort(key=lambda r: r["member"])
    out = dict(source="oracle (FP64 restatement of pyofss ARK4IP); input rounded to complex64",
               local_error=1e-6, results=res)
    with open(os.path.join(HERE, "ensemble_conditioning.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
