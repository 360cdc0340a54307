"""Train and evaluate the segment surrogate end to end on one GPU.

    python -m pyofsschanged_gb300.surrogate_run [--train 20000] [--test 2000] [--epochs 10]
        [--tol 1e-3] [--out result.json]

1. seeded pulses (sech, FWHM 30-200 fs, P0 1-20 kW, quadratic spectral phase
   +-500 fs^2) on the 2^13-point 835 nm grid;
2. their propagation through 5 cm of the supercontinuum fibre by the batched
   RK4IP engine (ARK4IP 1e-6, mixed precision) -- training data, calibration
   data and the reference outputs of the test set;
3. two networks trained from different seeds on the training split; the error
   estimate's scale calibrated on the calibration split;
4. the test set through the surrogate with RK4IP fallback at the tolerance:
   acceptance, true spectral errors of the accepted members, and solves/s of
   surrogate-with-fallback against the engine alone on the same members.
"""

import argparse
import json
import time

import numpy as np
import torch

from . import surrogate as sg


def solve_chunked(A0, z, chunk=4096):
    out = np.empty_like(A0)
    for s in range(0, len(A0), chunk):
        out[s:s + chunk], st = sg.propagate(A0[s:s + chunk], z)
        bad = [i for i, x in enumerate(st) if x["status"] != 0]
        if bad:
            raise RuntimeError(f"engine failed on members {bad[:5]}")
    return out


def main(argv=None):
    run(argv)
    return 0


def run(argv=None):
    """The whole experiment; returns the result dictionary (also printed as one JSON line)."""
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--calib", type=int, default=1000)
    ap.add_argument("--test", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--length-km", type=float, default=sg.SEGMENT_KM)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    z = a.length_km
    res = {"config": vars(a)}
    n_all = a.train + a.calib + a.test
    t0 = time.time()
    params, A0 = sg.sample_pulses(n_all, seed=20261205)
    res["sample_s"] = time.time() - t0

    torch.cuda.synchronize()
    t0 = time.time()
    AL = solve_chunked(A0, z)
    torch.cuda.synchronize()
    res["engine_solves_per_s_all"] = n_all / (time.time() - t0)

    pic, a0, aL, scale = sg.make_dataset(A0, AL, z)
    tr = slice(0, a.train)
    ca = slice(a.train, a.train + a.calib)
    te = slice(a.train + a.calib, n_all)
    nets, hist = [], []
    t0 = time.time()
    for seed in (0, 1):
        net = sg.SpectralNeuralOperator(seed=seed)
        hist.append(sg.train(net, pic, a0[tr], aL[tr], epochs=a.epochs, batch=a.batch, lr=a.lr, seed=seed,
                             log=lambda s: print(s, flush=True)))
        nets.append(net)
    torch.cuda.synchronize()
    res["train_s"] = time.time() - t0
    res["train_loss"] = hist

    sur = sg.SurrogateWithFallback(nets, pic, tol=a.tol)
    err_c, dis_c = sur.calibrate(a0[ca], aL[ca])
    res["kappa"] = sur.kappa
    # errors on the test split: network mean, each network, linear propagation alone
    mean, est = sur.estimate(a0[te])
    err_net = sg.rel_err(mean, aL[te])
    err_lin = sg.rel_err(a0[te], aL[te])
    res["test_error"] = {"network_median": float(np.median(err_net)), "network_p90": float(np.quantile(err_net, 0.9)),
                         "linear_only_median": float(np.median(err_lin)),
                         "estimate_vs_true_corr": float(np.corrcoef(np.log(est + 1e-30), np.log(err_net))[0, 1])}
    # end-to-end: surrogate with fallback vs the engine alone on the test members (host fields in/out)
    A_te = A0[te]
    torch.cuda.synchronize()
    t0 = time.time()
    ref_te = solve_chunked(A_te, z)
    torch.cuda.synchronize()
    t_engine = time.time() - t0
    by_tol = {}
    for tol in sorted({a.tol, 1e-2, 1e-1, 3e-1}):
        sur.tol = tol
        torch.cuda.synchronize()
        t0 = time.time()
        out, accept, _ = sur(A_te, z)
        torch.cuda.synchronize()
        t_sur = time.time() - t0
        s_ref = np.fft.ifft(ref_te, axis=1)
        s_out = np.fft.ifft(out, axis=1)
        e = np.linalg.norm(s_out - s_ref, axis=1) / np.linalg.norm(s_ref, axis=1)
        by_tol[str(tol)] = {"accepted": float(accept.mean()),
                            "max_error_accepted": float(e[accept].max()) if accept.any() else None,
                            "median_error_accepted": float(np.median(e[accept])) if accept.any() else None,
                            "frac_accepted_within_tol": float((e[accept] <= tol).mean()) if accept.any() else None,
                            "solves_per_s": len(A_te) / t_sur,
                            "speedup_vs_engine": t_engine / t_sur}
    res["engine_solves_per_s_test"] = len(A_te) / t_engine
    res["surrogate_with_fallback"] = by_tol
    line = json.dumps(res)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")
    return res


if __name__ == "__main__":
    raise SystemExit(main())
