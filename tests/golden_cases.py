"""Load the golden fixtures made by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    """Reference-run cases (fixtures with a parameter record; other .npz files in the
    directory hold oracle-only vectors with their own readers)."""
    out = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            with np.load(os.path.join(GOLDEN, f)) as z:
                if "params" in z.files:
                    out.append(f[:-4])
    return out


# methods of the reference that the CUDA engine runs (the oracle restates more)
ENGINE_METHODS = {"rk4ip", "ark4ip", "ss_sym_rk4", "ss_symmetric", "ss_simple", "ss_reduced",
                  "ss_sym_midpoint", "ss_agrawal", "ass_sym_rk4", "ass_symmetric", "ass_simple",
                  "ass_reduced", "ass_sym_midpoint", "ass_agrawal"}


def engine_names():
    """Golden cases whose method the engine runs."""
    return [n for n in names() if load(n)["params"]["fibre"]["method"] in ENGINE_METHODS]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = {k: z[k] for k in z.files if k != "params"}
    case["params"] = json.loads(str(z["params"]))
    case["name"] = name
    if "yb_sigma12_s" in case:  # the reference's cross sections interpolated on the grid
        case["params"]["fibre"]["yb_cross_sections"] = (case["yb_sigma12_s"], case["yb_sigma21_s"])
    return case


def domain_kwargs(params):
    d = dict(params["domain"])
    if "lambda_nm" in d:
        lam = d.pop("lambda_nm")
        d["centre_nu"] = 1.0e-3 * 299792458.0 / lam
    return d


def fibre_kwargs(params):
    return dict(params["fibre"])


def accepted_steps(calls, adaptive):
    """(z, h) of the accepted steps from the logged rk4ip calls of a reference run."""
    if not adaptive:
        return calls
    att = calls.reshape(-1, 3, 2)
    zs, hs = att[:, 0, 0], att[:, 2, 1]
    acc = [i for i in range(len(zs) - 1) if zs[i + 1] > zs[i]] + [len(zs) - 1]
    return np.stack([zs[acc], hs[acc]], axis=1)


def expected_evals(case):
    """Solver evaluations of the reference run: its logged rk4ip calls, or one per fixed
    step for the split-step method (which makes no rk4ip calls)."""
    fk = case["params"]["fibre"]
    if fk["method"].startswith("ss_"):
        return fk["total_steps"]
    return len(case["rk4ip_calls"])
