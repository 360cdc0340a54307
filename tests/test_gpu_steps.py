"""Step logs and step replay through the C ABI (gnlse_set_step_log, gnlse_set_replay).

The log of an ARK4IP instance holds (z, h) of every accepted step, the pairs the
reference's adaptive stepper appends to Storage.step_sizes (pyofss/modules/stepper.py:
339-345), where pyofss keeps only the steps that store a trace; Fibre applies that rule.
Replay makes an instance follow a given step sequence with every attempt accepted: with
the reference's own accepted steps the fp64 engine reproduces the reference output, and
the mixed mode's error then measures its arithmetic alone, with no controller decision
of its own.
"""

import numpy as np
import pytest

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, Fibre, Sech
from test_gpu_parity import make_plan, rel_l2, spec_err

pytestmark = pytest.mark.gpu


def accepted(case):
    return gc.accepted_steps(case["rk4ip_calls"], True)


@pytest.mark.parametrize("precision", ["fp64", "df"])
@pytest.mark.parametrize("name", ["sc_blowwood_ark4ip_1024", "gain_ark4ip_1024", "sc_hollenbeck_ark4ip_2048"])
def test_step_log_is_the_reference_step_sequence(cuda_ready, name, precision):
    case = gc.load(name)
    plan = make_plan(case, precision)
    plan.set_step_log(0, 100000)
    f = plan.pack([case["A0"]])
    plan.propagate(f)
    st = plan.stats()[0]
    log = plan.step_log(0, [st])
    want = accepted(case)
    assert len(log) == st["steps"] == len(want)
    # h follows the error estimate, a norm of the difference of two solutions that agree
    # to ~1e-6, so round-off enters it ~1e6 times amplified: the engine's step sizes agree
    # with the reference's to ~1e-11 .. 1.3e-9 (measured); the last step is the remainder
    # L - z, a difference of nearly equal numbers, compared to L instead
    L = float(np.sum(want[:, 1]))
    rel = np.abs(log[:-1, 1] - want[:-1, 1]) / want[:-1, 1]
    assert rel.max() <= 1e-8, (rel.max(), int(rel.argmax()), len(rel))
    assert abs(log[-1, 1] - want[-1, 1]) <= 1e-9 * L
    np.testing.assert_allclose(log[:, 0], np.cumsum(want[:, 1]), rtol=1e-9)


def test_fibre_step_sizes_follow_the_reference(cuda_ready):
    case = gc.load("sc_blowwood_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    fib = Fibre(precision="fp64", **{k: v for k, v in fk.items() if k != "method"}, method="cuda_ark4ip")
    pulse = dict(prm["pulse"])
    pulse.pop("kind")
    a0 = Sech(**pulse)(d, np.zeros(d.total_samples, complex))
    np.testing.assert_allclose(a0, case["A0"], rtol=1e-14, atol=1e-14 * np.abs(a0).max())
    fib(d, case["A0"].copy())
    # (absolute 1e-15 km for the final remainder step, see above)
    np.testing.assert_allclose(np.array(fib.stepper.storage.step_sizes), case["step_sizes"], rtol=1e-9,
                               atol=1e-15)


@pytest.mark.parametrize("name", ["sc_blowwood_ark4ip_1024", "sc_hollenbeck_ark4ip_2048", "sc_cfg_8192"])
def test_replay_of_the_reference_steps(cuda_ready, name):
    """fp64 with the reference's accepted steps replayed: the reference output, one attempt
    per step; mixed on the same sequence: the error of its arithmetic alone, which stays
    within the mixed bound while its own step-size decisions are taken out."""
    case = gc.load(name)
    h = accepted(case)[:, 1]
    for precision, tol in (("fp64", 1e-9), ("mixed", 1.5e-4)):
        plan = make_plan(case, precision)
        plan.set_replay(0, h)
        f = plan.pack([case["A0"]])
        plan.propagate(f)
        st = plan.stats()[0]
        out = plan.unpack(f)[0].cpu().numpy().astype(complex)
        assert st["status"] == 0 and st["steps"] == len(h) and st["rejected"] == 0
        assert st["evals"] == 3 * len(h)
        err = spec_err(out, case["A_out"])
        assert err <= tol, (precision, err)
        print(f"{name} {precision} replayed: {err:.2e}")
    # the oracle restates the same replay
    grid = go.Grid(**gc.domain_kwargs(case["params"]))
    fk = gc.fibre_kwargs(case["params"])
    if name != "sc_cfg_8192":  # (the oracle's 7061-step replay takes minutes on one core)
        L = fk.pop("length")
        for k in ("method", "traces", "local_error", "total_steps"):
            fk.pop(k, None)
        want, _ = go.Propagator(grid, L, **fk).adaptive(case["A0"].copy(), 1e-6, replay=h)
        assert rel_l2(want, case["A_out"]) <= 1e-12
