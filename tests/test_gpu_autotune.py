"""The launch-class autotuner: measured costs steer the class plans choose."""

import numpy as np
import pytest

from pyofsschanged_gb300 import _native as nat
from pyofsschanged_gb300 import autotune as at
from pyofsschanged_gb300.engine import Instance, Plan
from pyofsschanged_gb300.ensemble import ensemble_plan_inputs, sc_ensemble

pytestmark = pytest.mark.gpu


def test_autotune_measures_and_steers_class_choice(cuda_ready, tmp_path):
    members, domains, fields = sc_ensemble(64)
    idx = [i for i, m in enumerate(members) if m.n == 4096][:2]
    grids, _ = ensemble_plan_inputs([members[i] for i in idx], {4096: domains[4096]})
    # many equal instances, so that no chain exceeds the work bound (no latency switch)
    many = [Instance(0, length=1e-6, local_error=1e-6) for _ in range(600)]
    try:
        res = at.autotune({4096: (grids[0], [fields[i] for i in idx])}, "mixed", attempts=4,
                          cache=str(tmp_path / "costs.json"))
        assert set(res) == {(4096, 1), (4096, 2)}
        assert all(us > 0 for us in res.values())
        # cached: the second call measures nothing and returns the same costs
        assert at.autotune({4096: (grids[0], [fields[i] for i in idx])}, "mixed",
                           cache=str(tmp_path / "costs.json")) == res
        # a measured cost decides: make the single-CTA class look expensive
        nat.check(nat.lib().gnlse_set_class_cost(nat.GNLSE_MIXED, 12, 1, 1e9), "set")
        assert {c[:2] for c in Plan(grids, many, precision="mixed").class_times()} == {(11, 2)}
    finally:
        at.clear("mixed")
    assert {c[:2] for c in Plan(grids, many, precision="mixed").class_times()} == {(12, 1)}
