"""gnlse_propagate captured in a CUDA graph: replays equal the eager call.

A ragged plan (three grid sizes, so several class launches forked onto side
streams and joined back) is captured with torch.cuda.graph, together with the
input copy; every replay must reproduce the eager result bit for bit.
"""

import numpy as np
import pytest
import torch

from pyofsschanged_gb300.engine import Plan
from pyofsschanged_gb300.ensemble import ensemble_plan_inputs, sc_ensemble

pytestmark = pytest.mark.gpu


def _plan():
    members, domains, fields = sc_ensemble(256)
    pick = []
    for n in (4096, 8192, 16384):
        pick += [i for i, m in enumerate(members) if m.n == n][:2]
    sub = [members[i] for i in pick]
    grids, inst = ensemble_plan_inputs(sub, {n: domains[n] for n in set(m.n for m in sub)})
    plan = Plan(grids, inst, precision="mixed")
    return plan, plan.pack([fields[i] for i in pick])


def test_graph_replay_matches_eager(cuda_ready):
    plan, src = _plan()
    budget = 25
    eager = src.clone()
    plan.set_timing(True)  # per-class timing events, eager and (below) captured
    plan.propagate(eager, max_attempts=budget)
    torch.cuda.synchronize()
    assert all(ms > 0 for (_, _, _, ms) in plan.class_times())
    ref = eager.cpu().numpy()
    ref_stats = [(s["attempts"], s["z"], s["h"]) for s in plan.stats()]
    assert len(plan.class_times()) >= 2  # several class launches: the fork/join path

    work = torch.empty_like(src)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # warm-up outside the capture
        work.copy_(src)
        plan.propagate(work, max_attempts=budget)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()  # the timing events become event-record nodes of the graph
    with torch.cuda.graph(g):
        work.copy_(src)
        plan.propagate(work, max_attempts=budget)
    for _ in range(2):
        work.zero_()
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(work.cpu().numpy(), ref)
        assert [(s["attempts"], s["z"], s["h"]) for s in plan.stats()] == ref_stats
        assert all(ms > 0 for (_, _, _, ms) in plan.class_times())
