"""The allocation-free entry point against the plan-based one.

gnlse_propagate_noalloc serves callers that must not allocate device memory
while they propagate (a loop sharing the GPU with latency-critical work, where
cudaMalloc/cudaFree would synchronise the device, or a process whose device
memory belongs to another allocator).  It keeps its tables and scratch in a
static device array, so two calls in a row must give the same answer as the
plan-based entry point: the second call must not see the first call's state.
This file sorts last so that a run stopping at the first failure has already
run every other test.
"""

import ctypes as ct

import numpy as np
import pytest
import torch

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, GridTables, Instance, Plan
from pyofsschanged_gb300 import _native as nat
from pyofsschanged_gb300.engine import METHODS, _ptr

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same kernel and algorithm; only the twiddle tables are built differently


def spec_err(a, b):
    return float(np.linalg.norm(go.fft(a) - go.fft(b)) / np.linalg.norm(go.fft(b)))


def descs(g, inst):
    gd = nat.GridDesc()
    gd.n, gd.cluster, gd.dt, gd.window_t = g.n, 0, g.dt, g.window_t
    gd.beta_w, gd.alpha, gd.gamma = _ptr(g.beta_w), g.alpha, g.gamma
    gd.ss_w, gd.f_R, gd.hR_re, gd.hR_im, gd.nu = (_ptr(g.ss_w), g.f_R, _ptr(g.hR_re),
                                                 _ptr(g.hR_im), _ptr(g.nu))
    gd.gain_on, gd.gain_log, gd.E_sat = 1 if g.gain_on else 0, g.gain_log, g.E_sat
    gd.gain_length, gd.gain_profile = g.gain_length, _ptr(g.gain_profile)
    idesc = nat.InstanceDesc()
    idesc.grid, idesc.method, idesc.total_steps = 0, METHODS[inst.method], inst.total_steps
    idesc.traces, idesc.max_traces, idesc.length = inst.traces, 0, inst.length
    idesc.local_error, idesc.h0 = inst.local_error, inst.h0
    return gd, idesc


@pytest.mark.parametrize("name", ["sc_blowwood_ark4ip_1024", "gain_ark4ip_1024",
                                  "sc_blowwood_fixed_4096"])
def test_noalloc_matches_plan_two_calls(cuda_ready, name):
    case = gc.load(name)
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    method = fk.pop("method")
    steps = fk.pop("total_steps", 100)
    fk.pop("traces", None)
    tol = fk.pop("local_error", 1e-6)
    g = GridTables(d, **fk)
    inst = Instance(0, method=method, length=fk["length"], local_error=tol, total_steps=steps,
                    traces=1)
    plan = Plan([g], [inst], precision="fp32")
    ref = plan.pack([case["A0"]])
    plan.propagate(ref)
    want = ref.cpu().numpy().astype(complex)
    n_want = plan.stats()[0]["evals"]
    gd, idesc = descs(g, inst)
    lib = nat.lib()
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        f = torch.as_tensor(case["A0"].astype(np.complex64)).cuda()
        st = nat.Stats()
        rc = lib.gnlse_propagate_noalloc(ct.byref(gd), ct.byref(idesc), ct.c_void_p(f.data_ptr()),
                                         ct.byref(st), stream)
        assert rc == nat.GNLSE_OK, nat.status_string(rc)
        assert st.status == 0 and st.finished == 1 and st.evals == n_want
        assert spec_err(f.cpu().numpy().astype(complex), want) <= TOL


def test_noalloc_rejects_large_grid(cuda_ready):
    d = Domain(bit_width=12.5, samples_per_bit=8192, centre_nu=359.0)
    g = GridTables(d, beta=[0, 0, -10.0], gamma=1.0)
    gd, idesc = descs(g, Instance(0, method="rk4ip", length=1e-6, total_steps=2))
    f = torch.zeros(8192, dtype=torch.complex64, device="cuda")
    rc = nat.lib().gnlse_propagate_noalloc(ct.byref(gd), ct.byref(idesc), ct.c_void_p(f.data_ptr()),
                                           None, ct.c_void_p(0))
    assert rc == nat.GNLSE_UNSUPPORTED


def test_noalloc_rejects_yb_model(cuda_ready):
    case = gc.load("yb_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    for k in ("method", "total_steps", "traces", "local_error"):
        fk.pop(k, None)
    g = GridTables(d, **fk)
    inst = Instance(0, method="ark4ip", length=fk["length"], local_error=1e-6, traces=1)
    gd, idesc = descs(g, inst)
    gd.yb_on = 1
    f = torch.as_tensor(case["A0"].astype(np.complex64)).cuda()
    rc = nat.lib().gnlse_propagate_noalloc(ct.byref(gd), ct.byref(idesc), ct.c_void_p(f.data_ptr()),
                                           None, ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == nat.GNLSE_UNSUPPORTED


def test_noalloc_ignores_previous_call_tables(cuda_ready):
    """A call that passes no Raman, self-steepening or frequency table must not use the
    ones a previous call left in the shared array: the second call here has to match a
    plan built from the same (absent) tables, and its photon numbers, taken with
    nu = 1 as the plan path does, must be finite."""
    case = gc.load("sc_blowwood_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    tol = fk.get("local_error", 1e-6)
    full = GridTables(d, beta=fk["beta"], gamma=fk["gamma"], self_steepening=True,
                      use_all="blowwood", length=fk["length"])
    bare = GridTables(d, beta=fk["beta"], gamma=fk["gamma"], length=fk["length"])
    bare.nu = None
    assert full.hR_re is not None and full.ss_w is not None and bare.hR_re is None and bare.ss_w is None
    inst = Instance(0, method="ark4ip", length=fk["length"], local_error=tol, traces=1)
    plan = Plan([bare], [inst], precision="fp32")
    ref = plan.pack([case["A0"]])
    plan.propagate(ref)
    want = ref.cpu().numpy().astype(complex)
    st_want = plan.stats()[0]
    lib = nat.lib()
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    for g, check in ((full, False), (bare, True)):
        gd, idesc = descs(g, inst)
        f = torch.as_tensor(case["A0"].astype(np.complex64)).cuda()
        st = nat.Stats()
        rc = lib.gnlse_propagate_noalloc(ct.byref(gd), ct.byref(idesc), ct.c_void_p(f.data_ptr()),
                                         ct.byref(st), stream)
        assert rc == nat.GNLSE_OK, nat.status_string(rc)
        assert st.status == 0 and st.finished == 1
        if check:
            assert st.evals == st_want["evals"]
            assert spec_err(f.cpu().numpy().astype(complex), want) <= TOL
            for k in ("photons_in", "photons_out", "energy_in", "energy_out"):
                v = getattr(st, k)
                assert np.isfinite(v) and v > 0, (k, v)
                assert abs(v - st_want[k]) <= 1e-5 * abs(st_want[k]), (k, v, st_want[k])
