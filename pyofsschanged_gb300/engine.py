"""Python handle on a libgnlse plan: many propagations, one launch graph.

A :class:`Plan` owns the device operator tables, per-instance state and
scratch of the C engine (include/gnlse.h).  Fields are torch tensors on the
current CUDA device: complex64 for ``precision="fp32"``, complex128 for
``"fp64"``, ``"mixed"`` (complex64 transforms with a double-float state) and
``"df"`` (double-float transforms, nonlinear term and state), concatenated per
instance in the order given.
"""

import ctypes as ct

import numpy as np
import torch

from . import _native as nat

PRECISIONS = {"fp32": nat.GNLSE_FP32, "fp64": nat.GNLSE_FP64, "mixed": nat.GNLSE_MIXED,
              "df": nat.GNLSE_DF}
METHODS = {"rk4ip": nat.GNLSE_RK4IP, "ark4ip": nat.GNLSE_ARK4IP, "ss_sym_rk4": nat.GNLSE_SS_SYM_RK4,
           "ss_symmetric": nat.GNLSE_SS_SYMMETRIC, "ss_simple": nat.GNLSE_SS_SIMPLE,
           "ss_reduced": nat.GNLSE_SS_REDUCED, "ss_sym_midpoint": nat.GNLSE_SS_SYM_MIDPOINT,
           "ss_agrawal": nat.GNLSE_SS_AGRAWAL}
# the reference's adaptive split steps ("a" + method, stepper.py:111-116)
METHODS.update({"a" + k: v | nat.GNLSE_ADAPTIVE for k, v in list(METHODS.items()) if k.startswith("ss_")})


def _ptr(a):
    if a is None:
        return ct.POINTER(ct.c_double)()
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


class Instance:
    """One propagation: a field on grid ``grid`` through ``length`` km of fibre."""

    def __init__(self, grid, method="ark4ip", length=1.0, local_error=1e-6, total_steps=100,
                 traces=1, max_traces=None, h0=0.0, weight=0.0):
        self.grid = int(grid)
        self.weight = float(weight)
        self.method = method.lower()
        if self.method not in METHODS:
            raise ValueError(f"unknown method {method!r} ({', '.join(METHODS)})")
        self.length = float(length)
        self.local_error = float(local_error)
        self.total_steps = int(total_steps)
        self.traces = int(traces)
        if max_traces is None:
            if self.traces == 1:
                max_traces = 0
            elif not self.method.startswith("a"):  # fixed-step trace rule
                step = self.total_steps // self.traces if self.traces else 0
                max_traces = (self.total_steps + step - 1) // step if step > 0 else 0
            else:
                max_traces = self.traces + 2
        self.max_traces = int(max_traces)
        self.h0 = float(h0)


class Plan:
    def __init__(self, grids, instances, precision="fp32", device=None):
        if precision not in PRECISIONS:
            raise ValueError("precision must be 'fp32', 'mixed', 'df' or 'fp64'")
        lib = nat.lib()
        self.precision = precision
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.dtype = torch.complex64 if precision == "fp32" else torch.complex128
        self.grids = list(grids)
        self.instances = list(instances)
        self._keep = []
        gd = (nat.GridDesc * len(self.grids))()
        for i, g in enumerate(self.grids):
            d = gd[i]
            d.n = g.n
            d.cluster = g.cluster
            d.dt = g.dt
            d.window_t = g.window_t
            d.beta_w = _ptr(g.beta_w)
            d.alpha = g.alpha
            d.gamma = g.gamma
            d.ss_w = _ptr(g.ss_w)
            d.f_R = g.f_R
            d.hR_re = _ptr(g.hR_re)
            d.hR_im = _ptr(g.hR_im)
            d.nu = _ptr(g.nu)
            d.gain_on = 1 if g.gain_on else 0
            d.gain_log = g.gain_log
            d.E_sat = g.E_sat
            d.gain_length = g.gain_length
            d.gain_profile = _ptr(g.gain_profile)
            yb = g.yb
            if yb is not None:
                d.yb_on = 1
                d.yb_pump_w, d.yb_pump_sat, d.yb_pump_ratio = yb.Pp_0, yb.Psat_p, yb.ratio_p
                d.yb_pump_alpha, d.yb_pump_eta = yb.alpha_p_N, yb.eta_p
                d.yb_alpha, d.yb_eta = _ptr(yb.alpha_s_N), _ptr(yb.eta_s)
                d.yb_w_ratio, d.yb_w_sat = _ptr(yb.w_ratio), _ptr(yb.w_sat)
        idesc = (nat.InstanceDesc * len(self.instances))()
        for i, s in enumerate(self.instances):
            d = idesc[i]
            d.grid = s.grid
            d.method = METHODS[s.method]
            d.total_steps = s.total_steps
            d.traces = s.traces
            d.max_traces = s.max_traces
            d.length = s.length
            d.local_error = s.local_error
            d.h0 = s.h0
            d.weight = s.weight
        handle = ct.c_void_p()
        with torch.cuda.device(self.device):
            nat.check(lib.gnlse_plan_create(PRECISIONS[precision], len(self.grids), gd,
                                            len(self.instances), idesc, ct.byref(handle)),
                      "gnlse_plan_create")
        self.handle = handle
        self.n = [self.grids[s.grid].n for s in self.instances]
        self.field_elems = lib.gnlse_plan_field_elems(handle)
        self.field_off = [lib.gnlse_plan_field_offset(handle, i) for i in range(len(self.instances))]
        self.trace_elems = lib.gnlse_plan_trace_elems(handle)
        self.trace_off = [lib.gnlse_plan_trace_offset(handle, i) for i in range(len(self.instances))]
        self.tracez_elems = lib.gnlse_plan_trace_z_elems(handle)
        self.tracez_off = [lib.gnlse_plan_trace_z_offset(handle, i) for i in range(len(self.instances))]
        self.scratch_bytes = lib.gnlse_plan_scratch_bytes(handle)
        self.traces = None
        self.trace_z = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and nat._lib is not None:
            nat._lib.gnlse_plan_destroy(h)
            self.handle = None

    # -- buffers ---------------------------------------------------------------
    def empty_fields(self):
        return torch.zeros(self.field_elems, dtype=self.dtype, device=self.device)

    def pack(self, fields):
        """Concatenate per-instance numpy/torch fields into one device tensor."""
        out = self.empty_fields()
        for i, f in enumerate(fields):
            t = torch.as_tensor(np.asarray(f) if not torch.is_tensor(f) else f)
            out[self.field_off[i]:self.field_off[i] + self.n[i]] = t.to(self.device, self.dtype)
        return out

    def unpack(self, flat):
        return [flat[self.field_off[i]:self.field_off[i] + self.n[i]] for i in range(len(self.n))]

    def _trace_buffers(self):
        if self.trace_elems > 0 and self.traces is None:
            self.traces = torch.zeros(self.trace_elems, dtype=self.dtype, device=self.device)
            self.trace_z = torch.zeros(self.tracez_elems, dtype=torch.float64, device=self.device)

    # -- execution -------------------------------------------------------------
    def reset(self, stream=None):
        s = stream or torch.cuda.current_stream(self.device)
        nat.check(nat.lib().gnlse_reset(self.handle, ct.c_void_p(s.cuda_stream)), "gnlse_reset")

    def propagate(self, fields, max_attempts=0, stream=None, reset=True):
        """Propagate in place on ``fields`` (device tensor from empty_fields/pack)."""
        if fields.dtype != self.dtype or fields.device != self.device or not fields.is_contiguous():
            raise ValueError("fields must be a contiguous %s tensor on %s" % (self.dtype, self.device))
        if fields.numel() != self.field_elems:
            raise ValueError("fields has the wrong number of elements")
        s = stream or torch.cuda.current_stream(self.device)
        if reset:
            self.reset(s)
        self._trace_buffers()
        tr = ct.c_void_p(self.traces.data_ptr()) if self.traces is not None else ct.c_void_p()
        tz = ct.c_void_p(self.trace_z.data_ptr()) if self.trace_z is not None else ct.c_void_p()
        nat.check(nat.lib().gnlse_propagate(self.handle, ct.c_void_p(fields.data_ptr()), tr, tz,
                                            int(max_attempts), ct.c_void_p(s.cuda_stream)),
                  "gnlse_propagate")
        return fields

    def propagate_host(self, host_in, host_out=None, stream=None):
        """End-to-end call on host arrays (numpy complex, concatenated)."""
        npdt = np.complex64 if self.precision == "fp32" else np.complex128
        hin = np.ascontiguousarray(host_in, dtype=npdt)
        hout = hin if host_out is None else host_out
        s = stream or torch.cuda.current_stream(self.device)
        nat.check(nat.lib().gnlse_propagate_host(self.handle, ct.c_void_p(hin.ctypes.data),
                                                 ct.c_void_p(hout.ctypes.data),
                                                 ct.c_void_p(s.cuda_stream)),
                  "gnlse_propagate_host")
        return hout

    def set_timing(self, enable=True):
        nat.check(nat.lib().gnlse_set_timing(self.handle, 1 if enable else 0), "gnlse_set_timing")

    def class_times(self):
        """[(log2 points per CTA, cluster size, instances, kernel ms)] of the last propagate."""
        k = 16
        lm, cl, cnt = (ct.c_int32 * k)(), (ct.c_int32 * k)(), (ct.c_int32 * k)()
        ms = (ct.c_double * k)()
        nc = nat.lib().gnlse_class_times(self.handle, k, lm, cl, cnt, ms)
        if nc < 0:
            raise nat.GnlseError(-nc, "gnlse_class_times")
        return [(lm[i], cl[i], cnt[i], ms[i]) for i in range(nc)]

    def class_members(self):
        """Instance indices of each launch, in the order of class_times()."""
        n = len(self.instances)
        order = (ct.c_int32 * n)()
        nat.check(nat.lib().gnlse_class_order(self.handle, order), "gnlse_class_order")
        out, k = [], 0
        for (_, _, cnt, _) in self.class_times():
            out.append(list(order[k:k + cnt]))
            k += cnt
        return out

    def set_step_log(self, i, capacity):
        """Record instance i's accepted steps (z, h) from the next propagate on
        (gnlse_set_step_log); capacity 0 stops.  step_log(i) reads them."""
        if not hasattr(self, "_step_logs"):
            self._step_logs = {}
        buf = torch.zeros(2 * max(int(capacity), 1), dtype=torch.float64, device=self.device)
        self._step_logs[i] = buf if capacity > 0 else None
        nat.check(nat.lib().gnlse_set_step_log(self.handle, int(i), ct.c_void_p(buf.data_ptr()),
                                               int(capacity)), "gnlse_set_step_log")

    def step_log(self, i, stats=None):
        """[(z, h)] of instance i's recorded accepted steps (numpy, k x 2)."""
        buf = getattr(self, "_step_logs", {}).get(i)
        if buf is None:
            return np.zeros((0, 2))
        k = min((stats or self.stats())[i]["steps"], buf.numel() // 2)
        return buf[:2 * k].view(k, 2).cpu().numpy()

    def set_replay(self, i, h):
        """Make ARK4IP instance i follow the step sizes h (every attempt accepted);
        None returns it to the step-size controller (gnlse_set_replay)."""
        if not hasattr(self, "_replays"):
            self._replays = {}
        if h is None:
            self._replays.pop(i, None)
            nat.check(nat.lib().gnlse_set_replay(self.handle, int(i), ct.c_void_p(), 0), "gnlse_set_replay")
            return
        t = torch.as_tensor(np.asarray(h, float), dtype=torch.float64).to(self.device).contiguous()
        self._replays[i] = t
        nat.check(nat.lib().gnlse_set_replay(self.handle, int(i), ct.c_void_p(t.data_ptr()), t.numel()),
                  "gnlse_set_replay")

    def stats(self, stream=None):
        s = stream or torch.cuda.current_stream(self.device)
        arr = (nat.Stats * len(self.instances))()
        nat.check(nat.lib().gnlse_get_stats(self.handle, arr, ct.c_void_p(s.cuda_stream)),
                  "gnlse_get_stats")
        return [arr[i].as_dict() for i in range(len(self.instances))]

    def instance_traces(self, i, stats=None, device=False):
        """(z values, fields) of instance i's stored traces, as numpy arrays
        (fields as a [k, n] device tensor view with ``device=True``)."""
        st = (stats or self.stats())[i]
        k = st["ntraces"]
        if self.traces is None or k == 0:
            empty = np.zeros((0, self.n[i]), complex)
            return np.zeros(0), (torch.as_tensor(empty, device=self.device) if device else empty)
        z = self.trace_z[self.tracez_off[i]:self.tracez_off[i] + k].cpu().numpy()
        f = self.traces[self.trace_off[i]:self.trace_off[i] + k * self.n[i]].view(k, self.n[i])
        return z, (f if device else f.cpu().numpy())
