"""ctypes binding of libgnlse.so (declared in include/gnlse.h).

The library is built in-tree by :mod:`pyofsschanged_gb300.build`.  Loading fails
loudly when it is missing: there is no CPU fallback for the propagation path.
"""

import ctypes as ct
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GNLSE_LIB", os.path.join(HERE, "libgnlse.so"))

GNLSE_OK = 0
GNLSE_SMALL_STEP = 1
GNLSE_SUITABLE_STEP = 2
GNLSE_MAX_STEPS = 3
GNLSE_BAD_ARGUMENT = 4
GNLSE_CUDA_ERROR = 5
GNLSE_UNSUPPORTED = 6
GNLSE_OUT_OF_MEMORY = 7
GNLSE_RUNNING = 8

GNLSE_RK4IP = 0
GNLSE_ARK4IP = 1
GNLSE_SS_SYM_RK4 = 2
GNLSE_SS_SYMMETRIC = 3
GNLSE_SS_SIMPLE = 4
GNLSE_SS_REDUCED = 5
GNLSE_SS_SYM_MIDPOINT = 6
GNLSE_SS_AGRAWAL = 7
GNLSE_ADAPTIVE = 16
GNLSE_FP32 = 0
GNLSE_FP64 = 1
GNLSE_MIXED = 2
GNLSE_DF = 3

_dp = ct.POINTER(ct.c_double)


class GridDesc(ct.Structure):
    _fields_ = [
        ("n", ct.c_int32), ("cluster", ct.c_int32),
        ("dt", ct.c_double), ("window_t", ct.c_double),
        ("beta_w", _dp), ("alpha", ct.c_double), ("gamma", ct.c_double),
        ("ss_w", _dp), ("f_R", ct.c_double), ("hR_re", _dp), ("hR_im", _dp),
        ("nu", _dp), ("gain_on", ct.c_int32), ("pad0", ct.c_int32),
        ("gain_log", ct.c_double), ("E_sat", ct.c_double), ("gain_length", ct.c_double),
        ("gain_profile", _dp),
        ("yb_on", ct.c_int32), ("pad1", ct.c_int32),
        ("yb_pump_w", ct.c_double), ("yb_pump_sat", ct.c_double), ("yb_pump_ratio", ct.c_double),
        ("yb_pump_alpha", ct.c_double), ("yb_pump_eta", ct.c_double),
        ("yb_alpha", _dp), ("yb_eta", _dp), ("yb_w_ratio", _dp), ("yb_w_sat", _dp),
    ]


class InstanceDesc(ct.Structure):
    _fields_ = [
        ("grid", ct.c_int32), ("method", ct.c_int32), ("total_steps", ct.c_int32),
        ("traces", ct.c_int32), ("max_traces", ct.c_int32), ("pad0", ct.c_int32),
        ("length", ct.c_double), ("local_error", ct.c_double), ("h0", ct.c_double),
        ("weight", ct.c_double),
    ]


class Stats(ct.Structure):
    _fields_ = [
        ("z", ct.c_double), ("h", ct.c_double), ("delta_last", ct.c_double),
        ("energy_in", ct.c_double), ("energy_out", ct.c_double),
        ("photons_in", ct.c_double), ("photons_out", ct.c_double),
        ("attempts", ct.c_int64), ("accepted", ct.c_int64), ("rejected", ct.c_int64),
        ("evals", ct.c_int64), ("steps", ct.c_int64),
        ("status", ct.c_int32), ("ntraces", ct.c_int32), ("trace_overflow", ct.c_int32),
        ("finished", ct.c_int32), ("pump_w", ct.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every function declared in include/gnlse.h: name -> (restype, argtypes).
SIGNATURES = {
    "gnlse_abi_version": (ct.c_int, []),
    "gnlse_status_string": (ct.c_char_p, [ct.c_int]),
    "gnlse_plan_create": (ct.c_int, [ct.c_int, ct.c_int, ct.POINTER(GridDesc), ct.c_int,
                                     ct.POINTER(InstanceDesc), ct.POINTER(ct.c_void_p)]),
    "gnlse_plan_destroy": (ct.c_int, [ct.c_void_p]),
    "gnlse_plan_field_elems": (ct.c_int64, [ct.c_void_p]),
    "gnlse_plan_field_offset": (ct.c_int64, [ct.c_void_p, ct.c_int]),
    "gnlse_plan_trace_elems": (ct.c_int64, [ct.c_void_p]),
    "gnlse_plan_trace_offset": (ct.c_int64, [ct.c_void_p, ct.c_int]),
    "gnlse_plan_trace_z_elems": (ct.c_int64, [ct.c_void_p]),
    "gnlse_plan_trace_z_offset": (ct.c_int64, [ct.c_void_p, ct.c_int]),
    "gnlse_plan_scratch_bytes": (ct.c_int64, [ct.c_void_p]),
    "gnlse_reset": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "gnlse_propagate": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                   ct.c_int64, ct.c_void_p]),
    "gnlse_propagate_host": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "gnlse_get_stats": (ct.c_int, [ct.c_void_p, ct.POINTER(Stats), ct.c_void_p]),
    "gnlse_set_step_log": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int64]),
    "gnlse_set_replay": (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int64]),
    "gnlse_set_timing": (ct.c_int, [ct.c_void_p, ct.c_int]),
    "gnlse_profile_counters": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_longlong)]),
    "gnlse_propagate_noalloc": (ct.c_int, [ct.POINTER(GridDesc), ct.POINTER(InstanceDesc),
                                           ct.c_void_p, ct.POINTER(Stats), ct.c_void_p]),
    "gnlse_class_times": (ct.c_int, [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_int32),
                                     ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int32),
                                     ct.POINTER(ct.c_double)]),
    "gnlse_last_cuda_error": (ct.c_char_p, []),
    "gnlse_class_order": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int32)]),
    "gnlse_class_supported": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int]),
    "gnlse_set_class_cost": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_double]),
    # spectral neural operator surrogate kernels (include/sno.h)
    "sno_gemm": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int,
                            ct.c_void_p, ct.c_longlong, ct.c_longlong,
                            ct.c_void_p, ct.c_longlong, ct.c_longlong,
                            ct.c_void_p, ct.c_longlong, ct.c_longlong, ct.c_int,
                            ct.c_float, ct.c_float, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                            ct.c_longlong, ct.c_int, ct.c_void_p]),
    "sno_gelu_backward": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                     ct.c_longlong, ct.c_void_p]),
    "sno_to_bf16": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_longlong, ct.c_void_p]),
    "sno_gemm_timeouts": (ct.c_int, [ct.POINTER(ct.c_uint)]),
    "sno_colsum": (ct.c_int, [ct.c_void_p, ct.c_longlong, ct.c_int, ct.c_void_p, ct.c_void_p]),
    "sno_adam": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                            ct.c_longlong, ct.c_float, ct.c_float, ct.c_float, ct.c_float,
                            ct.c_int, ct.c_float, ct.c_void_p]),
    "sno_rel_l2": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_longlong, ct.c_int, ct.c_void_p,
                              ct.c_void_p, ct.c_void_p]),
}

OPTIONAL = {"gnlse_propagate_noalloc", "sno_gemm", "sno_gemm_timeouts", "sno_gelu_backward", "sno_to_bf16", "sno_colsum",
            "sno_adam", "sno_rel_l2"}

_lib = None
_lock = threading.Lock()


class GnlseError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = status_string(code) if _lib is not None else str(code)
        if _lib is not None and code in (GNLSE_CUDA_ERROR, GNLSE_OUT_OF_MEMORY):
            msg += " [" + _lib.gnlse_last_cuda_error().decode() + "]"
        super().__init__(f"{what}: {msg} (status {code})" if what else f"{msg} (status {code})")


def load(path=LIB_PATH):
    """Load the library (building nothing); raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"libgnlse.so not found at {path}; build it with "
                "`python -m pyofsschanged_gb300.build` (no CPU fallback exists)")
        lib = ct.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            if name in OPTIONAL and not hasattr(lib, name):
                continue  # reduced tuning builds leave these out
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def lib():
    return _lib if _lib is not None else load()


def status_string(code):
    return lib().gnlse_status_string(int(code)).decode()


def check(code, what=""):
    if code != GNLSE_OK:
        raise GnlseError(code, what)
