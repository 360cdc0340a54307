/*
 * gnlse.h -- C ABI of the GB300 GNLSE propagation engine (libgnlse.so).
 *
 * The engine replaces the propagation core of pyofss's Fibre module: the
 * stepper loop, the RK4IP solver and the linear/nonlinear operators it calls.
 * A host binding (the Python package pyofsschanged_gb300, or a ctypes/cffi
 * stub in pyofss itself) builds the operator tables exactly as pyofss does and
 * hands them over through this interface; the whole propagation of one or many
 * fields then runs on the GPU.
 *
 * Reference interfaces each entry point stands in for (paths inside the pyofss
 * project):
 *   gnlse_plan_create   Linearity.__call__ / default_linearity
 *                       (pyofss/modules/linearity.py:158-186),
 *                       Nonlinearity.__call__ (pyofss/modules/nonlinearity.py:160-185),
 *                       Amplifier.set_domain / spectal_filtration_array
 *                       (pyofss/modules/amplifier.py:110-147),
 *                       Amplifier2LevelModel.set_domain and its tables
 *                       (amplifier.py:247-344),
 *                       Stepper.__init__ (pyofss/modules/stepper.py:87-145)
 *   gnlse_propagate     Fibre.__call__ (pyofss/modules/fibre.py:136-148) ->
 *                       Stepper.__call__ (stepper.py:147-156) ->
 *                       standard_stepper (stepper.py:164-221) /
 *                       adaptive_stepper (stepper.py:247-376) ->
 *                       Solver.rk4ip (pyofss/modules/solver.py:339-354)
 *   gnlse_get_stats     Storage.step_sizes / fft_total (pyofss/modules/storage.py:160-181)
 *                       and the stepper exceptions (stepper.py:33-47, 350-354, 376)
 *   traces              Storage.append (storage.py:183-192): z and A(z) per trace
 *
 * Conventions: units as pyofss (t ps, nu THz, omega rad/ps, z km, beta_k
 * ps^k/km, gamma 1/(W km), power W, energy nJ).  Fields are complex
 * (interleaved re, im) in the time domain, natural order (t from -T/2),
 * complex64 for GNLSE_FP32 plans and complex128 for GNLSE_FP64 and
 * GNLSE_MIXED plans.
 * Spectral tables are in FFT order (pyofss fftshift order).
 *
 * All device pointers are plain CUDA device pointers; stream arguments are
 * cudaStream_t values passed as void*.  Every call returns a status code.
 * A plan is not thread safe; use one plan per host thread.
 */
#ifndef GNLSE_H
#define GNLSE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GNLSE_ABI_VERSION 2

/* status codes (per call and per instance) */
enum {
  GNLSE_OK = 0,
  GNLSE_SMALL_STEP = 1,      /* SmallStepSizeError (stepper.py:350-351) */
  GNLSE_SUITABLE_STEP = 2,   /* SuitableStepSizeError (stepper.py:353-354) */
  GNLSE_MAX_STEPS = 3,       /* MaximumStepsAllocatedError (stepper.py:376) */
  GNLSE_BAD_ARGUMENT = 4,
  GNLSE_CUDA_ERROR = 5,
  GNLSE_UNSUPPORTED = 6,
  GNLSE_OUT_OF_MEMORY = 7,
  GNLSE_RUNNING = 8          /* instance not finished (attempt budget reached) */
};

/* Methods: Solver.rk4ip with the fixed-step or the adaptive (step-doubling) driver;
 * the split steps Solver.ss_sym_rk4 (pyofss/modules/solver.py:330-337: linear half step,
 * classical RK4 on the nonlinear term, linear half step), Solver.ss_symmetric
 * (solver.py:267-275: linear half step, exponential nonlinear step evaluated with the
 * unpropagated field, linear half step; not with self-steepening, whose exponent in the
 * reference divides by the field), ss_simple, ss_reduced, ss_sym_midpoint and
 * ss_agrawal, with the fixed-step driver or -- a split-step method OR'ed with
 * GNLSE_ADAPTIVE, the reference's "a"-prefixed methods (stepper.py:111-116) -- the
 * adaptive driver with the method's order from Solver.errors (solver.py:57-70).  No
 * split step runs with gain or the Yb model (GNLSE_UNSUPPORTED). */
enum {
  GNLSE_RK4IP = 0, GNLSE_ARK4IP = 1, GNLSE_SS_SYM_RK4 = 2, GNLSE_SS_SYMMETRIC = 3,
  GNLSE_SS_SIMPLE = 4,  /* Solver.ss_simple (solver.py:256-265): exponential nonlinear step, then a
                           full linear step; fixed step, no gain, no self-steepening */
  GNLSE_SS_REDUCED = 5,  /* Solver.ss_reduced (solver.py:277-287): ss_symmetric with the exponent
                            from the half-step-propagated field; same limits */
  GNLSE_SS_SYM_MIDPOINT = 6,  /* Solver.ss_sym_midpoint (solver.py:323-328): linear half step,
                                 Solver.midpoint on the nonlinear term, linear half step */
  GNLSE_SS_AGRAWAL = 7,       /* Solver.ss_agrawal (solver.py:290-320): iterated symmetric split
                                 step with the exponent n(Y)/Y (0 where |Y| <= 1e-5) */
  GNLSE_ADAPTIVE = 16         /* flag: the adaptive step-doubling driver for a split step */
};
/* precision: GNLSE_FP32 complex64 throughout (fields complex64);
 * GNLSE_FP64 complex128 throughout (fields complex128);
 * GNLSE_MIXED complex64 transforms and nonlinear evaluations with the
 * propagation state, RK accumulator and exp(hD) factors in double-float
 * (about 48 bits) and FP64 input/output transforms (fields complex128);
 * GNLSE_DF double-float (about 48 bits, on FP32 instructions) throughout:
 * transforms, nonlinear term, state and stage algebra, with the linear phase,
 * error norm and step control in FP64 (fields complex128; grids of 1024 to
 * 32768 points). */
enum { GNLSE_FP32 = 0, GNLSE_FP64 = 1, GNLSE_MIXED = 2, GNLSE_DF = 3 };

/* One grid (pyofss Domain) with the fibre operators built on it. */
typedef struct {
  int32_t n;                  /* samples: power of two, 256 .. 65536 (GNLSE_DF: 1024 ..) */
  int32_t cluster;            /* CTAs per field: 0 = automatic, else 1, 2, 4, 8 or 16 (a
                                 non-portable cluster: 65536-point fp64 / df grids) */
  double dt;                  /* Domain.dt, ps */
  double window_t;            /* Domain.window_t, ps */
  const double* beta_w;       /* [n] fftshift(sum_k beta_k (w - w0)^k / k!), 1/km */
  double alpha;               /* linear attenuation, 1/km (0: none) */
  double gamma;               /* 1/(W km) */
  const double* ss_w;         /* [n] 1 + omega * s (FFT order); NULL: no self-steepening */
  double f_R;                 /* Raman fraction */
  const double* hR_re;        /* [n] Re fft(h_R) * window_t (FFT order); NULL: no Raman */
  const double* hR_im;        /* [n] Im of the same */
  const double* nu;           /* [n] absolute frequency, THz (FFT order); diagnostics */
  int32_t gain_on;            /* saturable gain (Amplifier) on/off */
  int32_t pad0;
  double gain_log;            /* ln(10^(small_signal_gain_dB / 10)) */
  double E_sat;               /* nJ */
  double gain_length;         /* amplifier length = fibre length, km */
  const double* gain_profile; /* [n] spectral gain profile (FFT order) */
  /* Yb two-level gain, Amplifier2LevelModel (pyofss/modules/amplifier.py:178-379);
   * excludes gain_on.  Every linear-operator call of the solver sets the inversion
   *   n2 = (yb_pump_ratio Pp / yb_pump_sat + sum_k yb_w_ratio[k] |X_k|^2)
   *      / (1 + Pp / yb_pump_sat + sum_k yb_w_sat[k] |X_k|^2)
   * from the spectrum X = n fft(x) (pyofss fft) of its argument x, applies the gain
   * exp(500 h (n2 yb_alpha[k] - yb_eta[k])) over the call's step h (km) and advances
   * the pump power Pp <- Pp exp(1000 h (n2 yb_pump_alpha - yb_pump_eta)). */
  int32_t yb_on;
  int32_t pad1;
  double yb_pump_w;           /* Pp_0: pump power entering the fibre, W */
  double yb_pump_sat;         /* Psat_p, W */
  double yb_pump_ratio;       /* sigma12_p / (sigma12_p + sigma21_p) */
  double yb_pump_alpha;       /* alpha_p N, 1/m */
  double yb_pump_eta;         /* eta_p, 1/m */
  const double* yb_alpha;     /* [n] alpha_s N = (sigma12_s + sigma21_s) rho_s N, 1/m (FFT order) */
  const double* yb_eta;       /* [n] eta_s = sigma12_s rho_s N, 1/m (FFT order) */
  const double* yb_w_ratio;   /* [n] ratio_s / Psat_s * dt / (n Tr), 0 where NaN (FFT order) */
  const double* yb_w_sat;     /* [n] 1 / Psat_s * dt / (n Tr), 0 where NaN (FFT order) */
} gnlse_grid_desc;

/* One propagation (one field through one fibre). */
typedef struct {
  int32_t grid;               /* index into the grid array */
  int32_t method;             /* GNLSE_RK4IP / GNLSE_SS_* (fixed step), GNLSE_ARK4IP */
  int32_t total_steps;        /* Fibre total_steps */
  int32_t traces;             /* Fibre traces (>= 1) */
  int32_t max_traces;         /* trace slots reserved for this instance (0: none) */
  int32_t pad0;
  double length;              /* km */
  double local_error;         /* adaptive tolerance */
  double h0;                  /* adaptive initial step, km; <= 0: the stepper's rule */
  double weight;              /* expected relative work (e.g. predicted attempts) used to
                                 start long propagations first; <= 0: the fibre length */
} gnlse_instance_desc;

typedef struct {
  double z;                   /* distance reached, km */
  double h;                   /* next step size, km */
  double delta_last;          /* last relative local error estimate */
  double energy_in, energy_out;      /* FP64 Parseval energy, nJ */
  double photons_in, photons_out;    /* FP64 photon number */
  int64_t attempts;           /* step attempts (adaptive) / steps (fixed) */
  int64_t accepted, rejected;
  int64_t evals;              /* RK4IP evaluations (3 per adaptive attempt) */
  int64_t steps;              /* accepted steps */
  int32_t status;             /* GNLSE_OK / error code / GNLSE_RUNNING */
  int32_t ntraces;            /* traces written */
  int32_t trace_overflow;     /* 1 if traces were dropped for lack of slots */
  int32_t finished;           /* 1 once the output field has been written */
  double pump_w;              /* Yb gain: pump power reached (Amplifier2LevelModel.Pp), W */
} gnlse_stats;

typedef struct gnlse_plan gnlse_plan;

int gnlse_abi_version(void);
const char* gnlse_status_string(int status);

/* Build device tables and scratch for n_instances propagations over n_grids
 * grids with the given precision (GNLSE_FP32, GNLSE_FP64 or GNLSE_MIXED). */
int gnlse_plan_create(int precision, int n_grids, const gnlse_grid_desc* grids,
                      int n_instances, const gnlse_instance_desc* instances,
                      gnlse_plan** plan_out);
int gnlse_plan_destroy(gnlse_plan* plan);

/* Layout of the caller's buffers: instance i's field occupies complex
 * elements [field_offset(i), field_offset(i) + n_i); its trace slots occupy
 * complex elements [trace_offset(i), trace_offset(i) + max_traces_i * n_i)
 * and its trace z values doubles [trace_z_offset(i), + max_traces_i). */
int64_t gnlse_plan_field_elems(const gnlse_plan* plan);
int64_t gnlse_plan_field_offset(const gnlse_plan* plan, int instance);
int64_t gnlse_plan_trace_elems(const gnlse_plan* plan);
int64_t gnlse_plan_trace_offset(const gnlse_plan* plan, int instance);
int64_t gnlse_plan_trace_z_elems(const gnlse_plan* plan);
int64_t gnlse_plan_trace_z_offset(const gnlse_plan* plan, int instance);
int64_t gnlse_plan_scratch_bytes(const gnlse_plan* plan);

/* Mark every instance as not started (the next propagate starts from the
 * fields it is given). */
int gnlse_reset(gnlse_plan* plan, void* stream);

/* Propagate all instances, in place on d_fields (device, time domain).
 * max_attempts > 0 bounds the attempts each instance may spend in this call;
 * unfinished instances report GNLSE_RUNNING and continue on the next call
 * (checkpoint / resume between calls).  Asynchronous on `stream`. */
int gnlse_propagate(gnlse_plan* plan, void* d_fields, void* d_traces, double* d_trace_z,
                    int64_t max_attempts, void* stream);

/* Same, from and to host memory: copies the fields in, propagates to the end
 * and copies the fields out (synchronous).  h_in and h_out may alias. */
int gnlse_propagate_host(gnlse_plan* plan, const void* h_in, void* h_out, void* stream);

/* Kernel timing.  With timing enabled every propagate records CUDA events
 * around each launch class (one kernel launch per distinct points-per-CTA and
 * cluster size) on the stream that class is launched on.  gnlse_class_times
 * waits for the last propagate's events and reports, per class, log2 of the
 * points per CTA, the cluster size, the number of instances and the kernel
 * duration in ms; it returns the number of classes (or a negative status). */
int gnlse_set_timing(gnlse_plan* plan, int enable);
int gnlse_class_times(gnlse_plan* plan, int max_classes, int32_t* logm, int32_t* cluster,
                      int32_t* count, double* ms);

/* Instance indices in launch order (n_instances entries): launch k of
 * gnlse_class_times covers the next count[k] entries. */
int gnlse_class_order(gnlse_plan* plan, int32_t* order);

/* Name of the CUDA error behind the calling thread's last GNLSE_CUDA_ERROR or
 * GNLSE_OUT_OF_MEMORY status ("none" before any). */
const char* gnlse_last_cuda_error(void);

/* Launch-class autotuning.  No counterpart in the reference (pyofss has no
 * launch configuration).  A class is a compiled (precision, points per CTA,
 * cluster size) instantiation; gnlse_class_supported tells whether one exists.
 * gnlse_set_class_cost records a measured SM time (us) per attempt of one field
 * in that class (sm_us <= 0 clears it); plans created afterwards choose each
 * instance's class from these measurements instead of the built-in GB300 table
 * (process-wide, thread-safe).  pyofsschanged_gb300.autotune measures them. */
int gnlse_class_supported(int precision, int log2_points_per_cta, int cluster);
int gnlse_set_class_cost(int precision, int log2_points_per_cta, int cluster, double sm_us);

/* Phase cycle counters of builds compiled with GNLSE_PROF=1 (8 per instance:
 * transforms, stage loops, exp(hD) tables, whole kernel); GNLSE_UNSUPPORTED
 * in normal builds.  Synchronises the device. */
int gnlse_profile_counters(gnlse_plan* plan, long long* out);

/* Record the accepted steps of adaptive instance `instance` on the following propagate
 * calls: entry k of d_steps (device, 2 * capacity doubles) is (z, h) of accepted step k,
 * the z reached and the step size used, as Stepper.adaptive_stepper appends them to
 * Storage.step_sizes (pyofss/modules/stepper.py:339-345; pyofss keeps only the steps
 * that store a trace, the log keeps every one).  gnlse_stats.steps counts them; steps
 * beyond `capacity` are not recorded.  capacity 0 stops the log.  Synchronous. */
int gnlse_set_step_log(gnlse_plan* plan, int instance, double* d_steps, int64_t capacity);

/* Replay: ARK4IP instance `instance` takes its step sizes from d_h (device, n doubles,
 * e.g. a step log) and accepts every attempt, ending after n steps; the step-doubling
 * error estimate is still formed (gnlse_stats.delta_last).  The oracle's
 * adaptive(replay=...) does the same on the CPU.  No counterpart in the reference's
 * stepper: it separates the effect of arithmetic precision on a propagation from that of
 * the step-size controller's decisions.  n 0 returns to the controller.  Synchronous. */
int gnlse_set_replay(gnlse_plan* plan, int instance, const double* d_h, int64_t n);

/* Copy per-instance statistics to host memory (synchronises `stream`). */
int gnlse_get_stats(gnlse_plan* plan, gnlse_stats* out, void* stream);

/* Propagate one complex64 field of 256..4096 points (power of two) without
 * allocating any memory.  No counterpart in the reference: pyofss has no GPU
 * path of this kind.  It serves callers that must not allocate device memory
 * while they propagate -- a host loop sharing the GPU with latency-critical
 * work (cudaMalloc/cudaFree synchronise the device), or a process whose device
 * memory is owned by another allocator or quota.  Tables, scratch and control
 * state live in one file-scope device array of 585 KiB that every GPU loading
 * the library keeps until exit; the caller passes the grid's host tables, the
 * instance description (max_traces must be 0) and the field d_field (device,
 * in place).  Larger grids and the Yb model return GNLSE_UNSUPPORTED.  All calls share the
 * array: calls whose GPU work overlaps (other streams or threads) race and
 * must be serialised by the caller.  The first call on each device looks up
 * the array's address.  The call waits for its host-to-device table copies;
 * stats_out (optional) waits for the result. */
int gnlse_propagate_noalloc(const gnlse_grid_desc* grid, const gnlse_instance_desc* instance,
                            void* d_field, gnlse_stats* stats_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GNLSE_H */
