// Shared host/device descriptors of the GNLSE engine.  Plain C structs: they
// cross the boundary between the C-ABI layer and the kernels only, never the
// public ABI (include/gnlse.h), which has its own descriptor types.
#pragma once
#include <stdint.h>

namespace gnlse {

// Per grid (one Domain + one set of fibre operators).  All spectral tables are
// stored in the cluster-permuted layout: entry a = c*M + k2 holds frequency
// index k = c + C*k2 (FFT order), where C is the cluster size and M = N/C.
struct GridDev {
  const double* beta;   // [N] sum_n beta_n (w-w0)^n/n!   (1/km), FP64
  const void* Kr;       // [N] real: gamma * (1 + omega * s)
  // Hp, lor and lor2 of a grid without Raman / gain / the Yb model point at another
  // table of the same type and length (read only under the raman and gain flags)
  const void* Hp;       // [N] complex: fft(h_R) * window_t / N
  const void* lor;      // [N] real: gain profile (Yb model: alpha_s N, 1/m)
  const void* lor2;     // [N] real: Yb model eta_s (1/m)
  const double* ybw;    // [2N] FP64: Yb model inversion weights (w_ratio, w_sat) per entry
  const double* nu;     // [N] absolute frequency (THz), FP64, for photon number
  const void* tw;       // [N] natural order: exp(+2 pi i j / N) (cross-CTA pass)
  const void* twl;      // [M] natural order: exp(+2 pi i j / M) (per-CTA transform)
  const void* tw64;     // extended-state plans: FP64 copies of tw and twl
  const void* twl64;
  const void* twp;      // per-pass twiddle rows of the M-point transform (gnlse_twiddle.h)
  const void* twp64;    // extended-state plans: FP64 copy of twp
  const void* cis_df;   // extended-state plans: [1024] double-float cis(j pi / 512)
  int n, logm, C, raman;
  int gain, pad0;       // gain 1: saturable amplifier, 2: Yb two-level model
  double alpha;         // 1/km, linear attenuation
  double fR;            // Raman fraction
  double gain_log;      // ln(10^(gain_dB/10))
  double E_sat;         // nJ
  double gain_len;      // km (amplifier length = fibre length)
  double dt;            // ps
  double window_t;      // ps
  double yb_pp0, yb_psat_p, yb_ratio_p, yb_alpha_p, yb_eta_p;  // Yb pump (W, W, -, 1/m, 1/m)
};

struct InstDev {
  int grid;             // index into GridDev array
  int method;           // 0: fixed-step RK4IP, 1: adaptive (ARK4IP)
  int total_steps;      // fixed-step count / adaptive initial-step rule
  int traces;           // pyofss 'traces' argument
  int max_traces;       // capacity of this instance's trace slots
  int pad0;
  double length;        // km
  double tol;           // local error (adaptive)
  double h0;            // initial step (adaptive), km
  long long field_off;  // element offset of the time-domain field (in/out)
  long long scratch_off;// element offset of the 8*N scratch block
  long long trace_off;  // element offset of max_traces*N trace slots
  long long tracez_off; // index of this instance's first trace z value
  double* step_log;     // adaptive: accepted steps (z, h), 2 doubles each (null: none)
  const double* replay; // adaptive RK4IP: step sizes to follow, every attempt accepted (null: none)
  long long step_cap;   // capacity of step_log in steps
  long long replay_n;   // entries of replay
};

enum : int {
  ST_OK = 0, ST_SMALL_STEP = 1, ST_SUITABLE_STEP = 2, ST_MAX_STEPS = 3,
  ST_BAD_ARG = 4, ST_RUNNING = 8
};

struct InstState {
  double z, h, z_ignore, delta_last;
  double E_in, E_out, Nph_in, Nph_out;
  double cache_eA, cache_eN;  // gain energies of the cached state
  double cache_y[4];          // Yb model: inversion sums of the cached state and its N(A)
  double pp;                  // Yb model: pump power, W
  long long attempts, accepted, rejected, evals, steps, ffts;
  int status, ntraces, phase, sidx;
  int ma_valid, ta, trace_overflow, pad0;
};

struct KParams {
  const InstDev* inst;
  InstState* state;
  const int* order;     // instance ids handled by this launch (one per cluster)
  int n_order;
  int pad0;
  const GridDev* grids;
  void* fields;         // base of time-domain fields (complex R)
  void* scratch;        // base of scratch (complex R)
  void* traces;         // base of trace slots (complex R)
  double* trace_z;      // trace z values, instance slots start at InstDev::tracez_off
  long long max_attempts;  // attempts this launch may spend per instance (<=0: unbounded)
  long long* prof;         // per-instance phase cycle counters (profiling builds only)
};

}  // namespace gnlse
