// C-ABI of the GNLSE engine: plan construction (device operator tables in the
// cluster-permuted layout), class dispatch and propagation driver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>

#include "../../include/gnlse.h"
#include "gnlse_launch.h"
#include "gnlse_twiddle.h"
#include "gnlse_types.h"

using namespace gnlse;

namespace {

// One kernel launch: the instances order[first, first + count) of one
// (points per CTA, cluster size) class at one start-priority level.
struct ClassRun {
  int logm, C;
  int first;  // offset into the order array
  int count;
  int level;  // 0 = longest predicted propagations (highest stream priority)
  int kinds;  // kernels its instances need: 1 RK4IP stage loop, 2 exponential split steps
};

// SM time (us) of one attempt of one field in class (logm, C), measured on
// GB300 in mixed precision with the GPU saturated by fields of that class;
// only ratios between classes are used.  Other classes: n log n scaling of the
// 4096-point single-CTA figure, plus half again for a cluster exchange.
// Measured costs set by the caller's autotuner (gnlse_set_class_cost) take
// precedence over the built-in table; process-wide, guarded by a mutex.
struct CostEntry { int precision, logm, C; double us; };
std::mutex g_cost_mu;
std::vector<CostEntry> g_cost;

bool tuned(int precision) {
  std::lock_guard<std::mutex> lk(g_cost_mu);
  for (const CostEntry& e : g_cost)
    if (e.precision == precision) return true;
  return false;
}

double sm_cost(int precision, int logm, int C) {
  {
    std::lock_guard<std::mutex> lk(g_cost_mu);
    for (const CostEntry& e : g_cost)
      if (e.precision == precision && e.logm == logm && e.C == C) return e.us;
  }
  struct Entry { int logm, C; double us; };
  static const Entry tab[] = {{12, 1, 171.4}, {11, 2, 198.3},  {13, 1, 495.2},  {12, 2, 514.9},
                              {11, 4, 457.9}, {13, 2, 1496.0}, {12, 4, 1158.3}, {11, 8, 992.6}};
  for (const Entry& e : tab)
    if (e.logm == logm && e.C == C) return e.us;
  const double n = (double)(1 << logm) * C;
  return 190.5 * (n / 4096.0) * (std::log2(n) / 12.0) * (C > 1 ? 1.5 : 1.0);
}

struct GridHost {
  int n, logm, C;
  void* d_beta = nullptr;
  void* d_Kr = nullptr;
  void* d_Hp = nullptr;
  void* d_lor = nullptr;
  void* d_nu = nullptr;
  void* d_tw = nullptr;
  void* d_twl = nullptr;
  void* d_tw64 = nullptr;
  void* d_twl64 = nullptr;
  void* d_cis = nullptr;
  void* d_lor2 = nullptr;
  void* d_ybw = nullptr;
  void* d_twp = nullptr;
  void* d_twp64 = nullptr;
};

bool supported(int precision, int logm, int C) {
#define GNLSE_MATCH(PREC, R, L, CC) \
  if (precision == (PREC) && logm == (L) && C == (CC)) return true;
#define GNLSE_M32(R, L, CC) GNLSE_MATCH(GNLSE_FP32, R, L, CC)
#define GNLSE_M64(R, L, CC) GNLSE_MATCH(GNLSE_FP64, R, L, CC)
#define GNLSE_MMX(R, L, CC) GNLSE_MATCH(GNLSE_MIXED, R, L, CC)
#define GNLSE_MDF(R, L, CC) GNLSE_MATCH(GNLSE_DF, R, L, CC)
  GNLSE_CLASSES_F32(GNLSE_M32)
  GNLSE_CLASSES_F64(GNLSE_M64)
  GNLSE_CLASSES_MIX(GNLSE_MMX)
  GNLSE_CLASSES_DF(GNLSE_MDF)
#undef GNLSE_MDF
#undef GNLSE_M32
#undef GNLSE_M64
#undef GNLSE_MMX
#undef GNLSE_MATCH
  return false;
}

cudaError_t dispatch1(int precision, int logm, int C, const KParams& kp, int n, cudaStream_t s, int kind) {
#define GNLSE_CALL(PREC, XS, R, L, CC)                                                 \
  if (precision == (PREC) && logm == (L) && C == (CC))                                 \
    return kind == 0 ? launch_class<R, L, CC, XS>(kp, n, s) : launch_class_ss<R, L, CC, XS>(kp, n, s);
#define GNLSE_C32(R, L, CC) GNLSE_CALL(GNLSE_FP32, false, R, L, CC)
#define GNLSE_C64(R, L, CC) GNLSE_CALL(GNLSE_FP64, false, R, L, CC)
#define GNLSE_CMX(R, L, CC) GNLSE_CALL(GNLSE_MIXED, true, R, L, CC)
#define GNLSE_CDF(R, L, CC) GNLSE_CALL(GNLSE_DF, false, R, L, CC)
  GNLSE_CLASSES_F32(GNLSE_C32)
  GNLSE_CLASSES_F64(GNLSE_C64)
  GNLSE_CLASSES_MIX(GNLSE_CMX)
  GNLSE_CLASSES_DF(GNLSE_CDF)
#undef GNLSE_CDF
#undef GNLSE_C32
#undef GNLSE_C64
#undef GNLSE_CMX
#undef GNLSE_CALL
  return cudaErrorInvalidValue;
}

// the class's kernels its instances need, in one stream
cudaError_t dispatch(int precision, int logm, int C, const KParams& kp, int n, cudaStream_t s, int kinds) {
  cudaError_t e = cudaSuccess;
  if ((kinds & 1) && (e = dispatch1(precision, logm, C, kp, n, s, 0)) != cudaSuccess) return e;
  if ((kinds & 2) && (e = dispatch1(precision, logm, C, kp, n, s, 1)) != cudaSuccess) return e;
  return e;
}

int ilog2i(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

}  // namespace

struct gnlse_plan {
  int precision = 0;
  size_t vsize = 8;    // bytes per field element
  size_t ssize = 8;    // bytes per scratch element
  int device = 0;
  std::vector<GridHost> grids;
  std::vector<InstDev> inst;
  std::vector<int> order;
  std::vector<ClassRun> classes;
  GridDev* d_grids = nullptr;
  InstDev* d_inst = nullptr;
  InstState* d_state = nullptr;
  int* d_order = nullptr;
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  int64_t field_elems = 0, trace_elems = 0, tracez_elems = 0;
  std::vector<int64_t> field_off, trace_off, tracez_off;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev;
  cudaEvent_t fork = nullptr;
  bool timing = false;
  long long* d_prof = nullptr;  // phase cycle counters (profiling builds)
  std::vector<cudaEvent_t> t0, t1;
  // host-buffer entry point staging
  void* d_io = nullptr;
  void* d_tr = nullptr;
  double* d_trz = nullptr;
  std::vector<void*> allocs;
};

namespace {

// Timing event record: under stream capture as an external event node (so the
// graph's replays record it), otherwise a plain record.
cudaError_t record_timing(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return e;
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

// name of the CUDA error behind the last GNLSE_CUDA_ERROR / GNLSE_OUT_OF_MEMORY
thread_local const char* g_last_cuda_error = "none";

int cuda_fail(cudaError_t e) {
  g_last_cuda_error = cudaGetErrorName(e);
  if (e == cudaErrorMemoryAllocation) return GNLSE_OUT_OF_MEMORY;
  return GNLSE_CUDA_ERROR;
}

template <class T>
cudaError_t upload(gnlse_plan* p, const std::vector<T>& h, void** d) {
  cudaError_t e = cudaMalloc(d, h.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  p->allocs.push_back(*d);
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Complex tables of double-float plans in the engine's layout {re.hi, im.hi, re.lo, im.lo}
// (gnlse_dd.cuh): each complex entry is built as two ddf (re, im) and rearranged.
template <class R>
void pack_complex(std::vector<R>& v) {
  if constexpr (std::is_same<R, ddf>::value) {
    for (size_t i = 0; i + 1 < v.size(); i += 2) {
      const ddf r = v[i], m = v[i + 1];
      v[i] = ddf(r.hi, m.hi);
      v[i + 1] = ddf(r.lo, m.lo);
    }
  }
}

// R: the transform element's real type (float, double or the double-float ddf);
// extended: mixed-precision plans (FP64 boundary twiddles); want_cis: the
// double-float cis(j pi / 512) table of the exp(hD) factors (mixed and df plans)
template <class R>
cudaError_t build_grid_tables(gnlse_plan* p, const gnlse_grid_desc& gd, GridHost& gh, GridDev& dv,
                              bool extended, bool want_cis) {
  const int n = gd.n, C = gh.C, M = n / C;
  auto perm = [&](int a) { return (a % M) * C + a / M; };  // slot a = c*M + k2  <-  k = c + C*k2
  std::vector<double> beta(n), nu(n);
  std::vector<R> Kr(n), lor, lor2, Hp;
  std::vector<double> ybw;
  std::vector<R> tw(2 * (size_t)n), twl(2 * (size_t)M);
  for (int a = 0; a < n; ++a) {
    const int k = perm(a);
    beta[a] = gd.beta_w[k];
    nu[a] = gd.nu ? gd.nu[k] : 1.0;
    Kr[a] = (R)(gd.gamma * (gd.ss_w ? gd.ss_w[k] : 1.0));
  }
  const bool raman = gd.hR_re != nullptr;
  if (raman) {
    Hp.resize(2 * (size_t)n);
    for (int a = 0; a < n; ++a) {
      const int k = perm(a);
      Hp[2 * a] = (R)(gd.hR_re[k] / n);
      Hp[2 * a + 1] = (R)((gd.hR_im ? gd.hR_im[k] : 0.0) / n);
    }
  }
  if (gd.gain_on) {
    lor.resize(n);
    for (int a = 0; a < n; ++a) lor[a] = (R)(gd.gain_profile ? gd.gain_profile[perm(a)] : 1.0);
  }
  const bool yb = gd.yb_on != 0;
  if (yb) {  // Yb model: lor = alpha_s N, lor2 = eta_s, inversion weights in FP64
    lor.resize(n);
    lor2.resize(n);
    ybw.resize(2 * (size_t)n);
    for (int a = 0; a < n; ++a) {
      const int k = perm(a);
      lor[a] = (R)gd.yb_alpha[k];
      lor2[a] = (R)gd.yb_eta[k];
      ybw[2 * (size_t)a] = gd.yb_w_ratio[k];
      ybw[2 * (size_t)a + 1] = gd.yb_w_sat[k];
    }
  }
  // exp(+2 pi i j / n), argument formed in long double
  for (int j = 0; j < n; ++j) {
    const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)j / (long double)n;
    tw[2 * (size_t)j] = (R)std::cos((double)ang);
    tw[2 * (size_t)j + 1] = (R)std::sin((double)ang);
  }
  for (int j = 0; j < M; ++j) {
    twl[2 * (size_t)j] = tw[2 * (size_t)j * C];
    twl[2 * (size_t)j + 1] = tw[2 * (size_t)j * C + 1];
  }
  pack_complex(tw);
  pack_complex(twl);
  pack_complex(Hp);
  // per-pass twiddle rows of the M-point transform
  const int rb = std::is_same<R, ddf>::value ? GNLSE_DF_RADIX_BITS : GNLSE_RADIX_BITS;  // the engine's radix
  const int logm = gh.logm, ntwp = twp_size(logm, rb);
  std::vector<R> twp(2 * (size_t)ntwp);
  std::vector<double> twp64(extended ? 2 * (size_t)ntwp : 0);
  for (int e2 = 0; e2 < ntwp; ++e2) {
    const long double ang = 2.0L * 3.14159265358979323846264338327950288L *
                            (long double)twp_exponent(logm, rb, e2) / (long double)M;
    const double c = (double)cosl(ang), sn = (double)sinl(ang);
    twp[2 * (size_t)e2] = (R)c;
    twp[2 * (size_t)e2 + 1] = (R)sn;
    if (extended) {
      twp64[2 * (size_t)e2] = c;
      twp64[2 * (size_t)e2 + 1] = sn;
    }
  }
  pack_complex(twp);
  cudaError_t e;
  if ((e = upload(p, twp, &gh.d_twp)) != cudaSuccess) return e;
  if (extended && (e = upload(p, twp64, &gh.d_twp64)) != cudaSuccess) return e;
  const long double PI_L = 3.14159265358979323846264338327950288L;
  if (want_cis) {
    // double-float cis(j pi/512), j < 1024, of the exp(hD) factors: float4
    // {cos hi, sin hi, cos lo, sin lo}
    std::vector<float> cis(4 * 1024);
    for (int j = 0; j < 1024; ++j) {
      const long double ang = PI_L * (long double)j / 512.0L;
      const long double c = cosl(ang), sn = sinl(ang);
      const float ch = (float)c, sh = (float)sn;
      cis[4 * j + 0] = ch;
      cis[4 * j + 1] = sh;
      cis[4 * j + 2] = (float)(c - (long double)ch);
      cis[4 * j + 3] = (float)(sn - (long double)sh);
    }
    if ((e = upload(p, cis, &gh.d_cis)) != cudaSuccess) return e;
  }
  if (extended) {
    // FP64 twiddles for the boundary transforms
    std::vector<double> tw64(2 * (size_t)n), twl64(2 * (size_t)M);
    for (int j = 0; j < n; ++j) {
      const long double ang = 2.0L * PI_L * (long double)j / (long double)n;
      tw64[2 * (size_t)j] = (double)std::cos((double)ang);
      tw64[2 * (size_t)j + 1] = (double)std::sin((double)ang);
    }
    for (int j = 0; j < M; ++j) {
      twl64[2 * (size_t)j] = tw64[2 * (size_t)j * C];
      twl64[2 * (size_t)j + 1] = tw64[2 * (size_t)j * C + 1];
    }
    if ((e = upload(p, tw64, &gh.d_tw64)) != cudaSuccess) return e;
    if ((e = upload(p, twl64, &gh.d_twl64)) != cudaSuccess) return e;
  }
  if ((e = upload(p, twl, &gh.d_twl)) != cudaSuccess) return e;
  if ((e = upload(p, beta, &gh.d_beta)) != cudaSuccess) return e;
  if ((e = upload(p, nu, &gh.d_nu)) != cudaSuccess) return e;
  if ((e = upload(p, Kr, &gh.d_Kr)) != cudaSuccess) return e;
  if ((e = upload(p, tw, &gh.d_tw)) != cudaSuccess) return e;
  if (raman && (e = upload(p, Hp, &gh.d_Hp)) != cudaSuccess) return e;
  if ((gd.gain_on || yb) && (e = upload(p, lor, &gh.d_lor)) != cudaSuccess) return e;
  if (yb && (e = upload(p, lor2, &gh.d_lor2)) != cudaSuccess) return e;
  if (yb && (e = upload(p, ybw, &gh.d_ybw)) != cudaSuccess) return e;
  dv.beta = (const double*)gh.d_beta;
  dv.Kr = gh.d_Kr;
  // Tables a grid does not use point at tables of the same type and length, never at
  // null: the kernels read them only under their flags (raman, gain), but the compiler
  // may issue such a read-only load ahead of its branch.
  dv.Hp = raman ? gh.d_Hp : gh.d_tw;
  dv.lor = (gd.gain_on || yb) ? gh.d_lor : gh.d_Kr;
  dv.lor2 = yb ? gh.d_lor2 : gh.d_Kr;
  dv.ybw = yb ? (const double*)gh.d_ybw : nullptr;
  dv.nu = (const double*)gh.d_nu;
  dv.tw = gh.d_tw;
  dv.twl = gh.d_twl;
  dv.tw64 = gh.d_tw64;
  dv.twl64 = gh.d_twl64;
  dv.cis_df = gh.d_cis;
  dv.twp = gh.d_twp;
  dv.twp64 = gh.d_twp64;
  dv.n = n;
  dv.logm = gh.logm;
  dv.C = C;
  dv.raman = raman ? 1 : 0;
  dv.gain = yb ? 2 : (gd.gain_on ? 1 : 0);
  dv.alpha = gd.alpha;
  dv.fR = gd.f_R;
  dv.gain_log = gd.gain_log;
  dv.E_sat = gd.E_sat;
  dv.gain_len = gd.gain_length;
  dv.dt = gd.dt;
  dv.window_t = gd.window_t;
  dv.yb_pp0 = yb ? gd.yb_pump_w : 0.0;
  dv.yb_psat_p = yb ? gd.yb_pump_sat : 1.0;
  dv.yb_ratio_p = yb ? gd.yb_pump_ratio : 0.0;
  dv.yb_alpha_p = yb ? gd.yb_pump_alpha : 0.0;
  dv.yb_eta_p = yb ? gd.yb_pump_eta : 0.0;
  return cudaSuccess;
}

void free_plan(gnlse_plan* p) {
  for (void* a : p->allocs) cudaFree(a);
  for (auto s : p->side) cudaStreamDestroy(s);
  for (auto e : p->ev) cudaEventDestroy(e);
  for (auto e : p->t0) cudaEventDestroy(e);
  for (auto e : p->t1) cudaEventDestroy(e);
  if (p->fork) cudaEventDestroy(p->fork);
  delete p;
}

}  // namespace

extern "C" {

int gnlse_abi_version(void) { return GNLSE_ABI_VERSION; }

const char* gnlse_status_string(int s) {
  switch (s) {
    case GNLSE_OK: return "ok";
    case GNLSE_SMALL_STEP: return "Step size is extremely small";
    case GNLSE_SUITABLE_STEP: return "Failed to set suitable step-size";
    case GNLSE_MAX_STEPS: return "Failed to complete with maximum steps allocated";
    case GNLSE_BAD_ARGUMENT: return "bad argument";
    case GNLSE_CUDA_ERROR: return "CUDA error";
    case GNLSE_UNSUPPORTED: return "unsupported grid size / precision / cluster size";
    case GNLSE_OUT_OF_MEMORY: return "out of device memory";
    case GNLSE_RUNNING: return "running (attempt budget reached)";
    default: return "unknown status";
  }
}

const char* gnlse_last_cuda_error(void) { return g_last_cuda_error; }

int gnlse_class_supported(int precision, int log2_points_per_cta, int cluster) {
  return supported(precision, log2_points_per_cta, cluster) ? 1 : 0;
}

int gnlse_set_class_cost(int precision, int log2_points_per_cta, int cluster, double sm_us) {
  if (precision != GNLSE_FP32 && precision != GNLSE_FP64 && precision != GNLSE_MIXED && precision != GNLSE_DF)
    return GNLSE_BAD_ARGUMENT;
  if (!supported(precision, log2_points_per_cta, cluster)) return GNLSE_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_cost_mu);
  for (size_t k = 0; k < g_cost.size(); ++k) {
    CostEntry& e = g_cost[k];
    if (e.precision == precision && e.logm == log2_points_per_cta && e.C == cluster) {
      if (sm_us > 0) e.us = sm_us;
      else g_cost.erase(g_cost.begin() + (long)k);
      return GNLSE_OK;
    }
  }
  if (sm_us > 0) g_cost.push_back({precision, log2_points_per_cta, cluster, sm_us});
  return GNLSE_OK;
}

int gnlse_plan_create(int precision, int n_grids, const gnlse_grid_desc* grids, int n_instances,
                      const gnlse_instance_desc* instances, gnlse_plan** plan_out) {
  if (!plan_out || !grids || !instances || n_grids <= 0 || n_instances <= 0) return GNLSE_BAD_ARGUMENT;
  if (precision != GNLSE_FP32 && precision != GNLSE_FP64 && precision != GNLSE_MIXED && precision != GNLSE_DF)
    return GNLSE_BAD_ARGUMENT;
  *plan_out = nullptr;
  gnlse_plan* p = new (std::nothrow) gnlse_plan();
  if (!p) return GNLSE_OUT_OF_MEMORY;
  p->precision = precision;
  p->vsize = precision == GNLSE_FP32 ? 8 : 16;
  p->ssize = precision == GNLSE_FP32 ? 8 : 16;
  cudaGetDevice(&p->device);
  // ---- grids: validation and the cluster sizes each may run with -------------
  std::vector<std::vector<int>> cands(n_grids);  // candidate cluster sizes, fixed or auto
  std::vector<int> tput(n_grids), lat(n_grids);   // throughput / latency choice (auto grids)
  for (int i = 0; i < n_grids; ++i) {
    const gnlse_grid_desc& gd = grids[i];
    const int n = gd.n;
    if (n < 256 || (n & (n - 1)) != 0 || !gd.beta_w || !(gd.dt > 0) || !(gd.window_t > 0) ||
        (gd.gain_on && !(gd.E_sat > 0 && gd.gain_length > 0)) ||
        (gd.yb_on && (gd.gain_on || !gd.yb_alpha || !gd.yb_eta || !gd.yb_w_ratio || !gd.yb_w_sat ||
                      !(gd.yb_pump_sat > 0) || !(gd.yb_pump_w >= 0)))) {
      free_plan(p);
      return GNLSE_BAD_ARGUMENT;
    }
    if (gd.cluster != 0) {
      const int C = gd.cluster;
      if ((C != 1 && C != 2 && C != 4 && C != 8 && C != 16) || n % C != 0 ||
          !supported(precision, ilog2i(n / C), C)) {
        free_plan(p);
        return GNLSE_UNSUPPORTED;
      }
      tput[i] = lat[i] = C;
      continue;
    }
    if ((precision == GNLSE_FP64 || precision == GNLSE_DF) && !tuned(precision)) {
      // 16-byte elements: 4096 points per CTA, larger grids span a cluster
      const int C = n <= 4096 ? 1 : n / 4096;
      if (C > 16 || !supported(precision, ilog2i(n / C), C)) {
        free_plan(p);
        return GNLSE_UNSUPPORTED;
      }
      tput[i] = lat[i] = C;
      continue;
    }
    // complex64 transforms: the cheapest class in SM time, and the class with the
    // least SM time per CTA (attempt latency) among those within 1.5x of it.
    // Slices of up to 4096 points per CTA only (8192-point CTAs fill an SM on
    // their own and pack badly beside the other classes of an ensemble),
    // except for grids above 8 x 4096 points.
    const int mcap = n > 8 * 4096 ? 13 : 12;
    int best = 0, fast = 0;
    for (int C = 1; C <= 16; C *= 2) {
      const int logm = ilog2i(n / C);
      if (n / C < 256 || logm > mcap || !supported(precision, logm, C)) continue;
      if (!best || sm_cost(precision, logm, C) < sm_cost(precision, ilog2i(n / best), best)) best = C;
    }
    if (!best) {
      free_plan(p);
      return GNLSE_UNSUPPORTED;
    }
    const double cb = sm_cost(precision, ilog2i(n / best), best);
    for (int C = 1; C <= 16; C *= 2) {
      const int logm = ilog2i(n / C);
      if (n / C < 256 || logm > mcap || !supported(precision, logm, C) || sm_cost(precision, logm, C) > 1.5 * cb) continue;
      if (!fast || sm_cost(precision, logm, C) / C < sm_cost(precision, ilog2i(n / fast), fast) / fast) fast = C;
    }
    tput[i] = best;
    lat[i] = fast;
  }

  // ---- instances -------------------------------------------------------------
  p->inst.resize(n_instances);
  p->field_off.resize(n_instances);
  p->trace_off.resize(n_instances);
  p->tracez_off.resize(n_instances);
  int64_t foff = 0, soff = 0, toff = 0, zoff = 0;
  for (int i = 0; i < n_instances; ++i) {
    const gnlse_instance_desc& id = instances[i];
    // base method and the adaptive flag (split steps only; GNLSE_ARK4IP is adaptive RK4IP)
    const int bm = id.method & ~GNLSE_ADAPTIVE;
    const bool flagged = (id.method & GNLSE_ADAPTIVE) != 0;
    if (id.grid < 0 || id.grid >= n_grids || bm < GNLSE_RK4IP || bm > GNLSE_SS_AGRAWAL ||
        (flagged && bm < GNLSE_SS_SYM_RK4) ||
        id.total_steps < 1 || id.traces < 1 || id.max_traces < 0 || !(id.length >= 0) ||
        ((id.method == GNLSE_ARK4IP || flagged) && !(id.local_error > 0))) {
      free_plan(p);
      return GNLSE_BAD_ARGUMENT;
    }
    const bool split = bm >= GNLSE_SS_SYM_RK4;
    if (split && (grids[id.grid].gain_on || grids[id.grid].yb_on)) {
      free_plan(p);  // the split-step paths have no amplifier step
      return GNLSE_UNSUPPORTED;
    }
    if (bm >= GNLSE_SS_SYMMETRIC && bm <= GNLSE_SS_REDUCED && grids[id.grid].ss_w) {
      free_plan(p);  // exponential step with self-steepening (see gnlse.h)
      return GNLSE_UNSUPPORTED;
    }
    const int n = grids[id.grid].n;
    InstDev& d = p->inst[i];
    memset(&d, 0, sizeof(d));
    d.grid = id.grid;
    d.method = id.method;
    d.total_steps = id.total_steps;
    d.traces = id.traces;
    d.max_traces = id.max_traces;
    d.length = id.length;
    d.tol = id.local_error;
    double h0 = id.h0;
    if (!(h0 > 0)) {  // stepper.py:256-264
      h0 = id.traces > id.total_steps ? id.length / id.traces : id.length / id.total_steps;
      if (h0 > 1e-6) h0 = 1e-6;
    }
    d.h0 = h0;
    d.field_off = foff;
    d.scratch_off = soff;
    d.trace_off = toff;
    d.tracez_off = zoff;
    p->field_off[i] = foff;
    p->trace_off[i] = toff;
    p->tracez_off[i] = zoff;
    foff += n;
    soff += 8 * (int64_t)n;
    toff += (int64_t)id.max_traces * n;
    zoff += id.max_traces;
  }
  p->field_elems = foff;
  p->trace_elems = toff;
  p->tracez_elems = zoff;
  p->scratch_bytes = (size_t)soff * p->ssize;

  // ---- class of each instance and launch schedule -----------------------------
  // Work w_i = the caller's weight (expected attempts) or the fibre length.
  // Every instance starts in its grid's cheapest class; the makespan is about
  // max(total SM time / SMs, longest chain), with a chain's time ~ 3 w_i x SM
  // time per attempt / C (about three CTAs share an SM when the GPU is full).
  // Instances whose chain exceeds the work bound move, longest first, to the
  // lower-latency class of their grid while that still shortens the longest chain.
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
  if (nsm <= 0) nsm = 1;
  std::vector<int> icl(n_instances);
  std::vector<double> w(n_instances);
  auto icost = [&](int i, int C) { return sm_cost(precision, ilog2i(grids[instances[i].grid].n / C), C); };
  auto chain = [&](int i, int C) { return 3.0 * w[i] * icost(i, C) / C; };
  double work = 0.0;
  for (int i = 0; i < n_instances; ++i) {
    w[i] = instances[i].weight > 0 ? instances[i].weight : (p->inst[i].length > 0 ? p->inst[i].length : 1.0);
    icl[i] = tput[instances[i].grid];
    work += w[i] * icost(i, icl[i]) / nsm;
  }
  std::vector<int> ids(n_instances);
  for (int i = 0; i < n_instances; ++i) ids[i] = i;
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return chain(a, icl[a]) > chain(b, icl[b]); });
  for (int i : ids) {
    const int L = lat[instances[i].grid];
    if (chain(i, icl[i]) <= work) break;
    if (L == icl[i] || chain(i, L) >= chain(i, icl[i])) continue;
    work += w[i] * (icost(i, L) - icost(i, icl[i])) / nsm;
    icl[i] = L;
  }
  // device tables for every (grid, cluster size) pair in use
  std::vector<GridDev> gdev;
  std::vector<int> vgrid, vC;
  for (int i = 0; i < n_instances; ++i) {
    const int g = instances[i].grid;
    int v = 0;
    while (v < (int)vgrid.size() && !(vgrid[v] == g && vC[v] == icl[i])) ++v;
    if (v == (int)vgrid.size()) {
      vgrid.push_back(g);
      vC.push_back(icl[i]);
    }
    p->inst[i].grid = v;
  }
  p->grids.resize(vgrid.size());
  gdev.resize(vgrid.size());
  for (size_t v = 0; v < vgrid.size(); ++v) {
    const gnlse_grid_desc& gd = grids[vgrid[v]];
    GridHost& gh = p->grids[v];
    gh.n = gd.n;
    gh.C = vC[v];
    gh.logm = ilog2i(gd.n / gh.C);
    cudaError_t e = precision == GNLSE_FP64
                        ? build_grid_tables<double>(p, gd, gh, gdev[v], false, false)
                        : precision == GNLSE_DF
                              ? build_grid_tables<ddf>(p, gd, gh, gdev[v], false, true)
                              : build_grid_tables<float>(p, gd, gh, gdev[v], precision == GNLSE_MIXED,
                                                         precision == GNLSE_MIXED);
    if (e != cudaSuccess) {
      free_plan(p);
      return cuda_fail(e);
    }
  }
  // Launches: each (level, class) pair is one launch on its own stream, and
  // levels map to decreasing stream priorities, so long propagations of every
  // grid size get SMs first.  With three levels, instances whose chain is
  // within 60% of the longest start at level 0, down to 30% at level 1;
  // with two, the split is at 50%.  Levels are limited so that the launches
  // need at most 8 streams: the device multiplexes streams onto 8 hardware
  // queues by default, and a launch sharing a queue waits behind the other.
  std::vector<double> dur(n_instances);
  double dmax = 0.0;
  for (int i = 0; i < n_instances; ++i) {
    dur[i] = chain(i, icl[i]);
    dmax = std::max(dmax, dur[i]);
  }
  int nclass = 0;
  {
    std::vector<int> seen;
    for (int i = 0; i < n_instances; ++i) {
      const GridHost& g = p->grids[p->inst[i].grid];
      const int k = g.logm * 16 + g.C;
      if (std::find(seen.begin(), seen.end(), k) == seen.end()) seen.push_back(k);
    }
    nclass = (int)seen.size();
  }
  const int nlevels = std::max(1, std::min(3, 8 / std::max(1, nclass)));
  auto level = [&](int i) {
    if (nlevels == 3) return dur[i] >= 0.6 * dmax ? 0 : (dur[i] >= 0.3 * dmax ? 1 : 2);
    if (nlevels == 2) return dur[i] >= 0.5 * dmax ? 0 : 1;
    return 0;
  };
  auto cls = [&](int i) { const GridHost& g = p->grids[p->inst[i].grid]; return g.logm * 16 + g.C; };
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) {
    if (level(a) != level(b)) return level(a) < level(b);
    if (cls(a) != cls(b)) return cls(a) < cls(b);
    return dur[a] > dur[b];
  });
  p->order = ids;
  for (int k = 0; k < n_instances;) {
    int j = k;
    while (j < n_instances && cls(ids[j]) == cls(ids[k]) && level(ids[j]) == level(ids[k])) ++j;
    const GridHost& g = p->grids[p->inst[ids[k]].grid];
    int kinds = 0;
    for (int q = k; q < j; ++q) kinds |= p->inst[ids[q]].method <= GNLSE_SS_SYM_RK4 ? 1 : 2;
    p->classes.push_back({g.logm, g.C, k, j - k, level(ids[k]), kinds});
    k = j;
  }
  cudaError_t e;
  void* ptr = nullptr;
  if ((e = upload(p, gdev, &ptr)) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  p->d_grids = (GridDev*)ptr;
  if ((e = upload(p, p->inst, &ptr)) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  p->d_inst = (InstDev*)ptr;
  if ((e = upload(p, p->order, &ptr)) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  p->d_order = (int*)ptr;
  if ((e = cudaMalloc(&ptr, sizeof(InstState) * n_instances)) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  p->allocs.push_back(ptr);
  p->d_state = (InstState*)ptr;
  cudaMemset(p->d_state, 0, sizeof(InstState) * n_instances);
  if ((e = cudaMalloc(&p->d_scratch, p->scratch_bytes)) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  p->allocs.push_back(p->d_scratch);
#if GNLSE_PROF
  if ((e = cudaMalloc((void**)&p->d_prof, sizeof(long long) * 8 * n_instances)) != cudaSuccess) {
    free_plan(p);
    return cuda_fail(e);
  }
  p->allocs.push_back(p->d_prof);
  cudaMemset(p->d_prof, 0, sizeof(long long) * 8 * n_instances);
#endif
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  for (size_t c = 0; c < p->classes.size(); ++c) {
    cudaStream_t s;
    cudaEvent_t ev;
    // level 0 -> greatest priority (numerically lowest), then one step per level
    int prio = prio_greatest + p->classes[c].level;
    if (prio > prio_least) prio = prio_least;
    if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      free_plan(p);
      return GNLSE_CUDA_ERROR;
    }
    p->side.push_back(s);
    p->ev.push_back(ev);
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      free_plan(p);
      return GNLSE_CUDA_ERROR;
    }
    p->t0.push_back(a);
    p->t1.push_back(b);
  }
  if (cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming) != cudaSuccess) {
    free_plan(p);
    return GNLSE_CUDA_ERROR;
  }
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) { free_plan(p); return cuda_fail(e); }
  *plan_out = p;
  return GNLSE_OK;
}

int gnlse_plan_destroy(gnlse_plan* p) {
  if (!p) return GNLSE_BAD_ARGUMENT;
  cudaDeviceSynchronize();
  free_plan(p);
  return GNLSE_OK;
}

int64_t gnlse_plan_field_elems(const gnlse_plan* p) { return p ? p->field_elems : -1; }
int64_t gnlse_plan_field_offset(const gnlse_plan* p, int i) {
  return (p && i >= 0 && i < (int)p->inst.size()) ? p->field_off[i] : -1;
}
int64_t gnlse_plan_trace_elems(const gnlse_plan* p) { return p ? p->trace_elems : -1; }
int64_t gnlse_plan_trace_offset(const gnlse_plan* p, int i) {
  return (p && i >= 0 && i < (int)p->inst.size()) ? p->trace_off[i] : -1;
}
int64_t gnlse_plan_trace_z_elems(const gnlse_plan* p) { return p ? p->tracez_elems : -1; }
int64_t gnlse_plan_trace_z_offset(const gnlse_plan* p, int i) {
  return (p && i >= 0 && i < (int)p->inst.size()) ? p->tracez_off[i] : -1;
}
int64_t gnlse_plan_scratch_bytes(const gnlse_plan* p) { return p ? (int64_t)p->scratch_bytes : -1; }

int gnlse_reset(gnlse_plan* p, void* stream) {
  if (!p) return GNLSE_BAD_ARGUMENT;
  cudaError_t e = cudaMemsetAsync(p->d_state, 0, sizeof(InstState) * p->inst.size(), (cudaStream_t)stream);
  return e == cudaSuccess ? GNLSE_OK : cuda_fail(e);
}

int gnlse_propagate(gnlse_plan* p, void* d_fields, void* d_traces, double* d_trace_z,
                    int64_t max_attempts, void* stream) {
  if (!p || !d_fields) return GNLSE_BAD_ARGUMENT;
  if (p->trace_elems > 0 && (!d_traces || !d_trace_z)) return GNLSE_BAD_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  KParams kp = {};
  kp.inst = p->d_inst;
  kp.state = p->d_state;
  kp.grids = p->d_grids;
  kp.fields = d_fields;
  kp.scratch = p->d_scratch;
  kp.traces = d_traces;
  kp.trace_z = d_trace_z;
  kp.max_attempts = max_attempts;
  kp.prof = p->d_prof;
  cudaError_t e;
  // Under stream capture the timing events are recorded as external events, so
  // that they become event-record nodes of the graph and still time each replay
  // (a plain record during capture only expresses a dependency).
  if (p->classes.size() == 1) {
    const ClassRun& c = p->classes[0];
    kp.order = p->d_order + c.first;
    kp.n_order = c.count;
    if (p->timing && (e = record_timing(p->t0[0], s)) != cudaSuccess) return cuda_fail(e);
    e = dispatch(p->precision, c.logm, c.C, kp, c.count, s, c.kinds);
    if (e != cudaSuccess) return cuda_fail(e);
    if (p->timing && (e = record_timing(p->t1[0], s)) != cudaSuccess) return cuda_fail(e);
    return GNLSE_OK;
  }
  // several classes: fork onto side streams so they share the GPU, then join
  if ((e = cudaEventRecord(p->fork, s)) != cudaSuccess) return cuda_fail(e);
  for (size_t k = 0; k < p->classes.size(); ++k) {
    const ClassRun& c = p->classes[k];
    if ((e = cudaStreamWaitEvent(p->side[k], p->fork, 0)) != cudaSuccess) return cuda_fail(e);
    kp.order = p->d_order + c.first;
    kp.n_order = c.count;
    if (p->timing && (e = record_timing(p->t0[k], p->side[k])) != cudaSuccess) return cuda_fail(e);
    if ((e = dispatch(p->precision, c.logm, c.C, kp, c.count, p->side[k], c.kinds)) != cudaSuccess)
      return cuda_fail(e);
    if (p->timing && (e = record_timing(p->t1[k], p->side[k])) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaEventRecord(p->ev[k], p->side[k])) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaStreamWaitEvent(s, p->ev[k], 0)) != cudaSuccess) return cuda_fail(e);
  }
  return GNLSE_OK;
}

int gnlse_propagate_host(gnlse_plan* p, const void* h_in, void* h_out, void* stream) {
  if (!p || !h_in || !h_out) return GNLSE_BAD_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)p->field_elems * p->vsize;
  cudaError_t e;
  if (!p->d_io) {
    if ((e = cudaMalloc(&p->d_io, bytes)) != cudaSuccess) return cuda_fail(e);
    p->allocs.push_back(p->d_io);
    if (p->trace_elems > 0) {
      if ((e = cudaMalloc(&p->d_tr, (size_t)p->trace_elems * p->vsize)) != cudaSuccess) return cuda_fail(e);
      p->allocs.push_back(p->d_tr);
      if ((e = cudaMalloc((void**)&p->d_trz, sizeof(double) * p->tracez_elems)) != cudaSuccess) return cuda_fail(e);
      p->allocs.push_back(p->d_trz);
    }
  }
  if ((e = cudaMemcpyAsync(p->d_io, h_in, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) return cuda_fail(e);
  int rc = gnlse_reset(p, stream);
  if (rc != GNLSE_OK) return rc;
  rc = gnlse_propagate(p, p->d_io, p->d_tr, p->d_trz, 0, stream);
  if (rc != GNLSE_OK) return rc;
  if ((e = cudaMemcpyAsync(h_out, p->d_io, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e);
  return GNLSE_OK;
}

int gnlse_profile_counters(gnlse_plan* p, long long* out) {
  if (!p || !out) return GNLSE_BAD_ARGUMENT;
  if (!p->d_prof) return GNLSE_UNSUPPORTED;
  cudaDeviceSynchronize();
  if (cudaMemcpy(out, p->d_prof, sizeof(long long) * 8 * p->inst.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GNLSE_CUDA_ERROR;
  return GNLSE_OK;
}

int gnlse_set_timing(gnlse_plan* p, int enable) {
  if (!p) return GNLSE_BAD_ARGUMENT;
  p->timing = enable != 0;
  return GNLSE_OK;
}

int gnlse_class_times(gnlse_plan* p, int max_classes, int32_t* logm, int32_t* cluster,
                      int32_t* count, double* ms) {
  if (!p || max_classes < 0) return -GNLSE_BAD_ARGUMENT;
  const int nc = (int)p->classes.size();
  for (int k = 0; k < nc && k < max_classes; ++k) {
    float t = 0.f;
    if (p->timing) {
      if (cudaEventSynchronize(p->t1[k]) != cudaSuccess ||
          cudaEventElapsedTime(&t, p->t0[k], p->t1[k]) != cudaSuccess)
        return -GNLSE_CUDA_ERROR;
    }
    if (logm) logm[k] = p->classes[k].logm;
    if (cluster) cluster[k] = p->classes[k].C;
    if (count) count[k] = p->classes[k].count;
    if (ms) ms[k] = p->timing ? (double)t : 0.0;
  }
  return nc;
}

int gnlse_class_order(gnlse_plan* p, int32_t* order) {
  if (!p || !order) return GNLSE_BAD_ARGUMENT;
  for (size_t i = 0; i < p->order.size(); ++i) order[i] = p->order[i];
  return GNLSE_OK;
}

int gnlse_set_step_log(gnlse_plan* p, int instance, double* d_steps, int64_t capacity) {
  if (!p || instance < 0 || instance >= (int)p->inst.size() || capacity < 0 || (capacity > 0 && !d_steps))
    return GNLSE_BAD_ARGUMENT;
  InstDev& d = p->inst[instance];
  d.step_log = capacity > 0 ? d_steps : nullptr;
  d.step_cap = capacity;
  cudaError_t e = cudaMemcpy(p->d_inst + instance, &d, sizeof(InstDev), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? GNLSE_OK : cuda_fail(e);
}

int gnlse_set_replay(gnlse_plan* p, int instance, const double* d_h, int64_t n) {
  if (!p || instance < 0 || instance >= (int)p->inst.size() || n < 0 || (n > 0 && !d_h))
    return GNLSE_BAD_ARGUMENT;
  InstDev& d = p->inst[instance];
  if (n > 0 && d.method != GNLSE_ARK4IP) return GNLSE_UNSUPPORTED;
  d.replay = n > 0 ? d_h : nullptr;
  d.replay_n = n;
  cudaError_t e = cudaMemcpy(p->d_inst + instance, &d, sizeof(InstDev), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? GNLSE_OK : cuda_fail(e);
}

int gnlse_get_stats(gnlse_plan* p, gnlse_stats* out, void* stream) {
  if (!p || !out) return GNLSE_BAD_ARGUMENT;
  const size_t n = p->inst.size();
  std::vector<InstState> st(n);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(st.data(), p->d_state, sizeof(InstState) * n, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e);
  for (size_t i = 0; i < n; ++i) {
    gnlse_stats& o = out[i];
    const InstState& t = st[i];
    o.z = t.z;
    o.h = t.h;
    o.delta_last = t.delta_last;
    o.energy_in = t.E_in;
    o.energy_out = t.E_out;
    o.photons_in = t.Nph_in;
    o.photons_out = t.Nph_out;
    o.attempts = t.attempts;
    o.accepted = t.accepted;
    o.rejected = t.rejected;
    o.evals = t.evals;
    o.steps = t.steps;
    o.status = t.phase == 0 ? GNLSE_RUNNING : (t.phase == 3 ? t.status : GNLSE_RUNNING);
    if (t.phase == 3 || t.phase == 2) o.status = t.status;
    o.ntraces = t.ntraces;
    o.trace_overflow = t.trace_overflow;
    o.finished = t.phase == 3 ? 1 : 0;
    o.pump_w = t.pp;
  }
  return GNLSE_OK;
}

}  // extern "C"
