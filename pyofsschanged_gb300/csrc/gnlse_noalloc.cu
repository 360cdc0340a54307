// gnlse_propagate_noalloc: one-field propagation that allocates no memory.
//
// Some callers cannot allocate device memory when they propagate: a host
// loop that shares the GPU with latency-critical work cannot afford
// cudaMalloc/cudaFree (they synchronise the device), and a process whose
// device memory is owned by another allocator (a framework's caching pool or
// a fixed per-process quota) must not take memory behind that allocator's
// back.  For them this entry point keeps everything it needs -- operator
// tables, twiddles, the 8 N-point work buffers and the control block -- in
// one file-scope __device__ array of kNoAllocBytes bytes, which every GPU
// that loads the library holds until the process exits.  The caller passes
// only the field (device, complex64, in place) and the host-side tables.
//
// Limits and rules: fields of 256..4096 points (power of two), complex64,
// no trace storage.  All calls share the array, so two calls whose work
// overlaps on the GPU (different streams, or different host threads) race
// and must be serialised by the caller; one call on one stream is ordered.
// The first call on a device looks up the array's device address (once per
// device, with that device current).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/gnlse.h"
#include "gnlse_launch.h"
#include "gnlse_twiddle.h"
#include "gnlse_types.h"

namespace {

constexpr int kNoAllocMaxN = 4096;
// layout (bytes, N = kNoAllocMaxN): scratch 8N complex64 | beta N f64 | nu N f64 |
// Kr N f32 | lor N f32 | Hp N c64 | tw N c64 | staging ss/hR_re/hR_im/gain 4N f64 |
// per-pass twiddle rows | control
constexpr size_t kScratch = 8ull * kNoAllocMaxN * 8;
constexpr size_t kBeta = kScratch;
constexpr size_t kNu = kBeta + 8ull * kNoAllocMaxN;
constexpr size_t kKr = kNu + 8ull * kNoAllocMaxN;
constexpr size_t kLor = kKr + 4ull * kNoAllocMaxN;
constexpr size_t kHp = kLor + 4ull * kNoAllocMaxN;
constexpr size_t kTw = kHp + 8ull * kNoAllocMaxN;
constexpr size_t kStage = kTw + 8ull * kNoAllocMaxN;
constexpr size_t kTwp = kStage + 4ull * 8 * kNoAllocMaxN;
constexpr int kTwpMax = 5120;  // >= twp_size(12, radix bits) for radix 8 and 16
constexpr size_t kCtl = kTwp + 8ull * kTwpMax;
constexpr size_t kNoAllocBytes = kCtl + 1024;  // 585 KiB in all

static __device__ __align__(256) unsigned char g_noalloc[kNoAllocBytes];

constexpr int kMaxDevices = 64;
static unsigned char* g_noalloc_dev[kMaxDevices];  // device address of g_noalloc, per device

// FP32 tables from the FP64 staging copies of the caller's host arrays.
__global__ void noalloc_tables(unsigned char* base, int n, double gamma, int has_ss, int raman,
                               int gain, int has_profile, int has_nu) {
  const double* stage = (const double*)(base + kStage);
  const double* ss = stage;
  const double* hre = stage + kNoAllocMaxN;
  const double* him = stage + 2 * kNoAllocMaxN;
  const double* gp = stage + 3 * kNoAllocMaxN;
  float* Kr = (float*)(base + kKr);
  float* lor = (float*)(base + kLor);
  float2* Hp = (float2*)(base + kHp);
  float2* tw = (float2*)(base + kTw);
  float2* twp = (float2*)(base + kTwp);
  double* nu = (double*)(base + kNu);
  int logm = 0;
  while ((1 << logm) < n) ++logm;
  const int ntwp = gnlse::twp_size(logm, GNLSE_RADIX_BITS);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ntwp; e += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)gnlse::twp_exponent(logm, GNLSE_RADIX_BITS, e) / (double)n, &s, &c);
    twp[e] = make_float2((float)c, (float)s);
  }
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    Kr[a] = (float)(gamma * (has_ss ? ss[a] : 1.0));
    if (raman) Hp[a] = make_float2((float)(hre[a] / n), (float)(him[a] / n));
    if (gain) lor[a] = has_profile ? (float)gp[a] : 1.0f;
    // without the caller's frequencies the photon number uses nu = 1, as the plan path
    // does (the array may still hold an earlier call's table)
    if (!has_nu) nu[a] = 1.0;
    double s, c;
    sincospi(2.0 * (double)a / (double)n, &s, &c);
    tw[a] = make_float2((float)c, (float)s);
  }
}

cudaError_t launch_fp32(int logm, const gnlse::KParams& kp, cudaStream_t s) {
  switch (logm) {
    case 8: return gnlse::launch_class<float, 8, 1, false>(kp, 1, s);
    case 9: return gnlse::launch_class<float, 9, 1, false>(kp, 1, s);
    case 10: return gnlse::launch_class<float, 10, 1, false>(kp, 1, s);
    case 11: return gnlse::launch_class<float, 11, 1, false>(kp, 1, s);
    case 12: return gnlse::launch_class<float, 12, 1, false>(kp, 1, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

extern "C" int gnlse_propagate_noalloc(const gnlse_grid_desc* gd, const gnlse_instance_desc* id,
                                       void* d_field, gnlse_stats* stats_out, void* stream) {
  if (!gd || !id || !d_field) return GNLSE_BAD_ARGUMENT;
  const int n = gd->n;
  if (n < 256 || n > kNoAllocMaxN || (n & (n - 1)) != 0) return GNLSE_UNSUPPORTED;
  if (gd->cluster > 1 || !gd->beta_w || !(gd->dt > 0) || !(gd->window_t > 0)) return GNLSE_BAD_ARGUMENT;
  if (gd->yb_on) return GNLSE_UNSUPPORTED;  // the Yb model's tables have no room in the static array
  if ((id->method != GNLSE_RK4IP && id->method != GNLSE_ARK4IP) || id->total_steps < 1 ||
      id->traces < 1 || id->max_traces != 0 || !(id->length >= 0) ||
      (id->method == GNLSE_ARK4IP && !(id->local_error > 0)) ||
      (gd->gain_on && !(gd->E_sat > 0 && gd->gain_length > 0)))
    return GNLSE_BAD_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GNLSE_CUDA_ERROR;
  if (!g_noalloc_dev[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc) != cudaSuccess || !ptr) return GNLSE_CUDA_ERROR;
    g_noalloc_dev[dev] = (unsigned char*)ptr;
  }
  unsigned char* base = g_noalloc_dev[dev];
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nb = sizeof(double) * (size_t)n;
  double* stage = (double*)(base + kStage);
  const bool raman = gd->hR_re != nullptr;
  const bool gain = gd->gain_on != 0;
  cudaError_t e = cudaSuccess;
  auto put = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && src) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  put(base + kBeta, gd->beta_w, nb);
  if (gd->nu) put(base + kNu, gd->nu, nb);
  put(stage, gd->ss_w, nb);
  put(stage + kNoAllocMaxN, gd->hR_re, nb);
  if (raman && gd->hR_im) put(stage + 2 * kNoAllocMaxN, gd->hR_im, nb);
  if (raman && !gd->hR_im && e == cudaSuccess) e = cudaMemsetAsync(stage + 2 * kNoAllocMaxN, 0, nb, s);
  if (gain) put(stage + 3 * kNoAllocMaxN, gd->gain_profile, nb);  // none: flat profile
  if (e != cudaSuccess) return GNLSE_CUDA_ERROR;
  static_assert(gnlse::twp_size(12, GNLSE_RADIX_BITS) <= kTwpMax, "twiddle rows");
  noalloc_tables<<<(n + 255) / 256, 256, 0, s>>>(base, n, gd->gamma, gd->ss_w != nullptr, raman, gain,
                                                  gd->gain_profile != nullptr, gd->nu != nullptr);
  if (cudaGetLastError() != cudaSuccess) return GNLSE_CUDA_ERROR;

  gnlse::GridDev g;
  memset(&g, 0, sizeof(g));
  g.beta = (const double*)(base + kBeta);
  g.Kr = base + kKr;
  // unused tables still point at valid memory: a read-only load may be issued ahead
  // of the flag that guards it
  g.Hp = base + kHp;
  g.lor = base + kLor;
  g.lor2 = base + kLor;
  g.nu = (const double*)(base + kNu);
  g.tw = base + kTw;
  g.twl = base + kTw;
  g.twp = base + kTwp;
  g.n = n;
  g.logm = 0;
  while ((1 << g.logm) < n) ++g.logm;
  g.C = 1;
  g.raman = raman ? 1 : 0;
  g.gain = gain ? 1 : 0;
  g.alpha = gd->alpha;
  g.fR = gd->f_R;
  g.gain_log = gd->gain_log;
  g.E_sat = gd->E_sat;
  g.gain_len = gd->gain_length;
  g.dt = gd->dt;
  g.window_t = gd->window_t;
  gnlse::InstDev d;
  memset(&d, 0, sizeof(d));
  d.method = id->method;
  d.total_steps = id->total_steps;
  d.traces = id->traces;
  d.length = id->length;
  d.tol = id->local_error;
  double h0 = id->h0;
  if (!(h0 > 0)) {  // stepper.py:256-264
    h0 = id->traces > id->total_steps ? id->length / id->traces : id->length / id->total_steps;
    if (h0 > 1e-6) h0 = 1e-6;
  }
  d.h0 = h0;
  // control block: GridDev | InstDev | InstState | order index, all in the array
  unsigned char* ctl = base + kCtl;
  gnlse::GridDev* dg = (gnlse::GridDev*)ctl;
  gnlse::InstDev* dd = (gnlse::InstDev*)(ctl + 256);
  gnlse::InstState* ds = (gnlse::InstState*)(ctl + 512);
  int* dorder = (int*)(ctl + 512 + 256);
  static_assert(sizeof(gnlse::GridDev) <= 256 && sizeof(gnlse::InstDev) <= 256 &&
                sizeof(gnlse::InstState) <= 256, "control block layout");
  if ((e = cudaMemcpyAsync(dg, &g, sizeof(g), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(dd, &d, sizeof(d), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(ds, 0, sizeof(gnlse::InstState), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(dorder, 0, sizeof(int), s)) != cudaSuccess)
    return GNLSE_CUDA_ERROR;
  // the host copies above read from this stack frame: wait for them
  if (cudaStreamSynchronize(s) != cudaSuccess) return GNLSE_CUDA_ERROR;
  gnlse::KParams kp;
  memset(&kp, 0, sizeof(kp));
  kp.inst = dd;
  kp.state = ds;
  kp.order = dorder;
  kp.n_order = 1;
  kp.grids = dg;
  kp.fields = d_field;
  kp.scratch = base;
  kp.max_attempts = 0;
  if (launch_fp32(g.logm, kp, s) != cudaSuccess) return GNLSE_CUDA_ERROR;
  if (stats_out) {
    gnlse::InstState st;
    if (cudaMemcpyAsync(&st, ds, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return GNLSE_CUDA_ERROR;
    stats_out->z = st.z;
    stats_out->h = st.h;
    stats_out->delta_last = st.delta_last;
    stats_out->energy_in = st.E_in;
    stats_out->energy_out = st.E_out;
    stats_out->photons_in = st.Nph_in;
    stats_out->photons_out = st.Nph_out;
    stats_out->attempts = st.attempts;
    stats_out->accepted = st.accepted;
    stats_out->rejected = st.rejected;
    stats_out->evals = st.evals;
    stats_out->steps = st.steps;
    stats_out->status = st.phase == 3 ? st.status : GNLSE_RUNNING;
    stats_out->ntraces = st.ntraces;
    stats_out->trace_overflow = st.trace_overflow;
    stats_out->finished = st.phase == 3 ? 1 : 0;
  }
  return GNLSE_OK;
}
