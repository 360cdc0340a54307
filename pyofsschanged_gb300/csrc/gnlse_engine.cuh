// Fused RK4IP / ARK4IP GNLSE engine for sm_103a.
//
// One thread-block cluster of C CTAs propagates one field of N = C*M points.
// CTA c keeps its M-point slice of the working field in shared memory:
//   time domain     : CTA c slot m  <-> sample n = c*M + m
//   spectral domain : CTA c slot k2 <-> frequency index k = c + C*k2 (FFT order)
// A transform is one cross-CTA radix-C pass through distributed shared memory
// (DSMEM) plus an M-point Stockham FFT in the CTA's own shared memory.  Every
// elementwise operation of the RK4IP step (exp(hD), SPM, Raman convolution,
// self-steepening, gain, the RK stage combination, the step-doubling error
// norm and the Richardson extrapolation) runs inside the first or last pass of
// a transform, so a stage never makes an extra pass over its data.
//
// The propagation state is kept in the spectral domain scaled by N
// (S = N * pyofss.fft(A)); the algebra is that of Solver.rk4ip
// (pyofss/modules/solver.py:339-354) with the linear operator applied in the
// spectral domain, which needs 4 transforms per nonlinear evaluation (16 per
// RK4IP evaluation) instead of the reference's 24.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "gnlse_dd.cuh"
#include "gnlse_df.cuh"
#include "gnlse_twiddle.h"
#include "gnlse_types.h"

// registers per thread the launch bounds aim for: CTAs per SM = 65536 / (T * this),
// limited by shared memory (GNLSE_MINB_CAP can lower it further)
#ifndef GNLSE_REGS_TARGET
#define GNLSE_REGS_TARGET 128
#endif
#ifndef GNLSE_MINB_CAP
#define GNLSE_MINB_CAP 16
#endif
// points each thread holds per pass (the radix is set in gnlse_twiddle.h)
#ifndef GNLSE_PPT
#define GNLSE_PPT 16
#endif
// fewest threads per CTA (slices below GNLSE_PPT * this many points leave threads
// idle in the radix passes)
#ifndef GNLSE_TMIN
#define GNLSE_TMIN 64
#endif

namespace cg = cooperative_groups;

// Phase cycle counters (GNLSE_PROF builds): thread 0 of each cluster's first
// CTA accumulates clock64() deltas of the attempt's phases into kp.prof.
#ifndef GNLSE_PROF
#define GNLSE_PROF 0
#endif
#if GNLSE_PROF
#define PROF_T0() long long _pt0 = clock64()
#define PROF_ADD(k) \
  do { if (threadIdx.x == 0) prof_acc[k] += clock64() - _pt0; _pt0 = clock64(); } while (0)
#else
#define PROF_T0() do {} while (0)
#define PROF_ADD(k) do {} while (0)
#endif

namespace gnlse {

template <class R> struct VT;
template <> struct VT<float> { using V = float2; };
template <> struct VT<double> { using V = double2; };
template <> struct VT<ddf> { using V = ddc; };  // double-float transforms ("df" plans)

// Read-only (non-coherent cache) load of a table entry of any element type.
template <class T>
__device__ __forceinline__ T ldro(const T* p) {
  if constexpr (std::is_same<T, ddf>::value) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return ddf(v.x, v.y);
  } else if constexpr (std::is_same<T, ddc>::value) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return ddc{make_float2(v.x, v.y), make_float2(v.z, v.w)};
  } else {
    return __ldg(p);
  }
}

// real type of a complex element type, its parts and construction
template <class V> struct RT { using type = decltype(V::x); };
template <> struct RT<ddc> { using type = ddf; };
template <class V> __device__ __forceinline__ V mk(typename RT<V>::type a, typename RT<V>::type b) {
  if constexpr (std::is_same<V, ddc>::value) {
    return mkdc(a, b);
  } else {
    V r;
    r.x = a;
    r.y = b;
    return r;
  }
}
template <class V> __device__ __forceinline__ auto re(const V& a) -> decltype(a.x) { return a.x; }
template <class V> __device__ __forceinline__ auto im(const V& a) -> decltype(a.y) { return a.y; }
template <class V> __device__ __forceinline__ V cconj(V a) { return mk<V>(a.x, -a.y); }
template <int SIGN, class V> __device__ __forceinline__ V cmul_i(V a) {  // SIGN i a
  return SIGN > 0 ? mk<V>(-a.y, a.x) : mk<V>(a.y, -a.x);
}
template <class V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <class V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <class V> __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class V> __device__ __forceinline__ V cmulc(V a, V b) {  // a * conj(b)
  return mk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <class V, class S> __device__ __forceinline__ V cscale(V a, S s) { return mk<V>(a.x * s, a.y * s); }
// inside a DFT butterfly: the plain operations, or for double-float values the variants
// that skip the renormalisation (gnlse_dd.cuh), with one cnorm of each output
template <class V> __device__ __forceinline__ V cadd_lazy(V a, V b) { return cadd(a, b); }
template <class V> __device__ __forceinline__ V csub_lazy(V a, V b) { return csub(a, b); }
template <class V> __device__ __forceinline__ V cmul_lazy(V a, V b) { return cmul(a, b); }
template <class V> __device__ __forceinline__ V cmulc_lazy(V a, V b) { return cmulc(a, b); }
template <class V> __device__ __forceinline__ V cnorm(V a) { return a; }
template <class V> __device__ __forceinline__ auto cabs2(V a) -> decltype(a.x) { return a.x * a.x + a.y * a.y; }

// Padded shared-memory slot: one spare element every 16 makes every Stockham
// pass (radix-16 strided stores included) free of bank conflicts for 8- and
// 16-byte elements.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }

// threadIdx.x read through an opaque instruction: index arithmetic derived from
// it is recomputed where it is used instead of being hoisted out of the
// propagation loop and kept live in registers across every transform.
// GNLSE_OPAQUE_TID selects where: bit 0 Stockham passes, bit 1 cross-CTA
// passes, bit 2 elementwise stage loops.
#ifndef GNLSE_OPAQUE_TID
#define GNLSE_OPAQUE_TID 1
#endif
template <int BIT>
__device__ __forceinline__ int tidx() {
  if constexpr ((GNLSE_OPAQUE_TID >> BIT) & 1) {
    int t;
    asm volatile("mov.u32 %0, %%tid.x;" : "=r"(t));
    return t;
  } else {
    return (int)threadIdx.x;
  }
}

__host__ __device__ constexpr int bitrev(int k, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((k >> b) & 1) << (bits - 1 - b);
  return r;
}
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// cos / sin of 2*pi*m/16.
__device__ __forceinline__ constexpr double c16(int m) {
  constexpr double t[16] = {1.0, 0.92387953251128674, 0.70710678118654752, 0.38268343236508977,
                            0.0, -0.38268343236508977, -0.70710678118654752, -0.92387953251128674,
                            -1.0, -0.92387953251128674, -0.70710678118654752, -0.38268343236508977,
                            0.0, 0.38268343236508977, 0.70710678118654752, 0.92387953251128674};
  return t[m & 15];
}
__device__ __forceinline__ constexpr double s16(int m) { return c16(m - 4); }

// In-register DFT of R points (R = 2..16): X[k] = sum_r v[r] exp(SIGN 2 pi i r k / R),
// radix-2 decimation in frequency with constant twiddles, output in natural order.
template <int RAD, int SIGN, class V>
__device__ __forceinline__ void dft(V (&v)[RAD]) {
  using S = typename RT<V>::type;
  constexpr int B = ilog2(RAD);
#pragma unroll
  for (int st = 0; st < B; ++st) {
    const int half = RAD >> (st + 1);
    const int L = half * 2;
#pragma unroll
    for (int blk = 0; blk < RAD; blk += L) {
#pragma unroll
      for (int j = 0; j < half; ++j) {
        V a = v[blk + j], b = v[blk + j + half];
        v[blk + j] = cadd_lazy(a, b);
        V d = csub_lazy(a, b);
        const int m = j * (16 / L);
        if (m == 0) {
          v[blk + j + half] = d;
        } else if (m == 4) {  // multiply by SIGN*i
          v[blk + j + half] = cmul_i<SIGN>(d);
        } else {
          const S c = (S)c16(m), s = (S)(SIGN * s16(m));
          v[blk + j + half] = cmul_lazy(d, mk<V>(c, s));  // d.x c - d.y s + i (d.x s + d.y c)
        }
      }
    }
  }
  V t[RAD];
#pragma unroll
  for (int k = 0; k < RAD; ++k) t[k] = v[bitrev(k, B)];
#pragma unroll
  for (int k = 0; k < RAD; ++k) v[k] = cnorm(t[k]);
}

// Simpson weight (units of dt) of sample n out of N, reproducing scipy's
// even-N composite Simpson with Cartwright's last-interval correction, as used
// by pyofss.field.energy (pyofss/field.py:161-172).
__device__ __forceinline__ double simpson_w(int n, int N) {
  if (n == 0) return 1.0 / 3.0;
  if (n == N - 1) return 5.0 / 12.0;
  if (n == N - 2) return 1.0;
  if (n == N - 3) return 4.0 / 3.0 - 1.0 / 12.0;
  return (n & 1) ? 4.0 / 3.0 : 2.0 / 3.0;
}

// XS ("extended state"): complex64 transforms and nonlinear evaluations with
// the propagation state, the RK accumulator and the exp(hD) factors held as
// double-float complex values (float4) and FP64 boundary transforms.
// INPLACE: cross-CTA passes exchange in place (no exchange buffer); used for
// the FP64 boundary transforms of extended-state kernels.
template <class R, int LOGM, int C, bool XS = false, bool INPLACE = false>
struct Engine {
  using V = typename VT<R>::V;
  // DD: double-float transforms, nonlinear term and state (complex128 user fields)
  static constexpr bool DD = std::is_same<R, ddf>::value;
  using SV = typename std::conditional<XS, float4, V>::type;  // state-like arrays
  using FV = typename std::conditional<XS || DD, double2, V>::type;  // user fields / traces
  static_assert(!XS || sizeof(R) == 4, "extended state runs on complex64 transforms");
  static constexpr int M = 1 << LOGM;
  static constexpr int N = M * C;
  static constexpr int RB = DD ? GNLSE_DF_RADIX_BITS : GNLSE_RADIX_BITS;  // log2 of the main radix
  static constexpr int PPT = DD ? (1 << GNLSE_DF_RADIX_BITS) : GNLSE_PPT;   // points per thread per pass
  static constexpr int T = (M / PPT) < GNLSE_TMIN ? GNLSE_TMIN : (M / PPT);
  static constexpr int MP = M + M / 16;
  static constexpr int RADIX = 1 << RB;
  static constexpr int NR16 = LOGM / RB;        // passes of the main radix
  static constexpr int REM = LOGM % RB;         // log2 of the final smaller radix
  static constexpr int RED = 64;  // doubles of reduction scratch
  // cluster_sum keeps up to 3 partial sums per warp at red[0, 48) and the totals at
  // red[48, 51): CTAs of at most 16 warps (a 1024-thread CTA would write past red into
  // the control block)
  static_assert(3 * (((M / PPT) < GNLSE_TMIN ? GNLSE_TMIN : (M / PPT)) / 32) <= 48,
                "reduction scratch holds the partial sums of at most 16 warps");
  static_assert(LOGM >= 8, "M >= 256 required");
  static_assert(C == 1 || C == 2 || C == 4 || C == 8 || C == 16, "cluster size 1, 2, 4, 8 or 16");
  static constexpr size_t ctl_bytes() { return 1024; }
  // CTAs that fit on one SM by shared memory (228 KB per SM, 1 KB reserved per CTA)
  static constexpr int NBUF = (C > 1 && !INPLACE) ? 3 : 2;  // X, P (+ W)
  static constexpr int MINB_RAW = (int)(233472 / (NBUF * MP * sizeof(V) + RED * sizeof(double) + 1024 + 1024));
  // ... and by the register target (128 registers: 2 CTAs of 256 threads, 4 of 128;
  // 64-thread CTAs of the small grids keep up to 255)
  static constexpr int TR = T < 128 ? 128 : T;
  static constexpr int MINB_TGT = 65536 / (TR * GNLSE_REGS_TARGET) < 1 ? 1 : 65536 / (TR * GNLSE_REGS_TARGET);
  static constexpr int MINB_REG = MINB_RAW < 1 ? 1 : (MINB_RAW < MINB_TGT ? MINB_RAW : MINB_TGT);
  static constexpr int MINB = MINB_REG < GNLSE_MINB_CAP ? MINB_REG : GNLSE_MINB_CAP;
  static constexpr size_t smem_bytes() {
    return NBUF * MP * sizeof(V) + RED * sizeof(double) + ctl_bytes();
  }

  struct Ctx {
    V* X;
    V* P;
    V* W;          // exchange buffer of the cross-CTA passes (C > 1)
    double* red;
    const V* tw;   // N-point table (cross-CTA pass)
    const V* twl;  // M-point table
    const V* twp;  // per-pass twiddle rows (per-CTA passes)
    int rank;
  };

  // Address of p's counterpart in CTA r of the cluster.  The mapping is an
  // opaque (volatile) instruction at every use, so the compiler recomputes it
  // instead of keeping the C remote bases of every buffer live across the
  // whole propagation loop (which spilled registers in the cluster classes).
  static __device__ __forceinline__ V* rmt(V* p, int r) {
    if constexpr (C > 1) {
      unsigned long long q;
      asm volatile("mapa.u64 %0, %1, %2;" : "=l"(q) : "l"(p), "r"(r));
      return reinterpret_cast<V*>(q);
    } else {
      return p;
    }
  }

  // Time-domain shared-memory layout: with C > 1 the CTA owning positions
  // n2 in [rank*M/C, (rank+1)*M/C) holds every sample n1*M + n2 of them (n1 < C),
  // at slot n1*M/C + n2 mod M/C, so both cross-CTA passes find their time-domain
  // operands locally.  With C = 1 the slot is the sample index.
  static __device__ __forceinline__ int tslot(int n1, int n2) {
    if constexpr (C > 1) {
      return n1 * (M / C) + (n2 & (M / C - 1));
    } else {
      return n2;
    }
  }
  // global sample index of local time slot s of CTA rank
  static __device__ __forceinline__ int tsample(int rank, int s) {
    if constexpr (C > 1) {
      constexpr int PM = M / C;
      return (s / PM) * M + rank * PM + (s & (PM - 1));
    } else {
      return rank * M + s;
    }
  }

  static __device__ __forceinline__ void csync() {
    if constexpr (C > 1) {
      cg::this_cluster().sync();
    } else {
      __syncthreads();
    }
  }

  // Twiddles are read with ordinary (L1-cached) loads rather than __ldg: the
  // non-coherent loads may be hoisted across the barriers into earlier
  // passes, which lengthens register lifetimes until the kernel spills.
  static __device__ __forceinline__ V twid(const V* tw, int idx, int sign) {
    const V w = tw[idx];
    return sign < 0 ? cconj(w) : w;
  }

  // ---- transforms ---------------------------------------------------------
  // One radix-RAD Stockham pass over the CTA's M points: all loads, barrier,
  // all stores (so src may equal dst).  FIRST: inputs from pro(owner, slot),
  // otherwise from src; LAST: outputs to epi(owner, slot, v), otherwise to dst.
  // twiddles of one butterfly: row[r] = W^{r k ...}, r < RAD, one 128-bit load per 16 bytes
  template <int RAD>
  static __device__ __forceinline__ void load_row(const V* row, V (&w)[RAD]) {
    if constexpr (sizeof(V) == 8) {
#pragma unroll
      for (int i = 0; i < RAD / 2; ++i) {
        const float4 q = *(reinterpret_cast<const float4*>(row) + i);
        w[2 * i] = mk<V>(q.x, q.y);
        w[2 * i + 1] = mk<V>(q.z, q.w);
      }
    } else {
#pragma unroll
      for (int r = 0; r < RAD; ++r) w[r] = row[r];
    }
  }

  template <int RAD, int SIGN, bool FIRST, bool LAST, int OFF, class Pro, class Epi>
  static __device__ __forceinline__ void pass(const Ctx& cx, const V* src, V* dst, int Ns, Pro& pro,
                                              Epi& epi) {
    constexpr int NB = M / RAD;
    constexpr int BPT = (NB + T - 1) / T;
    V v[BPT][RAD];
    const int tid = tidx<0>();
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = tid + b * T;
      if (NB % T == 0 || j < NB) {
#pragma unroll
        for (int r = 0; r < RAD; ++r) {
          const int i = j + r * NB;
          if constexpr (FIRST) v[b][r] = pro(cx.rank, i);
          else v[b][r] = src[pad(i)];
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = tid + b * T;
      if (NB % T == 0 || j < NB) {
        const int k = j & (Ns - 1);
        if (Ns > 1) {
          V w[RAD];
          load_row<RAD>(cx.twp + OFF + k * RAD, w);
#pragma unroll
          for (int r = 1; r < RAD; ++r)
            v[b][r] = SIGN > 0 ? cmul_lazy(v[b][r], w[r]) : cmulc_lazy(v[b][r], w[r]);
        }
        dft<RAD, SIGN>(v[b]);
        const int base = (j - k) * RAD + k;
#pragma unroll
        for (int r = 0; r < RAD; ++r) {
          const int o = base + r * Ns;
          if constexpr (LAST) epi(cx.rank, o, v[b][r]);
          else dst[pad(o)] = v[b][r];
        }
      }
    }
    __syncthreads();
  }

  template <int SIGN, bool PRO, bool EPI, int P16, class Pro, class Epi>
  static __device__ __forceinline__ void passes(const Ctx& cx, const V* src, V* buf, V* dst, int Ns,
                                                Pro& pro, Epi& epi) {
    if constexpr (P16 < NR16) {
      constexpr bool first = PRO && (P16 == 0);
      constexpr bool last_pass = (P16 == NR16 - 1) && (REM == 0);
      constexpr bool last = EPI && last_pass;
      pass<RADIX, SIGN, first, last, twp_offset(LOGM, RB, P16)>(cx, P16 == 0 ? src : buf,
                                                                 last_pass ? dst : buf, Ns, pro, epi);
      passes<SIGN, PRO, EPI, P16 + 1>(cx, src, buf, dst, Ns * RADIX, pro, epi);
    } else if constexpr (REM > 0) {
      pass<(1 << REM), SIGN, false, EPI, twp_offset(LOGM, RB, NR16)>(cx, buf, dst, Ns, pro, epi);
    }
  }

  // M-point Stockham transform of the CTA's own slice: src -> (buf) -> dst.
  template <int SIGN, bool PRO, bool EPI, class Pro, class Epi>
  static __device__ __forceinline__ void local_fft(const Ctx& cx, const V* src, V* buf, V* dst, Pro& pro,
                                                   Epi& epi) {
    passes<SIGN, PRO, EPI, 0>(cx, src, buf, dst, 1, pro, epi);
  }

  // Forward cross-CTA pass, streaming into the exchange buffers: slot n2 of
  // every CTA r (= x[r*M + n2], from pro) -> radix-C DFT -> twiddle W_N^{n2 k1}
  // -> exchange slot n2 of CTA k1.  lead: a cluster barrier is needed first
  // (inputs written since the last one).
  template <class Pro>
  static __device__ __forceinline__ void cross_fwd(const Ctx& cx, Pro& pro, bool lead, bool wfree = true) {
    constexpr int PM = M / C;
    const int tid = tidx<1>();
    if constexpr (INPLACE) {
      // in place: all reads, cluster barrier, all writes (into cx.W == cx.X)
      constexpr int BP = (PM + T - 1) / T;
      V v[BP][C];
      csync();
#pragma unroll
      for (int b = 0; b < BP; ++b) {
        const int q = tid + b * T;
        if (PM % T == 0 || q < PM)
#pragma unroll
          for (int r = 0; r < C; ++r) v[b][r] = pro(r, cx.rank * PM + q);
      }
      csync();
#pragma unroll
      for (int b = 0; b < BP; ++b) {
        const int q = tid + b * T;
        if (PM % T == 0 || q < PM) {
          const int n2 = cx.rank * PM + q;
          dft<C, +1>(v[b]);
#pragma unroll
          for (int k1 = 0; k1 < C; ++k1)
            rmt(cx.W, k1)[pad(n2)] = k1 ? cmul(v[b][k1], twid(cx.tw, n2 * k1, +1)) : v[b][k1];
        }
      }
      csync();
      return;
    }
    // Time-domain inputs are local (this CTA owns all C samples of its positions,
    // see tslot), so the loads, the radix-C DFT and the twiddles run before the
    // barrier that frees the other CTAs' exchange buffers; then the pushes.
    constexpr int BP = (PM + T - 1) / T;
    V v[BP][C];
    __syncthreads();  // inputs written by this CTA's threads
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = tid + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int r = 0; r < C; ++r) v[b][r] = pro(r, n2);
        dft<C, +1>(v[b]);
#pragma unroll
        for (int k1 = 1; k1 < C; ++k1) v[b][k1] = cmul(v[b][k1], twid(cx.tw, n2 * k1, +1));
      }
    }
    if (wfree) csync();  // every CTA is done reading its exchange buffer
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = tid + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int k1 = 0; k1 < C; ++k1) rmt(cx.W, k1)[pad(n2)] = v[b][k1];
      }
    }
    csync();
    (void)lead;
  }

  // Inverse cross-CTA pass from the exchange buffers: exchange slot n2 of
  // every CTA k1 -> twiddle W_N^{-n2 k1} -> radix-C DFT -> epi(n1, n2, x[n1*M + n2]).
  template <class Epi>
  static __device__ __forceinline__ void cross_inv(const Ctx& cx, Epi& epi, bool trail = true) {
    constexpr int PM = M / C;
    const int tid = tidx<1>();
    if constexpr (INPLACE) {
      constexpr int BP = (PM + T - 1) / T;
      V v[BP][C];
      csync();
#pragma unroll
      for (int b = 0; b < BP; ++b) {
        const int q = tid + b * T;
        if (PM % T == 0 || q < PM)
#pragma unroll
          for (int k1 = 0; k1 < C; ++k1) v[b][k1] = rmt(cx.W, k1)[pad(cx.rank * PM + q)];
      }
      csync();
#pragma unroll
      for (int b = 0; b < BP; ++b) {
        const int q = tid + b * T;
        if (PM % T == 0 || q < PM) {
          const int n2 = cx.rank * PM + q;
#pragma unroll
          for (int k1 = 1; k1 < C; ++k1) v[b][k1] = cmul_lazy(v[b][k1], twid(cx.tw, n2 * k1, -1));
          dft<C, -1>(v[b]);
#pragma unroll
          for (int n1 = 0; n1 < C; ++n1) epi(n1, n2, v[b][n1]);
        }
      }
      csync();
      return;
    }
    constexpr int BP = (PM + T - 1) / T;
    V v[BP][C];
    V w[BP][C];  // W_N^{-n2 k1}, requested before the barrier
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = tid + b * T;
      if (PM % T == 0 || q < PM)
#pragma unroll
        for (int k1 = 1; k1 < C; ++k1) w[b][k1] = twid(cx.tw, (cx.rank * PM + q) * k1, -1);
    }
    csync();
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = tid + b * T;
      if (PM % T == 0 || q < PM)
#pragma unroll
        for (int k1 = 0; k1 < C; ++k1) v[b][k1] = rmt(cx.W, k1)[pad(cx.rank * PM + q)];
    }
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = tid + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int k1 = 1; k1 < C; ++k1) v[b][k1] = cmul_lazy(v[b][k1], w[b][k1]);
        dft<C, -1>(v[b]);
#pragma unroll
        for (int n1 = 0; n1 < C; ++n1) epi(n1, n2, v[b][n1]);
      }
    }
    // The outputs are local (tslot); the cluster barrier is needed only when the
    // next write into an exchange buffer is not a forward cross pass (which frees
    // the buffers itself) -- trail = false skips it.
    if (trail) {
      csync();
    } else {
      __syncthreads();
    }
  }

  // Forward transform G+(x)[k] = sum_n x[n] e^{+2 pi i k n / N} (= N * pyofss fft),
  // result in buf (or to epi).  pro(n1, n2): time sample n1*M + n2, asked for only
  // in the CTA owning position n2 (tslot); epi(owner, slot, v): spectral output,
  // always called in the owner CTA.  lead (in-place cross passes only): inputs were
  // written since the last cluster barrier.  wfree = false: the caller guarantees that
  // no CTA still reads its exchange buffer (its last readers finished before a cluster
  // barrier already passed).
  template <class Pro, class Epi>
  static __device__ __forceinline__ void fwd(const Ctx& cx, V* buf, Pro& pro, Epi& epi, bool lead = true,
                                             bool wfree = true) {
    if constexpr (C == 1) {
      local_fft<+1, true, true>(cx, buf, buf, buf, pro, epi);
    } else {
      cross_fwd(cx, pro, lead, wfree);
      local_fft<+1, false, true>(cx, cx.W, buf, buf, pro, epi);
    }
  }

  // Inverse transform whose exchange goes through the P buffers: local passes in place
  // on buf, the last one pushing each output to the CTA owning its position (P slot
  // tslot(rank, n2)), one cluster barrier, then the radix-C pass on this CTA's own P
  // (each thread reads and rewrites only the C slots of its positions, so epi may write
  // P).  Needs P free in every CTA until the barrier; the exchange buffers W are not
  // touched.
  template <class Pro, class Epi>
  static __device__ __forceinline__ void inv_via_p(const Ctx& cx, V* buf, Pro& pro, Epi& epi) {
    if constexpr (C == 1) {
      local_fft<-1, true, true>(cx, buf, buf, buf, pro, epi);
    } else {
      constexpr int PM = M / C;
      auto push = [&](int, int o, V v) { rmt(cx.P, o / PM)[pad(tslot(cx.rank, o))] = v; };
      local_fft<-1, true, true>(cx, buf, buf, buf, pro, push);
      csync();
      const int tid = tidx<1>();
      constexpr int BP = (PM + T - 1) / T;
      V v[BP][C];
#pragma unroll
      for (int b = 0; b < BP; ++b) {
        const int q = tid + b * T;
        if (PM % T == 0 || q < PM) {
          const int n2 = cx.rank * PM + q;
#pragma unroll
          for (int k1 = 0; k1 < C; ++k1) v[b][k1] = cx.P[pad(tslot(k1, n2))];
#pragma unroll
          for (int k1 = 1; k1 < C; ++k1) v[b][k1] = cmul_lazy(v[b][k1], twid(cx.tw, n2 * k1, -1));
          dft<C, -1>(v[b]);
#pragma unroll
          for (int n1 = 0; n1 < C; ++n1) epi(n1, n2, v[b][n1]);
        }
      }
      __syncthreads();
    }
  }

  // Inverse transform G-(X)[n] = sum_k X[k] e^{-2 pi i k n / N} (= pyofss ifft).
  // pro(owner, slot): spectral input (owner CTA); epi(n1, n2, v): time sample
  // n1*M + n2, called in the CTA owning position n2 (tslot).
  template <class Pro, class Epi>
  static __device__ __forceinline__ void inv(const Ctx& cx, V* buf, Pro& pro, Epi& epi, bool trail = true) {
    if constexpr (C == 1) {
      local_fft<-1, true, true>(cx, buf, buf, buf, pro, epi);
    } else {
      local_fft<-1, true, false>(cx, buf, buf, cx.W, pro, epi);
      cross_inv(cx, epi, trail);
    }
  }

  // ---- reductions ---------------------------------------------------------
  // Sum of K values over the cluster; every thread of every CTA gets the same
  // result in the same summation order, so cluster-wide decisions agree.
  template <int K>
  static __device__ void cluster_sum(const Ctx& cx, double (&v)[K]) {
    static_assert(K <= 3, "");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = T / 32;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) cx.red[k * NW + wid] = v[k];
    __syncthreads();
    if (threadIdx.x < K) {
      double s = 0.0;
      for (int w = 0; w < NW; ++w) s += cx.red[threadIdx.x * NW + w];
      cx.red[48 + threadIdx.x] = s;
    }
    if constexpr (C > 1) {
      cg::cluster_group cl = cg::this_cluster();
      cl.sync();
#pragma unroll
      for (int k = 0; k < K; ++k) {
        double s = 0.0;
        for (int r = 0; r < C; ++r) s += cl.map_shared_rank(cx.red, r)[48 + k];
        v[k] = s;
      }
      cl.sync();
    } else {
      __syncthreads();
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] = cx.red[48 + k];
      __syncthreads();
    }
  }

  // ---- RK4IP stage algebra (Solver.rk4ip, solver.py:339-354) ---------------
  // Elementwise loops over this CTA's spectral slice between the transforms
  // of consecutive stages; each loop fuses the end of one stage with the
  // start of the next.
  struct Op {
    const SV* S0;
    const V* MA0;
    const SV* Et;
    SV* acc;
    SV* out;
    const SV* Sf;
    const R* Kr;
    const R* lor;
    const R* lor2;
    R h, aA, ak0, a3, ao, gb;
    double hh;
    int gain;
  };

  // gain exponent of one linear-operator call: ga lor (saturable amplifier), or
  // ga alpha_s N + gb eta_s (Yb model; ga = 500 h n2, gb = -500 h)
  static __device__ __forceinline__ R gexp(const Op& op, int a, R ga) {
    R x = ga * ldro(&op.lor[a]);
    if (op.gain == 2) x = fma(op.gb, ldro(&op.lor2[a]), x);
    return x;
  }
  static __device__ __forceinline__ V mult(const Op& op, int a, V e, R ga) {
    if (op.gain) e = cscale(e, (R)exp(gexp(op, a, ga)));
    return e;
  }
  // complex64 value (or the leading part of a double-float value) of a state-like array
  static __device__ __forceinline__ V ldv(const SV* p, int a) {
    if constexpr (XS) {
      return ld_hi(p, a);
    } else {
      return p[a];
    }
  }
  // gain factor exp(ga * lor) as a double-float real, 1 + expm1(x)
  static __device__ __forceinline__ dff gain_df(const Op& op, int a, R ga) {
    return fast_two_sum(1.0f, expm1f(gexp(op, a, ga)));
  }
  static __device__ __forceinline__ dfc mult_df(const Op& op, int a, dfc e, R ga) {
    if (op.gain) e = dfc_scale(e, gain_df(op, a, ga));
    return e;
  }

  // ---- the nonlinear operator ---------------------------------------------
  // On entry X holds the stage input xhat (spectral, this CTA's slice).  With
  // x = G-(xhat)/N and R(x) = (1-fR)|x|^2 + fR G-(Hp G+(|x|^2)) (Raman) or
  // |x|^2, on exit X holds G+(x R(x)) (spectral).  The transforms carry only
  // light per-element work in their first / last passes; with want_e the
  // Simpson energy (nJ) of x is returned.
  // keep_x (split-step kernel): also store x, sample n at keep_x[n]
  static __device__ __forceinline__ double nonlinear(const Ctx& cx, const GridDev& g, bool want_e,
                                                     V* keep_x = nullptr) {
    const R invN = (R)(1.0 / (double)N);
    const bool raman = g.raman != 0;
    V* X = cx.X;
    V* P = cx.P;
    // spectral operands are read by the local passes of this CTA (slot l), time-domain
    // ones by the cross-CTA passes as sample (n1, n2) at local slot tslot(n1, n2)
    auto rdXs = [&](int, int l) -> V { return X[pad(l)]; };
    auto rdXt = [&](int n1, int n2) -> V { return X[pad(tslot(n1, n2))]; };
    const bool keep_p = raman || want_e;
    auto e1 = [&](int n1, int n2, V v) {
      const int s = pad(tslot(n1, n2));
      V x = cscale(v, invN);
      R p = cabs2(x);
      if (keep_p) P[s] = mk<V>(p, (R)0);
      if (keep_x) keep_x[n1 * M + n2] = x;
      X[s] = raman ? x : cscale(x, p);
    };
    // The P buffers are free here (their last use, the Raman inverse or an energy
    // of the previous step, ended before a cluster barrier), so this inverse exchanges
    // through them and leaves the exchange buffers W untouched; W was last read by the
    // local passes of the previous forward transform, before the barrier of this
    // inverse, so the next forward cross pass needs no barrier of its own to free W.
    inv_via_p(cx, X, rdXs, e1);
    double energy = 0.0;
    if (want_e) energy = simpson_energy(cx, g, P);
    if (raman) {
      const V* Hp = (const V*)g.Hp;
      const R fR = (R)g.fR, f1 = (R)(1.0 - g.fR);
      auto rdPt = [&](int n1, int n2) -> V { return P[pad(tslot(n1, n2))]; };
      auto wrP = [&](int, int l, V v) { P[pad(l)] = v; };
      fwd(cx, P, rdPt, wrP, false, false);
      auto rdPH = [&](int o, int l) -> V { return cmul(P[pad(l)], ldro(&Hp[o * M + l])); };
      auto e3 = [&](int n1, int n2, V conv) {
        const int s = pad(tslot(n1, n2));
        V x = X[s];
        R p = cabs2(x);
        X[s] = cmul(x, mk<V>(f1 * p + fR * re(conv), fR * im(conv)));
      };
      inv(cx, P, rdPH, e3, false);
    }
    auto wrX = [&](int, int l, V v) { X[pad(l)] = v; };
    fwd(cx, X, rdXt, wrX, false, raman);  // without Raman, W is still free (see above)
    return energy;
  }

  // Simpson energy (nJ) of the time-domain powers held in buf[].x (this CTA's
  // local time slots, sample tsample(rank, slot)), summed over the cluster.
  static __device__ double simpson_energy(const Ctx& cx, const GridDev& g, const V* buf) {
    double e = 0.0;
    for (int l = threadIdx.x; l < M; l += T) e += simpson_w(tsample(cx.rank, l), N) * (double)re(buf[pad(l)]);
    double s[1] = {e * g.dt * 1e-3};
    cluster_sum<1>(cx, s);
    return s[0];
  }

  // Simpson energy (nJ) of G-(xhat)/N with xhat = pro(a, l), in the P buffer.
  // src 0: op.MA0, 1: op.acc (global), 2: the X buffer.
  static __device__ double energy_of(const Ctx& cx, const GridDev& g, const Op& op, int src) {
    const R invN = (R)(1.0 / (double)N);
    V* P = cx.P;
    auto pl = [&](int o, int l) -> V {
      return src == 0 ? op.MA0[o * M + l] : (src == 1 ? ldv(op.acc, o * M + l) : cx.X[pad(l)]);
    };
    auto ep = [&](int n1, int n2, V v) { P[pad(tslot(n1, n2))] = mk<V>(cabs2(cscale(v, invN)), (R)0); };
    inv(cx, P, pl, ep);
    return simpson_energy(cx, g, P);
  }

  // ---- boundary transforms --------------------------------------------------
  // The extended-state mode runs them in FP64, reusing the complex128
  // transform code on the same shared memory (X and P together hold one
  // double2 slice of M padded points).
  using E64 = Engine<double, LOGM, C, false, true>;
  static __device__ __forceinline__ typename E64::Ctx ctx64(const Ctx& cx, const GridDev& g) {
    typename E64::Ctx c;
    c.X = reinterpret_cast<double2*>(cx.X);
    c.P = c.X;
    c.W = c.X;  // in-place cross passes
    c.red = cx.red;
    c.tw = (const double2*)g.tw64;
    c.twl = (const double2*)g.twl64;
    c.twp = (const double2*)g.twp64;
    c.rank = cx.rank;
    return c;
  }

  // user field element <-> transform element (double-float plans convert complex128)
  static __device__ __forceinline__ V fv2v(const FV& f) {
    if constexpr (DD) {
      return mk<V>(R(f.x), R(f.y));
    } else {
      return f;
    }
  }
  static __device__ __forceinline__ FV v2fv(const V& v) {
    if constexpr (DD) {
      return make_double2((double)re(v), (double)im(v));
    } else {
      return v;
    }
  }

  // time -> spectral state: S = G+(field)
  static __device__ __noinline__ void to_spectral(const Ctx& cx, const GridDev& g, const FV* field, SV* S) {
    if constexpr (XS) {
      const typename E64::Ctx c = ctx64(cx, g);
      auto pro = [&](int o, int l) -> double2 { return field[o * M + l]; };
      auto epi = [&](int o, int l, double2 v) {
        dfc_store(S, o * M + l, dfc{df_from_double(v.x), df_from_double(v.y)});
      };
      E64::fwd(c, c.X, pro, epi);
    } else {
      auto pro = [&](int o, int l) -> V { return fv2v(field[o * M + l]); };
      auto epi = [&](int o, int l, V v) { S[o * M + l] = v; };
      fwd(cx, cx.P, pro, epi);
    }
  }

  // spectral state -> time field: field = G-(S)/N
  static __device__ __noinline__ void to_time(const Ctx& cx, const GridDev& g, const SV* S, FV* field) {
    if constexpr (XS) {
      const typename E64::Ctx c = ctx64(cx, g);
      const double invN = 1.0 / (double)N;
      auto pro = [&](int o, int l) -> double2 {
        const dfc v = dfc_load(S, o * M + l);
        return make_double2(df_to_double(v.re), df_to_double(v.im));
      };
      auto epi = [&](int o, int l, double2 v) { field[o * M + l] = make_double2(v.x * invN, v.y * invN); };
      E64::inv(c, c.X, pro, epi);
    } else {
      const R invN = (R)(1.0 / (double)N);
      auto pro = [&](int o, int l) -> V { return S[o * M + l]; };
      auto epi = [&](int o, int l, V v) { field[o * M + l] = v2fv(cscale(v, invN)); };
      inv(cx, cx.P, pro, epi);
    }
  }

  // exp(hh (i beta - alpha/2)) for this CTA's slice into E1; with E2 != null
  // also E2 = exp(2 hh (i beta - alpha/2)).  The phase beta*hh is formed in
  // FP64.  complex64 plans reduce it to [-pi, pi] before sincosf; complex128
  // plans call sincos; extended-state plans reduce it modulo pi/512 in FP64
  // (two-constant Cody-Waite), take cis(j pi/512) from a double-float table
  // and cis(t), |t| <= pi/1024, from its Taylor series in double-float, and
  // square the result for E2.
  static __device__ __noinline__ void exp_table(const Ctx& cx, const GridDev& g, double hh, SV* E1, SV* E2) {
    // the attenuation factor is 1 for a lossless fibre (skips an FP64 exp per thread)
    const double mag = g.alpha != 0.0 ? exp(-0.5 * g.alpha * hh) : 1.0;
    const int base = cx.rank * M;
    if constexpr (XS || DD) {
      const float4* tab = (const float4*)g.cis_df;
      const dff magd = df_from_double(mag);
      const bool lossy = g.alpha != 0.0;
      for (int l = threadIdx.x; l < M; l += T) {
        const int a = base + l;
        const double ph = g.beta[a] * hh;
        const double j = rint(ph * 0x1.45f306dc9c883p+7);          // 512 / pi
        double t = fma(-j, 0x1.921fb54000000p-8, ph);                // pi/512, high part
        t = fma(-j, 0x1.10b4611a62633p-38, t);                       // pi/512, low part
        const int ji = (int)(((long long)j) & 1023);
        const dff td = df_from_double(t);
        const float t2 = td.hi * td.hi;
        // sin t = t - t^3/6 + t^5/120 ; cos t = 1 - t^2/2 + t^4/24
        const dff sn = df_add_f(td, -td.hi * t2 * (1.0f / 6.0f) * (1.0f - t2 * 0.05f));
        dff tt = two_prod(td.hi, td.hi);
        tt.lo = fmaf(2.0f * td.hi, td.lo, tt.lo);
        dff cs = two_sum(1.0f, -0.5f * tt.hi);
        cs.lo += -0.5f * tt.lo + t2 * t2 * (1.0f / 24.0f);
        cs = fast_two_sum(cs.hi, cs.lo);
        const float4 tv = __ldg(&tab[ji]);
        dfc e = dfc_mul(dfc{{tv.x, tv.z}, {tv.y, tv.w}}, dfc{cs, sn});
        if (lossy) e = dfc_scale(e, magd);
        if constexpr (XS) {
          dfc_store(E1, a, e);
          if (E2) dfc_store(E2, a, dfc_mul(e, e));
        } else {
          E1[a] = mk<V>(ddf(e.re.hi, e.re.lo), ddf(e.im.hi, e.im.lo));
          if (E2) {
            const dfc e2 = dfc_mul(e, e);
            E2[a] = mk<V>(ddf(e2.re.hi, e2.re.lo), ddf(e2.im.hi, e2.im.lo));
          }
        }
      }
    } else {
      for (int l = threadIdx.x; l < M; l += T) {
        const int a = base + l;
        const double ph = g.beta[a] * hh;
        R s, c;
        if constexpr (sizeof(R) == 4) {
          const double TWO_PI = 6.283185307179586476925286766559;
          sincosf((float)(ph - TWO_PI * rint(ph * (1.0 / TWO_PI))), &s, &c);
        } else {
          sincos(ph, &s, &c);
        }
        E1[a] = mk<V>((R)mag * c, (R)mag * s);
        if (E2) {
          const double ph2 = g.beta[a] * (2.0 * hh);
          const double mag2 = g.alpha != 0.0 ? exp(-g.alpha * hh) : 1.0;
          if constexpr (sizeof(R) == 4) {
            const double TWO_PI = 6.283185307179586476925286766559;
            sincosf((float)(ph2 - TWO_PI * rint(ph2 * (1.0 / TWO_PI))), &s, &c);
          } else {
            sincos(ph2, &s, &c);
          }
          E2[a] = mk<V>((R)mag2 * c, (R)mag2 * s);
        }
      }
    }
    __syncthreads();
  }

  static __device__ __forceinline__ R gain_a(const GridDev& g, double hh, double energy) {
    return (R)(g.gain_log * hh / (2.0 * g.gain_len) / (1.0 + energy / g.E_sat));
  }

  // Yb two-level model (Amplifier2LevelModel.factor, amplifier.py:346-379) for one
  // linear-operator call over the step hh whose argument has inversion sums (sr, ss):
  // the inversion n2 = N2 / N, the pump update Pp <- Pp exp(1000 hh g_p), and the
  // coefficient 500 hh n2 of alpha_s N in the gain exponent (thread 0).
  static __device__ __forceinline__ R yb_call(const GridDev& g, InstState& st, double hh, double sr,
                                              double ss) {
    const double tp = st.pp / g.yb_psat_p;
    const double n2 = (g.yb_ratio_p * tp + sr) / (1.0 + tp + ss);
    st.pp *= exp((g.yb_alpha_p * n2 - g.yb_eta_p) * hh * 1e3);
    return (R)(500.0 * hh * n2);
  }

  // Yb model inversion sums sum_k w_ratio |X_k|^2, sum_k w_sat |X_k|^2 of a spectrum
  // X = n fft(x) held in src (0: op.MA0, 1: op.acc, 2: the X buffer), over the cluster,
  // into out[0..1] (shared memory; written by thread 0 before the closing barrier)
  static __device__ __forceinline__ void yb_sums(const Ctx& cx, const GridDev& g, const Op& op, int src,
                                              double* out) {
    const double2* w = (const double2*)g.ybw;
    const int base = cx.rank * M;
    double s0 = 0.0, s1 = 0.0;
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = base + l;
      const V v = src == 0 ? op.MA0[a] : (src == 1 ? ldv(op.acc, a) : cx.X[pad(l)]);
      const double p = (double)re(v) * (double)re(v) + (double)im(v) * (double)im(v);
      const double2 ww = __ldg(&w[a]);
      s0 += ww.x * p;
      s1 += ww.y * p;
    }
    double s[2] = {s0, s1};
    cluster_sum<2>(cx, s);
    if (threadIdx.x == 0) {
      out[0] = s[0];
      out[1] = s[1];
    }
    __syncthreads();
  }

  // ---- elementwise stage loops (fused end of one stage / start of the next) --
  // Each loop visits this CTA's M slots in batches of U per thread: every load
  // of a batch (global state arrays and the shared X slot) is issued before
  // the batch's arithmetic and stores, so U slots' loads are in flight at once.
  // (Loads cannot be hoisted above the previous slot's stores by the compiler,
  // which must assume they may alias.)  M is a multiple of 4 T for every class.
  using SL = typename std::conditional<XS, dfc, V>::type;  // full-precision state value
  static __device__ __forceinline__ SL lds(const SV* p, int a) {
    if constexpr (XS) {
      return dfc_load(p, a);
    } else {
      return p[a];
    }
  }
  static __device__ __forceinline__ V slhi(const SL& v) {
    if constexpr (XS) {
      return dfc_hi(v);
    } else {
      return v;
    }
  }
  static __device__ __forceinline__ V ik(R k, V v) { return cscale(cmul_i<1>(v), k); }  // i k v

  template <int U, class In, class Ld, class St>
  static __device__ __forceinline__ void each_slot(Ld&& ld, St&& st) {
    static_assert(M % (U * T) == 0, "slot batches must tile the slice");
    for (int l0 = tidx<2>(); l0 < M; l0 += U * T) {
      In in[U];
#pragma unroll
      for (int u = 0; u < U; ++u) in[u] = ld(l0 + u * T);
#pragma unroll
      for (int u = 0; u < U; ++u) st(l0 + u * T, in[u]);
    }
  }

  // X = Z (stage input of N(A) for state Z)
  static __device__ __forceinline__ void load_state(const Ctx& cx, const SV* Z) {
    const int base = cx.rank * M;
    V* X = cx.X;
    each_slot<4, V>([&](int l) { return ldv(Z, base + l); }, [&](int l, const V& v) { X[pad(l)] = v; });
    __syncthreads();
  }

  // MA = i K X  (N(A) of the state, unscaled by h)
  static __device__ __forceinline__ void store_ma(const Ctx& cx, const GridDev& g, V* MA) {
    const R* Kr = (const R*)g.Kr;
    const int base = cx.rank * M;
    V* X = cx.X;
    struct In { V x; R k; };
    each_slot<4, In>([&](int l) { return In{X[pad(l)], ldro(&Kr[base + l])}; },
                     [&](int l, const In& r) { MA[base + l] = ik(r.k, r.x); });
    __syncthreads();
  }

  // stage 1 input: S_I + k0/2 with S_I = L(A), k0 = L(h N(A))
  static __device__ __forceinline__ void pre_stage1(const Ctx& cx, const Op& ops) {
    const Op op = ops;
    const R half = (R)0.5;
    const int base = cx.rank * M;
    V* X = cx.X;
    struct In { V e, s0, ma; };
    each_slot<4, In>(
        [&](int l) {
          const int a = base + l;
          return In{ldv(op.Et, a), ldv(op.S0, a), op.MA0[a]};
        },
        [&](int l, const In& r) {
          const int a = base + l;
          const V si = cmul(mult(op, a, r.e, op.aA), r.s0);
          const V k0 = cscale(cmul(mult(op, a, r.e, op.ak0), r.ma), op.h);
          X[pad(l)] = cadd(si, cscale(k0, half));
        });
    __syncthreads();
  }

  // k1 = h N; acc = S_I + k0/6 + k1/3; stage 2 input S_I + k1/2
  static __device__ __forceinline__ void post_stage1(const Ctx& cx, const Op& ops) {
    const Op op = ops;
    const R half = (R)0.5, sixth = (R)(1.0 / 6.0), third = (R)(1.0 / 3.0);
    const int base = cx.rank * M;
    V* X = cx.X;
    struct In { V x; R k; SL e, s0; V ma; };
    each_slot<4, In>(
        [&](int l) {
          const int a = base + l;
          return In{X[pad(l)], ldro(&op.Kr[a]), lds(op.Et, a), lds(op.S0, a), op.MA0[a]};
        },
        [&](int l, const In& r) {
          const int a = base + l;
          const V k1 = ik(op.h * r.k, r.x);
          if constexpr (XS) {
            const dfc si = dfc_mul(mult_df(op, a, r.e, op.aA), r.s0);
            const V k0 = cscale(cmul(mult(op, a, dfc_hi(r.e), op.ak0), r.ma), op.h);
            dfc_store(op.acc, a, dfc_add_f(si, cadd(cscale(k0, sixth), cscale(k1, third))));
            X[pad(l)] = cadd(dfc_hi(si), cscale(k1, half));
          } else {
            const V si = cmul(mult(op, a, r.e, op.aA), r.s0);
            const V k0 = cscale(cmul(mult(op, a, r.e, op.ak0), r.ma), op.h);
            op.acc[a] = cadd(cadd(si, cscale(k0, sixth)), cscale(k1, third));
            X[pad(l)] = cadd(si, cscale(k1, half));
          }
        });
    __syncthreads();
  }

  // k2 = h N; acc += k2/3; stage 3 input L(S_I + k2) (gain: S_I + k2, scaled after)
  static __device__ __forceinline__ void post_stage2(const Ctx& cx, const Op& ops) {
    const Op op = ops;
    const R third = (R)(1.0 / 3.0);
    const int base = cx.rank * M;
    V* X = cx.X;
    struct In { V x; R k; SL acc; V e, s0; };
    each_slot<4, In>(
        [&](int l) {
          const int a = base + l;
          return In{X[pad(l)], ldro(&op.Kr[a]), lds(op.acc, a), ldv(op.Et, a), ldv(op.S0, a)};
        },
        [&](int l, const In& r) {
          const int a = base + l;
          const V k2 = ik(op.h * r.k, r.x);
          if constexpr (XS) {
            dfc_store(op.acc, a, dfc_add_f(r.acc, cscale(k2, third)));
          } else {
            op.acc[a] = cadd(r.acc, cscale(k2, third));
          }
          const V u = cadd(cmul(mult(op, a, r.e, op.aA), r.s0), k2);
          X[pad(l)] = op.gain ? u : cmul(r.e, u);
        });
    __syncthreads();
  }

  // One step of the exponential split-step methods without self-steepening:
  //   S_L = E1 S                                  (first linear step)
  //   B = G-(S_L)/N, a = G-(S or S_L)/N           (time domain; B kept in global Bt)
  //   t = (1 - fR)|a|^2 + fR G-(Hp G+(|a|^2))     (or |a|^2; default_exp_f[_all],
  //                                                 nonlinearity.py:209-221,269-270)
  //   A_N = exp(i gamma h t) B ;  S' = E2 G+(A_N) (second linear step)
  // computed as S' = E2 (S_L + G+((exp(i gamma h t) - 1) B)), which keeps the
  // propagation state's precision when the nonlinear phase per step is small.
  //   Solver.ss_symmetric (solver.py:267-275): E1 = E2 = exp(hD/2), a from S
  //   Solver.ss_reduced   (solver.py:277-287): E1 = E2 = exp(hD/2), a from S_L
  //   Solver.ss_simple    (solver.py:256-265): E1 = 1, E2 = exp(hD), a from S
  static __device__ __forceinline__ void ss_symmetric_step(const Ctx& cx, const GridDev& g, const SV* S, SV* Sh,
                                                        V* Bt, const SV* E, const SV* E2, double h,
                                                        bool t_from_sl) {
    const R invN = (R)(1.0 / (double)N);
    const int base = cx.rank * M;
    V* X = cx.X;
    V* P = cx.P;
    if (E) {  // S_L = E S -> Sh
      struct In { SL e, s; };
      each_slot<4, In>([&](int l) { return In{lds(E, base + l), lds(S, base + l)}; },
                       [&](int l, const In& r) {
                         if constexpr (XS) {
                           dfc_store(Sh, base + l, dfc_mul(r.e, r.s));
                         } else {
                           Sh[base + l] = cmul(r.e, r.s);
                         }
                       });
      __syncthreads();
    } else {  // no first linear step (ss_simple): S_L = S
      each_slot<4, SL>([&](int l) { return lds(S, base + l); }, [&](int l, const SL& v) { sts(Sh, base + l, v); });
      __syncthreads();
    }
    auto rdSh = [&](int o, int l) -> V { return ldv(Sh, o * M + l); };
    auto wrB = [&](int n1, int n2, V v) { Bt[n1 * M + n2] = cscale(v, invN); };
    inv(cx, X, rdSh, wrB);  // B = G-(S_L)/N
    const SV* Sa = t_from_sl ? Sh : S;
    auto rdS = [&](int o, int l) -> V { return ldv(Sa, o * M + l); };
    auto e1 = [&](int n1, int n2, V v) {
      const int sl = pad(tslot(n1, n2));
      const V x = cscale(v, invN);
      X[sl] = x;
      P[sl] = mk<V>(cabs2(x), (R)0);
    };
    inv(cx, X, rdS, e1);  // a = G-(S or S_L)/N, |a|^2
    if (g.raman) {
      const V* Hp = (const V*)g.Hp;
      const R fR = (R)g.fR, f1 = (R)(1.0 - g.fR);
      auto rdPt = [&](int n1, int n2) -> V { return P[pad(tslot(n1, n2))]; };
      auto wrP = [&](int, int l, V v) { P[pad(l)] = v; };
      fwd(cx, P, rdPt, wrP);
      auto rdPH = [&](int o, int l) -> V { return cmul(P[pad(l)], ldro(&Hp[o * M + l])); };
      auto e3 = [&](int n1, int n2, V conv) {
        const int sl = pad(tslot(n1, n2));
        P[sl] = mk<V>(f1 * cabs2(X[sl]) + fR * re(conv), fR * im(conv));
      };
      inv(cx, P, rdPH, e3);
    }
    __syncthreads();
    // Delta = (exp(i gamma h t) - 1) B in X: exp(x + iy) - 1 = expm1(x) cos y - 2 sin^2(y/2) + i e^x sin y
    const double gh = h * (double)ldro((const R*)g.Kr);  // gamma h (Kr = gamma without self-steepening)
    for (int l = threadIdx.x; l < M; l += T) {
      const V t = P[pad(l)];
      const V b = Bt[tsample(cx.rank, l)];
      const R px = (R)(-gh) * im(t), py = (R)gh * re(t);
      V ephi;
      if constexpr (DD) {  // the phase factor in FP64, ~1e-16, rounded to double-float
        double sn, cs;
        sincos((double)py, &sn, &cs);
        const double hs = sin(0.5 * (double)py), em1 = expm1((double)px);
        ephi = mk<V>(R(em1 * cs - 2.0 * hs * hs), R((em1 + 1.0) * sn));
      } else {
        R sn, cs;
        if constexpr (sizeof(R) == 4) {
          sincosf(py, &sn, &cs);
        } else {
          sincos(py, &sn, &cs);
        }
        const R hs = sizeof(R) == 4 ? sinf(0.5f * (float)py) : (R)sin(0.5 * (double)py);
        const R em1 = sizeof(R) == 4 ? expm1f((float)px) : (R)expm1((double)px);
        ephi = mk<V>(em1 * cs - (R)2 * hs * hs, (em1 + (R)1) * sn);
      }
      X[pad(l)] = cmul(ephi, b);
    }
    __syncthreads();
    // S' = E2 (S_L + G+(Delta))
    auto rdXt = [&](int n1, int n2) -> V { return X[pad(tslot(n1, n2))]; };
    auto wrS = [&](int, int l, V v) {
      const int a = base + l;
      if constexpr (XS) {
        dfc_store(Sh, a, dfc_mul(dfc_load(E2, a), dfc_add_f(dfc_load(Sh, a), v)));
      } else {
        Sh[a] = cmul(E2[a], cadd(Sh[a], v));
      }
    };
    fwd(cx, X, rdXt, wrS);
  }

  // ---- split-step kernel: the remaining step methods and their adaptive driver ----
  static __device__ __forceinline__ SL sl_mul(const SL& a, const SL& b) {
    if constexpr (XS) {
      return dfc_mul(a, b);
    } else {
      return cmul(a, b);
    }
  }
  static __device__ __forceinline__ SL sl_add(const SL& a, const V& b) {
    if constexpr (XS) {
      return dfc_add_f(a, b);
    } else {
      return cadd(a, b);
    }
  }
  static __device__ __forceinline__ void sts(SV* p, int a, const SL& v) {
    if constexpr (XS) {
      dfc_store(p, a, v);
    } else {
      p[a] = v;
    }
  }
  // nonlinear operator shared by every step of the split-step kernel (one copy of its code)
  static __device__ __noinline__ void nonlinear_ss(const Ctx& cx, const GridDev& g, V* keep_x) {
    nonlinear(cx, g, false, keep_x);
  }

  // Solver.ss_sym_midpoint / ss_sym_rk4 (solver.py:323-337) with Solver.midpoint / rk4
  // (solver.py:101-116) on the nonlinear term, on the spectral state:
  //   S_L = E S;  k_j = h N(S_L + c_j k_{j-1});  S' = E (S_L + sum_j b_j k_j)
  // NS = 2: midpoint (c = 0, 1/2; b = 0, 1); NS = 4: classical RK4.  acc: RK4 sum.
  template <int NS>
  static __device__ __forceinline__ void ss_rk_step(const Ctx& cx, const GridDev& g, const SV* S, SV* Sh,
                                                    SV* acc, const SV* E, double hd) {
    const int base = cx.rank * M;
    V* X = cx.X;
    const R* Kr = (const R*)g.Kr;
    const R h = (R)hd, half = (R)0.5, sixth = (R)(1.0 / 6.0), third = (R)(1.0 / 3.0);
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = base + l;
      const SL sl = sl_mul(lds(E, a), lds(S, a));
      sts(Sh, a, sl);
      X[pad(l)] = slhi(sl);
    }
    __syncthreads();
    for (int j = 0; j < NS; ++j) {
      nonlinear_ss(cx, g, nullptr);
      for (int l = threadIdx.x; l < M; l += T) {
        const int a = base + l;
        const V k = ik(h * ldro(&Kr[a]), X[pad(l)]);
        const SL sl = lds(Sh, a);
        if (NS == 2) {
          if (j == 0) {
            X[pad(l)] = cadd(slhi(sl), cscale(k, half));
          } else {
            sts(Sh, a, sl_mul(lds(E, a), sl_add(sl, k)));
          }
        } else if (j == 0) {
          sts(acc, a, sl_add(sl, cscale(k, sixth)));
          X[pad(l)] = cadd(slhi(sl), cscale(k, half));
        } else if (j < 3) {
          sts(acc, a, sl_add(lds(acc, a), cscale(k, third)));
          X[pad(l)] = cadd(slhi(sl), j == 1 ? cscale(k, half) : k);
        } else {
          sts(Sh, a, sl_mul(lds(E, a), sl_add(lds(acc, a), cscale(k, sixth))));
        }
      }
      __syncthreads();
    }
  }

  // ss_agrawal's ratio n(y)/y where |y| > 1e-5, else 0 (solver.py:295-316), in FP64
  // (out of line: FP64 library code, called from every transform epilogue site)
  static __device__ __noinline__ V agr_ratio(V n, V y) {
    const double yr = (double)re(y), yi = (double)im(y);
    if (!(hypot(yr, yi) > 1.0e-5)) return mk<V>(R(0.0), R(0.0));
    const double nr = (double)re(n), ni = (double)im(n), d = yr * yr + yi * yi;
    return mk<V>(R((nr * yr + ni * yi) / d), R((ni * yr - nr * yi) / d));
  }
  // exp(hh r) - 1 = expm1(x) cos y - 2 sin^2(y/2) + i e^x sin y, x + i y = hh r, in FP64
  static __device__ __noinline__ V cexpm1_scaled(double hh, V r) {
    const double x = hh * (double)re(r), y = hh * (double)im(r);
    double sn, cs;
    sincos(y, &sn, &cs);
    const double hs = sin(0.5 * y), em1 = expm1(x);
    return mk<V>(R(em1 * cs - 2.0 * hs * hs), R((em1 + 1.0) * sn));
  }

  // Solver.ss_agrawal (solver.py:290-320), with r(Y) = n(Y)/Y (0 where |Y| <= 1e-5):
  //   A_L = L(A, h/2);  Y_1 = L(exp(h r(A)) A_L, h/2);  S' = L(exp(h/2 (r(Y_1) + r(A))) A_L, h/2)
  // in the spectral state, each exponential step as S_L + G+((exp(.) - 1) a_L) so that a
  // small nonlinear phase keeps the state's precision.  Time-domain scratch (N samples
  // each): y (the field whose ratio is taken, then Delta_2), rA = r(A), aL = a_L.
  static __device__ __forceinline__ void ss_agrawal_step(const Ctx& cx, const GridDev& g, const SV* S, SV* Sh,
                                                         V* y, V* rA, V* aL, const SV* E, double h) {
    const int base = cx.rank * M;
    const R invN = (R)(1.0 / (double)N);
    V* X = cx.X;
    const R* Kr = (const R*)g.Kr;
    auto rdKX = [&](int, int l) -> V { return ik(ldro(&Kr[base + l]), X[pad(l)]); };
    // r(A): x -> y and X = G+(x R(x)) by the nonlinear operator, n(A) = G-(i K X)/N
    load_state(cx, S);
    nonlinear_ss(cx, g, y);
    auto wr_rA = [&](int n1, int n2, V v) {
      const int t = n1 * M + n2;
      rA[t] = agr_ratio(cscale(v, invN), y[t]);
    };
    inv(cx, X, rdKX, wr_rA);
    // S_L = E S -> Sh, a_L = G-(S_L)/N
    auto rdSL = [&](int, int l) -> V {
      const int a = base + l;
      const SL sl = sl_mul(lds(E, a), lds(S, a));
      sts(Sh, a, sl);
      return slhi(sl);
    };
    auto wr_aL = [&](int n1, int n2, V v) { aL[n1 * M + n2] = cscale(v, invN); };
    inv(cx, X, rdSL, wr_aL);
    // Y_1 = E (S_L + G+((exp(h r(A)) - 1) a_L)) into X, the nonlinear operator's input
    auto rdD1 = [&](int n1, int n2) -> V {
      const int t = n1 * M + n2;
      return cmul(cexpm1_scaled(h, rA[t]), aL[t]);
    };
    auto wrY1 = [&](int, int l, V v) {
      const int a = base + l;
      X[pad(l)] = slhi(sl_mul(lds(E, a), sl_add(lds(Sh, a), v)));
    };
    fwd(cx, X, rdD1, wrY1);
    // r(Y_1), then Delta_2 = (exp(h/2 (r(Y_1) + r(A))) - 1) a_L into y
    nonlinear_ss(cx, g, y);
    auto wrD2 = [&](int n1, int n2, V v) {
      const int t = n1 * M + n2;
      const V r1 = agr_ratio(cscale(v, invN), y[t]);
      y[t] = cmul(cexpm1_scaled(0.5 * h, cadd(r1, rA[t])), aL[t]);
    };
    inv(cx, X, rdKX, wrD2);
    // S' = E (S_L + G+(Delta_2))
    auto rdD2 = [&](int n1, int n2) -> V { return y[n1 * M + n2]; };
    auto wrS = [&](int, int l, V v) {
      const int a = base + l;
      sts(Sh, a, sl_mul(lds(E, a), sl_add(lds(Sh, a), v)));
    };
    fwd(cx, X, rdD2, wrS);
  }

  // one step of split-step method sm from S to Sh; E = exp(hD/2) (exp(hD) for
  // ss_simple); tmp: three N-element scratch slots.  Out of line: the fixed and the
  // adaptive driver call it from four sites.
  static __device__ __noinline__ void ss_step(const Ctx& cx, const GridDev& g, int sm, const SV* S, SV* Sh,
                                              SV* tmp, const SV* E, double h) {
    if (sm >= 3 && sm <= 5) {
      ss_symmetric_step(cx, g, S, Sh, reinterpret_cast<V*>(tmp), sm == 4 ? nullptr : E, E, h, sm == 5);
    } else if (sm == 2) {
      ss_rk_step<4>(cx, g, S, Sh, tmp, E, h);
    } else if (sm == 6) {
      ss_rk_step<2>(cx, g, S, Sh, tmp, E, h);
    } else {
      ss_agrawal_step(cx, g, S, Sh, reinterpret_cast<V*>(tmp), reinterpret_cast<V*>(tmp + N),
                      reinterpret_cast<V*>(tmp + 2 * N), E, h);
    }
  }

  // Solver.errors (solver.py:57-70): the order of each split step in the adaptive driver
  static __device__ __forceinline__ int ss_order(int sm) {
    return (sm == 4 || sm == 5) ? 2 : (sm == 2 ? 5 : 3);
  }

  // step-doubling error norms of F (fine) against Cc (coarse) over the cluster, and the
  // local extrapolation fa F - fb Cc into Cc (stepper.py:231-245, 272-274, 338)
  static __device__ void ss_extrapolate(const Ctx& cx, const SV* F, SV* Cc, double fa, double fb, double (&s)[3]) {
    const int base = cx.rank * M;
    double d2 = 0.0, f2 = 0.0, bad = 0.0;
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = base + l;
      if constexpr (XS) {
        const dfc f = dfc_load(F, a), c = dfc_load(Cc, a);
        const double fr = df_to_double(f.re), fi = df_to_double(f.im);
        const double dr = fr - df_to_double(c.re), di = fi - df_to_double(c.im);
        d2 += dr * dr + di * di;
        f2 += fr * fr + fi * fi;
        if (!isfinite(f.re.hi) || !isfinite(f.im.hi)) bad = 1.0;
        dfc_store(Cc, a, dfc_add(dfc_scale(f, df_from_double(fa)), dfc_scale(c, df_from_double(-fb))));
      } else {
        const V f = F[a], c = Cc[a];
        const double fr = (double)re(f), fi = (double)im(f);
        const double dr = fr - (double)re(c), di = fi - (double)im(c);
        d2 += dr * dr + di * di;
        f2 += fr * fr + fi * fi;
        if (!isfinite(fr) || !isfinite(fi)) bad = 1.0;
        Cc[a] = mk<V>(R(fa) * re(f) - R(fb) * re(c), R(fa) * im(f) - R(fb) * im(c));
      }
    }
    s[0] = d2;
    s[1] = f2;
    s[2] = bad;
    cluster_sum<3>(cx, s);
  }

  // dst = E dst over this CTA's slice: the linear half steps of the split-step method
  static __device__ __noinline__ void scale_state(const Ctx& cx, SV* dst, const SV* E) {
    const int base = cx.rank * M;
    struct In { SL e, s; };
    each_slot<4, In>([&](int l) { return In{lds(E, base + l), lds(dst, base + l)}; },
                     [&](int l, const In& r) {
                       if constexpr (XS) {
                         dfc_store(dst, base + l, dfc_mul(r.e, r.s));
                       } else {
                         dst[base + l] = cmul(r.e, r.s);
                       }
                     });
    __syncthreads();
  }

  static __device__ __forceinline__ void scale_stage3(const Ctx& cx, const Op& op) {
    const int base = cx.rank * M;
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = base + l;
      cx.X[pad(l)] = cmul(mult(op, a, ldv(op.Et, a), op.a3), cx.X[pad(l)]);
    }
    __syncthreads();
  }

  // k3 = h N; result = L(acc) + k3/6 -> out; coarse: error norms against Sf and
  // the local extrapolation (stepper.py:272-274,338) (16 A_fine - A_coarse)/15 -> out.
  static __device__ __forceinline__ void post_stage3(const Ctx& cx, const Op& ops, bool coarse,
                                                     double (&s)[3]) {
    const Op op = ops;
    const R sixth = (R)(1.0 / 6.0);
    const R fa = (R)(16.0 / 15.0), fb = (R)(1.0 / 15.0);
    const int base = cx.rank * M;
    V* X = cx.X;
    R d2 = 0, f2 = 0;
    double bad = 0.0;
    struct In { V x; R k; SL e, acc, sf; };
    each_slot<4, In>(
        [&](int l) {
          const int a = base + l;
          In r;
          r.x = X[pad(l)];
          r.k = ldro(&op.Kr[a]);
          r.e = lds(op.Et, a);
          r.acc = lds(op.acc, a);
          if (coarse) r.sf = lds(op.Sf, a);
          return r;
        },
        [&](int l, const In& r) {
          const int a = base + l;
          const V k3 = ik(op.h * r.k, r.x);
          if constexpr (XS) {
            const dfc res = dfc_add_f(dfc_mul(mult_df(op, a, r.e, op.ao), r.acc), cscale(k3, sixth));
            if (!coarse) {
              dfc_store(op.out, a, res);
            } else {
              const dfc sf = r.sf;
              const dfc d = dfc_sub(sf, res);
              d2 += d.re.hi * d.re.hi + d.im.hi * d.im.hi;
              f2 += sf.re.hi * sf.re.hi + sf.im.hi * sf.im.hi;
              if (!isfinite(sf.re.hi) || !isfinite(sf.im.hi)) bad = 1.0;
              const dff FA = {(float)(16.0 / 15.0), (float)(16.0 / 15.0 - (double)(float)(16.0 / 15.0))};
              const dff FB = {(float)(-1.0 / 15.0), (float)(-1.0 / 15.0 - (double)(float)(-1.0 / 15.0))};
              dfc_store(op.out, a, dfc_add(dfc_scale(sf, FA), dfc_scale(res, FB)));
            }
          } else {
            const V res = cadd(cmul(mult(op, a, r.e, op.ao), r.acc), cscale(k3, sixth));
            if (!coarse) {
              op.out[a] = res;
            } else {
              const V sf = r.sf;
              const V d = csub(sf, res);
              d2 += cabs2(d);
              f2 += cabs2(sf);
              if (!isfinite(re(sf)) || !isfinite(im(sf))) bad = 1.0;
              op.out[a] = mk<V>(fa * re(sf) - fb * re(res), fa * im(sf) - fb * im(res));
            }
          }
        });
    s[0] = (double)d2;
    s[1] = (double)f2;
    s[2] = bad;
    if (coarse) {
      cluster_sum<3>(cx, s);
    } else {
      __syncthreads();
    }
  }

  // FP64 energy (Parseval, nJ) and photon number of state S.
  static __device__ __noinline__ void diagnostics(const Ctx& cx, const GridDev& g, const SV* S,
                                                  double* E, double* Nph) {
    double e = 0.0, p = 0.0;
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = cx.rank * M + l;
      double s2;
      if constexpr (XS) {
        const dfc v = dfc_load(S, a);
        const double re = df_to_double(v.re), im = df_to_double(v.im);
        s2 = re * re + im * im;
      } else {
        s2 = (double)cabs2(S[a]);
      }
      e += s2;
      p += s2 / g.nu[a];
    }
    double s[2] = {e, p};
    cluster_sum<2>(cx, s);
    const double scale = g.window_t / ((double)N * (double)N);
    *E = s[0] * scale * 1e-3;
    *Nph = s[1] * scale / 6.62607015e-10;
  }

  // Per-CTA control block in shared memory: uniform state read by all
  // threads, written by thread 0 between barriers.
  struct Ctl {
    GridDev g;
    InstDev d;
    InstState st;
    Op op;
    double eA[2], eN[2];
    double yA[2][2], yN[2][2];  // Yb model: inversion sums of the states and their N(A)
    double yT[2][2];            // Yb model: sums of the third and fourth linear-call arguments
  };
  static_assert(sizeof(Ctl) <= 1024, "control block size");

  static __device__ void store_trace(const Ctx& cx, const KParams& kp, Ctl& c, const SV* S, double z) {
    if (c.st.ntraces >= c.d.max_traces) {
      __syncthreads();
      if (threadIdx.x == 0) c.st.trace_overflow = 1;
      __syncthreads();
      return;
    }
    FV* tr = (FV*)kp.traces + c.d.trace_off + (long long)c.st.ntraces * N;
    to_time(cx, c.g, S, tr);
    if (cx.rank == 0 && threadIdx.x == 0) kp.trace_z[c.d.tracez_off + c.st.ntraces] = z;
    __syncthreads();
    if (threadIdx.x == 0) c.st.ntraces += 1;
    __syncthreads();
  }

  // Fixed-step driver after a step (stepper.py:164-221): z from the linspace mesh,
  // the new state becomes current, traces every int(steps/traces) steps.
  static __device__ __forceinline__ void fixed_step_done(const Ctx& cx, const KParams& kp, Ctl& c, SV* base,
                                                         double h) {
    const InstDev& d = c.d;
    InstState& st = c.st;
    const double dz = d.length / d.total_steps;  // numpy linspace step of the z mesh
    const int storage_step = d.traces > 0 ? d.total_steps / d.traces : 0;
    const long long i = st.steps;
    __syncthreads();
    if (threadIdx.x == 0) {
      st.attempts += 1;
      st.sidx ^= 1;
      st.accepted += 1;
      st.steps += 1;
      st.z = (st.steps == d.total_steps) ? d.length : (double)st.steps * dz;
      if (st.steps >= d.total_steps) {
        st.status = ST_OK;
        st.phase = 2;
      }
    }
    __syncthreads();
    if (d.traces != 1 && storage_step > 0 && (i % storage_step) == 0)
      store_trace(cx, kp, c, base + (long long)st.sidx * N, (double)i * dz + h);
  }

  // The whole propagation of one instance.  Every CTA of a cluster evaluates
  // the same control decisions from the same cluster-reduced values, so all
  // CTAs follow one path.  An attempt is a loop over its nonlinear
  // evaluations ("slots"), so the transform code is inlined once:
  //   adaptive: N(A) of S, 3 stages of rk4ip(S, h/2) -> Sh, N(A) of Sh,
  //             3 stages of rk4ip(Sh, h/2) -> Sf, 3 stages of rk4ip(S, h) -> Sh'
  //   fixed   : N(A) of S, 3 stages of rk4ip(S, h) -> S'
  // Methods of the RK4IP stage loop (kernel kind 0): RK4IP fixed step, ARK4IP and
  // ss_sym_rk4; the exponential split steps (kind 1) run in a kernel of their own, so that
  // neither step loop's code weighs on the other's register allocation.
  static __device__ __forceinline__ bool rk_method(int method) { return method <= 2; }

  template <int KIND>
  static __device__ __forceinline__ void run(const KParams& kp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int cid = blockIdx.x / C;
    if (cid >= kp.n_order) return;
    Ctx cx;
    cx.X = (V*)smem_raw;
    cx.P = cx.X + MP;
    cx.W = C > 1 ? cx.P + MP : nullptr;
    cx.red = (double*)(cx.X + NBUF * MP);
    Ctl& c = *(Ctl*)(cx.red + RED);
    if constexpr (C > 1) {
      cx.rank = (int)cg::this_cluster().block_rank();
    } else {
      cx.rank = 0;
    }
    const int id = kp.order[cid];
    if (threadIdx.x == 0) {
      c.d = kp.inst[id];
      c.g = kp.grids[c.d.grid];
      c.st = kp.state[id];
      c.eA[0] = c.st.cache_eA;
      c.eN[0] = c.st.cache_eN;
      c.eA[1] = c.eN[1] = 0.0;
      c.yA[0][0] = c.st.cache_y[0];
      c.yA[0][1] = c.st.cache_y[1];
      c.yN[0][0] = c.st.cache_y[2];
      c.yN[0][1] = c.st.cache_y[3];
      c.yA[1][0] = c.yA[1][1] = c.yN[1][0] = c.yN[1][1] = 0.0;
    }
    __syncthreads();
    // an instance of the other kernel's kind: every CTA of the cluster leaves here, before
    // any cluster barrier
    if (rk_method(c.d.method) != (KIND == 0)) return;
    const GridDev& g = c.g;
    const InstDev& d = c.d;
    InstState& st = c.st;
    Op& op = c.op;
    cx.tw = (const V*)g.tw;
    cx.twl = (const V*)g.twl;
    cx.twp = (const V*)g.twp;
    FV* field = (FV*)kp.fields + d.field_off;
    SV* base = (SV*)kp.scratch + d.scratch_off;
    long long budget = kp.max_attempts > 0 ? kp.max_attempts : (1ll << 62);
#if GNLSE_PROF
    long long prof_acc[4] = {0, 0, 0, 0};
    const long long prof_start = clock64();
#endif

    if (st.phase == 0) {
      int ntr = 0, ovf = 0;
      if ((d.method == 1 || (d.method & 16)) && d.traces != 1) {
        if (d.max_traces > 0) {
          FV* tr = (FV*)kp.traces + d.trace_off;
          for (int l = threadIdx.x; l < M; l += T) tr[cx.rank * M + l] = field[cx.rank * M + l];
          if (cx.rank == 0 && threadIdx.x == 0) kp.trace_z[d.tracez_off] = 0.0;
          ntr = 1;
        } else {
          ovf = 1;
        }
      }
      to_spectral(cx, g, field, base);
      double e_in, n_in;
      diagnostics(cx, g, base, &e_in, &n_in);
      if (threadIdx.x == 0) {
        st.ntraces = ntr;
        st.trace_overflow = ovf;
        st.E_in = e_in;
        st.Nph_in = n_in;
        st.sidx = 0;
        st.z = 0.0;
        st.h = (d.method == 1 || (d.method & 16)) ? d.h0 : d.length / d.total_steps;
        st.z_ignore = d.length / d.traces;
        st.ma_valid = 0;
        st.ta = 0;
        st.pp = g.yb_pp0;
        st.status = ST_RUNNING;
        st.phase = 1;
      }
      __syncthreads();
    }

    const bool adaptive = d.method == 1;
    // Solver.ss_sym_rk4 (solver.py:330-337), fixed step: S <- E S, classical RK4 on the
    // nonlinear term (the RK4IP stage algebra with the exp(hD/2) factors replaced by an
    // exact 1, table 6), result <- E result, E = exp(hD/2) (table 7)
    const bool ssrk = d.method == 2;
    if (KIND == 0 && st.phase == 1 && !adaptive) {
      exp_table(cx, g, 0.5 * (d.length / d.total_steps), base + 7 * N, nullptr);
      if (ssrk) exp_table(cx, g, 0.0, base + 6 * N, nullptr);
    }

    if constexpr (KIND == 1) {
      // Split steps (method & 15): ss_symmetric (3), ss_simple (4), ss_reduced (5),
      // ss_sym_midpoint (6), ss_agrawal (7), and with the adaptive flag (16) also
      // ss_sym_rk4 (2).  Scratch: state slots 0/1, fine step 2, step scratch 3-5,
      // exp(hD) tables 6-7.
      const int sm = d.method & 15;
      const bool sadapt = (d.method & 16) != 0;
      SV* tmp = base + 3 * N;
      if (!sadapt) {
        // fixed step (stepper.py:164-221): exp(hD/2), or exp(hD) for ss_simple
        const double hf = d.length / d.total_steps;
        if (st.phase == 1) exp_table(cx, g, (sm == 4 ? 1.0 : 0.5) * hf, base + 7 * N, nullptr);
        while (st.phase == 1 && budget > 0) {
          const int sidx = st.sidx;
          ss_step(cx, g, sm, base + (long long)sidx * N, base + (long long)(sidx ^ 1) * N, tmp, base + 7 * N, hf);
          if (threadIdx.x == 0) st.evals += 1;
          budget -= 1;
          fixed_step_done(cx, kp, c, base, hf);
        }
      }
      // adaptive step doubling (stepper.py:247-376) with the method's order (Solver.errors)
      while (sadapt && st.phase == 1 && budget > 0) {
        if (threadIdx.x == 0 && st.ta == 0) {
          if (st.steps >= 99999) {
            st.status = ST_MAX_STEPS;
            st.phase = 2;
          } else if (st.z + st.h > d.length) {
            st.h = d.length - st.z;
          }
        }
        __syncthreads();
        if (st.phase != 1) break;
        const double h = st.h;
        const int sidx = st.sidx;
        SV* S = base + (long long)sidx * N;
        SV* Cc = base + (long long)(sidx ^ 1) * N;
        SV* F = base + 2 * N;
        // half steps' linear factor (table 6) and the coarse step's (table 7)
        exp_table(cx, g, (sm == 4 ? 0.5 : 0.25) * h, base + 6 * N, base + 7 * N);
        ss_step(cx, g, sm, S, Cc, tmp, base + 6 * N, 0.5 * h);  // A_half
        ss_step(cx, g, sm, Cc, F, tmp, base + 6 * N, 0.5 * h);  // A_fine
        ss_step(cx, g, sm, S, Cc, tmp, base + 7 * N, h);        // A_coarse
        const int eta = ss_order(sm);
        const double f_eta = (double)(1 << (eta - 1));
        double nrm[3];
        ss_extrapolate(cx, F, Cc, f_eta / (f_eta - 1.0), 1.0 / (f_eta - 1.0), nrm);
        budget -= 1;
        double delta;  // relative_local_error (stepper.py:231-245)
        if (nrm[2] != 0.0 || !isfinite(nrm[1])) {
          delta = 1.0;
        } else {
          const double nf = sqrt(nrm[1]);
          delta = nf != 0.0 ? sqrt(nrm[0]) / nf : sqrt(nrm[0]);
        }
        const bool accept = delta < 2.0 * d.tol;
        __syncthreads();
        if (threadIdx.x == 0) {
          if (accept && d.step_log && st.steps < d.step_cap && cx.rank == 0) {
            d.step_log[2 * st.steps] = st.z + h;
            d.step_log[2 * st.steps + 1] = h;
          }
          st.evals += 3;
          st.attempts += 1;
          st.ta += 1;
          st.delta_last = delta;
          if (delta > 0.0) {
            st.h = h * fmin(10.0, fmax(0.2, 0.9 * pow(d.tol / delta, 1.0 / (double)eta)));
          } else {
            st.h = h * 10.0;
          }
          if (accept) {
            st.z += h;
            st.sidx ^= 1;  // Cc holds the extrapolated solution
            st.accepted += 1;
            st.steps += 1;
            st.ta = 0;
            if (st.z >= d.length) {
              st.status = ST_OK;
              st.phase = 2;
            }
          } else {
            st.rejected += 1;
            if (st.h < 1e-37) {
              st.status = ST_SMALL_STEP;
              st.phase = 2;
            } else if (st.ta >= 1000) {
              st.status = ST_SUITABLE_STEP;
              st.phase = 2;
            }
          }
        }
        __syncthreads();
        if (accept && st.z > st.z_ignore) {
          store_trace(cx, kp, c, base + (long long)st.sidx * N, st.z);
          if (threadIdx.x == 0) st.z_ignore += d.length / d.traces;
          __syncthreads();
        }
      }
    }

    while (KIND == 0 && st.phase == 1 && budget > 0) {
      // ---- one attempt (adaptive) or one step (fixed) ------------------------
      if (threadIdx.x == 0) {
        if (adaptive) {
          if (d.replay) {  // follow the given step sizes; the list ends the propagation
            if (st.steps >= d.replay_n) {
              st.status = ST_OK;
              st.phase = 2;
            } else {
              st.h = d.replay[st.steps];
            }
          } else if (st.ta == 0) {
            if (st.steps >= 99999) {  // for s in range(1, steps_max) (stepper.py:289)
              st.status = ST_MAX_STEPS;
              st.phase = 2;
            } else if (st.z + st.h > d.length) {
              st.h = d.length - st.z;
            }
          }
        } else {
          st.ma_valid = 0;
        }
      }
      __syncthreads();
      if (st.phase != 1) break;
      const double h = adaptive ? st.h : d.length / d.total_steps;
      const int sidx = st.sidx;
      PROF_T0();
      if (adaptive) exp_table(cx, g, 0.25 * h, base + 6 * N, base + 7 * N);
      PROF_ADD(2);
      const int q_end = adaptive ? 11 : 4;
      double nrm[3] = {0.0, 0.0, 0.0};
      if (ssrk) scale_state(cx, base + (long long)sidx * N, base + 7 * N);  // linear half step
      for (int q = st.ma_valid ? 1 : 0; q < q_end; ++q) {
        // slot q: kind 0 = N(A) of state mi, kind 1..3 = stage of evaluation e
        const int kind = (q == 0 || q == 4) ? 0 : (q < 4 ? q : (q < 8 ? q - 4 : q - 7));
        const int mi = q == 4 ? 1 : 0;
        SV* S = base + (long long)sidx * N;
        SV* Sh = base + (long long)(sidx ^ 1) * N;
        if (kind == 1) {
          if (threadIdx.x == 0) {
            const int e = q < 4 ? 0 : (q < 8 ? 1 : 2);
            const double he = (adaptive && e < 2) ? 0.5 * h : h;
            const int m = e == 1 ? 1 : 0;
            op.Kr = (const R*)g.Kr;
            op.lor = (const R*)g.lor;
            op.lor2 = (const R*)g.lor2;
            op.gain = g.gain;
            op.acc = base + 5 * N;
            op.Sf = base + 2 * N;
            op.S0 = e == 1 ? Sh : S;
            op.MA0 = reinterpret_cast<V*>(base + (3 + m) * N);
            op.Et = base + ((ssrk || (adaptive && e < 2)) ? 6 : 7) * N;
            op.out = e == 1 ? base + 2 * N : Sh;
            op.h = (R)he;
            op.hh = 0.5 * he;
            if (g.gain == 2) {  // linear calls 1 (S_I = L(A)) and 2 (k0 = L(h N(A)))
              op.aA = yb_call(g, st, 0.5 * he, c.yA[m][0], c.yA[m][1]);
              op.ak0 = yb_call(g, st, 0.5 * he, he * he * c.yN[m][0], he * he * c.yN[m][1]);
              op.gb = (R)(-250.0 * he);
            } else {
              op.aA = g.gain ? gain_a(g, 0.5 * he, c.eA[m]) : (R)0;
              op.ak0 = g.gain ? gain_a(g, 0.5 * he, he * he * c.eN[m]) : (R)0;
            }
            op.a3 = op.ao = (R)0;
          }
          __syncthreads();
          pre_stage1(cx, op);
        } else if (kind == 0) {
          load_state(cx, mi == 0 ? S : Sh);
          if (g.gain == 2) yb_sums(cx, g, op, 2, c.yA[mi]);
        }
        PROF_ADD(1);
        const double en = nonlinear(cx, g, kind == 0 && g.gain == 1);
        PROF_ADD(0);
        if (kind == 0) {
          V* MA = reinterpret_cast<V*>(base + (3 + mi) * N);
          store_ma(cx, g, MA);
          double eN = 0.0;
          if (g.gain) {
            if (threadIdx.x == 0) op.MA0 = MA;
            __syncthreads();
            if (g.gain == 2) {
              yb_sums(cx, g, op, 0, c.yN[mi]);
            } else {
              eN = energy_of(cx, g, op, 0);
            }
          }
          if (threadIdx.x == 0) {
            c.eA[mi] = en;
            c.eN[mi] = eN;
            if (mi == 0) {
              st.ma_valid = 1;
              st.cache_eA = en;
              st.cache_eN = eN;
              st.cache_y[0] = c.yA[0][0];
              st.cache_y[1] = c.yA[0][1];
              st.cache_y[2] = c.yN[0][0];
              st.cache_y[3] = c.yN[0][1];
            }
          }
          __syncthreads();
        } else if (kind == 1) {
          post_stage1(cx, op);
        } else if (kind == 2) {
          post_stage2(cx, op);
          if (g.gain == 2) {
            yb_sums(cx, g, op, 2, c.yT[0]);
            yb_sums(cx, g, op, 1, c.yT[1]);
            if (threadIdx.x == 0) {  // linear call 3 (L(S_I + k2)), then call 4 (L(acc))
              op.a3 = yb_call(g, st, op.hh, c.yT[0][0], c.yT[0][1]);
              op.ao = yb_call(g, st, op.hh, c.yT[1][0], c.yT[1][1]);
            }
            __syncthreads();
            scale_stage3(cx, op);
          } else if (g.gain) {
            const double e_acc = energy_of(cx, g, op, 1);
            const double e_u = energy_of(cx, g, op, 2);
            if (threadIdx.x == 0) {
              op.ao = gain_a(g, op.hh, e_acc);
              op.a3 = gain_a(g, op.hh, e_u);
            }
            __syncthreads();
            scale_stage3(cx, op);
          }
        } else {
          post_stage3(cx, op, adaptive && q == 10, nrm);
          if (threadIdx.x == 0) st.evals += 1;
        }
        PROF_ADD(1);
      }
      if (ssrk) scale_state(cx, base + (long long)(sidx ^ 1) * N, base + 7 * N);  // linear half step
      budget -= 1;

      if (!adaptive) {
        fixed_step_done(cx, kp, c, base, h);
        continue;
      }

      // Adaptive driver (stepper.py:247-376); relative_local_error (stepper.py:231-245)
      double delta;
      if (nrm[2] != 0.0 || !isfinite(nrm[1])) {
        delta = 1.0;
      } else {
        const double nf = sqrt(nrm[1]);
        delta = nf != 0.0 ? sqrt(nrm[0]) / nf : sqrt(nrm[0]);
      }
      const bool accept = d.replay != nullptr || delta < 2.0 * d.tol;
      __syncthreads();
      if (threadIdx.x == 0) {
        if (accept && d.step_log && st.steps < d.step_cap && cx.rank == 0) {
          d.step_log[2 * st.steps] = st.z + h;
          d.step_log[2 * st.steps + 1] = h;
        }
        st.attempts += 1;
        st.ta += 1;
        st.delta_last = delta;
        const double h_temp = h;
        if (delta > 0.0) {
          const double factor = 0.9 * pow(d.tol / delta, 1.0 / 5.0);
          st.h = h_temp * fmin(10.0, fmax(0.2, factor));
        } else {
          st.h = h_temp * 10.0;
        }
        if (accept) {
          st.z += h_temp;
          st.sidx ^= 1;  // Sh holds the extrapolated solution
          st.ma_valid = 0;
          st.accepted += 1;
          st.steps += 1;
          st.ta = 0;
          if (st.z >= d.length) {
            st.status = ST_OK;
            st.phase = 2;
          }
        } else {
          st.rejected += 1;
          if (st.h < 1e-37) {
            st.status = ST_SMALL_STEP;
            st.phase = 2;
          } else if (st.ta >= 1000) {
            st.status = ST_SUITABLE_STEP;
            st.phase = 2;
          }
        }
      }
      __syncthreads();
      if (accept && st.z > st.z_ignore) {
        store_trace(cx, kp, c, base + (long long)st.sidx * N, st.z);
        if (threadIdx.x == 0) st.z_ignore += d.length / d.traces;
        __syncthreads();
      }
    }

    if (st.phase == 2) {
      const SV* S = base + (long long)st.sidx * N;
      to_time(cx, g, S, field);
      double e_out, n_out;
      diagnostics(cx, g, S, &e_out, &n_out);
      if (threadIdx.x == 0) {
        st.E_out = e_out;
        st.Nph_out = n_out;
        st.phase = 3;
      }
    }
    __syncthreads();
    if (cx.rank == 0 && threadIdx.x == 0) kp.state[id] = st;
#if GNLSE_PROF
    if (kp.prof && cx.rank == 0 && threadIdx.x == 0) {
      for (int k = 0; k < 3; ++k) kp.prof[8 * id + k] += prof_acc[k];
      kp.prof[8 * id + 3] += clock64() - prof_start;
    }
#endif
  }
};

template <class R, int LOGM, int C, bool XS>
__global__ void __launch_bounds__(Engine<R, LOGM, C, XS>::T, Engine<R, LOGM, C, XS>::MINB)
    gnlse_kernel(KParams kp) {
  Engine<R, LOGM, C, XS>::template run<0>(kp);
}

// the exponential split-step methods (ss_symmetric, ss_simple, ss_reduced)
template <class R, int LOGM, int C, bool XS>
__global__ void __launch_bounds__(Engine<R, LOGM, C, XS>::T, Engine<R, LOGM, C, XS>::MINB)
    gnlse_ss_kernel(KParams kp) {
  Engine<R, LOGM, C, XS>::template run<1>(kp);
}

// One cluster per instance of kernel k of class (R, M, C).
template <class R, int LOGM, int C, bool XS>
cudaError_t launch_kernel(void (*k)(KParams), const KParams& kp, int n_clusters, cudaStream_t stream) {
  using E = Engine<R, LOGM, C, XS>;
  const size_t smem = E::smem_bytes();
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  if (C > 8) {  // 16-CTA clusters are beyond the portable limit of 8
    err = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (err != cudaSuccess) return err;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_clusters * C);
  cfg.blockDim = dim3(E::T);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  int na = 0;
  if (C > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    na = 1;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  return cudaLaunchKernelEx(&cfg, k, kp);
}

// Host launchers for one (precision, M, C) class: the RK4IP-loop kernel, and the
// split-step kernel.
template <class R, int LOGM, int C, bool XS>
cudaError_t launch_class(const KParams& kp, int n_clusters, cudaStream_t stream) {
  return launch_kernel<R, LOGM, C, XS>(gnlse_kernel<R, LOGM, C, XS>, kp, n_clusters, stream);
}
template <class R, int LOGM, int C, bool XS>
cudaError_t launch_class_ss(const KParams& kp, int n_clusters, cudaStream_t stream) {
  return launch_kernel<R, LOGM, C, XS>(gnlse_ss_kernel<R, LOGM, C, XS>, kp, n_clusters, stream);
}

}  // namespace gnlse
