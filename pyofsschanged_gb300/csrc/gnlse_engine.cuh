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

#include "gnlse_types.h"

namespace cg = cooperative_groups;

namespace gnlse {

template <class R> struct VT;
template <> struct VT<float> { using V = float2; };
template <> struct VT<double> { using V = double2; };

template <class V> __device__ __forceinline__ V mk(decltype(V::x) a, decltype(V::x) b) { V r; r.x = a; r.y = b; return r; }
template <class V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <class V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <class V> __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class V> __device__ __forceinline__ V cmulc(V a, V b) {  // a * conj(b)
  return mk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <class V, class S> __device__ __forceinline__ V cscale(V a, S s) { return mk<V>(a.x * s, a.y * s); }
template <class V> __device__ __forceinline__ auto cabs2(V a) -> decltype(a.x) { return a.x * a.x + a.y * a.y; }

// Padded shared-memory slot: one spare element every 16 makes every Stockham
// pass (radix-16 strided stores included) free of bank conflicts for 8- and
// 16-byte elements.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }

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
  using S = decltype(V::x);
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
        v[blk + j] = cadd(a, b);
        V d = csub(a, b);
        const int m = j * (16 / L);
        if (m == 0) {
          v[blk + j + half] = d;
        } else if (m == 4) {  // multiply by SIGN*i
          v[blk + j + half] = SIGN > 0 ? mk<V>(-d.y, d.x) : mk<V>(d.y, -d.x);
        } else {
          const S c = (S)c16(m), s = (S)(SIGN * s16(m));
          v[blk + j + half] = mk<V>(d.x * c - d.y * s, d.x * s + d.y * c);
        }
      }
    }
  }
  V t[RAD];
#pragma unroll
  for (int k = 0; k < RAD; ++k) t[k] = v[bitrev(k, B)];
#pragma unroll
  for (int k = 0; k < RAD; ++k) v[k] = t[k];
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

// What the prologue of a nonlinear evaluation reads and what its epilogue
// writes (selected at run time so the transform code is compiled once).
enum StageKind : int {
  SK_MA = 0,   // in: Z = S0            out: MA = i K G+(x R)          (N(A) of a state)
  SK_S1 = 1,   // in: S_I + k0/2        out: k1 -> X, acc = S_I + k0/6 + k1/3
  SK_S2 = 2,   // in: S_I + k1/2        out: k2 -> X, acc += k2/3
  SK_S3 = 3,   // in: L(S_I + k2)       out: L(acc) + k3/6
  SK_S3C = 4,  // as SK_S3, then error norms vs Sf and local extrapolation
  SK_E_ACC = 5,  // energy of G-(acc)/N
  SK_E_U = 6,    // energy of G-(S_I + k2)/N
  SK_E_MA = 7    // energy of G-(MA)/N
};

template <class R, int LOGM, int C>
struct Engine {
  using V = typename VT<R>::V;
  static constexpr int M = 1 << LOGM;
  static constexpr int N = M * C;
  static constexpr int T = (M / 16) < 64 ? 64 : (M / 16);
  static constexpr int MP = M + M / 16;
  static constexpr int NR16 = LOGM / 4;
  static constexpr int REM = LOGM % 4;
  static constexpr int RED = 64;  // doubles of reduction scratch
  static_assert(LOGM >= 8, "M >= 256 required");
  static_assert(C == 1 || C == 2 || C == 4 || C == 8, "cluster size 1, 2, 4 or 8");
  static constexpr size_t ctl_bytes() { return 512; }
  static constexpr size_t smem_bytes() {
    return 2 * MP * sizeof(V) + RED * sizeof(double) + ctl_bytes();
  }

  struct Ctx {
    V* X;
    V* P;
    double* red;
    const V* tw;
    int rank;
  };

  // Runtime description of one nonlinear evaluation (see StageKind).
  struct Op {
    int kind;
    int gain;
    const V* S0;
    const V* MA0;
    const V* Et;
    V* acc;
    V* out;
    const V* Sf;
    const R* Kr;
    const R* lor;
    R h, aA, ak0, a3, ao;
  };

  static __device__ __forceinline__ V* rmt(V* p, int r) {
    if constexpr (C > 1) {
      return cg::this_cluster().map_shared_rank(p, r);
    } else {
      return p;
    }
  }

  static __device__ __forceinline__ void csync() {
    if constexpr (C > 1) {
      cg::this_cluster().sync();
    } else {
      __syncthreads();
    }
  }

  static __device__ __forceinline__ V twid(const V* tw, int idx, int sign) {
    V w = __ldg(&tw[idx]);
    if (sign < 0) w.y = -w.y;
    return w;
  }

  // ---- transforms ---------------------------------------------------------
  // One in-place radix-RAD Stockham pass over the CTA's M points (all loads,
  // barrier, all stores).  FIRST: inputs from pro(owner, slot); LAST: outputs
  // to epi(owner, slot, v); otherwise the padded shared buffer.
  template <int RAD, int SIGN, bool FIRST, bool LAST, class Pro, class Epi>
  static __device__ __forceinline__ void pass(const Ctx& cx, V* buf, int Ns, Pro& pro, Epi& epi) {
    constexpr int NB = M / RAD;
    constexpr int BPT = (NB + T - 1) / T;
    V v[BPT][RAD];
    const int tid = threadIdx.x;
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = tid + b * T;
      if (NB % T == 0 || j < NB) {
#pragma unroll
        for (int r = 0; r < RAD; ++r) {
          const int i = j + r * NB;
          if constexpr (FIRST) v[b][r] = pro(cx.rank, i);
          else v[b][r] = buf[pad(i)];
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
          const int step = C * k * (M / (Ns * RAD));
#pragma unroll
          for (int r = 1; r < RAD; ++r) v[b][r] = cmul(v[b][r], twid(cx.tw, r * step, SIGN));
        }
        dft<RAD, SIGN>(v[b]);
        const int base = (j - k) * RAD + k;
#pragma unroll
        for (int r = 0; r < RAD; ++r) {
          const int o = base + r * Ns;
          if constexpr (LAST) epi(cx.rank, o, v[b][r]);
          else buf[pad(o)] = v[b][r];
        }
      }
    }
    __syncthreads();
  }

  template <int SIGN, bool PRO, bool EPI, int P16, class Pro, class Epi>
  static __device__ __forceinline__ void passes16(const Ctx& cx, V* buf, int Ns, Pro& pro, Epi& epi) {
    if constexpr (P16 < NR16) {
      constexpr bool first = PRO && (P16 == 0);
      constexpr bool last = EPI && (P16 == NR16 - 1) && (REM == 0);
      pass<16, SIGN, first, last>(cx, buf, Ns, pro, epi);
      passes16<SIGN, PRO, EPI, P16 + 1>(cx, buf, Ns * 16, pro, epi);
    } else if constexpr (REM > 0) {
      pass<(1 << REM), SIGN, false, EPI>(cx, buf, Ns, pro, epi);
    }
  }

  template <int SIGN, bool PRO, bool EPI, class Pro, class Epi>
  static __device__ __forceinline__ void local_fft(const Ctx& cx, V* buf, Pro& pro, Epi& epi) {
    passes16<SIGN, PRO, EPI, 0>(cx, buf, 1, pro, epi);
  }

  // Forward cross-CTA pass: slot n2 of every CTA r (= x[r*M + n2]) -> radix-C
  // DFT -> twiddle W_N^{n2 k1} -> slot n2 of CTA k1.
  template <class Pro>
  static __device__ __forceinline__ void cross_fwd(const Ctx& cx, V* buf, Pro& pro) {
    constexpr int PM = M / C;
    constexpr int BP = (PM + T - 1) / T;
    V v[BP][C];
    csync();
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = threadIdx.x + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int r = 0; r < C; ++r) v[b][r] = pro(r, n2);
      }
    }
    csync();
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = threadIdx.x + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
        dft<C, +1>(v[b]);
#pragma unroll
        for (int k1 = 0; k1 < C; ++k1) {
          V val = k1 ? cmul(v[b][k1], twid(cx.tw, n2 * k1, +1)) : v[b][k1];
          rmt(buf, k1)[pad(n2)] = val;
        }
      }
    }
    csync();
  }

  // Inverse cross-CTA pass: slot n2 of every CTA k1 -> twiddle W_N^{-n2 k1}
  // -> radix-C DFT -> epi(n1, n2, x[n1*M + n2]).
  template <class Epi>
  static __device__ __forceinline__ void cross_inv(const Ctx& cx, V* buf, Epi& epi) {
    constexpr int PM = M / C;
    constexpr int BP = (PM + T - 1) / T;
    V v[BP][C];
    csync();
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = threadIdx.x + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int k1 = 0; k1 < C; ++k1) v[b][k1] = rmt(buf, k1)[pad(n2)];
      }
    }
    csync();
#pragma unroll
    for (int b = 0; b < BP; ++b) {
      const int q = threadIdx.x + b * T;
      if (PM % T == 0 || q < PM) {
        const int n2 = cx.rank * PM + q;
#pragma unroll
        for (int k1 = 1; k1 < C; ++k1) v[b][k1] = cmul(v[b][k1], twid(cx.tw, n2 * k1, -1));
        dft<C, -1>(v[b]);
#pragma unroll
        for (int n1 = 0; n1 < C; ++n1) epi(n1, n2, v[b][n1]);
      }
    }
    csync();
  }

  // Forward transform G+(x)[k] = sum_n x[n] e^{+2 pi i k n / N} (= N * pyofss fft).
  // pro(owner, slot): time-domain input; epi(owner, slot, v): spectral output,
  // always called in the owner CTA.
  template <class Pro, class Epi>
  static __device__ __forceinline__ void fwd(const Ctx& cx, V* buf, Pro& pro, Epi& epi) {
    if constexpr (C == 1) {
      local_fft<+1, true, true>(cx, buf, pro, epi);
    } else {
      cross_fwd(cx, buf, pro);
      local_fft<+1, false, true>(cx, buf, pro, epi);
    }
  }

  // Inverse transform G-(X)[n] = sum_k X[k] e^{-2 pi i k n / N} (= pyofss ifft).
  // pro(owner, slot): spectral input (owner CTA); epi(owner, slot, v): time
  // output, possibly for a remote CTA of the cluster.
  template <class Pro, class Epi>
  static __device__ __forceinline__ void inv(const Ctx& cx, V* buf, Pro& pro, Epi& epi) {
    if constexpr (C == 1) {
      local_fft<-1, true, true>(cx, buf, pro, epi);
    } else {
      local_fft<-1, true, false>(cx, buf, pro, epi);
      cross_inv(cx, buf, epi);
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

  // ---- stage prologue / epilogue algebra (Solver.rk4ip, solver.py:339-354) --
  static __device__ __forceinline__ V mult(const Op& op, int a, R ga) {
    V e = op.Et[a];
    if (op.gain) e = cscale(e, (R)exp(ga * op.lor[a]));
    return e;
  }
  static __device__ __forceinline__ V hK(const Op& op, int a, V v) {  // h * i * K * v
    const R k = op.h * op.Kr[a];
    return mk<V>(-k * v.y, k * v.x);
  }
  static __device__ __forceinline__ V s_I(const Op& op, int a) { return cmul(mult(op, a, op.aA), op.S0[a]); }
  static __device__ __forceinline__ V k_0(const Op& op, int a) {
    return cscale(cmul(mult(op, a, op.ak0), op.MA0[a]), op.h);
  }

  static __device__ __forceinline__ V stage_pro(const Ctx& cx, const Op& op, int a, int l) {
    const R half = (R)0.5;
    switch (op.kind) {
      case SK_MA: return op.S0[a];
      case SK_S1: return cadd(s_I(op, a), cscale(k_0(op, a), half));
      case SK_S2: return cadd(s_I(op, a), cscale(cx.X[pad(l)], half));
      case SK_E_ACC: return op.acc[a];
      case SK_E_U: return cadd(s_I(op, a), cx.X[pad(l)]);
      case SK_E_MA: return op.MA0[a];
      default: return cmul(mult(op, a, op.a3), cadd(s_I(op, a), cx.X[pad(l)]));  // SK_S3, SK_S3C
    }
  }

  static __device__ __forceinline__ void stage_fin(const Ctx& cx, const Op& op, int a, int l, V v,
                                                   double& d2, double& f2, double& bad) {
    const R sixth = (R)(1.0 / 6.0), third = (R)(1.0 / 3.0);
    switch (op.kind) {
      case SK_MA: {
        const R k = op.Kr[a];
        op.out[a] = mk<V>(-k * v.y, k * v.x);
        break;
      }
      case SK_S1: {
        V k1 = hK(op, a, v);
        cx.X[pad(l)] = k1;
        op.acc[a] = cadd(cadd(s_I(op, a), cscale(k_0(op, a), sixth)), cscale(k1, third));
        break;
      }
      case SK_S2: {
        V k2 = hK(op, a, v);
        cx.X[pad(l)] = k2;
        op.acc[a] = cadd(op.acc[a], cscale(k2, third));
        break;
      }
      case SK_S3: {
        V k3 = hK(op, a, v);
        op.out[a] = cadd(cmul(mult(op, a, op.ao), op.acc[a]), cscale(k3, sixth));
        break;
      }
      default: {  // SK_S3C
        V k3 = hK(op, a, v);
        V res = cadd(cmul(mult(op, a, op.ao), op.acc[a]), cscale(k3, sixth));
        V sf = op.Sf[a];
        V d = csub(sf, res);
        d2 += (double)cabs2(d);
        f2 += (double)cabs2(sf);
        if (!isfinite(sf.x) || !isfinite(sf.y)) bad = 1.0;
        // local extrapolation (stepper.py:272-274,338): (16 A_fine - A_coarse) / 15
        const R fa = (R)(16.0 / 15.0), fb = (R)(1.0 / 15.0);
        op.out[a] = mk<V>(fa * sf.x - fb * res.x, fa * sf.y - fb * res.y);
        break;
      }
    }
  }

  // ---- the nonlinear operator ---------------------------------------------
  // x = G-(xhat)/N for the stage input xhat; y = x R(x) with
  // R = (1-fR)|x|^2 + fR G-(Hp G+(|x|^2)) (Raman) or |x|^2; then G+(y) is
  // handed to the stage epilogue.  res[0] returns the Simpson energy of x
  // (SK_MA with gain) or res[0..2] the error norms (SK_S3C).
  static __device__ __noinline__ void nonlinear(const Ctx& cx, const GridDev& g, const Op& op_in,
                                                double* res) {
    const Op op = op_in;
    const R invN = (R)(1.0 / (double)N);
    const bool raman = g.raman != 0;
    const bool want_e = (op.kind == SK_MA) && op.gain;
    const int n_tot = N;
    double eacc = 0.0;
    V* X = cx.X;
    V* P = cx.P;
    auto pro = [&](int o, int l) -> V { return stage_pro(cx, op, o * M + l, l); };
    auto e1 = [&](int o, int l, V v) {
      V x = cscale(v, invN);
      R p = cabs2(x);
      if (want_e) eacc += simpson_w(o * M + l, n_tot) * (double)p;
      if (raman) {
        rmt(X, o)[pad(l)] = x;
        rmt(P, o)[pad(l)] = mk<V>(p, (R)0);
      } else {
        rmt(X, o)[pad(l)] = cscale(x, p);
      }
    };
    inv(cx, X, pro, e1);
    if (raman) {
      const V* Hp = (const V*)g.Hp;
      const R fR = (R)g.fR, f1 = (R)(1.0 - g.fR);
      auto rdP = [&](int o, int l) -> V { return rmt(P, o)[pad(l)]; };
      auto mulH = [&](int o, int l, V v) { P[pad(l)] = cmul(v, Hp[o * M + l]); };
      fwd(cx, P, rdP, mulH);
      auto e3 = [&](int o, int l, V conv) {
        V* Xo = rmt(X, o);
        V x = Xo[pad(l)];
        R p = cabs2(x);
        Xo[pad(l)] = cmul(x, mk<V>(f1 * p + fR * conv.x, fR * conv.y));
      };
      inv(cx, P, rdP, e3);
    }
    double d2 = 0.0, f2 = 0.0, bad = 0.0;
    auto rdX = [&](int o, int l) -> V { return rmt(X, o)[pad(l)]; };
    auto fin = [&](int o, int l, V v) { stage_fin(cx, op, o * M + l, l, v, d2, f2, bad); };
    fwd(cx, X, rdX, fin);
    if (want_e) {
      double s[1] = {eacc * g.dt * 1e-3};
      cluster_sum<1>(cx, s);
      res[0] = s[0];
    }
    if (op.kind == SK_S3C) {
      double s[3] = {d2, f2, bad};
      cluster_sum<3>(cx, s);
      res[0] = s[0];
      res[1] = s[1];
      res[2] = s[2];
    }
  }

  // Simpson energy (nJ) of G-(xhat)/N for a prologue kind SK_E_*, computed in
  // the P buffer (X is left untouched).
  static __device__ __noinline__ double energy_of(const Ctx& cx, const GridDev& g, const Op& op_in) {
    const Op op = op_in;
    const double invN2 = 1.0 / ((double)N * (double)N);
    const int n_tot = N;
    double eacc = 0.0;
    auto pro = [&](int o, int l) -> V { return stage_pro(cx, op, o * M + l, l); };
    auto ep = [&](int o, int l, V v) { eacc += simpson_w(o * M + l, n_tot) * (double)cabs2(v) * invN2; };
    inv(cx, cx.P, pro, ep);
    double s[1] = {eacc * g.dt * 1e-3};
    cluster_sum<1>(cx, s);
    return s[0];
  }

  // time -> spectral state: S = G+(field)
  static __device__ __noinline__ void to_spectral(const Ctx& cx, const V* field, V* S) {
    auto pro = [&](int o, int l) -> V { return field[o * M + l]; };
    auto epi = [&](int o, int l, V v) { S[o * M + l] = v; };
    fwd(cx, cx.P, pro, epi);
  }

  // spectral state -> time field: field = G-(S)/N
  static __device__ __noinline__ void to_time(const Ctx& cx, const V* S, V* field) {
    const R invN = (R)(1.0 / (double)N);
    auto pro = [&](int o, int l) -> V { return S[o * M + l]; };
    auto epi = [&](int o, int l, V v) { field[o * M + l] = cscale(v, invN); };
    inv(cx, cx.P, pro, epi);
  }

  // exp(hh (i beta - alpha/2)) for this CTA's slice.  FP32 plans form the
  // phase beta*hh in FP64 and reduce it to [-pi, pi] before the FP32 sincos.
  static __device__ __noinline__ void exp_table(const Ctx& cx, const GridDev& g, double hh, V* Et) {
    const double mag = exp(-0.5 * g.alpha * hh);
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = cx.rank * M + l;
      double ph = g.beta[a] * hh;
      R s, c;
      if constexpr (sizeof(R) == 4) {
        const double TWO_PI = 6.283185307179586476925286766559;
        ph -= TWO_PI * rint(ph * (1.0 / TWO_PI));
        sincosf((float)ph, &s, &c);
      } else {
        sincos(ph, &s, &c);
      }
      Et[a] = mk<V>((R)mag * c, (R)mag * s);
    }
    __syncthreads();
  }

  static __device__ __forceinline__ R gain_a(const GridDev& g, double hh, double energy) {
    return (R)(g.gain_log * hh / (2.0 * g.gain_len) / (1.0 + energy / g.E_sat));
  }

  // N(A) of state Z (unscaled by h) into MA, plus the gain energies of A and N(A).
  static __device__ void state_cache(const Ctx& cx, const GridDev& g, const V* Z, V* MA,
                                     double& eA, double& eN) {
    Op op = {};
    op.kind = SK_MA;
    op.gain = g.gain;
    op.S0 = Z;
    op.out = MA;
    op.MA0 = MA;
    op.Kr = (const R*)g.Kr;
    double res[3] = {0, 0, 0};
    nonlinear(cx, g, op, res);
    eA = res[0];
    eN = 0.0;
    if (g.gain) {
      op.kind = SK_E_MA;
      eN = energy_of(cx, g, op);
    }
  }

  // One RK4IP evaluation of step h from state S0 (cached N(A) in MA0, gain
  // energies eA / eN) with Et = exp(D h/2).  COARSE = false: result to out;
  // COARSE = true: error norms against Sf in norms[0..2] and the local
  // extrapolation of (Sf, coarse result) to out.
  static __device__ __noinline__ void rk4ip(const Ctx& cx, const GridDev& g, const V* S0, const V* MA0,
                                            double eA, double eN, const V* Et, V* acc, double h,
                                            V* out, const V* Sf, bool coarse, double* norms) {
    const double hh = 0.5 * h;
    Op op = {};
    op.gain = g.gain;
    op.S0 = S0;
    op.MA0 = MA0;
    op.Et = Et;
    op.acc = acc;
    op.out = out;
    op.Sf = Sf;
    op.Kr = (const R*)g.Kr;
    op.lor = (const R*)g.lor;
    op.h = (R)h;
    op.aA = g.gain ? gain_a(g, hh, eA) : (R)0;
    op.ak0 = g.gain ? gain_a(g, hh, h * h * eN) : (R)0;
    double res[3] = {0, 0, 0};
    op.kind = SK_S1;
    nonlinear(cx, g, op, res);
    op.kind = SK_S2;
    nonlinear(cx, g, op, res);
    if (g.gain) {
      op.kind = SK_E_ACC;
      op.ao = gain_a(g, hh, energy_of(cx, g, op));
      op.kind = SK_E_U;
      op.a3 = gain_a(g, hh, energy_of(cx, g, op));
    }
    op.kind = coarse ? SK_S3C : SK_S3;
    nonlinear(cx, g, op, res);
    if (coarse) {
      norms[0] = res[0];
      norms[1] = res[1];
      norms[2] = res[2];
    }
  }

  // FP64 energy (Parseval, nJ) and photon number of state S.
  static __device__ __noinline__ void diagnostics(const Ctx& cx, const GridDev& g, const V* S,
                                                  double* E, double* Nph) {
    double e = 0.0, p = 0.0;
    for (int l = threadIdx.x; l < M; l += T) {
      const int a = cx.rank * M + l;
      const double s2 = (double)cabs2(S[a]);
      e += s2;
      p += s2 / g.nu[a];
    }
    double s[2] = {e, p};
    cluster_sum<2>(cx, s);
    const double scale = g.window_t / ((double)N * (double)N);
    *E = s[0] * scale * 1e-3;
    *Nph = s[1] * scale / 6.62607015e-10;
  }

  static __device__ void store_trace(const Ctx& cx, const KParams& kp, const InstDev& d,
                                     InstState& st, const V* S, double z) {
    if (st.ntraces >= d.max_traces) {
      st.trace_overflow = 1;
      return;
    }
    V* tr = (V*)kp.traces + d.trace_off + (long long)st.ntraces * N;
    to_time(cx, S, tr);
    if (cx.rank == 0 && threadIdx.x == 0) kp.trace_z[d.tracez_off + st.ntraces] = z;
    st.ntraces += 1;
  }

  // The whole propagation of one instance.  Control state lives in shared
  // memory; every thread evaluates the same decisions from the same
  // cluster-reduced values, so all CTAs of a cluster follow one path.
  static __device__ void run(const KParams& kp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int cid = blockIdx.x / C;
    if (cid >= kp.n_order) return;
    Ctx cx;
    cx.X = (V*)smem_raw;
    cx.P = cx.X + MP;
    cx.red = (double*)(cx.P + MP);
    unsigned char* ctl = (unsigned char*)(cx.red + RED);
    GridDev& g = *(GridDev*)ctl;
    InstDev& d = *(InstDev*)(ctl + 192);
    static_assert(sizeof(GridDev) <= 192 && sizeof(InstDev) <= 128, "control block layout");
    if constexpr (C > 1) {
      cx.rank = (int)cg::this_cluster().block_rank();
    } else {
      cx.rank = 0;
    }
    const int id = kp.order[cid];
    if (threadIdx.x == 0) {
      d = kp.inst[id];
      g = kp.grids[d.grid];
    }
    __syncthreads();
    cx.tw = (const V*)g.tw;
    InstState st = kp.state[id];
    V* field = (V*)kp.fields + d.field_off;
    V* base = (V*)kp.scratch + d.scratch_off;
    V* Sbuf[2] = {base, base + N};
    V* Sf = base + 2 * N;
    V* MA = base + 3 * N;
    V* MAh = base + 4 * N;
    V* acc = base + 5 * N;
    V* E1 = base + 6 * N;
    V* E2 = base + 7 * N;
    long long budget = kp.max_attempts > 0 ? kp.max_attempts : (1ll << 62);

    if (st.phase == 0) {
      st.ntraces = 0;
      st.trace_overflow = 0;
      if (d.method == 1 && d.traces != 1) {
        if (d.max_traces > 0) {
          V* tr = (V*)kp.traces + d.trace_off;
          for (int l = threadIdx.x; l < M; l += T) tr[cx.rank * M + l] = field[cx.rank * M + l];
          if (cx.rank == 0 && threadIdx.x == 0) kp.trace_z[d.tracez_off] = 0.0;
          st.ntraces = 1;
        } else {
          st.trace_overflow = 1;
        }
      }
      to_spectral(cx, field, Sbuf[0]);
      diagnostics(cx, g, Sbuf[0], &st.E_in, &st.Nph_in);
      st.sidx = 0;
      st.z = 0.0;
      st.h = d.method == 1 ? d.h0 : d.length / d.total_steps;
      st.z_ignore = d.length / d.traces;
      st.ma_valid = 0;
      st.ta = 0;
      st.status = ST_RUNNING;
      st.phase = 1;
    }

    if (st.phase == 1 && d.method == 0) {
      // Fixed-step driver (stepper.py:164-221); exp(D h/2) is computed once,
      // as Linearity.default_exp_f_cached does (linearity.py:258-262).
      const double h = d.length / d.total_steps;
      const double dz = d.length / d.total_steps;  // numpy linspace step of the z mesh
      const int storage_step = d.traces > 0 ? d.total_steps / d.traces : 0;
      exp_table(cx, g, 0.5 * h, E2);
      while (st.steps < d.total_steps && budget > 0) {
        V* S = Sbuf[st.sidx];
        V* Sn = Sbuf[st.sidx ^ 1];
        double eA = 0, eN = 0;
        state_cache(cx, g, S, MA, eA, eN);
        rk4ip(cx, g, S, MA, eA, eN, E2, acc, h, Sn, nullptr, false, nullptr);
        st.sidx ^= 1;
        st.evals += 1;
        st.attempts += 1;
        st.accepted += 1;
        budget -= 1;
        const long long i = st.steps;
        st.steps += 1;
        st.z = (st.steps == d.total_steps) ? d.length : (double)st.steps * dz;
        if (d.traces != 1 && storage_step > 0 && (i % storage_step) == 0)
          store_trace(cx, kp, d, st, Sbuf[st.sidx], (double)i * dz + h);
      }
      if (st.steps >= d.total_steps) {
        st.status = ST_OK;
        st.phase = 2;
      }
    }

    if (st.phase == 1 && d.method == 1) {
      // Adaptive driver (stepper.py:247-376): step doubling, eta = 5.
      const double tol = d.tol;
      const double step_storage = d.length / d.traces;
      while (st.phase == 1 && budget > 0) {
        if (st.ta == 0) {
          if (st.steps >= 99999) {  // for s in range(1, steps_max)
            st.status = ST_MAX_STEPS;
            st.phase = 2;
            break;
          }
          if (st.z + st.h > d.length) st.h = d.length - st.z;
        }
        V* S = Sbuf[st.sidx];
        V* Sh = Sbuf[st.sidx ^ 1];
        if (!st.ma_valid) {
          state_cache(cx, g, S, MA, st.cache_eA, st.cache_eN);
          st.ma_valid = 1;
        }
        const double h = st.h;
        const double h_half = 0.5 * h;
        exp_table(cx, g, 0.5 * h_half, E1);
        exp_table(cx, g, 0.5 * h, E2);
        rk4ip(cx, g, S, MA, st.cache_eA, st.cache_eN, E1, acc, h_half, Sh, nullptr, false, nullptr);
        double eAh = 0, eNh = 0;
        state_cache(cx, g, Sh, MAh, eAh, eNh);
        rk4ip(cx, g, Sh, MAh, eAh, eNh, E1, acc, h_half, Sf, nullptr, false, nullptr);
        double nrm[3];
        rk4ip(cx, g, S, MA, st.cache_eA, st.cache_eN, E2, acc, h, Sh, Sf, true, nrm);
        st.evals += 3;
        st.attempts += 1;
        st.ta += 1;
        budget -= 1;
        // relative_local_error (stepper.py:231-245)
        double delta;
        if (nrm[2] != 0.0 || !isfinite(nrm[1])) {
          delta = 1.0;
        } else {
          const double nf = sqrt(nrm[1]);
          delta = nf != 0.0 ? sqrt(nrm[0]) / nf : sqrt(nrm[0]);
        }
        st.delta_last = delta;
        const double h_temp = h;
        if (delta > 0.0) {
          const double factor = 0.9 * pow(tol / delta, 1.0 / 5.0);
          st.h = h_temp * fmin(10.0, fmax(0.2, factor));
        } else {
          st.h = h_temp * 10.0;
        }
        if (delta < 2.0 * tol) {
          st.z += h_temp;
          st.sidx ^= 1;  // Sh now holds the extrapolated solution
          st.ma_valid = 0;
          st.accepted += 1;
          st.steps += 1;
          st.ta = 0;
          if (st.z > st.z_ignore) {
            store_trace(cx, kp, d, st, Sbuf[st.sidx], st.z);
            st.z_ignore += step_storage;
          }
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
    }

    if (st.phase == 2) {
      to_time(cx, Sbuf[st.sidx], field);
      diagnostics(cx, g, Sbuf[st.sidx], &st.E_out, &st.Nph_out);
      st.phase = 3;
    }
    __syncthreads();
    if (cx.rank == 0 && threadIdx.x == 0) kp.state[id] = st;
  }
};

template <class R, int LOGM, int C>
__global__ void __launch_bounds__(Engine<R, LOGM, C>::T) gnlse_kernel(KParams kp) {
  Engine<R, LOGM, C>::run(kp);
}

// Host launcher for one (precision, M, C) class: one cluster per instance.
template <class R, int LOGM, int C>
cudaError_t launch_class(const KParams& kp, int n_clusters, cudaStream_t stream) {
  using E = Engine<R, LOGM, C>;
  const size_t smem = E::smem_bytes();
  cudaError_t err = cudaFuncSetAttribute(gnlse_kernel<R, LOGM, C>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
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
  return cudaLaunchKernelEx(&cfg, gnlse_kernel<R, LOGM, C>, kp);
}

}  // namespace gnlse
