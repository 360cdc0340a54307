// Kernels of the spectral neural operator (SNO) surrogate: a batched BF16
// tensor-core GEMM with FP32 accumulation and fused epilogues, and the
// elementwise pieces of training (GELU backward, bias gradients, Adam, the
// relative-L2 loss).  Every network layer -- the truncated forward DFT, the
// per-mode spectral mixing, the truncated inverse DFT, the pointwise channel
// mixing and the weight gradients of each -- is one call of sno_gemm.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sno.h"

namespace {


__device__ __forceinline__ float gelu_f(float z) {
  // tanh form of GELU (Hendrycks & Gimpel)
  const float c = 0.7978845608028654f;
  return 0.5f * z * (1.0f + tanhf(c * (z + 0.044715f * z * z * z)));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float c = 0.7978845608028654f;
  const float u = c * (z + 0.044715f * z * z * z);
  const float th = tanhf(u);
  const float du = c * (1.0f + 3.0f * 0.044715f * z * z);
  return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * du;
}

// ---- tcgen05 GEMM -----------------------------------------------------------
// One CTA of 128 threads computes a 128 x 64 tile of C with the 5th-generation tensor
// cores: BF16 tiles of op(A) (128 x 64) and op(B)^T (64 x 64) are staged in shared
// memory in the canonical K-major layout without swizzle (8 x 8 "core matrices" of
// 128 contiguous bytes), one thread issues tcgen05.mma (kind::f16, FP32 accumulator in
// tensor memory, M = 128, N = 64, K = 16 per instruction) and commits to an mbarrier;
// after the last K tile each warp reads its 32 accumulator lanes (rows) with
// tcgen05.ld and applies the epilogue.  Every wait is bounded: on a timeout the kernel
// records it (sno_gemm_timeouts) and skips the rest of its work.
constexpr int TM = 128, TN = 64, TK = 64, KG = TK / 8;  // KG: 8-element K groups per tile row
constexpr int TMEM_COLS = 64;                             // FP32 accumulator columns (N)
constexpr unsigned long long WAIT_LIMIT = 1ull << 26;

__device__ unsigned int g_gemm_timeouts;

// byte offset of element (row, k) of a tile in the canonical K-major layout
__device__ __forceinline__ int core_off(int row, int k) {
  return ((row >> 3) * KG + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, leading byte offset (between core
// matrices adjacent in K), stride byte offset (between 8-row groups), version 1,
// no swizzle
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
  const unsigned long long lbo = 128, sbo = KG * 128;
  return (unsigned long long)((addr >> 4) & 0x3FFF) | (((lbo >> 4) & 0x3FFF) << 16) |
         (((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, N = 64, M = 128
constexpr unsigned IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(TN >> 3) << 17) |
                           ((unsigned)(TM >> 4) << 24);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned phase) {
  for (unsigned long long it = 0; it < WAIT_LIMIT; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// C[z] (M x N, row-major, ldc) = alpha * op(A[z]) op(B[z]) + beta * C[z] (+ bias[n]);
// op(A) is M x K: A[m*lda + k] (ta = 0) or A[k*lda + m] (ta = 1);
// op(B) is K x N: B[k*ldb + n] (tb = 0) or B[n*ldb + k] (tb = 1).
// Grid: (ceil(N/TN), ceil(M/TM), batch * splits).  With splits > 1 each CTA sums
// a K range and adds alpha * partial into C atomically (C prepared by the caller).
// Epilogue (splits == 1): Z = result is stored to C; if gelu_out, GELU(Z) is
// also stored as BF16 to gelu_out (same ldc); if bf16_out, Z as BF16.
struct GemmArgs {
  int M, N, K, ta, tb;
  const __nv_bfloat16* A;
  long long lda, sA;
  const __nv_bfloat16* B;
  long long ldb, sB;
  float* C;
  long long ldc, sC;
  float alpha, beta;
  const float* bias;
  __nv_bfloat16* gelu_out;
  __nv_bfloat16* bf16_out;
  long long sO;
  int batch, splits;
};

__global__ void __launch_bounds__(128) sno_gemm_kernel(GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* As = sm;                      // TM x TK BF16, canonical layout (16 KB)
  unsigned char* Bs = sm + TM * TK * 2;        // TN x TK BF16 (8 KB)
  unsigned long long* bar = (unsigned long long*)(Bs + TN * TK * 2);
  unsigned* tmem_slot = (unsigned*)(bar + 1);
  const int z = blockIdx.z / g.splits, sp = blockIdx.z % g.splits;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const __nv_bfloat16* A = g.A + (long long)z * g.sA;
  const __nv_bfloat16* B = g.B + (long long)z * g.sB;
  float* C = g.C + (long long)z * g.sC;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nk = (g.K + TK - 1) / TK;
  const int per = (nk + g.splits - 1) / g.splits;
  const int kb0 = sp * per, kb1 = min(nk, kb0 + per);
  const unsigned bar_a = smem_u32(bar);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {  // tensor-memory accumulator: 128 lanes x 64 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = *tmem_slot;

  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  unsigned phase = 0;
  bool ok = true;
  for (int kb = kb0; kb < kb1 && ok; ++kb) {
    const int k0 = kb * TK;
    // global -> shared in the canonical layout: op(A) rows m, op(B)^T rows n, k inner
    for (int e = tid; e < TM * TK; e += 128) {
      int m, k;
      if (g.ta) { m = e % TM; k = e / TM; } else { k = e % TK; m = e / TK; }
      const int gm = m0 + m, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gm < g.M && gk < g.K) v = g.ta ? A[(long long)gk * g.lda + gm] : A[(long long)gm * g.lda + gk];
      *reinterpret_cast<__nv_bfloat16*>(As + core_off(m, k)) = v;
    }
    for (int e = tid; e < TN * TK; e += 128) {
      int n, k;
      if (g.tb) { k = e % TK; n = e / TK; } else { n = e % TN; k = e / TN; }
      const int gn = n0 + n, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gn < g.N && gk < g.K) v = g.tb ? B[(long long)gn * g.ldb + gk] : B[(long long)gk * g.ldb + gn];
      *reinterpret_cast<__nv_bfloat16*>(Bs + core_off(n, k)) = v;
    }
    // the generic-proxy stores must be visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      for (int j = 0; j < TK / 16; ++j) {
        const unsigned long long ad = smem_desc(smem_u32(As) + j * 256);
        const unsigned long long bd = smem_desc(smem_u32(Bs) + j * 256);
        const unsigned acc = (kb > kb0 || j > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar_a)
                   : "memory");
    }
    // the MMAs have read the tiles before they are overwritten or the result is read
    ok = mbar_wait(bar_a, phase);
    phase ^= 1;
    __syncthreads();
  }
  if (!ok && lane == 0) atomicAdd(&g_gemm_timeouts, 1u);
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

  if (ok && kb1 > kb0) {
    // this warp's 32 accumulator lanes = rows 32 warp + lane, columns 0..63
    float acc[TN];
    {
      unsigned r[TN];
      const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
          "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
          "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
            "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
            "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
            "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]),
            "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
            "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]),
            "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
            "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int c = 0; c < TN; ++c) acc[c] = __uint_as_float(r[c]);
    }
    const int m = m0 + 32 * warp + lane;
    if (m < g.M) {
#pragma unroll 8
      for (int c = 0; c < TN; ++c) {
        const int n = n0 + c;
        if (n >= g.N) break;
        float* cp = C + (long long)m * g.ldc + n;
        const float v = g.alpha * acc[c];
        if (g.splits > 1) {
          atomicAdd(cp, v);
          continue;
        }
        const float zv = v + (g.beta != 0.f ? g.beta * *cp : 0.f) + (g.bias ? g.bias[n] : 0.f);
        *cp = zv;
        const long long o = (long long)z * g.sO + (long long)m * g.ldc + n;
        if (g.gelu_out) g.gelu_out[o] = __float2bfloat16(gelu_f(zv));
        if (g.bf16_out) g.bf16_out[o] = __float2bfloat16(zv);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

__global__ void gelu_backward_kernel(const float* dy, const float* zpre, float* dz, __nv_bfloat16* dz16,
                                     long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = dy[i] * gelu_grad(zpre[i]);
    dz[i] = v;
    if (dz16) dz16[i] = __float2bfloat16(v);
  }
}

__global__ void to_bf16_kernel(const float* x, __nv_bfloat16* y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

// column sums of a rows x cols row-major matrix, added into out[cols]
__global__ void colsum_kernel(const float* x, long long rows, int cols, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const long long r0 = blockIdx.y * (long long)((rows + gridDim.y - 1) / gridDim.y);
  const long long r1 = min(rows, r0 + (rows + gridDim.y - 1) / gridDim.y);
  float s = 0.f;
  for (long long r = r0; r < r1; ++r) s += x[r * cols + c];
  atomicAdd(out + c, s);
}

// Adam with bias correction (Kingma & Ba); refreshes the BF16 copy of the weights
__global__ void adam_kernel(float* w, const float* gr, float* m, float* v, __nv_bfloat16* w16, long long n,
                            float lr, float b1, float b2, float eps, float c1, float c2, float wd) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float g = gr[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16(wi);
  }
}

// Per sample b (rows of `len` floats): e_b = |pred - tgt|^2 / |tgt|^2 (into err[b]);
// grad = 2 (pred - tgt) / (|tgt|^2 * batch) when grad != null.
__global__ void rel_l2_kernel(const float* pred, const float* tgt, long long len, int batch, float* err,
                              float* grad) {
  const int b = blockIdx.x;
  const float* p = pred + (long long)b * len;
  const float* t = tgt + (long long)b * len;
  __shared__ float sd[256], st[256];
  float d2 = 0.f, t2 = 0.f;
  for (long long i = threadIdx.x; i < len; i += blockDim.x) {
    const float d = p[i] - t[i];
    d2 += d * d;
    t2 += t[i] * t[i];
  }
  sd[threadIdx.x] = d2;
  st[threadIdx.x] = t2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sd[threadIdx.x] += sd[threadIdx.x + s];
      st[threadIdx.x] += st[threadIdx.x + s];
    }
    __syncthreads();
  }
  const float tn = st[0] > 0.f ? st[0] : 1.f;
  if (threadIdx.x == 0) err[b] = sd[0] / tn;
  if (grad) {
    const float sc = 2.f / (tn * (float)batch);
    for (long long i = threadIdx.x; i < len; i += blockDim.x) grad[(long long)b * len + i] = sc * (p[i] - t[i]);
  }
}

int grid1(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

}  // namespace

extern "C" {

int sno_gemm_timeouts(unsigned* out) {
  if (!out) return SNO_BAD_ARGUMENT;
  return cudaMemcpyFromSymbol(out, g_gemm_timeouts, sizeof(unsigned)) == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_gemm(int M, int N, int K, int ta, int tb, const void* A, long long lda, long long sA, const void* B,
             long long ldb, long long sB, float* C, long long ldc, long long sC, int batch, float alpha,
             float beta, const float* bias, void* gelu_out, void* bf16_out, long long sO, int splits,
             void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || batch <= 0 || !A || !B || !C || splits < 1 || splits > 1024)
    return SNO_BAD_ARGUMENT;
  if (splits > 1 && (bias || gelu_out || bf16_out || beta != 1.0f)) return SNO_BAD_ARGUMENT;
  GemmArgs g;
  g.M = M; g.N = N; g.K = K; g.ta = ta; g.tb = tb;
  g.A = (const __nv_bfloat16*)A; g.lda = lda; g.sA = sA;
  g.B = (const __nv_bfloat16*)B; g.ldb = ldb; g.sB = sB;
  g.C = C; g.ldc = ldc; g.sC = sC;
  g.alpha = alpha; g.beta = beta; g.bias = bias;
  g.gelu_out = (__nv_bfloat16*)gelu_out; g.bf16_out = (__nv_bfloat16*)bf16_out; g.sO = sO;
  g.batch = batch; g.splits = splits;
  const long long gz = (long long)batch * splits;
  if (gz > 65535) return SNO_BAD_ARGUMENT;
  dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, (unsigned)gz);
  if (grid.y > 65535) return SNO_BAD_ARGUMENT;
  // 24 KB of tiles plus the barrier; 36 KB requested keeps at most 6 CTAs (384 of the 512
  // tensor-memory columns) on an SM
  const int smem = 36 * 1024;
  if (cudaFuncSetAttribute(sno_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return SNO_CUDA_ERROR;
  sno_gemm_kernel<<<grid, 128, smem, (cudaStream_t)stream>>>(g);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_gelu_backward(const float* dy, const float* zpre, float* dz, void* dz_bf16, long long n, void* stream) {
  if (!dy || !zpre || !dz || n < 0) return SNO_BAD_ARGUMENT;
  if (n == 0) return SNO_OK;
  gelu_backward_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(dy, zpre, dz, (__nv_bfloat16*)dz_bf16, n);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_to_bf16(const float* x, void* y, long long n, void* stream) {
  if (!x || !y || n < 0) return SNO_BAD_ARGUMENT;
  if (n == 0) return SNO_OK;
  to_bf16_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(x, (__nv_bfloat16*)y, n);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_colsum(const float* x, long long rows, int cols, float* out, void* stream) {
  if (!x || !out || rows < 0 || cols <= 0) return SNO_BAD_ARGUMENT;
  if (rows == 0) return SNO_OK;
  long long parts = rows / 256;
  if (parts < 1) parts = 1;
  if (parts > 1024) parts = 1024;
  dim3 grid((cols + 63) / 64, (unsigned)parts);
  colsum_kernel<<<grid, 64, 0, (cudaStream_t)stream>>>(x, rows, cols, out);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float beta1,
             float beta2, float eps, int step, float weight_decay, void* stream) {
  if (!w || !g || !m || !v || n < 0 || step < 1) return SNO_BAD_ARGUMENT;
  if (n == 0) return SNO_OK;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16*)w_bf16, n, lr, beta1,
                                                          beta2, eps, c1, c2, weight_decay);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

int sno_rel_l2(const float* pred, const float* target, long long len, int batch, float* err, float* grad,
               void* stream) {
  if (!pred || !target || !err || len <= 0 || batch <= 0) return SNO_BAD_ARGUMENT;
  rel_l2_kernel<<<batch, 256, 0, (cudaStream_t)stream>>>(pred, target, len, batch, err, grad);
  return cudaGetLastError() == cudaSuccess ? SNO_OK : SNO_CUDA_ERROR;
}

}  // extern "C"
