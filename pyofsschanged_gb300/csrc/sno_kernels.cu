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

constexpr int BM = 64, BN = 64, BK = 32, KP = BK + 8;  // padded k stride (bank-conflict free)

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

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[z] (M x N, row-major, ldc) = alpha * op(A[z]) op(B[z]) + beta * C[z] (+ bias[n]);
// op(A) is M x K: A[m*lda + k] (ta = 0) or A[k*lda + m] (ta = 1);
// op(B) is K x N: B[k*ldb + n] (tb = 0) or B[n*ldb + k] (tb = 1).
// Grid: (ceil(N/BN), ceil(M/BM), batch * splits).  With splits > 1 each CTA sums
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
  __shared__ __align__(16) __nv_bfloat16 As[BM][KP];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][KP];
  const int z = blockIdx.z / g.splits, sp = blockIdx.z % g.splits;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const __nv_bfloat16* A = g.A + (long long)z * g.sA;
  const __nv_bfloat16* B = g.B + (long long)z * g.sB;
  float* C = g.C + (long long)z * g.sC;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gq = lane >> 2, tq = lane & 3;
  // K range of this split, in BK chunks
  const int nk = (g.K + BK - 1) / BK;
  const int per = (nk + g.splits - 1) / g.splits;
  const int kb0 = sp * per, kb1 = min(nk, kb0 + per);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int kb = kb0; kb < kb1; ++kb) {
    const int k0 = kb * BK;
    // global -> shared: BM x BK of op(A) and BN x BK of op(B)^T, k contiguous in shared
    for (int e = tid; e < BM * BK; e += 128) {
      int m, k;
      if (g.ta) { m = e % BM; k = e / BM; } else { k = e % BK; m = e / BK; }
      const int gm = m0 + m, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gm < g.M && gk < g.K) v = g.ta ? A[(long long)gk * g.lda + gm] : A[(long long)gm * g.lda + gk];
      As[m][k] = v;
    }
    for (int e = tid; e < BN * BK; e += 128) {
      int n, k;
      if (g.tb) { k = e % BK; n = e / BK; } else { n = e % BN; k = e / BN; }
      const int gn = n0 + n, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gn < g.N && gk < g.K) v = g.tb ? B[(long long)gn * g.ldb + gk] : B[(long long)gk * g.ldb + gn];
      Bs[n][k] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + gq;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8 + gq;
        bf[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq]);
        bf[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm + i * 16 + gq + (r >> 1) * 8;
        const int n = n0 + wn + j * 8 + 2 * tq + (r & 1);
        if (m >= g.M || n >= g.N) continue;
        float* cp = C + (long long)m * g.ldc + n;
        const float v = g.alpha * acc[i][j][r];
        if (g.splits > 1) {
          atomicAdd(cp, v);
          continue;
        }
        float zv = v + (g.beta != 0.f ? g.beta * *cp : 0.f) + (g.bias ? g.bias[n] : 0.f);
        *cp = zv;
        const long long o = (long long)z * g.sO + (long long)m * g.ldc + n;
        if (g.gelu_out) g.gelu_out[o] = __float2bfloat16(gelu_f(zv));
        if (g.bf16_out) g.bf16_out[o] = __float2bfloat16(zv);
      }
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
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, (unsigned)gz);
  if (grid.y > 65535) return SNO_BAD_ARGUMENT;
  sno_gemm_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(g);
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
