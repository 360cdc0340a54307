/*
 * C ABI of the spectral neural operator (SNO) surrogate kernels.
 *
 * No pyofss counterpart: the surrogate maps an input pulse to the field after a
 * fixed fibre segment and falls back to the RK4IP engine (gnlse.h) when its
 * error estimate exceeds a tolerance.  Matrices are row-major; BF16 operands
 * are raw 16-bit bfloat16 arrays; every call is stream-ordered on `stream`
 * (a cudaStream_t) and returns an SNO_* status.
 */
#ifndef SNO_H
#define SNO_H

#ifdef __cplusplus
extern "C" {
#endif

enum { SNO_OK = 0, SNO_BAD_ARGUMENT = 4, SNO_CUDA_ERROR = 5 };

/* Batched GEMM on the BF16 tensor cores (tcgen05.mma, kind::f16, FP32 accumulator in
 * tensor memory; 128 x 64 output tiles, 64-deep K tiles staged in shared memory):
 *   C[z] = alpha * op(A[z]) * op(B[z]) + beta * C[z] (+ bias[n]),  z < batch,
 * op(A) = A (M x K, A[m*lda + k]) or, with ta = 1, A^T stored K x M (A[k*lda + m]);
 * op(B) = B (K x N, B[k*ldb + n]) or, with tb = 1, B^T stored N x K (B[n*ldb + k]).
 * sA, sB, sC: element strides between batch entries (0 = shared operand).
 * splits > 1 splits K over CTAs that add alpha * partial into C atomically
 * (then beta must be 1 and bias / outputs NULL).  Optional outputs, stride sO:
 * gelu_out = BF16 GELU(result), bf16_out = BF16 result. */
int sno_gemm(int M, int N, int K, int ta, int tb, const void* A, long long lda, long long sA, const void* B,
             long long ldb, long long sB, float* C, long long ldc, long long sC, int batch, float alpha,
             float beta, const float* bias, void* gelu_out, void* bf16_out, long long sO, int splits,
             void* stream);

/* Number of GEMM CTAs (since the library was loaded) whose wait for the tensor cores
 * ran out of its iteration bound; they skipped the rest of their tile.  Synchronous. */
int sno_gemm_timeouts(unsigned* out);

/* dz = dy * GELU'(zpre) (tanh form), optionally also as BF16 into dz_bf16. */
int sno_gelu_backward(const float* dy, const float* zpre, float* dz, void* dz_bf16, long long n, void* stream);

/* y = BF16(x). */
int sno_to_bf16(const float* x, void* y, long long n, void* stream);

/* out[c] += sum_r x[r*cols + c]  (bias gradients). */
int sno_colsum(const float* x, long long rows, int cols, float* out, void* stream);

/* One Adam step (bias-corrected, decoupled-free L2 term weight_decay * w added to
 * the gradient) on FP32 weights w with moments m, v; refreshes w_bf16 if not NULL. */
int sno_adam(float* w, const float* g, float* m, float* v, void* w_bf16, long long n, float lr, float beta1,
             float beta2, float eps, int step, float weight_decay, void* stream);

/* Per row b of `len` values: err[b] = |pred - target|^2 / |target|^2; with grad
 * != NULL also grad = d(mean_b err_b)/d pred. */
int sno_rel_l2(const float* pred, const float* target, long long len, int batch, float* err, float* grad,
               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SNO_H */
