/* geoflac_fno.h -- tensor-core kernels of the learned surrogate (Fourier
 * neural operator) that screens and fast-forwards ensemble members.
 *
 * No reference counterpart: GeoFLAC has no learned component.  Device
 * pointers throughout; every call is asynchronous on `stream` (a
 * cudaStream_t, NULL = default stream).
 */
#ifndef GEOFLAC_FNO_H
#define GEOFLAC_FNO_H

#ifdef __cplusplus
extern "C" {
#endif

#define GF_FNO_OK 0
#define GF_FNO_ERR_CUDA (-1)
#define GF_FNO_ERR_ARG (-2)
#define GF_FNO_ERR_ALIGN (-3)   /* TMA needs 16-byte aligned bases and strides */
#define GF_FNO_ERR_TIMEOUT (-6) /* a bounded wait inside a kernel gave up */

/* C[z][m][n] = alpha * sum_k A[z][m][k] * B[z][n][k] + beta * C[z][m][n] + bias[n]
 * A: BF16, row stride lda, batch stride sA (elements); B: BF16, ldb, sB;
 * C: FP32 (c_bf16 = 0) or BF16 (c_bf16 = 1, beta must be 0), ldc, sC
 * (sA/sB/sC = 0: dense batches).  K % 8 == 0, lda and ldb multiples of 8.
 * tcgen05 MMA with FP32 accumulation in tensor memory, TMA operand loads. */
int gf_gemm_bf16(const void *A, const void *B, void *C, int batch, int M, int N, int K, long long lda, long long sA,
                 long long ldb, long long sB, long long ldc, long long sC, int c_bf16, float alpha, float beta,
                 const float *bias, void *stream);
/* GF_FNO_ERR_TIMEOUT if a GEMM kernel gave up a wait since the last call. */
int gf_gemm_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GEOFLAC_FNO_H */
