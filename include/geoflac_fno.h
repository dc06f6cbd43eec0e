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
/* The same with three extensions: sA = -1 shares one A among all batches;
 * (FP32 C only) aux, if not NULL, receives a BF16 copy of the final C
 * (act = 0) or of GELU(C) (act = 1) in the same layout; and c_bf16 = 2
 * (with aux) leaves C unwritten: C is then only read, for beta != 0, or
 * may be NULL with beta = 0 (inference, where only the BF16 activation
 * is kept). */
int gf_gemm_bf16_ex(const void *A, const void *B, void *C, int batch, int M, int N, int K, long long lda,
                    long long sA, long long ldb, long long sB, long long ldc, long long sC, int c_bf16, float alpha,
                    float beta, const float *bias, void *aux, int act, void *stream);
/* GF_FNO_ERR_TIMEOUT if a GEMM kernel gave up a wait since the last call. */
int gf_gemm_error(void);

/* Element types below: 0 = FP32, 1 = BF16. */
/* dst[b][c][r] = src[b][r][c] for batch matrices of rows x cols. */
int gf_fno_transpose(const void *src, void *dst, int batch, long long rows, int cols, int src_bf16, int dst_bf16,
                     void *stream);
int gf_fno_cast(const void *src, void *dst, long long n, int src_bf16, int dst_bf16, void *stream);
/* a = GELU(z) (erf form); dz = da * GELU'(z), with an optional BF16 copy. */
int gf_fno_gelu(const float *z, void *a, long long n, int a_bf16, void *stream);
int gf_fno_gelu_bwd(const float *z, const void *da, int da_bf16, float *dz, void *dz_bf16, long long n, void *stream);
/* Complex bookkeeping of the truncated 2-D DFT.  Y[(b, c, kp)][q]: for the
 * W-transformed row kp (kp < m2 real part, kp >= m2 imaginary part of W-mode
 * kp mod m2), cosine (q < Q) and sine (q >= Q) sums over the rows h of the Q
 * kept H-modes.  U[(k2, q)][b][(c, re|im)] (BF16) is the 2-D DFT coefficient;
 * the _bwd form maps dU (FP32, same layout) back to dY (BF16). */
int gf_fno_spec_combine(const float *Y, void *U, int B, int C, int m2, int Q, void *stream);
int gf_fno_spec_combine_bwd(const float *dU, void *dY, int B, int C, int m2, int Q, void *stream);
/* Complex mode weights R[mode][i][o][re, im] (FP32) to the real 2C x 2C
 * blocks Rm[mode][(o, part)][(i, part)] and RmT = transpose (BF16), and the
 * gradient of R from the gradient of Rm. */
int gf_fno_expand_modes(const float *R, void *Rm, void *RmT, int modes, int C, void *stream);
int gf_fno_modes_grad(const float *dRm, float *dR, int modes, int C, void *stream);
/* out[c] (+)= sum_r X[r][c]; dst[i] (+)= sum_b src[b][i]. */
int gf_fno_colsum(const float *X, float *out, long long rows, int cols, int accum, void *stream);
int gf_fno_sum_batches(const float *src, float *dst, int nb, long long n, int accum, void *stream);
/* Adam (bias-corrected, decoupled from the loss scale), step counts from 1. */
int gf_fno_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                int step, float weight_decay, void *stream);
/* loss += mean((pred - target)^2); dpred = scale * 2 (pred - target) / n. */
int gf_fno_mse(const float *pred, const float *target, void *dpred, int dpred_bf16, double *loss, long long n,
               float scale, void *stream);
/* Surrogate input from a sampled grid raw [n][H][W][9] and member
 * parameters [n][4]: (raw - mean) / std per channel, (params - pmean) /
 * pstd, two grid coordinates in [-1, 1], one zero channel -> BF16
 * [n][H][W][16].  stats = {mean[9], std[9], pmean[4], pstd[4]}. */
int gf_fno_pack_input(const float *raw, const float *params, const float *stats, void *out, int n, int H, int W,
                      void *stream);
/* Training target from the later grid y and the earlier x: (y - x - mean_d) /
 * std_d in channels 0..8 of 16 (FP32); stats_d = {mean_d[9], std_d[9]}. */
int gf_fno_pack_target(const float *y, const float *x, const float *stats_d, float *out, long long points,
                       void *stream);
/* dst[r] = src[idx[r]] for nrows rows of row_bytes bytes (idx on the device). */
int gf_fno_gather_rows(const void *src, void *dst, const long long *idx, int nrows, long long row_bytes,
                       void *stream);
/* Prediction back to fields: y = x + mean_d + std_d * pred. */
int gf_fno_unpack(const float *pred, const float *x, const float *stats_d, float *y, long long points, void *stream);
/* The same with weights: term i weighted by w[(i / w_period) % w_len]. */
int gf_fno_mse_weighted(const float *pred, const float *target, void *dpred, int dpred_bf16, double *loss,
                        long long n, float scale, const float *w, long long w_period, int w_len, void *stream);
/* out = x + y (y may be NULL), FP32 and/or BF16 outputs. */
int gf_fno_add(const float *x, const float *y, float *out, void *out_bf16, long long n, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GEOFLAC_FNO_H */
