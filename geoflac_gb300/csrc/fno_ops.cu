// Memory-bound kernels of the surrogate around the tensor-core GEMMs:
// layout changes between the channel-last activations and the DFT / mode
// layouts, the complex bookkeeping of the truncated 2-D DFT, activation,
// reductions, loss and the Adam update.  All elementwise work is one pass
// over the data with vectorised or shared-memory-tiled access.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/geoflac_fno.h"

namespace {

constexpr int TB = 256;

inline unsigned nblk(long long n, int t = TB) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ float ldv(const void *p, long long i, int type) {
    return type ? __bfloat162float(reinterpret_cast<const __nv_bfloat16 *>(p)[i]) : reinterpret_cast<const float *>(p)[i];
}
__device__ __forceinline__ void stv(void *p, long long i, int type, float v) {
    if (type)
        reinterpret_cast<__nv_bfloat16 *>(p)[i] = __float2bfloat16_rn(v);
    else
        reinterpret_cast<float *>(p)[i] = v;
}

// dst[b][c][r] = src[b][r][c], 32x32 tiles through shared memory
__global__ void k_transpose(const void *__restrict__ src, void *__restrict__ dst, long long rows, int cols, int st,
                            int dt) {
    __shared__ float tile[32][33];
    const long long b = blockIdx.z;
    const long long off = b * (long long)rows * cols;
    const long long r0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        long long r = r0 + k;
        int c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[k][threadIdx.x] = ldv(src, off + r * cols + c, st);
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int c = c0 + k;
        long long r = r0 + threadIdx.x;
        if (r < rows && c < cols) stv(dst, off + (long long)c * rows + r, dt, tile[threadIdx.x][k]);
    }
}

__global__ void k_cast(const void *__restrict__ src, void *__restrict__ dst, long long n, int st, int dt) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) stv(dst, i, dt, ldv(src, i, st));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void k_gelu(const float *__restrict__ z, void *__restrict__ a, long long n, int at) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) stv(a, i, at, gelu(z[i]));
}

__global__ void k_gelu_bwd(const float *__restrict__ z, const void *__restrict__ da, int dat, float *__restrict__ dz,
                           __nv_bfloat16 *__restrict__ dzb, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = ldv(da, i, dat) * gelu_d(z[i]);
    dz[i] = g;
    if (dzb) dzb[i] = __float2bfloat16_rn(g);
}

// Forward DFT bookkeeping.  Y[(b, c, kp)][q] holds, for the W-transformed
// row kp (kp < m2: real part of mode kp, kp >= m2: imaginary part), the
// cosine (q < Q) and sine (q >= Q) sums over h of the Q kept H-modes.
// U[(k2, q)][b][(c, part)] = sum_h (Xr + i Xi) e^{-i phi}.
__global__ void k_spec_combine(const float *__restrict__ Y, __nv_bfloat16 *__restrict__ U, int B, int C, int m2,
                               int Q) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)Q * m2 * B * C;
    if (t >= total) return;
    int c = (int)(t % C);
    long long r = t / C;
    int b = (int)(r % B);
    r /= B;
    int k2 = (int)(r % m2);
    int q = (int)(r / m2);
    long long rre = ((long long)b * C + c) * (2 * m2) + k2, rim = rre + m2;
    const float *yre = Y + rre * (2 * Q), *yim = Y + rim * (2 * Q);
    float ure = yre[q] + yim[Q + q];
    float uim = yim[q] - yre[Q + q];
    long long o = (((long long)k2 * Q + q) * B + b) * (2 * C) + 2 * c;
    U[o] = __float2bfloat16_rn(ure);
    U[o + 1] = __float2bfloat16_rn(uim);
}

// its adjoint: dY from dU (dU FP32 [(k2, q)][b][(c, part)])
__global__ void k_spec_combine_bwd(const float *__restrict__ dU, __nv_bfloat16 *__restrict__ dY, int B, int C,
                                   int m2, int Q) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)Q * m2 * B * C;
    if (t >= total) return;
    int c = (int)(t % C);
    long long r = t / C;
    int b = (int)(r % B);
    r /= B;
    int k2 = (int)(r % m2);
    int q = (int)(r / m2);
    long long o = (((long long)k2 * Q + q) * B + b) * (2 * C) + 2 * c;
    float gre = dU[o], gim = dU[o + 1];
    long long rre = ((long long)b * C + c) * (2 * m2) + k2, rim = rre + m2;
    __nv_bfloat16 *yre = dY + rre * (2 * Q), *yim = dY + rim * (2 * Q);
    yre[q] = __float2bfloat16_rn(gre);
    yim[Q + q] = __float2bfloat16_rn(gre);
    yim[q] = __float2bfloat16_rn(gim);
    yre[Q + q] = __float2bfloat16_rn(-gim);
}

// complex mode weights R[mode][i][o][re, im] -> the real 2C x 2C blocks of
// the per-mode product, Rm[mode][(o, part)][(i, part)] and its transpose
__global__ void k_expand_modes(const float *__restrict__ R, __nv_bfloat16 *__restrict__ Rm,
                               __nv_bfloat16 *__restrict__ RmT, int modes, int C) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)modes * C * C;
    if (t >= total) return;
    int o = (int)(t % C);
    long long r = t / C;
    int i = (int)(r % C);
    long long mo = r / C;
    const float *w = R + ((mo * C + i) * C + o) * 2;
    float re = w[0], im = w[1];
    const long long n2 = 2LL * C;
    __nv_bfloat16 *M = Rm + mo * n2 * n2, *T = RmT + mo * n2 * n2;
    const __nv_bfloat16 bre = __float2bfloat16_rn(re), bim = __float2bfloat16_rn(im), nim = __float2bfloat16_rn(-im);
    // out_re = sum_i ure*re - uim*im ; out_im = sum_i ure*im + uim*re
    M[(2 * o) * n2 + 2 * i] = bre;
    M[(2 * o) * n2 + 2 * i + 1] = nim;
    M[(2 * o + 1) * n2 + 2 * i] = bim;
    M[(2 * o + 1) * n2 + 2 * i + 1] = bre;
    T[(2 * i) * n2 + 2 * o] = bre;
    T[(2 * i + 1) * n2 + 2 * o] = nim;
    T[(2 * i) * n2 + 2 * o + 1] = bim;
    T[(2 * i + 1) * n2 + 2 * o + 1] = bre;
}

// gradient of the complex weights from the gradient of the real blocks
__global__ void k_modes_grad(const float *__restrict__ dRm, float *__restrict__ dR, int modes, int C) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)modes * C * C;
    if (t >= total) return;
    int o = (int)(t % C);
    long long r = t / C;
    int i = (int)(r % C);
    long long mo = r / C;
    const long long n2 = 2LL * C;
    const float *M = dRm + mo * n2 * n2;
    float gre = M[(2 * o) * n2 + 2 * i] + M[(2 * o + 1) * n2 + 2 * i + 1];
    float gim = M[(2 * o + 1) * n2 + 2 * i] - M[(2 * o) * n2 + 2 * i + 1];
    float *w = dR + ((mo * C + i) * C + o) * 2;
    w[0] = gre;
    w[1] = gim;
}

// out[c] (+)= sum over rows of X[r][c]; one block per column group
__global__ void k_colsum(const float *__restrict__ X, float *__restrict__ out, long long rows, int cols, int accum) {
    __shared__ float red[TB];
    const int c = blockIdx.x;
    float s = 0.0f;
    for (long long r = threadIdx.x; r < rows; r += blockDim.x) s += X[r * cols + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = TB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = (accum ? out[c] : 0.0f) + red[0];
}

// column sums, stage 1: block b sums rows [b*rpb, (b+1)*rpb) of a row-major
// matrix whose column count divides the block size (coalesced reads; each
// thread stays on one column), partial[b][c]
__global__ void k_colsum_part(const float *__restrict__ X, float *__restrict__ part, long long rows, int cols,
                              long long rpb) {
    __shared__ float red[TB];
    const long long r0 = (long long)blockIdx.x * rpb, r1 = min(rows, r0 + rpb);
    const int per = TB / cols; // rows per pass
    const int c = threadIdx.x % cols, rr = threadIdx.x / cols;
    float s = 0.0f;
    for (long long r = r0 + rr; r < r1; r += per) s += X[r * cols + c];
    red[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < cols) {
        float t = 0.0f;
        for (int q = 0; q < per; ++q) t += red[q * cols + threadIdx.x];
        part[(long long)blockIdx.x * cols + threadIdx.x] = t;
    }
}

__global__ void k_sum_batches(const float *__restrict__ src, float *__restrict__ dst, int nb, long long n, int accum) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int b = 0; b < nb; ++b) s += src[(long long)b * n + i];
    dst[i] = (accum ? dst[i] : 0.0f) + s;
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float c1, float c2, float wd) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i] + wd * p[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// mean-squared error over n values; loss accumulated in FP64, gradient
// scale * 2 (pred - target) / n written as BF16 for the backward GEMMs
__global__ void k_mse(const float *__restrict__ pred, const float *__restrict__ target, void *__restrict__ dpred,
                      int dt, double *__restrict__ loss, long long n, float scale, const float *__restrict__ w,
                      long long w_period, int w_len) {
    __shared__ double red[TB];
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < n) {
        float d = pred[i] - target[i];
        float wi = w ? w[(i / w_period) % w_len] : 1.0f;
        e = (double)wi * d * d;
        if (dpred) stv(dpred, i, dt, scale * 2.0f * wi * d / (float)n);
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int w = TB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / (double)n);
}

// a = x + y (FP32) written as FP32 and/or BF16
__global__ void k_add(const float *__restrict__ x, const float *__restrict__ y, float *__restrict__ out,
                      __nv_bfloat16 *__restrict__ outb, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = x[i] + (y ? y[i] : 0.0f);
    if (out) out[i] = s;
    if (outb) outb[i] = __float2bfloat16_rn(s);
}

// surrogate input: 9 normalised fields, 4 normalised member parameters,
// 2 grid coordinates in [-1, 1], one zero channel (16, BF16)
__global__ void k_pack_input(const float *__restrict__ raw, const float *__restrict__ prm,
                             const float *__restrict__ stats, __nv_bfloat16 *__restrict__ out, int n, int H, int W) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * H * W) return;
    const int gx = (int)(t % W), gy = (int)((t / W) % H), m = (int)(t / ((long long)W * H));
    const float *r = raw + t * 9;
    __nv_bfloat16 *o = out + t * 16;
    for (int c = 0; c < 9; ++c) o[c] = __float2bfloat16_rn((r[c] - stats[c]) / stats[9 + c]);
    for (int c = 0; c < 4; ++c) o[9 + c] = __float2bfloat16_rn((prm[m * 4 + c] - stats[18 + c]) / stats[22 + c]);
    o[13] = __float2bfloat16_rn(2.0f * (gx + 0.5f) / W - 1.0f);
    o[14] = __float2bfloat16_rn(2.0f * (gy + 0.5f) / H - 1.0f);
    o[15] = __float2bfloat16_rn(0.0f);
}

// training target: normalised increments (y - x - mean_d) / std_d in 9 of 16 channels
__global__ void k_pack_target(const float *__restrict__ y, const float *__restrict__ x, const float *__restrict__ sd,
                              float *__restrict__ out, long long pts) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pts) return;
    for (int c = 0; c < 16; ++c)
        out[t * 16 + c] = c < 9 ? (y[t * 9 + c] - x[t * 9 + c] - sd[c]) / sd[9 + c] : 0.0f;
}

// prediction back to fields: y = x + mean_d + std_d * pred
__global__ void k_unpack(const float *__restrict__ pred, const float *__restrict__ x, const float *__restrict__ sd,
                         float *__restrict__ y, long long pts) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= pts) return;
    for (int c = 0; c < 9; ++c) y[t * 9 + c] = x[t * 9 + c] + sd[c] + sd[9 + c] * pred[t * 16 + c];
}

// dst[r] = src[idx[r]] for rows of `row_words` 32-bit words
__global__ void k_gather_rows(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
                              const long long *__restrict__ idx, int nrows, long long row_words) {
    const int r = blockIdx.y;
    const long long s = idx[r];
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < row_words; w += (long long)gridDim.x * blockDim.x)
        dst[(long long)r * row_words + w] = src[s * row_words + w];
    (void)nrows;
}

} // namespace

#define FNO_RET(s) return cudaGetLastError() == cudaSuccess ? GF_FNO_OK : GF_FNO_ERR_CUDA

extern "C" {

int gf_fno_pack_input(const float *raw, const float *params, const float *stats, void *out, int n, int H, int W,
                      void *stream) {
    if (!raw || !params || !stats || !out || n < 1 || H < 1 || W < 1) return GF_FNO_ERR_ARG;
    long long pts = (long long)n * H * W;
    k_pack_input<<<nblk(pts), TB, 0, (cudaStream_t)stream>>>(raw, params, stats, (__nv_bfloat16 *)out, n, H, W);
    FNO_RET(stream);
}

int gf_fno_pack_target(const float *y, const float *x, const float *stats_d, float *out, long long points,
                       void *stream) {
    if (!y || !x || !stats_d || !out || points < 1) return GF_FNO_ERR_ARG;
    k_pack_target<<<nblk(points), TB, 0, (cudaStream_t)stream>>>(y, x, stats_d, out, points);
    FNO_RET(stream);
}

int gf_fno_gather_rows(const void *src, void *dst, const long long *idx, int nrows, long long row_bytes,
                       void *stream) {
    if (!src || !dst || !idx || nrows < 1 || nrows > 65535 || row_bytes < 4 || row_bytes % 4) return GF_FNO_ERR_ARG;
    long long words = row_bytes / 4;
    unsigned gx = (unsigned)((words + TB - 1) / TB);
    if (gx > 1024) gx = 1024;
    k_gather_rows<<<dim3(gx, (unsigned)nrows), TB, 0, (cudaStream_t)stream>>>((const uint32_t *)src, (uint32_t *)dst,
                                                                             idx, nrows, words);
    FNO_RET(stream);
}

int gf_fno_unpack(const float *pred, const float *x, const float *stats_d, float *y, long long points, void *stream) {
    if (!pred || !x || !stats_d || !y || points < 1) return GF_FNO_ERR_ARG;
    k_unpack<<<nblk(points), TB, 0, (cudaStream_t)stream>>>(pred, x, stats_d, y, points);
    FNO_RET(stream);
}



int gf_fno_transpose(const void *src, void *dst, int batch, long long rows, int cols, int src_bf16, int dst_bf16,
                     void *stream) {
    if (!src || !dst || batch < 1 || rows < 1 || cols < 1 || batch > 65535 || (cols + 31) / 32 > 65535 ||
        (rows + 31) / 32 > 2147483647LL)
        return GF_FNO_ERR_ARG;
    dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((cols + 31) / 32), (unsigned)batch);
    k_transpose<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>(src, dst, rows, cols, src_bf16, dst_bf16);
    FNO_RET(stream);
}

int gf_fno_cast(const void *src, void *dst, long long n, int src_bf16, int dst_bf16, void *stream) {
    if (!src || !dst || n < 0) return GF_FNO_ERR_ARG;
    if (n) k_cast<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(src, dst, n, src_bf16, dst_bf16);
    FNO_RET(stream);
}

int gf_fno_gelu(const float *z, void *a, long long n, int a_bf16, void *stream) {
    if (!z || !a || n < 0) return GF_FNO_ERR_ARG;
    if (n) k_gelu<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(z, a, n, a_bf16);
    FNO_RET(stream);
}

int gf_fno_gelu_bwd(const float *z, const void *da, int da_bf16, float *dz, void *dz_bf16, long long n, void *stream) {
    if (!z || !da || !dz || n < 0) return GF_FNO_ERR_ARG;
    if (n) k_gelu_bwd<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(z, da, da_bf16, dz, (__nv_bfloat16 *)dz_bf16, n);
    FNO_RET(stream);
}

int gf_fno_spec_combine(const float *Y, void *U, int B, int C, int m2, int Q, void *stream) {
    if (!Y || !U || B < 1 || C < 1 || m2 < 1 || Q < 1) return GF_FNO_ERR_ARG;
    long long n = (long long)Q * m2 * B * C;
    k_spec_combine<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(Y, (__nv_bfloat16 *)U, B, C, m2, Q);
    FNO_RET(stream);
}

int gf_fno_spec_combine_bwd(const float *dU, void *dY, int B, int C, int m2, int Q, void *stream) {
    if (!dU || !dY || B < 1 || C < 1 || m2 < 1 || Q < 1) return GF_FNO_ERR_ARG;
    long long n = (long long)Q * m2 * B * C;
    k_spec_combine_bwd<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(dU, (__nv_bfloat16 *)dY, B, C, m2, Q);
    FNO_RET(stream);
}

int gf_fno_expand_modes(const float *R, void *Rm, void *RmT, int modes, int C, void *stream) {
    if (!R || !Rm || !RmT || modes < 1 || C < 1) return GF_FNO_ERR_ARG;
    long long n = (long long)modes * C * C;
    k_expand_modes<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(R, (__nv_bfloat16 *)Rm, (__nv_bfloat16 *)RmT, modes, C);
    FNO_RET(stream);
}

int gf_fno_modes_grad(const float *dRm, float *dR, int modes, int C, void *stream) {
    if (!dRm || !dR || modes < 1 || C < 1) return GF_FNO_ERR_ARG;
    long long n = (long long)modes * C * C;
    k_modes_grad<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(dRm, dR, modes, C);
    FNO_RET(stream);
}

int gf_fno_colsum(const float *X, float *out, long long rows, int cols, int accum, void *stream) {
    if (!X || !out || rows < 1 || cols < 1) return GF_FNO_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cols <= TB && TB % cols == 0 && rows >= 4096) {
        // two stages through a fixed scratch of 1024 partial rows
        static float *part = nullptr;
        static int part_cols = 0;
        const int nb = 1024;
        if (!part || part_cols < cols) {
            if (part) cudaFree(part);
            part = nullptr;
            if (cudaMalloc(&part, sizeof(float) * nb * TB) != cudaSuccess) return GF_FNO_ERR_CUDA;
            part_cols = TB;
        }
        long long rpb = (rows + nb - 1) / nb;
        k_colsum_part<<<nb, TB, 0, st>>>(X, part, rows, cols, rpb);
        k_sum_batches<<<nblk(cols), TB, 0, st>>>(part, out, nb, cols, accum);
    } else {
        k_colsum<<<(unsigned)cols, TB, 0, st>>>(X, out, rows, cols, accum);
    }
    FNO_RET(stream);
}

int gf_fno_sum_batches(const float *src, float *dst, int nb, long long n, int accum, void *stream) {
    if (!src || !dst || nb < 1 || n < 1) return GF_FNO_ERR_ARG;
    k_sum_batches<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(src, dst, nb, n, accum);
    FNO_RET(stream);
}

int gf_fno_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                int step, float weight_decay, void *stream) {
    if (!p || !g || !m || !v || n < 1 || step < 1) return GF_FNO_ERR_ARG;
    float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2, weight_decay);
    FNO_RET(stream);
}

int gf_fno_mse(const float *pred, const float *target, void *dpred, int dpred_bf16, double *loss, long long n,
               float scale, void *stream) {
    if (!pred || !target || !loss || n < 1) return GF_FNO_ERR_ARG;
    k_mse<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(pred, target, dpred, dpred_bf16, loss, n, scale, nullptr, 1, 1);
    FNO_RET(stream);
}

int gf_fno_mse_weighted(const float *pred, const float *target, void *dpred, int dpred_bf16, double *loss,
                        long long n, float scale, const float *w, long long w_period, int w_len, void *stream) {
    if (!pred || !target || !loss || !w || n < 1 || w_period < 1 || w_len < 1) return GF_FNO_ERR_ARG;
    k_mse<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(pred, target, dpred, dpred_bf16, loss, n, scale, w, w_period,
                                                   w_len);
    FNO_RET(stream);
}

int gf_fno_add(const float *x, const float *y, float *out, void *out_bf16, long long n, void *stream) {
    if (!x || (!out && !out_bf16) || n < 0) return GF_FNO_ERR_ARG;
    if (n) k_add<<<nblk(n), TB, 0, (cudaStream_t)stream>>>(x, y, out, (__nv_bfloat16 *)out_bf16, n);
    FNO_RET(stream);
}

} // extern "C"
