// BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation
// in tensor memory: the matrix products of the surrogate (1x1 channel
// mixing, truncated DFTs written as products with DFT matrices, per-mode
// spectral mixing, and their gradients).
//
//   C[z][m][n] = alpha * sum_k A[z][m][k] * B[z][n][k] + beta * C[z][m][n] + bias[n]
//
// A and B are K-major BF16 (row stride lda/ldb elements, batch stride
// sA/sB; sA = -1 shares one A among all batches), C is row-major FP32 or
// BF16, with an optional BF16 copy of C or of GELU(C) (fused activation).
// One CTA computes a 128 x BN tile: one thread issues TMA loads of 128x64
// (A) and BNx64 (B) BF16 tiles into a ring of up to 4 (as many as the
// K-blocks) 128-byte-swizzled shared-memory buffers, one thread issues
// tcgen05.mma (M=128, N=BN, K=16) from shared-memory descriptors into a TMEM
// accumulator, and the four warps read the accumulator back with
// tcgen05.ld for the epilogue.  Every wait on an mbarrier is bounded; a
// timed-out wait raises the error flag read by gf_gemm_error().

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/geoflac_fno.h"

namespace {

constexpr int BM = 128, BK = 64, STAGES = 4, GEMM_THREADS = 128;
constexpr long long WAIT_LIMIT = 1LL << 22;

__device__ int g_gemm_err;

// shared memory of one CTA with a ring of `stages` operand buffers:
// A stages, B stages (each 1024-byte aligned), then the mbarriers
template <int BN> struct SmemLayout {
    static constexpr uint32_t a_bytes = BM * BK * 2, b_bytes = BN * BK * 2;
    __host__ __device__ static uint32_t bars(int stages) { return (uint32_t)stages * (a_bytes + b_bytes); }
    __host__ __device__ static uint32_t total(int stages) { return bars(stages) + (2 * stages + 2) * 8 + 16; }
};

struct Epilogue {
    void *C;
    long long ldc, sC;
    int M, N, c_bf16;
    float alpha, beta;
    const float *bias;
    __nv_bfloat16 *aux; // optional second output act(z) in BF16 (same layout as C)
    int act;            // 0: aux = z, 1: aux = GELU(z)
    int a_bcast;        // A shared by every batch (loaded at batch coordinate 0)
    int stages;
};

__device__ __forceinline__ float act_gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (long long it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
                 : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (start address and offsets in 16-byte units)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// instruction descriptor: BF16 x BF16 -> FP32, both K-major, M = 128
template <int BN> __device__ __forceinline__ uint32_t idesc() {
    return (1u << 4)                      // D format F32
           | (1u << 7)                    // A format BF16
           | (1u << 10)                   // B format BF16
           | ((uint32_t)(BN >> 3) << 17)  // N
           | ((uint32_t)(BM >> 4) << 24); // M
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t id, uint32_t accum) {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                 "l"(da), "l"(db), "r"(id), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BN>
__global__ void __launch_bounds__(GEMM_THREADS)
    k_gemm_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int K, Epilogue ep) {
    extern __shared__ uint8_t dsmem[];
    typedef SmemLayout<BN> L;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~static_cast<uintptr_t>(1023));
    const int stages = ep.stages;
    uint8_t *sa = base, *sb = base + (size_t)stages * L::a_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(base + L::bars(stages));
    uint64_t *empty = full + stages, *done = empty + stages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, z = blockIdx.z;
    const int nk = (K + BK - 1) / BK;
    __shared__ int fail;
    if (threadIdx.x == 0) {
        fail = 0;
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) { // TMA producer
            const uint32_t bytes = (uint32_t)(BM + BN) * BK * sizeof(__nv_bfloat16);
            const int za = ep.a_bcast ? 0 : z;
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % stages;
                if (kb >= stages && !mbar_wait(&empty[s], ((kb / stages) - 1) & 1)) {
                    fail = 1;
                    break;
                }
                mbar_expect_tx(&full[s], bytes);
                tma_load_3d(sa + (size_t)s * L::a_bytes, &tmA, kb * BK, m0, za, &full[s]);
                tma_load_3d(sb + (size_t)s * L::b_bytes, &tmB, kb * BK, n0, z, &full[s]);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) { // MMA issuer
            const uint32_t id = idesc<BN>();
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % stages;
                if (!mbar_wait(&full[s], (kb / stages) & 1)) {
                    fail = 1;
                    break;
                }
                fence_after();
                const uint64_t da = sdesc(smem_u32(sa + (size_t)s * L::a_bytes)),
                               db = sdesc(smem_u32(sb + (size_t)s * L::b_bytes));
#pragma unroll
                for (int k = 0; k < BK / 16; ++k)
                    mma(tmem, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), id, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(&empty[s]);
            }
            mma_commit(done);
        }
        __syncwarp();
    }
    const bool ok = mbar_wait(done, 0);
    fence_after();
    if (ok && !fail) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tmem_ld32(trow + (uint32_t)c0, v);
            const int col0 = n0 + c0;
            if (row >= ep.M || col0 >= ep.N) continue;
            const long long off = (long long)z * ep.sC + (long long)row * ep.ldc + col0;
            const bool full32 = col0 + 32 <= ep.N;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                float x = ep.alpha * v[i];
                if (ep.bias && col0 + i < ep.N) x += ep.bias[col0 + i];
                v[i] = x;
            }
            if (ep.c_bf16 == 1) {
                __nv_bfloat16 *C = reinterpret_cast<__nv_bfloat16 *>(ep.C) + off;
                if (full32 && ((reinterpret_cast<uintptr_t>(C) & 15) == 0)) {
#pragma unroll
                    for (int i = 0; i < 32; i += 8) {
                        uint4 w;
                        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&w);
#pragma unroll
                        for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(v[i + 2 * q], v[i + 2 * q + 1]);
                        *reinterpret_cast<uint4 *>(C + i) = w;
                    }
                } else {
                    for (int i = 0; i < 32 && col0 + i < ep.N; ++i) C[i] = __float2bfloat16_rn(v[i]);
                }
            } else {
                float *C = reinterpret_cast<float *>(ep.C) + off;
                if (full32 && ((reinterpret_cast<uintptr_t>(C) & 15) == 0)) {
#pragma unroll
                    for (int i = 0; i < 32; i += 4) {
                        float4 o = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                        if (ep.beta != 0.0f) {
                            float4 c = *reinterpret_cast<const float4 *>(C + i);
                            o.x += ep.beta * c.x;
                            o.y += ep.beta * c.y;
                            o.z += ep.beta * c.z;
                            o.w += ep.beta * c.w;
                        }
                        if (ep.c_bf16 != 2) *reinterpret_cast<float4 *>(C + i) = o;
                        v[i] = o.x;
                        v[i + 1] = o.y;
                        v[i + 2] = o.z;
                        v[i + 3] = o.w;
                    }
                } else {
                    for (int i = 0; i < 32 && col0 + i < ep.N; ++i) {
                        float x = v[i];
                        if (ep.beta != 0.0f) x += ep.beta * C[i];
                        if (ep.c_bf16 != 2) C[i] = x;
                        v[i] = x;
                    }
                }
                if (ep.aux) {
                    __nv_bfloat16 *X = ep.aux + off;
                    if (full32 && ((reinterpret_cast<uintptr_t>(X) & 15) == 0)) {
#pragma unroll
                        for (int i = 0; i < 32; i += 8) {
                            uint4 w;
                            __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&w);
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                float a0 = v[i + 2 * q], a1 = v[i + 2 * q + 1];
                                if (ep.act) {
                                    a0 = act_gelu(a0);
                                    a1 = act_gelu(a1);
                                }
                                h[q] = __floats2bfloat162_rn(a0, a1);
                            }
                            *reinterpret_cast<uint4 *>(X + i) = w;
                        }
                    } else {
                        for (int i = 0; i < 32 && col0 + i < ep.N; ++i)
                            X[i] = __float2bfloat16_rn(ep.act ? act_gelu(v[i]) : v[i]);
                    }
                }
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(&g_gemm_err, 1);
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN));
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return g_encode;
}

// 3-D map {K, rows, batch} of a K-major BF16 operand, box {64, box_rows, 1}
bool make_map(CUtensorMap *m, const void *p, int K, int rows, int batch, long long ld, long long sbatch,
              int box_rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
    cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)(sbatch > 0 ? sbatch : (long long)rows * ld) * 2};
    cuuint32_t box[3] = {BK, (cuuint32_t)box_rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(p), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int BN> int launch(const CUtensorMap &ta, const CUtensorMap &tb, int batch, int M, int N, int K,
                             Epilogue ep, cudaStream_t s) {
    const int nk = (K + BK - 1) / BK;
    ep.stages = nk < STAGES ? nk : STAGES;
    const size_t smem = SmemLayout<BN>::total(ep.stages) + 1024;
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_gemm_bf16<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(SmemLayout<BN>::total(STAGES) + 1024)) != cudaSuccess)
            return GF_FNO_ERR_CUDA;
        attr_set = true;
    }
    dim3 grid((unsigned)((M + BM - 1) / BM), (unsigned)((N + BN - 1) / BN), (unsigned)batch);
    k_gemm_bf16<BN><<<grid, GEMM_THREADS, smem, s>>>(ta, tb, K, ep);
    return cudaGetLastError() == cudaSuccess ? GF_FNO_OK : GF_FNO_ERR_CUDA;
}

} // namespace

extern "C" {

int gf_gemm_bf16(const void *A, const void *B, void *C, int batch, int M, int N, int K, long long lda, long long sA,
                 long long ldb, long long sB, long long ldc, long long sC, int c_bf16, float alpha, float beta,
                 const float *bias, void *stream) {
    return gf_gemm_bf16_ex(A, B, C, batch, M, N, K, lda, sA, ldb, sB, ldc, sC, c_bf16, alpha, beta, bias, nullptr, 0,
                           stream);
}

int gf_gemm_bf16_ex(const void *A, const void *B, void *C, int batch, int M, int N, int K, long long lda,
                    long long sA, long long ldb, long long sB, long long ldc, long long sC, int c_bf16, float alpha,
                    float beta, const float *bias, void *aux, int act, void *stream) {
    if (!A || !B || (!C && !(c_bf16 == 2 && beta == 0.0f)) || batch < 1 || M < 1 || N < 1 || K < 1)
        return GF_FNO_ERR_ARG;
    if (batch > 65535 || (M + BM - 1) / BM > 2147483647LL) return GF_FNO_ERR_ARG;
    // TMA: 16-byte aligned base addresses and row / batch strides
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return GF_FNO_ERR_ALIGN;
    const int a_bcast = sA < 0 ? 1 : 0; // sA = -1: one A for every batch
    if ((lda * 2) % 16 || (ldb * 2) % 16 || ((a_bcast ? 0 : sA) * 2) % 16 || (sB * 2) % 16 || K % 8)
        return GF_FNO_ERR_ALIGN;
    if (lda < K || ldb < K || ldc < N) return GF_FNO_ERR_ARG;
    if (c_bf16 == 1 && (beta != 0.0f || aux)) return GF_FNO_ERR_ARG;
    if (c_bf16 == 2 && !aux) return GF_FNO_ERR_ARG; // nothing would be stored
    if (c_bf16 < 0 || c_bf16 > 2) return GF_FNO_ERR_ARG;
    if (aux && (reinterpret_cast<uintptr_t>(aux) & 15)) return GF_FNO_ERR_ALIGN;
    const int bn = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, K, M, a_bcast ? 1 : batch, lda, a_bcast ? 0 : sA, BM) ||
        !make_map(&tb, B, K, N, batch, ldb, sB, bn))
        return GF_FNO_ERR_CUDA;
    Epilogue ep{C, ldc, sC > 0 ? sC : (long long)M * ldc, M, N, c_bf16, alpha, beta, bias,
                reinterpret_cast<__nv_bfloat16 *>(aux), act, a_bcast, STAGES};
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (bn == 64) return launch<64>(ta, tb, batch, M, N, K, ep, s);
    if (bn == 128) return launch<128>(ta, tb, batch, M, N, K, ep, s);
    return launch<256>(ta, tb, batch, M, N, K, ep, s);
}

int gf_gemm_error(void) {
    int h = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&h, g_gemm_err, sizeof h) != cudaSuccess) return GF_FNO_ERR_CUDA;
    if (h) cudaMemcpyToSymbol(g_gemm_err, &zero, sizeof zero);
    return h ? GF_FNO_ERR_TIMEOUT : GF_FNO_OK;
}

} // extern "C"
