// BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation
// in tensor memory: the matrix products of the surrogate (1x1 channel
// mixing, truncated DFTs written as products with DFT matrices, per-mode
// spectral mixing, and their gradients).
//
//   C[z][m][n] = alpha * sum_k A[z][m][k] * B[z][n][k] + beta * C[z][m][n] + bias[n]
//
// A and B are K-major BF16 (row stride lda/ldb elements, batch stride
// sA/sB), C is row-major FP32 or BF16.  One CTA computes a 128 x BN tile:
// one thread issues TMA loads of 128x64 (A) and BNx64 (B) BF16 tiles into a
// 4-stage ring of 128-byte-swizzled shared-memory buffers, one thread issues
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

template <int BN> struct __align__(1024) GemmSmem {
    __nv_bfloat16 a[STAGES][BM * BK]; // 16 KB per stage, 1024-byte aligned
    __nv_bfloat16 b[STAGES][BN * BK];
    uint64_t full[STAGES], empty[STAGES], done;
    uint32_t tmem_base;
};

struct Epilogue {
    void *C;
    long long ldc, sC;
    int M, N, c_bf16;
    float alpha, beta;
    const float *bias;
};

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
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int K, Epilogue ep) {
    extern __shared__ uint8_t dsmem[];
    GemmSmem<BN> &S = *reinterpret_cast<GemmSmem<BN> *>((reinterpret_cast<uintptr_t>(dsmem) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, z = blockIdx.z;
    const int nk = (K + BK - 1) / BK;
    __shared__ int fail;
    if (threadIdx.x == 0) {
        fail = 0;
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&S.full[s], 1);
            mbar_init(&S.empty[s], 1);
        }
        mbar_init(&S.done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"((uint32_t)BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem_base;

    if (warp == 0) {
        if (lane == 0) { // TMA producer
            const uint32_t bytes = (uint32_t)(BM + BN) * BK * sizeof(__nv_bfloat16);
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % STAGES;
                if (kb >= STAGES && !mbar_wait(&S.empty[s], ((kb / STAGES) - 1) & 1)) {
                    fail = 1;
                    break;
                }
                mbar_expect_tx(&S.full[s], bytes);
                tma_load_3d(S.a[s], &tmA, kb * BK, m0, z, &S.full[s]);
                tma_load_3d(S.b[s], &tmB, kb * BK, n0, z, &S.full[s]);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) { // MMA issuer
            const uint32_t id = idesc<BN>();
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % STAGES;
                if (!mbar_wait(&S.full[s], (kb / STAGES) & 1)) {
                    fail = 1;
                    break;
                }
                fence_after();
                const uint64_t da = sdesc(smem_u32(S.a[s])), db = sdesc(smem_u32(S.b[s]));
#pragma unroll
                for (int k = 0; k < BK / 16; ++k)
                    mma(tmem, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), id, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(&S.empty[s]);
            }
            mma_commit(&S.done);
        }
        __syncwarp();
    }
    const bool ok = mbar_wait(&S.done, 0);
    fence_after();
    if (ok && !fail) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tmem_ld32(trow + (uint32_t)c0, v);
            if (row >= ep.M) continue;
            const int col0 = n0 + c0;
            if (col0 >= ep.N) continue;
            if (ep.c_bf16) {
                __nv_bfloat16 *C = reinterpret_cast<__nv_bfloat16 *>(ep.C) + (long long)z * ep.sC + (long long)row * ep.ldc;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int col = col0 + i;
                    if (col < ep.N) {
                        float x = ep.alpha * v[i];
                        if (ep.bias) x += ep.bias[col];
                        C[col] = __float2bfloat16_rn(x);
                    }
                }
            } else {
                float *C = reinterpret_cast<float *>(ep.C) + (long long)z * ep.sC + (long long)row * ep.ldc;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int col = col0 + i;
                    if (col < ep.N) {
                        float x = ep.alpha * v[i];
                        if (ep.beta != 0.0f) x += ep.beta * C[col];
                        if (ep.bias) x += ep.bias[col];
                        C[col] = x;
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
                             const Epilogue &ep, cudaStream_t s) {
    const size_t smem = sizeof(GemmSmem<BN>) + 1024;
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_gemm_bf16<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
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
    if (!A || !B || !C || batch < 1 || M < 1 || N < 1 || K < 1) return GF_FNO_ERR_ARG;
    if (batch > 65535 || (M + BM - 1) / BM > 2147483647LL) return GF_FNO_ERR_ARG;
    // TMA: 16-byte aligned base addresses and row / batch strides
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return GF_FNO_ERR_ALIGN;
    if ((lda * 2) % 16 || (ldb * 2) % 16 || (sA * 2) % 16 || (sB * 2) % 16 || K % 8) return GF_FNO_ERR_ALIGN;
    if (lda < K || ldb < K || ldc < N) return GF_FNO_ERR_ARG;
    if (c_bf16 && beta != 0.0f) return GF_FNO_ERR_ARG;
    const int bn = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, K, M, batch, lda, sA, BM) || !make_map(&tb, B, K, N, batch, ldb, sB, bn))
        return GF_FNO_ERR_CUDA;
    Epilogue ep{C, ldc, sC > 0 ? sC : (long long)M * ldc, M, N, c_bf16, alpha, beta, bias};
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
