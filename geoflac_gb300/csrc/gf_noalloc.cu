// Mesh-quality test without any device allocation: gf_min_angle_noalloc.
//
// Some callers cannot allocate device memory while they run the model.  A
// host code whose device arrays live in an OpenACC data region (the
// reference's own GPU build) or in a caching allocator (PyTorch's) hands all
// of its memory to that runtime: a cudaMalloc from this library would bypass
// it and can fail once the pool holds the device's memory, and cudaFree waits
// for the whole device, stalling the caller's asynchronous queues.  Those
// callers pass the coordinates they already hold on the device and get the
// smallest triangle angle of src/rem_test.f90:77-118 back, computed by a
// variant of the context's min-angle kernel whose per-block partial minima go
// to a fixed array compiled into this library instead of context memory.
//
// The array g_min_angle_scratch below is that scratch (65,792 bytes):
//   bytes   0..3    completion ticket (unsigned int)
//   bytes   8..15   the result (double)
//   bytes 256..     one partial minimum per block, overwritten by every call
// Before each launch the call clears the ticket and sets the result to a NaN
// (two cudaMemsetAsync on the caller's stream; they allocate nothing), and
// the last block of the launch writes the minimum there.  A result that is
// still NaN after the launch (the last block never ran) is an error, never a
// stale angle.  Every call shares the array: two calls in flight at the same
// time on one device (different streams or host threads) corrupt each
// other's ticket, partials and result.  Callers serialise them (one stream,
// or wait between calls).
//
// The array's device address is looked up once per CUDA context (a module
// loaded into a caller-made driver context has its own copy of the array),
// on the first call made while that context is current.  Each call ends with
// a cudaStreamSynchronize and a copy into host memory, so it cannot be made
// while its stream is being captured into a graph.

#include <cuda.h>
#include <cuda_runtime.h>

#include <math.h>

#include <mutex>

#include "../../include/geoflac_gb300.h"
#include "gf_index.h"

#define GF_MA_THREADS 256
#define GF_MA_MAX_BLOCKS 8192 // at most 8192 * 256 = 2,097,152 elements
#define GF_MA_HEADER 32       // doubles ahead of the partials (256 bytes)
#define GF_MA_MAX_SLOTS 64     // contexts whose scratch address is cached

static __device__ __align__(256) double g_min_angle_scratch[GF_MA_HEADER + GF_MA_MAX_BLOCKS];

namespace {

__device__ __forceinline__ double warp_fmin(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// One element per thread; the block's minimum goes to scratch, and the last
// block to finish folds the partials into the result and clears the ticket.
__global__ void __launch_bounds__(GF_MA_THREADS) k_min_angle_scratch(const double *__restrict__ cord, GfDims d,
                                                                     double *scratch) {
    unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch);
    double *partial = scratch + GF_MA_HEADER;
    __shared__ double wmin[GF_MA_THREADS / 32];
    __shared__ int last;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double amin = 180.0;
    if (e < d.E) {
        int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
        long long n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
        // quad nodes (j,i), (j+1,i), (j,i+1), (j+1,i+1)
        const double x[4] = {cord[n1], cord[n1 + 1], cord[n3], cord[n3 + 1]};
        const double y[4] = {cord[d.N + n1], cord[d.N + n1 + 1], cord[d.N + n3], cord[d.N + n3 + 1]};
        const double raddeg = 180.0 / 3.14159265358979323846;
        const int tv[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 1, 3}, {0, 3, 2}};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int v[4] = {tv[t][0], tv[t][1], tv[t][2], tv[t][0]};
            double ang[3];
#pragma unroll
            for (int k = 1; k <= 2; ++k) {
                double xa = x[v[k + 1]] - x[v[k]], ya = y[v[k + 1]] - y[v[k]];
                double xxal = sqrt(xa * xa + ya * ya);
                double xb = x[v[k - 1]] - x[v[k]], yb = y[v[k - 1]] - y[v[k]];
                double xxbl = sqrt(xb * xb + yb * yb);
                ang[k] = raddeg * acos((xa * xb + ya * yb) / (xxal * xxbl));
            }
            ang[0] = 180.0 - ang[1] - ang[2];
            amin = fmin(amin, fmin(ang[0], fmin(ang[1], ang[2])));
        }
    }
    amin = warp_fmin(amin);
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = amin;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = wmin[0];
        for (int w = 1; w < GF_MA_THREADS / 32; ++w) b = fmin(b, wmin[w]);
        partial[blockIdx.x] = fmax(b, 0.0);
        __threadfence();
        last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double m = 180.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += GF_MA_THREADS) m = fmin(m, __ldcg(&partial[b]));
    m = warp_fmin(m);
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        m = wmin[0];
        for (int w = 1; w < GF_MA_THREADS / 32; ++w) m = fmin(m, wmin[w]);
        scratch[1] = m;
        *ticket = 0u;
    }
}

std::mutex g_setup_mu;
struct ScratchSlot {
    CUcontext ctx;
    int dev;
    double *ptr;
};
ScratchSlot g_slots[GF_MA_MAX_SLOTS] = {};
int g_nslots = 0;
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
bool g_ctx_fn_looked_up = false;

// Current driver context (nullptr when the driver entry point is unavailable:
// the cache is then keyed by the device alone).  Caller holds g_setup_mu.
CUcontext current_context() {
    if (!g_ctx_fn_looked_up) {
        g_ctx_fn_looked_up = true;
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current && g_ctx_get_current(&c) != CUDA_SUCCESS) c = nullptr;
    return c;
}

// Device address of the scratch array in the current context (looked up
// once per context with cudaGetSymbolAddress).
int scratch_of_current_context(double **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    CUcontext ctx = current_context();
    for (int k = 0; k < g_nslots; ++k)
        if (g_slots[k].ctx == ctx && g_slots[k].dev == dev) {
            *out = g_slots[k].ptr;
            return GF_OK;
        }
    if (g_nslots == GF_MA_MAX_SLOTS) return GF_ERR_LIMIT;
    double *ptr = nullptr;
    if (cudaGetSymbolAddress((void **)&ptr, g_min_angle_scratch) != cudaSuccess || !ptr) return GF_ERR_CUDA;
    // the lookup may have made the runtime's primary context current (no
    // context was current before it): key the address on the context now set
    ctx = current_context();
    g_slots[g_nslots++] = ScratchSlot{ctx, dev, ptr};
    *out = ptr;
    return GF_OK;
}

} // namespace

extern "C" int gf_min_angle_noalloc(const double *d_cord, int nx, int nz, void *stream, double *min_angle) {
    if (!d_cord || !min_angle || nx < 2 || nz < 2) return GF_ERR_ARG;
    long long E = (long long)(nx - 1) * (nz - 1);
    long long blocks = (E + GF_MA_THREADS - 1) / GF_MA_THREADS;
    if (blocks > GF_MA_MAX_BLOCKS) return GF_ERR_LIMIT;
    double *scratch = nullptr;
    int rc = scratch_of_current_context(&scratch);
    if (rc != GF_OK) return rc;
    GfDims d{nx, nz, 0, (long long)nx * nz, E};
    cudaStream_t s = (cudaStream_t)stream;
    // ticket = 0 and result = NaN (all bits set) before the launch, so that
    // neither an earlier aborted launch nor the previous call's result leaks
    if (cudaMemsetAsync(scratch, 0, sizeof(double), s) != cudaSuccess) return GF_ERR_CUDA;
    if (cudaMemsetAsync(scratch + 1, 0xff, sizeof(double), s) != cudaSuccess) return GF_ERR_CUDA;
    k_min_angle_scratch<<<(unsigned)blocks, GF_MA_THREADS, 0, s>>>(d_cord, d, scratch);
    if (cudaGetLastError() != cudaSuccess) return GF_ERR_CUDA;
    double a = 0.0;
    if (cudaMemcpyAsync(&a, scratch + 1, sizeof a, cudaMemcpyDeviceToHost, s) != cudaSuccess) return GF_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return GF_ERR_CUDA;
    if (isnan(a)) return GF_ERR_CUDA; // the launch ended before its last block folded the partials
    *min_angle = a;
    return GF_OK;
}
