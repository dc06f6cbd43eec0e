// Ensemble driver: hundreds of independent models of uneven size advanced
// by one persistent kernel per step.
//
// Each member is an ordinary mixed-precision context; a packed member table
// (device pointers, dimensions, constants) and per-kind tile tables (element,
// node, 2x node, marker and max(element, node) items) describe the ensemble.
// A tile is `threads * items_per_thread` consecutive items of ONE member, so
// a warp never mixes members and the per-member reductions stay warp-local.
// Every phase of the step (fl_therm, change_phase, fl_rheol, fl_node,
// fl_move, rmasses, dt_mass) walks all tiles of all members, each CTA a
// contiguous run of tiles, and the phases are separated by a grid barrier:
// the ensemble shares the step's phase order, not its dt or its size.  The
// per-item work is the same device code as the single-model kernels; a
// member's result does not depend on the other members, the tile depth or
// the residency (FP32 contraction may differ from the separately compiled
// single-model kernels at rounding level).
//
// The grid is co-resident (cooperative launch), sized from the occupancy of
// the chosen CTA shape; the barrier gives up after a bounded wait and raises
// an error flag instead of hanging.

// Items written in one phase are read in the next within the same kernel:
// no pointer here may be treated as read-only for the kernel's lifetime.
#define __restrict__
// 32-bit indices, as in the mixed instantiation (members are mixed contexts)
#define GF_IDX int
#include "gf_kernels_impl.cuh"
#include "gf_member.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

enum { K_E = 0, K_N, K_N2, K_M, K_EN, K_KINDS };

struct BatchMember {
    const DevParams *P;
    DevClock *C;
    DevArrays A;
    GfDims d;
    int idt_scale, movegrid, nmarkers, pad;
    double z0, rzbo; // undeformed surface and depth of the regular start-up mesh
};

struct BatchSync {
    unsigned count, gen;
    int err, pad;
};

struct BatchArgs {
    const BatchMember *members;
    int nmembers;
    const int2 *tile[K_KINDS]; // (member, first item) per tile
    int ntile[K_KINDS];
    BatchSync *sync;
    unsigned sig;
    int ipt;   // items per thread
    int merge; // every member allows the thermal sweeps beside fl_rheol / fl_node
};

// Bounded grid barrier (gf_grid_barrier: arrivals, generation counter,
// error flag -- BatchSync has that layout).  Returns false if any CTA gave
// up waiting; the kernel then returns at once.
__device__ bool grid_sync(BatchSync *s) { return gfk::gf_grid_barrier(reinterpret_cast<unsigned *>(s), 1LL << 24); }

// Check of the bounded barrier: CTA `absent` of a two-CTA co-resident launch
// never arrives; the other waits at most `limit` polls and leaves with the
// error flag set (absent = -1: both arrive and pass).
__global__ void k_barrier_probe(unsigned *bar, int absent, long long limit, int *passed) {
    if ((int)blockIdx.x == absent) return;
    bool ok = gfk::gf_grid_barrier(bar, limit);
    if (threadIdx.x == 0) passed[blockIdx.x] = ok ? 1 : 0;
}

// All tiles of one item kind, a contiguous run per CTA; the member record is
// staged in shared memory whenever the run crosses into the next member.
template <class F> __device__ void for_tiles(const BatchArgs &a, int kind, BatchMember &sm, int &cur, F &&f) {
    const int nt = a.ntile[kind];
    const int per = (nt + gridDim.x - 1) / gridDim.x;
    const int t0 = blockIdx.x * per, t1 = min(nt, t0 + per);
    for (int t = t0; t < t1; ++t) {
        const int2 tl = a.tile[kind][t];
        if (tl.x != cur) {
            __syncthreads();
            const int *src = reinterpret_cast<const int *>(a.members + tl.x);
            int *dst = reinterpret_cast<int *>(&sm);
            for (int w = threadIdx.x; w < (int)(sizeof(BatchMember) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
            __syncthreads();
            cur = tl.x;
        }
        for (int r = 0; r < a.ipt; ++r) f(sm, (long long)tl.y + (long long)r * blockDim.x + threadIdx.x);
    }
}

// Per-member scalar work, one thread per member.
template <class F> __device__ void for_members(const BatchArgs &a, F &&f) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < a.nmembers; m += gridDim.x * blockDim.x) f(a.members[m]);
}

// rmasses, dt_mass and par.f90's time advance after fl_move (shared by both
// schedules of k_batch_step)
template <class R> __device__ __forceinline__ void mech_tail(const BatchArgs &a, BatchMember &sm, int &cur, unsigned sig) {
    using namespace gfk;
#define GF_SYNC()                                                                                                      \
    do {                                                                                                               \
        if (!grid_sync(a.sync)) return;                                                                                \
    } while (0)
    const int dtm = (sig & 32u) ? 1 : 0;
    if (sig & 16u) { // rmasses
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_elem_dens<R>(m.P, m.C, m.A, m.d, i);
        });
        GF_SYNC();
        for_members(a, [&](const BatchMember &m) { b_k_frac_fix<R>(m.P, m.C, m.A, m.d); });
        GF_SYNC();
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_node_gather_tri<R>((const R *)m.A.e_tri, m.A.rmass, m.d, i);
        });
        GF_SYNC();
    }
    if (dtm) { // dt_mass
        for_members(a, [&](const BatchMember &m) { b_k_dt_reset(m.C); });
        GF_SYNC();
        for_tiles(a, K_EN, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_dt_reduce<R>(m.P, m.C, m.A, m.d, i);
        });
        GF_SYNC();
        for_members(a, [&](const BatchMember &m) { b_k_dt_scalars(m.P, m.C); });
        GF_SYNC();
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.idt_scale != 0) b_k_elem_am3<R>(m.P, m.C, m.A, m.d, i);
        });
        GF_SYNC();
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.idt_scale != 0)
                b_k_node_gather_tri<R>((const R *)m.A.e_tri, m.A.amass, m.d, i);
            else if (i < m.d.N)
                m.A.amass[i] = m.A.rmass[i];
        });
        GF_SYNC();
    }
    // par.f90:86: time advanced inside fl_move on steps without dt_mass
    for_members(a, [&](const BatchMember &m) {
        if (!m.movegrid || dtm) m.C->time = m.C->time + m.C->dt;
    });
#undef GF_SYNC
}

// One FLAC step (flac.f90:5-91, mixed precision) of every member.
// MINB: resident CTAs per SM the register allocation is sized for (the whole
// step is one kernel, so its register count is that of its heaviest phase;
// a cap trades spills in fl_rheol for occupancy in every phase)
template <int THREADS, int MINB> __global__ void __launch_bounds__(THREADS, MINB) k_batch_step(BatchArgs a) {
    using namespace gfk;
    typedef float R;
    __shared__ BatchMember sm;
    int cur = -1;
    const unsigned sig = a.sig;
#define GF_SYNC()                                                                                                      \
    do {                                                                                                               \
        if (!grid_sync(a.sync)) return;                                                                                \
    } while (0)
    // fl_therm
    for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
        b_k_therm_prep32(m.P, m.A, m.d, (float *)m.A.t_coef, i);
    });
    GF_SYNC();
    // Steps whose fl_rheol / fl_node read nothing the thermal update writes
    // (no viscosity update, no change_phase; every member without thermal
    // stress, Winkler foundation or flux bottom condition): the sweeps share
    // phases with fl_rheol, fl_node and the coordinate update, which saves
    // three grid barriers and lets CTAs go on to the next kind of tile.
    if (a.merge && (sig & 1u) && !(sig & 2u) && !(sig & 4u)) {
        const int avg = (sig & (8u << 8)) ? 2 : ((sig & (4u << 8)) ? 1 : 0);
        const int dtm = (sig & 32u) ? 1 : 0;
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_therm_sweep32(m.P, m.C, m.A, m.d, (const float *)m.A.t_coef, (float *)m.A.t_delta0, m.A.t_delta1,
                              0, i);
        });
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) { b_k_rheol<R>(m.P, m.C, m.A, m.d, 0, 0, i); });
        GF_SYNC();
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_therm_sweep32(m.P, m.C, m.A, m.d, (const float *)m.A.t_coef, (float *)m.A.t_delta0, m.A.t_delta1,
                              1, i);
        });
        if (avg > 0)
            for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
                b_k_rheol_avg<R>(m.C, m.A, m.d, avg == 2 ? 1 : 0, i);
            });
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) { b_k_node<R>(m.P, m.C, m.A, m.d, i); });
        GF_SYNC();
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_therm_apply32(m.P, m.A, m.d, m.A.t_delta1, i);
        });
        if (avg == 2) for_members(a, [&](const BatchMember &m) { b_k_rheol_clock(m.C, 1); });
        for_tiles(a, K_N2, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.movegrid) b_k_move_cord(m.C, m.A, m.d, i);
        });
        GF_SYNC();
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.movegrid) b_k_move_elem<R>(m.C, m.A, m.d, dtm ? 0 : 1, i);
        });
        GF_SYNC();
        mech_tail<R>(a, sm, cur, sig);
        return;
    }
    for (int sweep = 0; sweep < 2; ++sweep) {
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_therm_sweep32(m.P, m.C, m.A, m.d, (const float *)m.A.t_coef, (float *)m.A.t_delta0, m.A.t_delta1,
                              sweep, i);
        });
        GF_SYNC();
    }
    for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) {
        b_k_therm_apply32(m.P, m.A, m.d, m.A.t_delta1, i);
    });
    GF_SYNC();
    if (sig & 1u) {
        if (sig & 2u) { // change_phase
            for_tiles(a, K_M, sm, cur, [&](const BatchMember &m, long long i) {
                b_k_phase_markers32(m.P, m.A, m.d, m.nmarkers, i);
            });
            GF_SYNC();
            for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
                b_k_phase_recount<R>(m.P, m.C, m.A, m.d, 0, i);
            });
            GF_SYNC();
        }
        const int upd = (sig & 4u) ? 1 : 0;
        const int avg = (sig & (8u << 8)) ? 2 : ((sig & (4u << 8)) ? 1 : 0);
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
            b_k_rheol<R>(m.P, m.C, m.A, m.d, upd, 0, i);
        });
        GF_SYNC();
        if (avg > 0) {
            for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
                b_k_rheol_avg<R>(m.C, m.A, m.d, avg == 2 ? 1 : 0, i);
            });
            GF_SYNC();
            if (avg == 2) {
                for_members(a, [&](const BatchMember &m) { b_k_rheol_clock(m.C, 1); });
                GF_SYNC();
            }
        }
        for_tiles(a, K_N, sm, cur, [&](const BatchMember &m, long long i) { b_k_node<R>(m.P, m.C, m.A, m.d, i); });
        GF_SYNC();
        const int dtm = (sig & 32u) ? 1 : 0;
        for_tiles(a, K_N2, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.movegrid) b_k_move_cord(m.C, m.A, m.d, i);
        });
        GF_SYNC();
        for_tiles(a, K_E, sm, cur, [&](const BatchMember &m, long long i) {
            if (m.movegrid) b_k_move_elem<R>(m.C, m.A, m.d, dtm ? 0 : 1, i);
        });
        GF_SYNC();
        mech_tail<R>(a, sm, cur, sig);
    } else {
        for_members(a, [&](const BatchMember &m) { m.C->time = m.C->time + m.C->dt; });
    }
#undef GF_SYNC
}

// ---------------------------------------------------------------- surrogate I/O
// Fields of every member resampled to an H x W grid (channels last, FP32):
// 0 vx, 1 vz, 2 sxx, 3 szz, 4 sxz (total stress, mean of the 4 triangles),
// 5 plastic strain, 6 temperature, 7 fraction of phase `phase_id`,
// 8 vertical displacement from the regular start-up mesh.  Bilinear in the
// node / element-centre index space of each member (the members' domains
// keep the grid's aspect).
constexpr int SAMPLE_CH = 9;

struct GridArgs {
    const BatchMember *members;
    int n, H, W, phase_id;
    float *grid;       // [n][H][W][SAMPLE_CH]
    const float *pred; // injection source, same layout
};

__device__ __forceinline__ void lerp_index(float f, int n, int &i0, float &w) {
    // f in [0, n-1] -> cell i0 in [0, n-2], weight of i0 + 1
    if (n < 2) {
        i0 = 0;
        w = 0.0f;
        return;
    }
    f = fminf(fmaxf(f, 0.0f), (float)(n - 1));
    i0 = min((int)f, n - 2);
    w = f - (float)i0;
}

__device__ double elem_value(const BatchMember &m, long long e, int ch, int phase_id) {
    const float *st = (const float *)m.A.stress0;
    const GfDims &d = m.d;
    const double pr = m.A.p_ref[e];
    switch (ch) {
    case 2: case 3: {
        int c = ch - 2;
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += (double)st[gf_s(d, e, c, k)];
        return 0.25 * s - pr;
    }
    case 4: {
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += (double)st[gf_s(d, e, 2, k)];
        return 0.25 * s;
    }
    case 5: return (double)((const float *)m.A.aps)[e];
    default: return m.A.phase_ratio[gf_pr(d, e, phase_id - 1)];
    }
}

__device__ double node_value(const BatchMember &m, long long n, int j, int ch) {
    const GfDims &d = m.d;
    switch (ch) {
    case 0: return m.A.vel[n];
    case 1: return m.A.vel[d.N + n];
    case 6: return m.A.temp[n];
    default: return m.A.cord[d.N + n] - (m.z0 + m.rzbo * (double)j / (double)(d.nz - 1));
    }
}

__global__ void k_sample(GridArgs g) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)g.n * g.H * g.W;
    if (t >= total) return;
    const int gx = (int)(t % g.W), gy = (int)((t / g.W) % g.H), mi = (int)(t / ((long long)g.W * g.H));
    const BatchMember &m = g.members[mi];
    const int nx = m.d.nx, nz = m.d.nz;
    float *out = g.grid + t * SAMPLE_CH;
    // nodes
    int i0, j0;
    float wx, wy;
    lerp_index((gx + 0.5f) * (nx - 1) / g.W, nx, i0, wx);
    lerp_index((gy + 0.5f) * (nz - 1) / g.H, nz, j0, wy);
    const int nch[4] = {0, 1, 6, 8};
    for (int q = 0; q < 4; ++q) {
        int ch = nch[q];
        double a = node_value(m, gf_node(m.d, j0, i0), j0, ch), b = node_value(m, gf_node(m.d, j0, i0 + 1), j0, ch);
        double c = node_value(m, gf_node(m.d, j0 + 1, i0), j0 + 1, ch),
               dd = node_value(m, gf_node(m.d, j0 + 1, i0 + 1), j0 + 1, ch);
        out[ch] = (float)((1 - wy) * ((1 - wx) * a + wx * b) + wy * ((1 - wx) * c + wx * dd));
    }
    // elements (centres)
    lerp_index((gx + 0.5f) * (nx - 1) / g.W - 0.5f, nx - 1, i0, wx);
    lerp_index((gy + 0.5f) * (nz - 1) / g.H - 0.5f, nz - 1, j0, wy);
    const int ech[5] = {2, 3, 4, 5, 7};
    const int i1 = min(i0 + 1, nx - 2), j1 = min(j0 + 1, nz - 2);
    for (int q = 0; q < 5; ++q) {
        int ch = ech[q];
        double a = elem_value(m, gf_elem(m.d, j0, i0), ch, g.phase_id), b = elem_value(m, gf_elem(m.d, j0, i1), ch, g.phase_id);
        double c = elem_value(m, gf_elem(m.d, j1, i0), ch, g.phase_id), dd = elem_value(m, gf_elem(m.d, j1, i1), ch, g.phase_id);
        out[ch] = (float)((1 - wy) * ((1 - wx) * a + wx * b) + wy * ((1 - wx) * c + wx * dd));
    }
}

// bilinear read of one channel of member mi's grid at grid coordinates (fy, fx)
__device__ float grid_at(const GridArgs &g, int mi, float fy, float fx, int ch) {
    int i0, j0;
    float wx, wy;
    lerp_index(fx, g.W, i0, wx);
    lerp_index(fy, g.H, j0, wy);
    const float *G = g.pred + (long long)mi * g.H * g.W * SAMPLE_CH;
    auto at = [&](int j, int i) { return G[((long long)j * g.W + i) * SAMPLE_CH + ch]; };
    return (1 - wy) * ((1 - wx) * at(j0, i0) + wx * at(j0, i0 + 1)) + wy * ((1 - wx) * at(j0 + 1, i0) + wx * at(j0 + 1, i0 + 1));
}

// grid -> member nodes: velocity, temperature, vertical position
__global__ void k_inject_nodes(GridArgs g, const int2 *tiles, int ntile, int ipt) {
    for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
        const int2 tl = tiles[t];
        const BatchMember &m = g.members[tl.x];
        for (int r = 0; r < ipt; ++r) {
            long long n = (long long)tl.y + (long long)r * blockDim.x + threadIdx.x;
            if (n >= m.d.N) continue;
            const int j = (int)(n % m.d.nz), i = (int)(n / m.d.nz);
            const float fx = (float)i * g.W / (m.d.nx - 1) - 0.5f, fy = (float)j * g.H / (m.d.nz - 1) - 0.5f;
            const double vx = grid_at(g, tl.x, fy, fx, 0), vz = grid_at(g, tl.x, fy, fx, 1);
            const double z = m.z0 + m.rzbo * (double)j / (double)(m.d.nz - 1) + (double)grid_at(g, tl.x, fy, fx, 8);
            m.A.vel[n] = vx;
            m.A.vel[m.d.N + n] = vz;
            const double tn = grid_at(g, tl.x, fy, fx, 6);
            m.A.temp[n] = tn;
            m.A.temp_hi[n] = (float)tn;
            m.A.temp_lo[n] = (float)(tn - (double)(float)tn);
            m.A.cord[m.d.N + n] = z;
            const float hx = (float)vx, hz = (float)vz, hc = (float)z;
            m.A.vel_hi[n] = hx;
            m.A.vel_lo[n] = (float)(vx - (double)hx);
            m.A.vel_hi[m.d.N + n] = hz;
            m.A.vel_lo[m.d.N + n] = (float)(vz - (double)hz);
            m.A.cord_hi[m.d.N + n] = hc;
            m.A.cord_lo[m.d.N + n] = (float)(z - (double)hc);
        }
    }
}

// grid -> member elements: stresses (the out-of-plane stress keeps its
// deviation from the in-plane mean), plastic strain; areas of the moved mesh
__global__ void k_inject_elems(GridArgs g, const int2 *tiles, int ntile, int ipt, DevClock *err) {
    for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
        const int2 tl = tiles[t];
        const BatchMember &m = g.members[tl.x];
        const GfDims &d = m.d;
        for (int r = 0; r < ipt; ++r) {
            long long e = (long long)tl.y + (long long)r * blockDim.x + threadIdx.x;
            if (e >= d.E) continue;
            const int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
            const float fx = (i + 0.5f) * g.W / (d.nx - 1) - 0.5f, fy = (j + 0.5f) * g.H / (d.nz - 1) - 0.5f;
            float *st = (float *)m.A.stress0;
            const double pr = m.A.p_ref[e];
            const double sxx = grid_at(g, tl.x, fy, fx, 2), szz = grid_at(g, tl.x, fy, fx, 3),
                         sxz = grid_at(g, tl.x, fy, fx, 4);
            for (int k = 0; k < 4; ++k) {
                double oxx = (double)st[gf_s(d, e, 0, k)] - pr, ozz = (double)st[gf_s(d, e, 1, k)] - pr;
                double oyy = (double)st[gf_s(d, e, 3, k)] - pr;
                double nyy = oyy + 0.5 * ((sxx - oxx) + (szz - ozz));
                st[gf_s(d, e, 0, k)] = (float)(sxx + pr);
                st[gf_s(d, e, 1, k)] = (float)(szz + pr);
                st[gf_s(d, e, 2, k)] = (float)sxz;
                st[gf_s(d, e, 3, k)] = (float)(nyy + pr);
            }
            ((float *)m.A.aps)[e] = fmaxf(0.0f, grid_at(g, tl.x, fy, fx, 5));
            gfk::Quad q;
            gfk::load_quad(m.A.cord, d, j, i, q);
            const double *x = q.x, *y = q.y;
            double det[4] = {((x[1] * y[2] - y[1] * x[2]) - (x[0] * y[2] - y[0] * x[2])) + (x[0] * y[1] - y[0] * x[1]),
                             ((x[1] * y[3] - y[1] * x[3]) - (x[2] * y[3] - y[2] * x[3])) + (x[2] * y[1] - y[2] * x[1]),
                             ((x[1] * y[3] - y[1] * x[3]) - (x[0] * y[3] - y[0] * x[3])) + (x[0] * y[1] - y[0] * x[1]),
                             ((x[3] * y[2] - y[3] * x[2]) - (x[0] * y[2] - y[0] * x[2])) + (x[0] * y[3] - y[0] * x[3])};
            for (int k = 0; k < 4; ++k) {
                ((float *)m.A.area)[gf_ek(d, e, k)] = (float)(1.0 / det[k]);
                if (det[k] <= 0.0) gfk::set_status(m.C, 41, (int)e);
            }
        }
    }
    (void)err;
}

// Force imbalance at the free nodes (fl_node.f90 without damping): per member
// sum |F| and sum (|gravity| + sum over triangles |stress-divergence term|).
__global__ void k_force_residual(const BatchMember *members, const int2 *tiles, int ntile, int ipt, double *acc,
                                 double g_acc) {
    for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
        const int2 tl = tiles[t];
        const BatchMember &m = members[tl.x];
        const GfDims &d = m.d;
        double sf = 0.0, ss = 0.0;
        for (int r = 0; r < ipt; ++r) {
            long long n = (long long)tl.y + (long long)r * blockDim.x + threadIdx.x;
            if (n >= d.N) continue;
            const int j = (int)(n % d.nz), i = (int)(n / d.nz);
            const int c0 = m.A.ncod[n], c1 = m.A.ncod[d.N + n];
            const int kk[4][3] = {{1, 2, 3}, {0, 1, 2}, {0, 1, 3}, {0, 2, 3}};
            const int mm[4][3] = {{2, 2, 1}, {1, 1, 1}, {2, 0, 2}, {0, 0, 0}};
            const float *st = (const float *)m.A.stress0;
            const float *area = (const float *)m.A.area;
            double fx = 0.0, fy = 0.0, mag = 0.0;
            for (int qd = 0; qd < 4; ++qd) {
                int je = j + (qd < 2 ? -1 : 0), ie = i + ((qd & 1) ? 0 : -1);
                if (je < 0 || ie < 0 || je > d.nz - 2 || ie > d.nx - 2) continue;
                long long e = gf_elem(d, je, ie);
                gfk::Quad q;
                gfk::load_quad(m.A.cord, d, je, ie, q);
                double ar[4];
                for (int k = 0; k < 4; ++k) ar[k] = (double)area[gf_ek(d, e, k)];
                double dx[3][4], dz[3][4];
                gfk::shape_derivs<double>(q, ar, dx, dz);
                const double pe = m.A.p_ref[e];
                for (int k = 0; k < 3; ++k) {
                    int tt = kk[qd][k], mq = mm[qd][k];
                    double factor = 0.25 / ar[tt];
                    double sxx = (double)st[gf_s(d, e, 0, tt)] - pe, szz = (double)st[gf_s(d, e, 1, tt)] - pe,
                           sxz = (double)st[gf_s(d, e, 2, tt)];
                    double tx = factor * (sxx * dx[mq][tt] + sxz * dz[mq][tt]);
                    double ty = factor * (sxz * dx[mq][tt] + szz * dz[mq][tt]);
                    fx -= tx;
                    fy -= ty;
                    mag += sqrt(tx * tx + ty * ty);
                }
            }
            const double grav = m.A.rmass[n] * g_acc;
            fy -= grav;
            if (c0 == 1) fx = 0.0; // fixed velocity components carry reactions
            if (c1 == 1) fy = 0.0;
            sf += sqrt(fx * fx + fy * fy);
            ss += mag + fabs(grav);
        }
        sf = gfk::warp_sum(sf);
        ss = gfk::warp_sum(ss);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&acc[2 * tl.x], sf);
            atomicAdd(&acc[2 * tl.x + 1], ss);
        }
    }
}

typedef void (*BatchKernel)(BatchArgs);

// the kernel for a CTA width and residency: register-capped builds where
// compiled, else the uncapped one
BatchKernel kernel_for(int threads, int cps) {
    switch (threads) {
    case 128: return k_batch_step<128, 1>;
    case 256:
        if (cps == 2) return k_batch_step<256, 2>;
        if (cps >= 3) return k_batch_step<256, 3>;
        return k_batch_step<256, 1>;
    case 512:
        if (cps >= 2) return k_batch_step<512, 2>;
        return k_batch_step<512, 1>;
    default: return nullptr;
    }
}

} // namespace

struct gf_batch {
    std::vector<gf_ctx *> members;
    std::vector<GfMemberView> views;
    BatchMember *d_members = nullptr;
    int2 *d_tiles[K_KINDS] = {};
    int ntile[K_KINDS] = {};
    BatchSync *d_sync = nullptr;
    cudaStream_t s = nullptr;
    gf_batch_config cfg{256, 2, 1, 10};
    double g = 10.0; // gravity of the members (one value; checked at creation)
    int grid = 0;
    int merge = 0;
    long long elements = 0;
    struct Graph {
        std::vector<unsigned> sigs;
        cudaGraphExec_t exec;
    };
    std::vector<Graph> graphs;
    // device copy of the fields gf_batch_inject overwrites (restore point)
    void *backup = nullptr;
    std::vector<size_t> backup_off;
};

namespace {
// (device pointer, bytes) of every field of member v that injection writes
std::vector<std::pair<void *, size_t>> injected_fields(const GfMemberView &v) {
    const size_t N = (size_t)v.d.N, E = (size_t)v.d.E;
    return {{v.A.vel, 2 * N * sizeof(double)},    {v.A.temp, N * sizeof(double)},
            {v.A.cord, 2 * N * sizeof(double)},   {v.A.stress0, 16 * E * sizeof(float)},
            {v.A.aps, E * sizeof(float)},         {v.A.area, 4 * E * sizeof(float)},
            {v.A.cord_hi, 2 * N * sizeof(float)}, {v.A.cord_lo, 2 * N * sizeof(float)},
            {v.A.vel_hi, 2 * N * sizeof(float)},  {v.A.vel_lo, 2 * N * sizeof(float)},
            {v.A.temp_hi, N * sizeof(float)},     {v.A.temp_lo, N * sizeof(float)}};
}
} // namespace

namespace {

int batch_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GF_OK;
    std::fprintf(stderr, "geoflac_gb300: CUDA error in %s: %s\n", what, cudaGetErrorString(e));
    return GF_ERR_CUDA;
}
#define GB_CK(call)                                                                                                    \
    do {                                                                                                               \
        int _rc = batch_cuda((call), #call);                                                                           \
        if (_rc) return _rc;                                                                                           \
    } while (0)

void drop_graphs(gf_batch *b) {
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
}

long long kind_count(const GfMemberView &v, int kind) {
    switch (kind) {
    case K_E: return v.d.E;
    case K_N: return v.d.N;
    case K_N2: return 2 * v.d.N;
    case K_M: return v.nmarkers;
    default: return std::max(v.d.E, v.d.N);
    }
}

// tile tables and the co-resident grid for the current configuration
int build_tables(gf_batch *b) {
    const gf_batch_config &c = b->cfg;
    BatchKernel k = kernel_for(c.threads, c.ctas_per_sm);
    if (!k || c.items_per_thread < 1 || c.items_per_thread > 64 || c.ctas_per_sm < 1) return GF_ERR_ARG;
    int dev = 0, sms = 0, occ = 0;
    GB_CK(cudaGetDevice(&dev));
    GB_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, c.threads, 0));
    if (occ < 1) return GF_ERR_UNSUPPORTED;
    const int full_grid = sms * std::min(occ, c.ctas_per_sm);
    const long long tile = (long long)c.threads * c.items_per_thread;
    for (int kind = 0; kind < K_KINDS; ++kind) {
        std::vector<int2> t;
        for (size_t m = 0; m < b->views.size(); ++m) {
            long long n = kind_count(b->views[m], kind);
            for (long long s = 0; s < n; s += tile) {
                if (s > 0x7fffffff) return GF_ERR_ARG;
                t.push_back(make_int2((int)m, (int)s));
            }
        }
        if (b->d_tiles[kind]) cudaFree(b->d_tiles[kind]);
        b->d_tiles[kind] = nullptr;
        b->ntile[kind] = (int)t.size();
        if (!t.empty()) {
            GB_CK(cudaMalloc(&b->d_tiles[kind], t.size() * sizeof(int2)));
            GB_CK(cudaMemcpy(b->d_tiles[kind], t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice));
        }
    }
    // a small batch (e.g. a few members rerun after screening) runs on no
    // more CTAs than it has element or node tiles: its grid barriers then
    // involve few CTAs
    const int work = std::max(1, std::max(b->ntile[K_E], b->ntile[K_N]));
    b->grid = std::min(full_grid, work);
    drop_graphs(b);
    return GF_OK;
}

int upload_members(gf_batch *b) {
    std::vector<BatchMember> h(b->views.size());
    for (size_t m = 0; m < h.size(); ++m) {
        const GfMemberView &v = b->views[m];
        std::memset(&h[m], 0, sizeof(BatchMember));
        h[m].P = v.P;
        h[m].C = v.C;
        h[m].A = v.A;
        h[m].d = v.d;
        h[m].idt_scale = v.idt_scale;
        h[m].movegrid = v.movegrid;
        h[m].nmarkers = v.nmarkers;
        h[m].z0 = v.z0;
        h[m].rzbo = v.rzbo;
    }
    GB_CK(cudaMemcpy(b->d_members, h.data(), h.size() * sizeof(BatchMember), cudaMemcpyHostToDevice));
    return GF_OK;
}

BatchArgs args_of(const gf_batch *b, unsigned sig) {
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.members = b->d_members;
    a.nmembers = (int)b->members.size();
    for (int k = 0; k < K_KINDS; ++k) {
        a.tile[k] = b->d_tiles[k];
        a.ntile[k] = b->ntile[k];
    }
    a.sync = b->d_sync;
    a.sig = sig;
    a.ipt = b->cfg.items_per_thread;
    a.merge = b->merge;
    return a;
}

int launch_step(gf_batch *b, unsigned sig) {
    BatchArgs a = args_of(b, sig);
    cudaLaunchConfig_t lc;
    std::memset(&lc, 0, sizeof lc);
    lc.gridDim = dim3((unsigned)b->grid);
    lc.blockDim = dim3((unsigned)b->cfg.threads);
    lc.stream = b->s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    GB_CK(cudaLaunchKernelEx(&lc, kernel_for(b->cfg.threads, b->cfg.ctas_per_sm), a));
    return GF_OK;
}

// Signatures of the next n steps (all members share them).
std::vector<unsigned> next_sigs(gf_batch *b, int n, std::vector<int> &nl, std::vector<int> &ns) {
    // simulate the host bookkeeping of member 0 without touching it
    const GfMemberView &v = b->views[0];
    std::vector<unsigned> sigs;
    int nloop = v.nloop, nsrate = v.nsrate;
    for (int k = 0; k < n; ++k) {
        unsigned sig = 0;
        if (v.itherm != 2) {
            sig |= 1u;
            if (nloop % v.ifreq_rmasses == 0) sig |= 2u | 16u;
            if (nloop % v.ifreq_visc == 0) sig |= 4u;
            if (nsrate == v.ifreq_avgsr) sig |= 8u << 8;
            else if (nsrate == -1) sig |= 4u << 8;
            if (nloop % v.ifreq_imasses == 0) sig |= 32u;
            if (sig & (8u << 8)) nsrate = 0;
            nsrate = nsrate + 1;
        }
        nloop = nloop + 1;
        sigs.push_back(sig);
    }
    nl.assign(1, nloop);
    ns.assign(1, nsrate);
    return sigs;
}

int refresh_views(gf_batch *b) {
    b->merge = 1;
    for (size_t m = 0; m < b->members.size(); ++m) {
        int rc = gf_ctx_view(b->members[m], &b->views[m]);
        if (rc) return rc;
        const gf_params &p = *b->views[m].hp;
        if (p.istress_therm != 0 || p.nyhydro != 0 || p.itemp_bc == 2) b->merge = 0;
        // surface processes (diff_topo / resurface) are not part of the
        // ensemble step
        if (p.topo_kappa > 0.0) return GF_ERR_UNSUPPORTED;
    }
    return GF_OK;
}

int check_status(gf_batch *b) {
    GB_CK(cudaStreamSynchronize(b->s));
    BatchSync hs;
    GB_CK(cudaMemcpy(&hs, b->d_sync, sizeof hs, cudaMemcpyDeviceToHost));
    if (hs.err) return GF_ERR_TIMEOUT;
    int first = GF_OK;
    for (gf_ctx *c : b->members) {
        int st = gf_ctx_take_status(c);
        if (st && !first) first = st;
    }
    return first;
}

} // namespace

extern "C" {

int gf_batch_create(gf_batch **out, gf_ctx **members, int n) {
    if (!out || !members || n <= 0) return GF_ERR_ARG;
    *out = nullptr;
    gf_batch *b = new (std::nothrow) gf_batch;
    if (!b) return GF_ERR_NOMEM;
    b->members.assign(members, members + n);
    b->views.resize(n);
    int rc = refresh_views(b);
    for (int m = 0; m < n && !rc; ++m) {
        const GfMemberView &v = b->views[m], &v0 = b->views[0];
        if (v.mode != GF_MODE_MIXED) rc = GF_ERR_UNSUPPORTED;
        else if (v.nloop != v0.nloop || v.nsrate != v0.nsrate || v.itherm != v0.itherm ||
                 v.ifreq_rmasses != v0.ifreq_rmasses || v.ifreq_visc != v0.ifreq_visc ||
                 v.ifreq_imasses != v0.ifreq_imasses || v.ifreq_avgsr != v0.ifreq_avgsr)
            rc = GF_ERR_ARG; // the members must share the step schedule
        b->elements += v.d.E;
        if (v.g != b->views[0].g) rc = GF_ERR_ARG;
    }
    if (!rc) b->g = b->views[0].g;
    if (!rc) rc = batch_cuda(cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking), "stream");
    if (!rc) rc = batch_cuda(cudaMalloc(&b->d_members, sizeof(BatchMember) * n), "members");
    if (!rc) rc = batch_cuda(cudaMalloc(&b->d_sync, sizeof(BatchSync)), "sync");
    if (!rc) rc = batch_cuda(cudaMemset(b->d_sync, 0, sizeof(BatchSync)), "sync");
    if (!rc) rc = upload_members(b);
    if (!rc) rc = build_tables(b);
    if (rc) {
        gf_batch_destroy(b);
        return rc;
    }
    *out = b;
    return GF_OK;
}

void gf_batch_destroy(gf_batch *b) {
    if (!b) return;
    if (b->s) cudaStreamSynchronize(b->s);
    drop_graphs(b);
    for (int k = 0; k < K_KINDS; ++k)
        if (b->d_tiles[k]) cudaFree(b->d_tiles[k]);
    if (b->d_members) cudaFree(b->d_members);
    if (b->d_sync) cudaFree(b->d_sync);
    if (b->backup) cudaFree(b->backup);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
}

int gf_batch_set_config(gf_batch *b, const gf_batch_config *cfg) {
    if (!b || !cfg) return GF_ERR_ARG;
    gf_batch_config old = b->cfg;
    b->cfg = *cfg;
    int rc = build_tables(b);
    if (rc) {
        b->cfg = old;
        build_tables(b);
    }
    return rc;
}

int gf_batch_get_config(gf_batch *b, gf_batch_config *cfg) {
    if (!b || !cfg) return GF_ERR_ARG;
    *cfg = b->cfg;
    return GF_OK;
}

long long gf_batch_elements(gf_batch *b) { return b ? b->elements : 0; }

int gf_batch_grid(gf_batch *b) { return b ? b->grid : 0; }

void *gf_batch_stream(gf_batch *b) { return b ? (void *)b->s : nullptr; }

int gf_batch_step(gf_batch *b, int nsteps) {
    if (!b || nsteps < 0) return GF_ERR_ARG;
    // members must be idle: their own streams may still hold work
    for (const GfMemberView &v : b->views) GB_CK(cudaStreamSynchronize(v.s));
    int rc = refresh_views(b);
    if (rc) return rc;
    int done = 0;
    const int G = b->cfg.graph_steps;
    while (done < nsteps) {
        int chunk = G > 0 ? std::min(G, nsteps - done) : 1;
        std::vector<int> nl, ns;
        std::vector<unsigned> sigs = next_sigs(b, chunk, nl, ns);
        if (G > 0) {
            cudaGraphExec_t exec = nullptr;
            for (auto &g : b->graphs)
                if (g.sigs == sigs) exec = g.exec;
            if (!exec) {
                cudaGraph_t graph;
                GB_CK(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
                int lrc = GF_OK;
                for (unsigned sig : sigs)
                    if (!lrc) lrc = launch_step(b, sig);
                cudaError_t e = cudaStreamEndCapture(b->s, &graph);
                if (lrc) return lrc;
                GB_CK(e);
                GB_CK(cudaGraphInstantiate(&exec, graph, 0));
                cudaGraphDestroy(graph);
                b->graphs.push_back(gf_batch::Graph{sigs, exec});
            }
            GB_CK(cudaGraphLaunch(exec, b->s));
        } else {
            rc = launch_step(b, sigs[0]);
            if (rc) return rc;
        }
        for (unsigned sig : sigs)
            for (gf_ctx *c : b->members) gf_ctx_advance(c, sig);
        rc = refresh_views(b);
        if (rc) return rc;
        done += chunk;
    }
    return check_status(b);
}

// Autotuner: every CTA shape (threads), tile depth (items per thread) and
// residency (CTAs per SM) that fits, each timed over `trial_steps` steps
// with CUDA events after one untimed step; the fastest is kept.  The trial
// steps advance the members like any other steps.
int gf_batch_tune(gf_batch *b, int trial_steps, gf_batch_config *best, double *best_ms) {
    if (!b || trial_steps < 1) return GF_ERR_ARG;
    gf_batch_config keep = b->cfg, win = b->cfg;
    double win_ms = 1e300;
    cudaEvent_t e0, e1;
    GB_CK(cudaEventCreate(&e0));
    GB_CK(cudaEventCreate(&e1));
    const int threads[3] = {128, 256, 512};
    const int ipts[4] = {1, 2, 4, 8};
    int rc = GF_OK;
    for (int t : threads) {
        for (int ipt : ipts)
            for (int cps = 1; cps <= 4; ++cps) {
                int occ = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_for(t, cps), t, 0);
                if (occ < cps) continue;
                gf_batch_config c{t, ipt, cps, 0}; // direct launches: no capture inside the timing
                b->cfg = c;
                if (build_tables(b)) continue;
                rc = gf_batch_step(b, 1);
                if (rc) break;
                cudaEventRecord(e0, b->s);
                rc = gf_batch_step(b, trial_steps);
                if (rc) break;
                cudaEventRecord(e1, b->s);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                double per = ms / trial_steps;
                if (per < win_ms) {
                    win_ms = per;
                    win = c;
                }
            }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    win.graph_steps = keep.graph_steps;
    b->cfg = rc ? keep : win;
    int rc2 = build_tables(b);
    if (rc) return rc;
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return rc2;
}

int gf_batch_sample(gf_batch *b, float *grid, int H, int W, int phase_id) {
    if (!b || !grid || H < 1 || W < 1 || phase_id < 1) return GF_ERR_ARG;
    GridArgs g{b->d_members, (int)b->members.size(), H, W, phase_id, grid, nullptr};
    long long n = (long long)g.n * H * W;
    k_sample<<<(unsigned)((n + 255) / 256), 256, 0, b->s>>>(g);
    GB_CK(cudaGetLastError());
    return GF_OK;
}

int gf_batch_inject(gf_batch *b, const float *grid, int H, int W) {
    if (!b || !grid || H < 2 || W < 2) return GF_ERR_ARG;
    for (gf_ctx *c : b->members) gf_ctx_invalidate_forces(c);
    GridArgs g{b->d_members, (int)b->members.size(), H, W, 1, nullptr, grid};
    const int T = b->cfg.threads, ipt = b->cfg.items_per_thread;
    if (b->ntile[K_N]) k_inject_nodes<<<b->ntile[K_N], T, 0, b->s>>>(g, b->d_tiles[K_N], b->ntile[K_N], ipt);
    if (b->ntile[K_E])
        k_inject_elems<<<b->ntile[K_E], T, 0, b->s>>>(g, b->d_tiles[K_E], b->ntile[K_E], ipt, nullptr);
    GB_CK(cudaGetLastError());
    return check_status(b);
}

int gf_batch_backup(gf_batch *b) {
    if (!b) return GF_ERR_ARG;
    for (const GfMemberView &v : b->views) GB_CK(cudaStreamSynchronize(v.s));
    if (!b->backup) {
        size_t total = 0;
        b->backup_off.clear();
        for (const GfMemberView &v : b->views) {
            b->backup_off.push_back(total);
            for (auto &f : injected_fields(v)) total += (f.second + 255) & ~(size_t)255;
        }
        GB_CK(cudaMalloc(&b->backup, total));
    }
    for (size_t m = 0; m < b->views.size(); ++m) {
        size_t off = b->backup_off[m];
        for (auto &f : injected_fields(b->views[m])) {
            GB_CK(cudaMemcpyAsync((char *)b->backup + off, f.first, f.second, cudaMemcpyDeviceToDevice, b->s));
            off += (f.second + 255) & ~(size_t)255;
        }
    }
    return GF_OK;
}

int gf_batch_restore(gf_batch *b, const int *members, int count) {
    if (!b || (count > 0 && !members)) return GF_ERR_ARG;
    if (!b->backup) return GF_ERR_ARG;
    for (int k = 0; k < count; ++k) {
        int m = members[k];
        if (m < 0 || m >= (int)b->views.size()) return GF_ERR_ARG;
        gf_ctx_invalidate_forces(b->members[m]);
        size_t off = b->backup_off[m];
        for (auto &f : injected_fields(b->views[m])) {
            GB_CK(cudaMemcpyAsync(f.first, (char *)b->backup + off, f.second, cudaMemcpyDeviceToDevice, b->s));
            off += (f.second + 255) & ~(size_t)255;
        }
    }
    GB_CK(cudaStreamSynchronize(b->s));
    return GF_OK;
}

int gf_batch_force_residual(gf_batch *b, double *residual) {
    if (!b || !residual) return GF_ERR_ARG;
    const int n = (int)b->members.size();
    double *acc = nullptr;
    GB_CK(cudaMalloc(&acc, sizeof(double) * 2 * n));
    cudaMemsetAsync(acc, 0, sizeof(double) * 2 * n, b->s);
    const double g_acc = b->g;
    if (b->ntile[K_N])
        k_force_residual<<<b->ntile[K_N], b->cfg.threads, 0, b->s>>>(b->d_members, b->d_tiles[K_N], b->ntile[K_N],
                                                                     b->cfg.items_per_thread, acc, g_acc);
    std::vector<double> h(2 * n);
    cudaError_t e = cudaMemcpyAsync(h.data(), acc, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, b->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->s);
    cudaFree(acc);
    GB_CK(e);
    for (int m = 0; m < n; ++m) residual[m] = h[2 * m] / (h[2 * m + 1] > 0 ? h[2 * m + 1] : 1.0);
    return GF_OK;
}

int gf_grid_barrier_selftest(int absent_cta, long long limit, int *passed) {
    if (!passed || absent_cta < -1 || absent_cta > 1 || limit < 1) return GF_ERR_ARG;
    unsigned *bar = nullptr;
    int *d_passed = nullptr;
    GB_CK(cudaMalloc(&bar, 4 * sizeof(unsigned)));
    cudaError_t e = cudaMalloc(&d_passed, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(bar, 0, 4 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(d_passed, 0xff, 2 * sizeof(int));
    unsigned err = 0;
    if (e == cudaSuccess) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(2);
        lc.blockDim = dim3(32);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        e = cudaLaunchKernelEx(&lc, k_barrier_probe, bar, absent_cta, limit, d_passed);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(passed, d_passed, 2 * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&err, bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(d_passed);
    GB_CK(e);
    return err ? GF_ERR_TIMEOUT : GF_OK;
}

} // extern "C"
