// Magma sub-model on the device (itype_melting = 1, FP64 contexts):
// melting after change_phase's phase recount (src/change_phase.f90:264-483),
// fl_therm's magma part (src/fl_therm.f90:56-391) and the magma blocks of
// diff_topo (src/fl_move.f90:213-302).  Included by gf_remesh.cu inside its
// kernel namespace (it shares check_inside, add_marker1 and
// count_phase_ratio1 with the surface processes); compiled without FMA
// contraction.
//
// The reference runs these loops serially (or with OpenMP atomics, whose
// order varies from run to run); this file reproduces the serial order:
//  * element-to-node sums become per-node gathers in serial element order;
//  * the melting loops cool an element's corners in place, so later
//    elements see earlier ones' cooling: the elements that can melt at all
//    (above their solidus at the start; temperatures only fall in these
//    loops) are listed in serial order and run by corner-dependency levels
//    (elements of one level share no corner), or walked by one thread when
//    the list is short;
//  * the weighted sums of the MOR melting zone are taken in serial order,
//    terms computed in parallel, each sum by its own warp;
//  * migration scatters many sources into many targets: each target walks
//    the ordered lists of the sources that can reach it (dike / cone sources
//    in its column window, MOR sources in the MOR cone), inserting the
//    reference's per-element clamp at its own serial position, one warp per
//    accumulated field;
//  * new markers are numbered in serial order by one thread walking the
//    list of elements that receive any.

constexpr int MG_SED1 = 1, MG_OCEAN1 = 3, MG_MANT1 = 4, MG_SCHIST = 5, MG_OCEAN2 = 7, MG_MANT2 = 8, MG_SERP = 9,
              MG_OCEANDRY = 10, MG_SED2 = 11, MG_ECLG = 13, MG_ARC1 = 14, MG_HYDMANT = 16, MG_METASED = 17;
constexpr double MG_W_BARRIER = 1.0e-4;
constexpr int MG_CB = 1024; // elements per block of the ordered compaction

// zone scalars (mg_s) and integer slots (mg_i)
enum { MS_VALID = 0, MS_XC, MS_ZC, MS_ZSURF, MS_H2, MS_TANL, MS_TANR, MS_TANM, MS_WSUM };
enum { MI_COUNT = 0, MI_FOUND, MI_IC, MI_JC, MI_IHWL, MI_IHWR, MI_IHW, MI_COUNT2, MI_MAXJ, MI_P0 };
// per-source terms (mg_src, GF_MG_SRC_W doubles per source)
enum { SR_E = 0, SR_FLAGS, SR_TERM_C, SR_II0, SR_II1, SR_TERM_M, SR_XMELT, SR_ZMELT, SR_J1, SR_I1, SR_TERM_R };
// Integer entries of the records are stored bit for bit (mg_pack / mg_int):
// a conversion from double would run on the FP64 pipe in every inner loop.
__device__ __forceinline__ double mg_pack(long long v) { return __longlong_as_double(v); }
__device__ __forceinline__ long long mg_int(double v) { return __double_as_longlong(v); }
// per-candidate record of the melting walk (mg_src): element, loop mask,
// corner nodes (j,i), (j,i+1), (j+1,i), (j+1,i+1), then the phase sum and
// solidus of each loop (mantle, sediments, basalt, flux)
enum { MR_E = 0, MR_MASK, MR_N00, MR_N01, MR_N10, MR_N11, MR_TPR };

// (j, i) of element e = i (nz-1) + j and of node n = i nz + j
__device__ __forceinline__ void mg_eji(const GfDims &d, long long e, int &j, int &i) {
    i = (int)(e / (d.nz - 1));
    j = (int)(e - (long long)i * (d.nz - 1));
}
__device__ __forceinline__ void mg_nji(const GfDims &d, long long n, int &j, int &i) {
    i = (int)(n / d.nz);
    j = (int)(n - (long long)i * d.nz);
}
__device__ __forceinline__ double mg_min(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double mg_max(double a, double b) { return b > a ? b : a; }
// ceiling() of a ratio that may be huge, held to +-2^29 (beyond every loop
// bound it feeds)
__device__ __forceinline__ int mg_ceil(double x) {
    double c = ceil(x);
    if (!(c < 536870912.0)) return 536870912;
    if (c < -536870912.0) return -536870912;
    return (int)c;
}
// phase_ratio(iph, e) with the reference's flat-memory reads for a phase id
// above nphase (the next element's entries; zero past the array)
__device__ __forceinline__ double mg_pr(const DevArrays &A, const GfDims &d, long long e, int iph1) {
    const long long off = (long long)(iph1 - 1) + (long long)d.nphase * e;
    if (off < 0 || off >= (long long)d.nphase * d.E) return 0.0;
    return A.phase_ratio[off];
}
__device__ __forceinline__ double mg_T(const DevArrays &A, const GfDims &d, int j, int i) {
    return A.temp[gf_node(d, j, i)];
}
__device__ __forceinline__ double mg_tmpr(const DevArrays &A, const GfDims &d, int j, int i) {
    return 0.25 * (mg_T(A, d, j, i) + mg_T(A, d, j, i + 1) + mg_T(A, d, j + 1, i) + mg_T(A, d, j + 1, i + 1));
}
__device__ __forceinline__ double mg_depth(const DevArrays &A, const GfDims &d, int j, int i) {
    const double *c = A.cord;
    double yy = 0.25 * (CY(c, d, j, i) + CY(c, d, j, i + 1) + CY(c, d, j + 1, i) + CY(c, d, j + 1, i + 1));
    return 0.5 * (CY(c, d, 0, i) + CY(c, d, 0, i + 1)) - yy;
}
__device__ __forceinline__ double mg_pmelt(const DevParams &P, int kph, double over, double span) {
    if (P.latent_heat_magma > 0.0) return mg_min(P.cp[kph - 1] * over / P.latent_heat_magma, 0.1);
    return mg_min(over / span * 0.1, 0.1);
}
__device__ __forceinline__ void mg_cool(DevArrays &A, const GfDims &d, int j, int i, double dt_melt) {
    double *T = A.temp;
    T[gf_node(d, j, i)] = T[gf_node(d, j, i)] - dt_melt;
    T[gf_node(d, j, i + 1)] = T[gf_node(d, j, i + 1)] - dt_melt;
    T[gf_node(d, j + 1, i)] = T[gf_node(d, j + 1, i)] - dt_melt;
    T[gf_node(d, j + 1, i + 1)] = T[gf_node(d, j + 1, i + 1)] - dt_melt;
}
// the four solidi (Katz 2003 hydrous mantle, Nichols 1994 sediments,
// Gutscher 2000 basalt / eclogite, Grove 2009 water-saturated mantle)
__device__ __forceinline__ double sol_mantle(const DevParams &P, double depth) {
    double press = fabs(3000.0 * P.g * depth * 1e-9);
    return -5.02 * (press * press) + 1.32e2 * press + 1.09e3;
}
__device__ __forceinline__ double sol_sed(double depth) {
    return mg_max(680 + 0.6e-3 * (depth - 140e3), 930 - 313 * (1 - gfm::exp(-depth / 7e3)));
}
__device__ __forceinline__ double sol_basalt(double depth) {
    double press = 3000 * 10 * depth / 1e9;
    if (press < 1.0) return 1050.0 - 420.0 * (1.0 - gfm::exp(-press * 3.3));
    if (press > 2.7) return (press + 14.0) * 43.0;
    return 630.0 + 13.0 * (press * press);
}
__device__ __forceinline__ double sol_wet(double depth) {
    if (depth > 80e3) return 800;
    return 800 + (double)6.2e-8f * ((depth - 80e3) * (depth - 80e3));
}
__device__ __forceinline__ double tpr_mantle(const DevArrays &A, const GfDims &d, long long e) {
    return mg_pr(A, d, e, MG_MANT1) + mg_pr(A, d, e, MG_MANT2);
}
__device__ __forceinline__ double tpr_sed(const DevArrays &A, const GfDims &d, long long e) {
    return mg_pr(A, d, e, MG_SED1) + mg_pr(A, d, e, MG_SED2) + mg_pr(A, d, e, MG_METASED) + mg_pr(A, d, e, MG_SCHIST);
}
__device__ __forceinline__ double tpr_basalt(const DevArrays &A, const GfDims &d, long long e) {
    return mg_pr(A, d, e, MG_OCEAN1) + mg_pr(A, d, e, MG_OCEAN2) + mg_pr(A, d, e, MG_OCEANDRY) + mg_pr(A, d, e, MG_ECLG);
}

// ---------------------------------------------------------------- ordered compaction
// Which elements a list holds.
enum { MG_PRED_MASK = 0, MG_PRED_W = 1, MG_PRED_MOR = 2, MG_PRED_ARC = 3 };
__device__ __forceinline__ bool mg_pred(int mode, const DevArrays &A, const GfDims &d, long long e) {
    if (mode == MG_PRED_MASK) return A.mg_mask[e] != 0;
    if (mode == MG_PRED_W) return A.fmelt2[e] > MG_W_BARRIER;
    // migration sources: MOR melt with a valid melting zone (MOR), melting
    // below the column's Moho (dikes and the mantle cone: ARC)
    if (mode == MG_PRED_MOR) return A.fmelt2[e] > 0 && A.mg_s[MS_VALID] != 0.0;
    int j, i;
    mg_eji(d, e, j, i);
    return j + 1 > A.jmoho[i] && A.fmelt[e] > 0;
}
// block b counts its MG_CB elements
__global__ void __launch_bounds__(MG_CB) k_mg_count(DevArrays A, GfDims d, int mode) {
    const long long e = (long long)blockIdx.x * MG_CB + threadIdx.x;
    const int v = (e < d.E && mg_pred(mode, A, d, e)) ? 1 : 0;
    const int c = __syncthreads_count(v);
    if (threadIdx.x == 0) A.mg_blk[blockIdx.x] = c;
}
// block b writes its elements after those of blocks 0..b-1; the last block
// stores the total in *count
__global__ void __launch_bounds__(MG_CB) k_mg_write(DevArrays A, GfDims d, int mode, int *list, int *count) {
    __shared__ int red[32];
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int part = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += MG_CB) part += A.mg_blk[b];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) red[w] = part;
    __syncthreads();
    int base = 0;
    for (int k = 0; k < MG_CB / 32; ++k) base += red[k];
    const long long e = (long long)blockIdx.x * MG_CB + threadIdx.x;
    const bool v = e < d.E && mg_pred(mode, A, d, e);
    const unsigned bal = __ballot_sync(0xffffffffu, v);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    int off = base;
    for (int k = 0; k < w; ++k) off += wsum[k];
    off += __popc(bal & ((1u << lane) - 1u));
    if (v) list[off] = (int)e;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        int tot = base;
        for (int k = 0; k < MG_CB / 32; ++k) tot += wsum[k];
        *count = tot;
    }
}

// ---------------------------------------------------------------- melting (change_phase)
// per column: the deepest serpentinite / chlorite element above the
// melting depth (flux melting starts there; -1: none), or fl_therm's
// topmost non-sediment row (1-based) for the dikes
__global__ void k_mg_cols(DevArrays A, GfDims d, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nx - 1) return;
    if (mode == 0) {
        int js = -1;
        for (int j = d.nz - 2; j >= 0; --j) {
            const long long e = gf_elem(d, j, i);
            if (mg_pr(A, d, e, MG_SERP) + mg_pr(A, d, e, MG_HYDMANT) > 0.6 && CY(A.cord, d, j, i) > -200e3) {
                js = j;
                break;
            }
        }
        A.mg_col[i] = js;
    } else {
        const int jm = A.jmoho[i] < d.nz - 1 ? A.jmoho[i] : d.nz - 1;
        int jtop = 1;
        while (jtop < jm) {
            const int iph = A.iphase[gf_elem(d, jtop - 1, i)];
            if (iph != MG_SED1 && iph != MG_SED2) break;
            ++jtop;
        }
        A.mg_col[d.nx + i] = jtop;
    }
}

// zero the melt fractions; mark the elements above a solidus at the start
// (bit 0 mantle, 1 sediments, 2 basalt, 3 flux melting)
__global__ void __launch_bounds__(GF_THREADS) k_melt_flags(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    int j, i;
    mg_eji(d, e, j, i);
    A.fmelt[e] = 0.0;
    A.fmelt2[e] = 0.0;
    const double z = CY(A.cord, d, j, i);
    const double tmpr = mg_tmpr(A, d, j, i), depth = mg_depth(A, d, j, i);
    unsigned m = 0;
    if (tpr_mantle(A, d, e) > 0.6 && z > -150e3 && tmpr > sol_mantle(P, depth)) m |= 1u;
    if (tpr_sed(A, d, e) > 0.6 && z > -200e3 && tmpr > sol_sed(depth)) m |= 2u;
    if (tpr_basalt(A, d, e) > 0.6 && z > -200e3 && tmpr > sol_basalt(depth)) m |= 4u;
    const int js = A.mg_col[i];
    if (js >= 0 && j <= js && tmpr > sol_wet(depth)) m |= 8u;
    A.mg_mask[e] = (uint8_t)m;
}

// the static part of each listed candidate: corner nodes, and per loop the
// phase sum and the solidus (depth and phases do not change while melting)
__global__ void __launch_bounds__(GF_THREADS) k_melt_prep(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.mg_i[MI_COUNT]) return;
    const DevParams &P = *Pp;
    const long long e = A.mg_list[k];
    int j, i;
    mg_eji(d, e, j, i);
    double *r = A.mg_src + (long long)k * GF_MG_SRC_W;
    const double depth = mg_depth(A, d, j, i);
    r[MR_E] = mg_pack(e);
    r[MR_MASK] = mg_pack(A.mg_mask[e]);
    r[MR_N00] = mg_pack(gf_node(d, j, i));
    r[MR_N01] = mg_pack(gf_node(d, j, i + 1));
    r[MR_N10] = mg_pack(gf_node(d, j + 1, i));
    r[MR_N11] = mg_pack(gf_node(d, j + 1, i + 1));
    r[MR_TPR + 0] = tpr_mantle(A, d, e);
    r[MR_TPR + 1] = sol_mantle(P, depth);
    r[MR_TPR + 2] = tpr_sed(A, d, e);
    r[MR_TPR + 3] = sol_sed(depth);
    r[MR_TPR + 4] = tpr_basalt(A, d, e);
    r[MR_TPR + 5] = sol_basalt(depth);
    r[MR_TPR + 6] = mg_pr(A, d, e, MG_MANT1) + mg_pr(A, d, e, MG_MANT2) + mg_pr(A, d, e, MG_SERP);
    r[MR_TPR + 7] = sol_wet(depth);
}

// each melting loop's candidates in processing order (one CTA): positions
// in the candidate list with the loop's bit, in list order; the flux loop
// then column by column, each column's run reversed (upwards).  Slot
// loop * E of mg_order, the flux order at 4 E; counts in mg_i[MI_P0 + loop].
__global__ void __launch_bounds__(MG_CB) k_melt_order(DevArrays A, GfDims d) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const int n = A.mg_i[MI_COUNT];
    const double *rec = A.mg_src;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int loop = 0; loop < 4; ++loop) {
        int *out = A.mg_order + (long long)loop * d.E;
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        for (int base = 0; base < n; base += MG_CB) {
            const int k = base + threadIdx.x;
            const bool v = k < n && (mg_int(rec[(long long)k * GF_MG_SRC_W + MR_MASK]) & (1LL << loop));
            const unsigned bal = __ballot_sync(0xffffffffu, v);
            if (lane == 0) wsum[w] = __popc(bal);
            __syncthreads();
            int off = carry;
            for (int q = 0; q < w; ++q) off += wsum[q];
            off += __popc(bal & ((1u << lane) - 1u));
            if (v) out[off] = k;
            __syncthreads();
            if (threadIdx.x == 0) {
                int t = 0;
                for (int q = 0; q < MG_CB / 32; ++q) t += wsum[q];
                carry += t;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) A.mg_i[MI_P0 + loop] = carry;
        __syncthreads();
    }
    const int n3 = A.mg_i[MI_P0 + 3];
    const int *o3 = A.mg_order + 3 * d.E;
    int *o4 = A.mg_order + 4 * d.E;
    const long long nz1 = d.nz - 1;
    auto elem = [&](int p) { return mg_int(rec[(long long)o3[p] * GF_MG_SRC_W + MR_E]); };
    for (int p = threadIdx.x; p < n3; p += MG_CB) {
        const long long col = elem(p) / nz1;
        int lo = 0, hi = n3; // first entry of the column
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (elem(mid) < col * nz1) lo = mid + 1;
            else hi = mid;
        }
        const int gs = lo;
        hi = n3; // first entry past the column
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (elem(mid) < (col + 1) * nz1) lo = mid + 1;
            else hi = mid;
        }
        o4[gs + (lo - 1 - p)] = o3[p];
    }
}

// melting loop `loop` over its candidates in processing order, one thread:
// the next candidate's corner temperatures are loaded while the current one
// is processed, then patched where the current one cooled a shared corner
__device__ void melt_walk(const DevParams &P, double *__restrict__ T, double *__restrict__ fmelt,
                          double *__restrict__ fmelt2, const double *__restrict__ rec, const int *__restrict__ order,
                          int cnt, int loop) {
    if (cnt <= 0) return;
    const double *r = rec + (long long)order[0] * GF_MG_SRC_W;
    long long n[4], m[4];
    double t[4], u[4];
    for (int q = 0; q < 4; ++q) {
        n[q] = mg_int(r[MR_N00 + q]);
        t[q] = T[n[q]];
    }
    long long e = mg_int(r[MR_E]);
    double fm = (loop >= 2) ? fmelt[e] : 0.0;
    for (int k = 0; k < cnt; ++k) {
        const double *rn = r;
        long long en = 0;
        double fmn = 0.0;
        if (k + 1 < cnt) {
            rn = rec + (long long)order[k + 1] * GF_MG_SRC_W;
            for (int q = 0; q < 4; ++q) {
                m[q] = mg_int(rn[MR_N00 + q]);
                u[q] = T[m[q]];
            }
            en = mg_int(rn[MR_E]);
            if (loop >= 2) fmn = fmelt[en];
        }
        const double tmpr = 0.25 * (t[0] + t[1] + t[2] + t[3]);
        const double sol = r[MR_TPR + 2 * loop + 1];
        if (tmpr > sol) {
            const double over = tmpr - sol;
            if (loop == 0) {
                fmelt2[e] = mg_pmelt(P, MG_MANT1, over, 35.0) * r[MR_TPR];
            } else if (loop == 1) {
                fmelt[e] = mg_pmelt(P, MG_SED2, over, 50.0) * r[MR_TPR + 2];
            } else if (loop == 2) {
                fmelt[e] = fm + mg_pmelt(P, MG_OCEAN1, over, 20.0) * r[MR_TPR + 4];
            } else {
                fmelt[e] = fm + mg_pmelt(P, MG_MANT1, over, 50.0) * r[MR_TPR + 6];
            }
            for (int q = 0; q < 4; ++q) {
                t[q] = t[q] - over;
                T[n[q]] = t[q];
            }
            if (k + 1 < cnt)
                for (int q = 0; q < 4; ++q)
                    for (int c = 0; c < 4; ++c)
                        if (m[q] == n[c]) u[q] = t[c];
        }
        r = rn;
        e = en;
        fm = fmn;
        for (int q = 0; q < 4; ++q) {
            n[q] = m[q];
            t[q] = u[q];
        }
    }
}

// one candidate of melting loop `loop` from the current corner temperatures
__device__ __forceinline__ void melt_one(const DevParams &P, double *__restrict__ T, double *__restrict__ fmelt,
                                         double *__restrict__ fmelt2, const double *__restrict__ r, int loop) {
    long long n[4];
    double t[4];
    for (int q = 0; q < 4; ++q) {
        n[q] = mg_int(r[MR_N00 + q]);
        t[q] = T[n[q]];
    }
    const double tmpr = 0.25 * (t[0] + t[1] + t[2] + t[3]);
    const double sol = r[MR_TPR + 2 * loop + 1];
    if (!(tmpr > sol)) return;
    const long long e = mg_int(r[MR_E]);
    const double over = tmpr - sol;
    if (loop == 0) fmelt2[e] = mg_pmelt(P, MG_MANT1, over, 35.0) * r[MR_TPR];
    else if (loop == 1) fmelt[e] = mg_pmelt(P, MG_SED2, over, 50.0) * r[MR_TPR + 2];
    else if (loop == 2) fmelt[e] = fmelt[e] + mg_pmelt(P, MG_OCEAN1, over, 20.0) * r[MR_TPR + 4];
    else fmelt[e] = fmelt[e] + mg_pmelt(P, MG_MANT1, over, 50.0) * r[MR_TPR + 6];
    for (int q = 0; q < 4; ++q) T[n[q]] = t[q] - over;
}

// The four melting loops, in the reference's order, by one CTA.  In a
// loop's serial order (columns ascending; rows downwards, or upwards for
// flux melting) an element depends on the earlier elements that share one of
// its corners: (j-1,i), (j-1,i-1), (j,i-1), (j+1,i-1) (rows mirrored for the
// flux loop).  Level 2i + j (2i - j for the flux loop) puts every such
// predecessor on a lower level, and elements of one level share no corner,
// so the levels run one after another, the elements of a level at once:
// the serial result, bit for bit.  Above MG_LEVELS levels, or for a short
// list, one thread walks the list instead.
constexpr int MG_LEVELS = 4096;
__global__ void __launch_bounds__(MG_CB) k_melt_serial(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    __shared__ int start[MG_LEVELS + 1];
    __shared__ int fill[MG_LEVELS];
    __shared__ int psum[MG_CB];
    const DevParams &P = *Pp;
    const long long nz1 = d.nz - 1;
    const int nlev = 2 * d.nx + d.nz;
    int *lvl = A.mg_order + 5 * d.E; // candidates sorted by level
    for (int loop = 0; loop < 4; ++loop) {
        const int *order = A.mg_order + (long long)(loop == 3 ? 4 : loop) * d.E;
        const int cnt = A.mg_i[MI_P0 + loop];
        if (cnt == 0) continue;
        if (nlev > MG_LEVELS || cnt < 64) { // a short list: the walk is cheaper than the level sort
            if (threadIdx.x == 0) melt_walk(P, A.temp, A.fmelt, A.fmelt2, A.mg_src, order, cnt, loop);
            __syncthreads();
            continue;
        }
        auto level = [&](int k) {
            const long long e = mg_int(A.mg_src[(long long)order[k] * GF_MG_SRC_W + MR_E]);
            const int i = (int)(e / nz1), j = (int)(e - (long long)i * nz1);
            return loop < 3 ? 2 * i + j : 2 * i - j + d.nz;
        };
        for (int l = threadIdx.x; l < nlev; l += MG_CB) fill[l] = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += MG_CB) atomicAdd(&fill[level(k)], 1);
        __syncthreads();
        // exclusive scan of the level counts: each thread a contiguous run
        const int per = (nlev + MG_CB - 1) / MG_CB, l0 = threadIdx.x * per;
        int sum = 0;
        for (int l = l0; l < l0 + per && l < nlev; ++l) sum += fill[l];
        psum[threadIdx.x] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int q = 0; q < MG_CB; ++q) {
                const int v = psum[q];
                psum[q] = acc;
                acc += v;
            }
        }
        __syncthreads();
        int acc = psum[threadIdx.x];
        for (int l = l0; l < l0 + per && l < nlev; ++l) {
            start[l] = acc;
            acc += fill[l];
            fill[l] = 0;
        }
        if (threadIdx.x == MG_CB - 1) start[nlev] = cnt;
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += MG_CB) {
            const int l = level(k);
            lvl[start[l] + atomicAdd(&fill[l], 1)] = order[k];
        }
        __syncthreads();
        for (int l = 0; l < nlev; ++l) {
            const int s0 = start[l], s1 = start[l + 1];
            if (s0 == s1) continue;
            for (int k = s0 + (int)threadIdx.x; k < s1; k += MG_CB)
                melt_one(P, A.temp, A.fmelt, A.fmelt2, A.mg_src + (long long)lvl[k] * GF_MG_SRC_W, loop);
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------- fl_therm's magma part
// freezing of both pools (temperature from temp0); the latent heat of the
// element's four corners kept for the node pass
__global__ void __launch_bounds__(GF_THREADS) k_mg_freeze(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A,
                                                          GfDims d) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    const double dt = C->dt;
    int j, i;
    mg_eji(d, e, j, i);
    const double *T0 = A.temp0;
    const double cp_eff = P.cp[A.iphase[e] - 1];
    const double tmpr = 0.25 * (T0[gf_node(d, j, i)] + T0[gf_node(d, j + 1, i)] + T0[gf_node(d, j, i + 1)] +
                                T0[gf_node(d, j + 1, i + 1)]);
    const double fr_lambda = P.lambda_freeze * gfm::exp(-P.lambda_freeze_tdep * (tmpr - P.t_top));
    const double f1 = A.fmagma[e], f2 = A.fmagma2[e];
    const double d1 = mg_min(f1, f1 * dt * fr_lambda), d2 = mg_min(f2, f2 * dt * fr_lambda);
    A.fmagma[e] = f1 - d1;
    A.fmagma2[e] = f2 - d2;
    A.mg_e[e] = d1 * P.latent_heat_magma / cp_eff / 4 + d2 * P.latent_heat_magma / cp_eff / 4;
}
// each node adds its elements' latent heat in serial element order, then
// temp = min(temp, t_bot)
__global__ void __launch_bounds__(GF_THREADS) k_mg_freeze_nodes(const DevParams *__restrict__ Pp, DevArrays A,
                                                                GfDims d) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    int J, I;
    mg_nji(d, n, J, I);
    const int nx = d.nx, nz = d.nz;
    double t = A.temp[n];
    if (J > 0 && I > 0) t = t + A.mg_e[gf_elem(d, J - 1, I - 1)];
    if (J < nz - 1 && I > 0) t = t + A.mg_e[gf_elem(d, J, I - 1)];
    if (J > 0 && I < nx - 1) t = t + A.mg_e[gf_elem(d, J - 1, I)];
    if (J < nz - 1 && I < nx - 1) t = t + A.mg_e[gf_elem(d, J, I)];
    A.temp[n] = mg_min(t, Pp->t_bot);
}

// element centre of the quad with the reference's corner order
// (j,i), (j,i+1), (j+1,i), (j+1,i+1)
__device__ __forceinline__ double mg_cx(const double *c, const GfDims &d, int j, int i) {
    return 0.25 * (CX(c, d, j, i) + CX(c, d, j, i + 1) + CX(c, d, j + 1, i) + CX(c, d, j + 1, i + 1));
}
__device__ __forceinline__ double mg_cz(const double *c, const GfDims &d, int j, int i) {
    return 0.25 * (CY(c, d, j, i) + CY(c, d, j, i + 1) + CY(c, d, j + 1, i) + CY(c, d, j + 1, i + 1));
}

// fmelt2-weighted centre of the MOR melting zone (one CTA: terms in
// parallel into shared memory, sums by one thread in serial order); also
// the mantle cone's tan and width
__global__ void __launch_bounds__(MG_CB) k_mg_zone1(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    __shared__ double sx[MG_CB], sz[MG_CB], sw[MG_CB];
    const DevParams &P = *Pp;
    const int n = A.mg_i[MI_COUNT];
    double xs = 0, zs = 0, ws = 0;
    for (int base = 0; base < n; base += MG_CB) {
        if (base + (int)threadIdx.x < n) {
            const long long e = A.mg_list[base + threadIdx.x];
            int j, i;
            mg_eji(d, e, j, i);
            const double w = A.fmelt2[e];
            sx[threadIdx.x] = mg_cx(A.cord, d, j, i) * w;
            sz[threadIdx.x] = mg_cz(A.cord, d, j, i) * w;
            sw[threadIdx.x] = w;
        }
        __syncthreads();
        // the three sums by the first lanes of warps 0-2 (on different SM
        // sub-partitions, whose FP64 pipes then run side by side)
        const int m = n - base < MG_CB ? n - base : MG_CB;
        if (threadIdx.x == 0)
            for (int k = 0; k < m; ++k) xs = xs + sx[k];
        else if (threadIdx.x == 32)
            for (int k = 0; k < m; ++k) zs = zs + sz[k];
        else if (threadIdx.x == 64)
            for (int k = 0; k < m; ++k) ws = ws + sw[k];
        __syncthreads();
    }
    if (threadIdx.x == 32) sx[0] = zs;
    if (threadIdx.x == 64) sx[1] = ws;
    __syncthreads();
    if (threadIdx.x == 0) {
        zs = sx[0];
        ws = sx[1];
        const double tan_m = gfm::tan(0.5 * P.angle_mzone * 3.14159265358979323846 / 180.0);
        A.mg_s[MS_TANM] = tan_m;
        A.mg_i[MI_IHW] = mg_ceil(tan_m * 200e3 / P.dxmin);
        A.mg_s[MS_WSUM] = ws;
        A.mg_s[MS_VALID] = 0.0;
        A.mg_i[MI_FOUND] = 0x7fffffff;
        A.mg_i[MI_MAXJ] = 0;
        if (ws > 0.0) {
            A.mg_s[MS_XC] = xs / ws;
            A.mg_s[MS_ZC] = zs / ws;
        }
    }
}
// the first element (serial order) holding the centre
__global__ void __launch_bounds__(GF_THREADS) k_mg_find(DevArrays A, GfDims d) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E || !(A.mg_s[MS_WSUM] > 0.0)) return;
    int j, i;
    mg_eji(d, e, j, i);
    const double xc = A.mg_s[MS_XC], zc = A.mg_s[MS_ZC];
    const double *c = A.cord;
    if (CX(c, d, j, i) <= xc && CX(c, d, j, i + 1) >= xc && CY(c, d, j, i) >= zc && CY(c, d, j + 1, i) <= zc)
        atomicMin(&A.mg_i[MI_FOUND], (int)e);
}
// widths on either side of the centre and the zone's cone (one CTA as above)
__global__ void __launch_bounds__(MG_CB) k_mg_zone2(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    __shared__ double sx[MG_CB], sw[MG_CB], sl[MG_CB], sr[MG_CB];
    const int found = A.mg_i[MI_FOUND];
    if (found == 0x7fffffff) return;
    const DevParams &P = *Pp;
    const int n = A.mg_i[MI_COUNT];
    const double xc = A.mg_s[MS_XC];
    double xl = 0, xr = 0, wl = 0, wr = 0;
    for (int base = 0; base < n; base += MG_CB) {
        if (base + (int)threadIdx.x < n) {
            const long long e = A.mg_list[base + threadIdx.x];
            int j, i;
            mg_eji(d, e, j, i);
            const double w = A.fmelt2[e], x = mg_cx(A.cord, d, j, i);
            sx[threadIdx.x] = x;
            sw[threadIdx.x] = w;
            sl[threadIdx.x] = (xc - x) * (xc - x) * w;
            sr[threadIdx.x] = (x - xc) * (x - xc) * w;
        }
        __syncthreads();
        // the four sums by the first lanes of warps 0-3
        const int m = n - base < MG_CB ? n - base : MG_CB;
        if (threadIdx.x == 0) {
            for (int k = 0; k < m; ++k)
                if (sx[k] < xc) xl = xl + sl[k];
        } else if (threadIdx.x == 32) {
            for (int k = 0; k < m; ++k)
                if (sx[k] < xc) wl = wl + sw[k];
        } else if (threadIdx.x == 64) {
            for (int k = 0; k < m; ++k)
                if (sx[k] > xc) xr = xr + sr[k];
        } else if (threadIdx.x == 96) {
            for (int k = 0; k < m; ++k)
                if (sx[k] > xc) wr = wr + sw[k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 32) sl[0] = wl;
    if (threadIdx.x == 64) sl[1] = xr;
    if (threadIdx.x == 96) sl[2] = wr;
    __syncthreads();
    if (threadIdx.x == 0) {
        wl = sl[0];
        xr = sl[1];
        wr = sl[2];
        int jc, ic;
        mg_eji(d, found, jc, ic);
        xl = 1.8 * sqrt(xl / wl);
        xr = 1.8 * sqrt(xr / wr);
        if (xl < P.dxmin) xl = P.dxmin;
        if (xr < P.dxmin) xr = P.dxmin;
        if (xl != xl) xl = P.dxmin;
        if (xr != xr) xr = P.dxmin;
        const double z_surf = 0.5 * (CY(A.cord, d, 0, ic) + CY(A.cord, d, 0, ic + 1));
        const double h2 = z_surf - A.mg_s[MS_ZC];
        const double tl = xl / h2, tr = xr / h2;
        A.mg_s[MS_ZSURF] = z_surf;
        A.mg_s[MS_H2] = h2;
        A.mg_s[MS_TANL] = tl;
        A.mg_s[MS_TANR] = tr;
        A.mg_i[MI_IC] = ic;
        A.mg_i[MI_JC] = jc;
        A.mg_i[MI_IHWL] = mg_ceil(tl * 150e3 / P.dxmin);
        A.mg_i[MI_IHWR] = mg_ceil(tr * 150e3 / P.dxmin);
        A.mg_s[MS_VALID] = 1.0;
    }
}

// the terms each listed migration source adds
__global__ void __launch_bounds__(GF_THREADS) k_mg_src(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A,
                                                       GfDims d, const int *list, const int *count, double *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const DevParams &P = *Pp;
    const double dt = C->dt;
    const long long e = list[k];
    int j, i;
    mg_eji(d, e, j, i);
    const int nx = d.nx, i1 = i + 1, j1 = j + 1;
    const int jm = A.jmoho[i] < 1 ? 1 : (A.jmoho[i] > d.nz - 1 ? d.nz - 1 : A.jmoho[i]); // a valid row
    const double *c = A.cord;
    const double area0 = ((const double *)A.area)[gf_ek(d, e, 0)], area1 = ((const double *)A.area)[gf_ek(d, e, 1)];
    const double quad_area = 0.5 / area0 + 0.5 / area1;
    double *s = out + (long long)k * GF_MG_SRC_W;
    unsigned flags = 0;
    s[SR_E] = mg_pack(e);
    s[SR_J1] = mg_pack(j1);
    s[SR_I1] = mg_pack(i1);
    if (j1 > jm && A.fmelt[e] > 0) {
        flags |= 1u;
        atomicMax(&A.mg_i[MI_MAXJ], j1);
        const double fm = A.fmelt[e];
        double area_ratio = (CY(c, d, 0, i) + CY(c, d, 0, i + 1) - CY(c, d, jm - 1, i) - CY(c, d, jm - 1, i + 1)) /
                            (CY(c, d, j, i) + CY(c, d, j, i + 1) - CY(c, d, j + 1, i) - CY(c, d, j + 1, i + 1));
        const int nd = P.nelem_dike;
        const int ihalf = (nd - 1) / 2 > 0 ? (nd - 1) / 2 : 0, nd1 = nd > 1 ? nd : 1;
        int ii_start = i1 - ihalf > 1 ? i1 - ihalf : 1;
        int ii_end = ii_start + nd1 - 1 < nx - 1 ? ii_start + nd1 - 1 : nx - 1;
        ii_start = ii_end - nd1 + 1 > 1 ? ii_end - nd1 + 1 : 1;
        const int ncol = ii_end - ii_start + 1;
        s[SR_TERM_C] = fm * P.ratio_crust_mzone * area_ratio * P.prod_magma * dt / ncol;
        s[SR_II0] = mg_pack(ii_start);
        s[SR_II1] = mg_pack(ii_end);
        const double z_moho = 0.5 * (CY(c, d, jm - 1, i) + CY(c, d, jm - 1, i + 1));
        const double z_melt = 0.5 * (CY(c, d, j + 1, i) + CY(c, d, j + 1, i + 1));
        const double x_melt = 0.5 * (CX(c, d, j + 1, i) + CX(c, d, j + 1, i + 1));
        const double h = z_moho - z_melt;
        area_ratio = h * h * A.mg_s[MS_TANM] / quad_area;
        s[SR_TERM_M] = fm * P.ratio_mantle_mzone * area_ratio * P.prod_magma * dt;
        s[SR_XMELT] = x_melt;
        s[SR_ZMELT] = z_melt;
    }
    if (A.fmelt2[e] > 0 && A.mg_s[MS_VALID] != 0.0) {
        flags |= 2u;
        const double h2 = A.mg_s[MS_H2];
        const double area_ratio =
            0.5 * (h2 * h2 * A.mg_s[MS_TANL] / quad_area + h2 * h2 * A.mg_s[MS_TANR] / quad_area);
        s[SR_TERM_R] = A.fmelt2[e] * area_ratio * P.prod_magma2 * dt;
    }
    s[SR_FLAGS] = mg_pack(flags);
}

// first position of the ordered source list whose element is >= e
__device__ __forceinline__ int mg_lower(const int *list, int n, long long e) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (list[mid] < e) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// every element as a migration target: the adds of the sources that reach
// it, in serial order, with its own clamp to fmagma_max at its place in
// that order.  fmagma takes only dike / mantle-cone adds and fmagma2 only
// MOR adds, so each is accumulated over its own ordered source list; four
// threads per element in consecutive warps (different SM sub-partitions,
// whose FP64 pipes run side by side) carry fmagma, fmagma2, dike_added and
// the MOR marker volume.
__global__ void __launch_bounds__(GF_THREADS) k_mg_migrate(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int part = (int)((gid >> 5) & 3);
    const long long t = ((gid >> 7) << 5) + (gid & 31);
    if (t >= d.E) return;
    const DevParams &P = *Pp;
    const int nx = d.nx, nz = d.nz;
    int jt, it;
    mg_eji(d, t, jt, it);
    const int jt1 = jt + 1, it1 = it + 1;
    const double fmax = P.fmagma_max;
    if (part == 1 || part == 3) { // MOR pool: fmagma2 (clamped) and the MOR marker volume
        bool in = false;
        if (A.mg_s[MS_VALID] != 0.0) {
            const int ic1 = A.mg_i[MI_IC] + 1, jc1 = A.mg_i[MI_JC] + 1;
            const int lo = ic1 - A.mg_i[MI_IHWL] > 1 ? ic1 - A.mg_i[MI_IHWL] : 1;
            const int hi = ic1 + A.mg_i[MI_IHWR] < nx - 1 ? ic1 + A.mg_i[MI_IHWR] : nx - 1;
            if (it1 >= lo && it1 <= hi && jt1 <= jc1) {
                // which side of the zone's cone the element lies in
                const double *c = A.cord;
                const double x = 0.5 * (CX(c, d, jt, it) + CX(c, d, jt, it + 1));
                const double z = 0.5 * (CY(c, d, jt, it) + CY(c, d, jt, it + 1));
                const double xc = A.mg_s[MS_XC], z_surf = A.mg_s[MS_ZSURF];
                in = (x < xc && fabs(xc - x) <= A.mg_s[MS_TANL] * (z_surf - z)) ||
                     (x >= xc && fabs(x - xc) <= A.mg_s[MS_TANR] * (z_surf - z));
            }
        }
        const int n = in ? A.mg_i[MI_COUNT] : 0;
        const double *src = A.mg_src;
        if (part == 1) {
            double f2 = A.fmagma2[t];
            bool clamped = false;
            for (int k = 0; k < n; ++k) {
                const double *s = src + (long long)k * GF_MG_SRC_W;
                const long long es = mg_int(s[SR_E]);
                if (!clamped && es > t) {
                    f2 = mg_min(f2, fmax);
                    clamped = true;
                }
                f2 = f2 + s[SR_TERM_R];
                if (es == t) {
                    f2 = mg_min(f2, fmax);
                    clamped = true;
                }
            }
            if (!clamped) f2 = mg_min(f2, fmax);
            A.fmagma2[t] = f2;
        } else {
            double mv = A.mor_marker_vol[t];
            for (int k = 0; k < n; ++k) mv = mv + src[(long long)k * GF_MG_SRC_W + SR_TERM_R];
            A.mor_marker_vol[t] = mv;
        }
        return;
    }
    // dikes and the mantle cone: fmagma (clamped) and dike_added, over the
    // sources in columns within max(nelem_dike, cone half width), none
    // when the element lies below its Moho and below every source
    const double *c = A.cord;
    const double x = 0.5 * (CX(c, d, jt, it) + CX(c, d, jt, it + 1));
    const double z = 0.5 * (CY(c, d, jt, it) + CY(c, d, jt, it + 1));
    const int jm_t = A.jmoho[it], jtop_t = A.mg_col[nx + it];
    const bool crust_row = jt1 >= jtop_t && jt1 <= jm_t;
    const int ihw = A.mg_i[MI_IHW];
    const double tan_m = A.mg_s[MS_TANM];
    const int *list = A.mg_list2;
    const double *src = A.mg_src2;
    int k0 = 0, k1 = 0;
    if (!(jt1 > jm_t && jt1 > A.mg_i[MI_MAXJ])) {
        const int n = A.mg_i[MI_COUNT2];
        const int reach = (P.nelem_dike > ihw ? P.nelem_dike : ihw) + 1;
        const long long clo = it - reach < 0 ? 0 : it - reach;
        const long long chi = it + reach + 1 > nx - 1 ? nx - 1 : it + reach + 1;
        k0 = mg_lower(list, n, clo * (nz - 1));
        k1 = mg_lower(list, n, chi * (nz - 1));
    }
    if (part == 0) {
        double f = A.fmagma[t];
        bool clamped = false;
        for (int k = k0; k < k1; ++k) {
            const double *s = src + (long long)k * GF_MG_SRC_W;
            const long long es = mg_int(s[SR_E]);
            if (!clamped && es > t) {
                f = mg_min(f, fmax);
                clamped = true;
            }
            if (crust_row && it1 >= mg_int(s[SR_II0]) && it1 <= mg_int(s[SR_II1])) f = f + s[SR_TERM_C];
            const int i1s = (int)mg_int(s[SR_I1]);
            const int lo = i1s - ihw > 1 ? i1s - ihw : 1, hi = i1s + ihw < nx - 1 ? i1s + ihw : nx - 1;
            if (it1 >= lo && it1 <= hi && jt1 >= jm_t + 1 && jt1 <= mg_int(s[SR_J1]) &&
                fabs(x - s[SR_XMELT]) <= tan_m * (z - s[SR_ZMELT]))
                f = f + s[SR_TERM_M];
            if (es == t) {
                f = mg_min(f, fmax);
                clamped = true;
            }
        }
        if (!clamped) f = mg_min(f, fmax);
        A.fmagma[t] = f;
    } else {
        double da = 0.0;
        for (int k = k0; k < k1; ++k) {
            const double *s = src + (long long)k * GF_MG_SRC_W;
            if (crust_row && it1 >= mg_int(s[SR_II0]) && it1 <= mg_int(s[SR_II1])) da = da + s[SR_TERM_C];
        }
        A.dike_added[t] = da;
    }
}

// rate-capped dike release; mark the elements that receive new markers
__global__ void __launch_bounds__(GF_THREADS) k_mg_release(const DevParams *__restrict__ Pp, DevArrays A, GfDims d) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    const double *area = (const double *)A.area;
    const double elem_area = 0.5 / area[gf_ek(d, e, 0)] + 0.5 / area[gf_ek(d, e, 1)];
    const double pending = A.dike_added[e] * elem_area + A.dike_backlog[e];
    const double released = mg_min(pending, 1.0e-4 * P.Amin);
    A.dike_backlog[e] = pending - released;
    A.dike_released[e] = released / elem_area;
    const double dmv = A.dike_marker_vol[e] + released;
    A.dike_marker_vol[e] = dmv;
    const int kinc = A.nmark_elem[e];
    bool add = false;
    if (kinc > 0 && kinc < GF_MAX_MARKERS_PER_ELEM) {
        const double unit = elem_area / kinc;
        // the MOR test with the count before any arc markers is exact when
        // no arc marker comes first and a superset otherwise
        add = dmv >= unit || A.mor_marker_vol[e] >= unit;
    }
    A.mg_mask[e] = add ? 1 : 0;
}
// new arc (karc1) and oceanic-crust (kocean1) markers at the centres of the
// listed elements, numbered in serial order
__global__ void k_mg_markers(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A, GfDims d, int max_markers) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const DevParams &P = *Pp;
    const int n = A.mg_i[MI_COUNT];
    const double *area = (const double *)A.area;
    const double time = C->time;
    for (int k = 0; k < n; ++k) {
        const long long e = A.mg_list[k];
        int j, i;
        mg_eji(d, e, j, i);
        const double elem_area = 0.5 / area[gf_ek(d, e, 0)] + 0.5 / area[gf_ek(d, e, 1)];
        for (int path = 0; path < 2; ++path) {
            double *vol = path == 0 ? &A.dike_marker_vol[e] : &A.mor_marker_vol[e];
            const int kinc = A.nmark_elem[e];
            if (kinc > 0 && kinc < GF_MAX_MARKERS_PER_ELEM) {
                const double unit = elem_area / kinc;
                if (*vol >= unit) {
                    const int room = GF_MAX_MARKERS_PER_ELEM - kinc, want = mg_ceil(*vol / unit);
                    const int n_to_add = want < room ? want : room;
                    const double *c = A.cord;
                    const double xc = 0.25 * (CX(c, d, j, i) + CX(c, d, j + 1, i) + CX(c, d, j, i + 1) + CX(c, d, j + 1, i + 1));
                    const double yc = 0.25 * (CY(c, d, j, i) + CY(c, d, j + 1, i) + CY(c, d, j, i + 1) + CY(c, d, j + 1, i + 1));
                    for (int m = 0; m < n_to_add; ++m)
                        add_marker1(A, d, xc, yc, path == 0 ? MG_ARC1 : MG_OCEAN1, time, j, i, max_markers);
                    *vol = 0.0;
                    count_phase_ratio1(P, C, A, d, e);
                }
            }
        }
    }
}

// ---------------------------------------------------------------- diff_topo's magma blocks
// the area-weighted column sum of f (rows in order): one warp, each lane
// one row of every 32, every lane adding the same terms in row order
__device__ __forceinline__ double mg_col_sum(const DevArrays &A, const GfDims &d, int i, const double *f, int lane) {
    const double *area = (const double *)A.area;
    double tot = 0;
    for (int j0 = 0; j0 < d.nz - 1; j0 += 32) {
        const int j = j0 + lane;
        double term = 0;
        if (j < d.nz - 1) {
            const long long e = gf_elem(d, j, i);
            const double quad_area = 0.5 / area[gf_ek(d, e, 0)] + 0.5 / area[gf_ek(d, e, 1)];
            term = quad_area * f[e];
        }
        const int m = d.nz - 1 - j0 < 32 ? d.nz - 1 - j0 : 32;
        for (int k = 0; k < m; ++k) tot = tot + __shfl_sync(0xffffffffu, term, k);
    }
    return tot;
}
// arc extrusion of each inner column (fl_move.f90:213-237), one warp per column
__global__ void __launch_bounds__(GF_THREADS) k_arc_cols(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A,
                                                         GfDims d, double rate) {
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) + 1, lane = threadIdx.x & 31;
    if (i >= d.nx - 2) return;
    const DevParams &P = *Pp;
    const double totalmelt = mg_col_sum(A, d, i, A.fmelt, lane);
    if (lane != 0) return;
    const double *c = A.cord;
    const double ext = rate * C->dt * totalmelt * P.prod_magma /
                       (CX(c, d, 0, i + 1) - CX(c, d, 0, i) +
                        0.5 * (CX(c, d, 0, i) - CX(c, d, 0, i - 1) + CX(c, d, 0, i + 2) - CX(c, d, 0, i + 1)));
    A.extrusion[i] = ext;
    A.extr_acc[i] = A.extr_acc[i] + ext;
    A.dhacc[i] = A.dhacc[i] + ext;
}
// each surface node takes the extrusion of the column on its left, then of
// the one on its right (serial column order)
__global__ void k_arc_nodes(DevArrays A, GfDims d) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= d.nx) return;
    const long long nz_ = d.N + gf_node(d, 0, I);
    double hc = A.dhacc_correction[I], z = A.cord[nz_];
    if (I - 1 >= 1 && I - 1 < d.nx - 2) {
        hc = hc + A.extrusion[I - 1];
        z = z + A.extrusion[I - 1];
    }
    if (I >= 1 && I < d.nx - 2) {
        hc = hc + A.extrusion[I];
        z = z + A.extrusion[I];
    }
    A.dhacc_correction[I] = hc;
    A.cord[nz_] = z;
}
// the MOR pool of each inner column: its volume, the erupted fraction
// taken from the pool, and the height it would form (fl_move.f90:247-264);
// one warp per column
__global__ void __launch_bounds__(GF_THREADS) k_mor_cols(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A,
                                                         GfDims d) {
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) + 1, lane = threadIdx.x & 31;
    if (i >= d.nx - 2) return;
    const DevParams &P = *Pp;
    const double dt = C->dt;
    const double total_melt = mg_col_sum(A, d, i, A.fmagma2, lane);
    for (int j = lane; j < d.nz - 1; j += 32) {
        const long long e = gf_elem(d, j, i);
        const double f2 = A.fmagma2[e];
        A.fmagma2[e] = f2 - mg_min(f2, f2 * P.prod_magma2 * dt);
    }
    if (lane == 0) A.mg_c[i] = dt * total_melt * P.prod_magma2 / (CX(A.cord, d, 0, i + 1) - CX(A.cord, d, 0, i));
}
// newphase2marker (marker_data.f90:107-137) on rows j1..j2, columns i1..i2 (1-based)
__device__ void mg_newphase(DevArrays &A, const GfDims &d, int j1, int j2, int i1, int i2, int iph) {
    const long long total = (long long)d.nphase * d.E;
    for (int i = i1; i <= i2; ++i)
        for (int j = j1; j <= j2; ++j) {
            const long long e = gf_elem(d, j - 1, i - 1);
            for (int n = 0; n < A.nmark_elem[e]; ++n)
                A.mark_phase[A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n] - 1] = (int8_t)iph;
            A.iphase[e] = iph;
            for (int k = 0; k < d.nphase; ++k) A.phase_ratio[gf_pr(d, e, k)] = 0.0;
            const long long off = (long long)(iph - 1) + (long long)d.nphase * e;
            if (off < total) A.phase_ratio[off] = 1.0;
        }
}
// the columns with MOR magma in serial order: one warp loads 32 columns'
// erupted heights and surface / second-row heights, its first lane walks the
// active ones, converting rows to oceanic crust (newphase2marker) when the
// erupted height reaches an element's, and adding the remainder to the
// column's two surface nodes; the left node of the next column is the one
// this column just raised
__global__ void k_mor_chain(DevArrays A, GfDims d) {
    __shared__ double s_eh[32], s_z0[32], s_z0n[32], s_z1[32], s_z1n[32], s_ea[32];
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int lane = threadIdx.x, nx = d.nx, nz = d.nz;
    double *c = A.cord;
    const long long N = d.N;
    int last = -1;       // the last column processed
    double last_z = 0.0; // its right surface node's new height
    for (int base = 1; base < nx - 2; base += 32) {
        const int ii = base + lane;
        const bool in = ii < nx - 2;
        const double eh = in ? A.mg_c[ii] : 0.0;
        if (in) {
            s_eh[lane] = eh;
            s_z0[lane] = CY(c, d, 0, ii);
            s_z0n[lane] = CY(c, d, 0, ii + 1);
            s_z1[lane] = CY(c, d, 1, ii);
            s_z1n[lane] = CY(c, d, 1, ii + 1);
            s_ea[lane] = A.extr_acc[ii];
        }
        unsigned bal = __ballot_sync(0xffffffffu, in && eh != 0.0);
        __syncwarp();
        if (lane == 0)
            while (bal) {
                const int l = __ffs(bal) - 1, i = base + l;
                bal &= bal - 1;
                const double h = s_eh[l];
                const double z0 = (last == i - 1) ? last_z : s_z0[l], z0n = s_z0n[l];
                double ele_height = fabs(0.5 * (s_z1n[l] + s_z1[l]) - 0.5 * (z0n + z0));
                double quotient = h / ele_height, remainder = fmod(h, ele_height);
                int j_oc = 1;
                if (!(quotient >= 0.0 && quotient < 2.0)) {
                    for (int j = 1; j < nz - 1; ++j) {
                        ele_height = ele_height + fabs(0.5 * (CY(c, d, j + 1, i + 1) + CY(c, d, j + 1, i)) -
                                                       0.5 * (CY(c, d, j, i + 1) + CY(c, d, j, i)));
                        quotient = h / ele_height;
                        remainder = fmod(h, ele_height);
                        if (quotient >= 0.0 && quotient < 2.0) {
                            j_oc = j + 1;
                            break;
                        }
                    }
                }
                if (quotient >= 1)
                    for (int j = 1; j <= nz - 1; ++j)
                        if (A.iphase[gf_elem(d, j - 1, i)] != MG_OCEAN1) {
                            const int j2 = j + j_oc - 1 < nz - 1 ? j + j_oc - 1 : nz - 1;
                            mg_newphase(A, d, j, j2, i + 1, i + 1, MG_OCEAN1);
                            break;
                        }
                A.extr_acc[i] = s_ea[l] + remainder / 2;
                c[N + gf_node(d, 0, i)] = z0 + remainder / 2;
                last_z = z0n + remainder / 2;
                c[N + gf_node(d, 0, i + 1)] = last_z;
                last = i;
            }
        __syncwarp();
    }
}
