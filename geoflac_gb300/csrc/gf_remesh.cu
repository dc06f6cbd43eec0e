// Remesh event on the device (src/par.f90:94-110): bar2euler, remesh,
// lpeuler2bar, marker2elem.  One thread per marker, node, element or new
// interpolation point; the reference's serial orders that decide results
// (marker numbering, per-element marker lists, the search order of the
// barycentric point location) are reproduced with scans and per-element
// sorts instead of a serial loop.  Compiled without FMA contraction: every
// FP64 expression rounds as in the serial Fortran.

#include "gf_kernels.cuh"

namespace {
namespace gfr {

using gfk::set_status;

inline unsigned blocks_for(long long n) { return (unsigned)((n + GF_THREADS - 1) / GF_THREADS); }

__device__ __forceinline__ double CX(const double *cord, const GfDims &d, int j, int i) { return cord[gf_node(d, j, i)]; }
__device__ __forceinline__ double CY(const double *cord, const GfDims &d, int j, int i) {
    return cord[d.N + gf_node(d, j, i)];
}

// check_inside (src/euler2bar.f90:102-161): the
// two triangles of element (j,i); bar1/bar2 and the 1-based triangle number
__device__ bool check_inside(const double *cord, const GfDims &d, double x, double y, double &bar1, double &bar2,
                             int &ntr, int i, int j) {
    for (int k = 0; k < 2; ++k) {
        double x1, x2, x3, y1, y2, y3;
        if (k == 0) {
            x1 = CX(cord, d, j, i); x2 = CX(cord, d, j + 1, i); x3 = CX(cord, d, j, i + 1);
            y1 = CY(cord, d, j, i); y2 = CY(cord, d, j + 1, i); y3 = CY(cord, d, j, i + 1);
        } else {
            x1 = CX(cord, d, j, i + 1); x2 = CX(cord, d, j + 1, i); x3 = CX(cord, d, j + 1, i + 1);
            y1 = CY(cord, d, j, i + 1); y2 = CY(cord, d, j + 1, i); y3 = CY(cord, d, j + 1, i + 1);
        }
        double det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
        double m11 = (x2 * y3 - y2 * x3) / det, m12 = (y2 - y3) / det, m13 = (x3 - x2) / det;
        double m21 = (x3 * y1 - y3 * x1) / det, m22 = (y3 - y1) / det, m23 = (x1 - x3) / det;
        bar1 = m11 + m12 * x + y * m13;
        bar2 = m21 + m22 * x + y * m23;
        if (bar1 >= 0.0 && bar2 >= 0.0 && bar1 + bar2 <= 1.0) {
            ntr = 2 * ((d.nz - 1) * i + j) + k + 1;
            return true;
        }
    }
    return false;
}

// ---------------------------------------------------------------- bar2euler
// marker2xy (src/bar2euler.f90:73-117): barycentric -> (x, y) in mark_a1/a2
__global__ void __launch_bounds__(GF_THREADS) k_bar2euler(DevArrays A, GfDims d, int nmarkers, int has_dhacc) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmarkers || A.mark_dead[m] == 0) return;
    const int nz = d.nz;
    int n = A.mark_ntriag[m];
    int k = (n - 1) % 2 + 1;
    int jj = ((n - k) / 2) % (nz - 1);
    int ii = (n - k) / 2 / (nz - 1);
    double ba1 = A.mark_a1[m], ba2 = A.mark_a2[m];
    double ba3 = 1.0 - ba1 - ba2;
    int i1, i2, i3, j1, j2, j3;
    if (k == 1) {
        i1 = ii; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj;
    } else {
        i1 = ii + 1; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj + 1;
    }
    const double *c = A.cord;
    double x = CX(c, d, j1, i1) * ba1 + CX(c, d, j2, i2) * ba2 + CX(c, d, j3, i3) * ba3;
    double y = CY(c, d, j1, i1) * ba1 + CY(c, d, j2, i2) * ba2 + CY(c, d, j3, i3) * ba3;
    if (has_dhacc) {
        if (j1 == 0) y = y - A.dhacc_correction[i1] * ba1;
        if (j2 == 0) y = y - A.dhacc_correction[i2] * ba2;
        if (j3 == 0) y = y - A.dhacc_correction[i3] * ba3;
    }
    A.mark_a1[m] = x;
    A.mark_a2[m] = y;
}

// ---------------------------------------------------------------- rem_cord
// New x of every node (rem_cord.f90:10-33): mesh1 between the row's ends
__global__ void __launch_bounds__(GF_THREADS) k_regrid_x(DevArrays A, GfDims d, GfRemeshArgs a, const double *tx) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.N) return;
    int j = (int)(t % d.nz), i = (int)(t / d.nz);
    const double *co = A.cord_old;
    double xl = 0.0, xr = 0.0;
    if (a.mode_rem == 1) {
        xl = CX(co, d, j, 0);
        xr = CX(co, d, j, d.nx - 1);
    } else if (a.mode_rem == 11 || a.mode_rem == 3) {
        xl = a.x0;
        xr = a.x0 + a.rxbo;
    } else if (a.mode_rem == 4) {
        // every row spans the surface row, which is regridded first
        xl = CX(co, d, 0, 0);
        xr = CX(co, d, 0, d.nx - 1);
        if (j > 0) {
            double x0n = xl + tx[0] * ((xr - xl) / a.ar_x);
            double x1n = xl + tx[d.nx - 1] * ((xr - xl) / a.ar_x);
            xl = x0n;
            xr = x1n;
        }
    }
    A.cord[gf_node(d, j, i)] = xl + tx[i] * ((xr - xl) / a.ar_x);
}

// New z (rem_cord.f90:34-79): surface and bottom by linear interpolation
// of the old rows at the new x, then mesh1 down each column.  One thread per column.
__global__ void __launch_bounds__(GF_THREADS) k_regrid_z(DevArrays A, GfDims d, GfRemeshArgs a, const double *tz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nx) return;
    const int nx = d.nx, nz = d.nz;
    const double *co = A.cord_old;
    double *cord = A.cord;
    for (int j = 0; j < nz; j += nz - 1) {
        double xx = CX(cord, d, j, i);
        double z = CY(co, d, j, i);
        if (xx <= CX(co, d, j, 0)) {
            z = CY(co, d, j, 0);
        } else if (xx >= CX(co, d, j, nx - 1)) {
            z = CY(co, d, j, nx - 1);
        } else {
            for (int ii = 0; ii < nx - 1; ++ii) {
                double xl = CX(co, d, j, ii), xr = CX(co, d, j, ii + 1);
                if (xx >= xl && xx <= xr) {
                    double zl = CY(co, d, j, ii), zr = CY(co, d, j, ii + 1);
                    z = zl + (xx - xl) * (zr - zl) / (xr - xl);
                    break;
                }
            }
        }
        cord[d.N + gf_node(d, j, i)] = z;
        if (nz == 1) break;
    }
    if (!a.is_flex && (a.mode_rem == 3 || a.mode_rem == 1)) cord[d.N + gf_node(d, nz - 1, i)] = a.z0 + a.rzbo;
    double zt = CY(cord, d, 0, i), zb = CY(cord, d, nz - 1, i);
    double mag = (zb - zt) / a.ar_z;
    for (int j = 0; j < nz; ++j) cord[d.N + gf_node(d, j, i)] = zt + tz[j] * mag;
}

// ---------------------------------------------------------------- interpolation
// Old/new element centres (remesh.f90:63-75), planes of E
__global__ void __launch_bounds__(GF_THREADS) k_centres(DevArrays A, GfDims d, double *cold, double *cnew) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
    const double *co = A.cord_old, *cn = A.cord;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        long long o = k * d.N;
        cold[k * d.E + e] = 0.25 * (co[o + gf_node(d, j, i)] + co[o + gf_node(d, j + 1, i)] +
                                    co[o + gf_node(d, j, i + 1)] + co[o + gf_node(d, j + 1, i + 1)]);
        cnew[k * d.E + e] = 0.25 * (cn[o + gf_node(d, j, i)] + cn[o + gf_node(d, j + 1, i)] +
                                    cn[o + gf_node(d, j, i + 1)] + cn[o + gf_node(d, j + 1, i + 1)]);
    }
}

// A (nzt x nxt) grid of points, point (j,i) at i*nzt + j, x plane then y plane.
struct PtGrid {
    const double *xy;
    int nzt, nxt;
    long long P;
    __device__ double X(int j, int i) const { return xy[(long long)i * nzt + j]; }
    __device__ double Y(int j, int i) const { return xy[P + (long long)i * nzt + j]; }
};

// rem_trpars (remesh.f90:267-320): 6 coefficients per old triangle
__global__ void __launch_bounds__(GF_THREADS) k_trpars(PtGrid g, double *pt) {
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long ntri = 2LL * (g.nzt - 1) * (g.nxt - 1);
    if (n >= ntri) return;
    long long cell = n / 2;
    int k = (int)(n % 2) + 1;
    int i = (int)(cell / (g.nzt - 1)), j = (int)(cell % (g.nzt - 1));
    double x1, x2, x3, y1, y2, y3;
    if (k == 1) {
        x1 = g.X(j, i); x2 = g.X(j + 1, i); x3 = g.X(j, i + 1);
        y1 = g.Y(j, i); y2 = g.Y(j + 1, i); y3 = g.Y(j, i + 1);
    } else {
        x1 = g.X(j, i + 1); x2 = g.X(j + 1, i); x3 = g.X(j + 1, i + 1);
        y1 = g.Y(j, i + 1); y2 = g.Y(j + 1, i); y3 = g.Y(j + 1, i + 1);
    }
    double det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
    double *q = pt + n * 6;
    q[0] = (x2 * y3 - y2 * x3) / det;
    q[1] = (y2 - y3) / det;
    q[2] = (x3 - x2) / det;
    q[3] = (x3 * y1 - y3 * x1) / det;
    q[4] = (y3 - y1) / det;
    q[5] = (x1 - x3) / det;
}

__device__ __forceinline__ void weights2(double da, double db, double &wa, double &wb) {
    wa = 1.0 / da / (1.0 / da + 1.0 / db);
    wb = 1.0 / db / (1.0 / da + 1.0 / db);
}

// rem_barcord (remesh.f90:327-439): containing old triangle of each new
// point within +-4 cells, in the reference's search order; else the two
// nearest vertices of the triangle with the smallest sum of squared weights
__global__ void __launch_bounds__(GF_THREADS) k_barcord(PtGrid old, const double *cnew, const double *pt, int *numtr,
                                                        double *bc) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nzt = old.nzt, nxt = old.nxt;
    if (p >= old.P) return;
    int j = (int)(p % nzt), i = (int)(p / nzt);
    double xx = cnew[p], yy = cnew[old.P + p];
    const double perr = 1e-4;
    const int mm = 4;
    double amodmin = 1e10;
    int nmin = 0;
    int io0 = max(0, i - mm), io1 = min(nxt - 2, i + mm), jo0 = max(0, j - mm), jo1 = min(nzt - 2, j + mm);
    for (int io = io0; io <= io1; ++io)
        for (int jo = jo0; jo <= jo1; ++jo)
            for (int k = 1; k <= 2; ++k) {
                int n1 = 2 * ((nzt - 1) * io + jo) + k;
                const double *q = pt + (long long)(n1 - 1) * 6;
                double a1 = q[0] + xx * q[1] + yy * q[2];
                double a2 = q[3] + xx * q[4] + yy * q[5];
                double a3 = 1.0 - a1 - a2;
                double amod = a1 * a1 + a2 * a2 + a3 * a3;
                if (amod < amodmin) {
                    amodmin = amod;
                    nmin = n1;
                }
                if (a1 <= -perr || a1 >= (1.0 + perr)) continue;
                if (a2 <= -perr || a2 >= (1.0 + perr)) continue;
                if (a3 <= -perr || a3 >= (1.0 + perr)) continue;
                numtr[p] = n1;
                bc[p] = a1;
                bc[old.P + p] = a2;
                bc[2 * old.P + p] = a3;
                return;
            }
    numtr[p] = nmin;
    if (nmin <= 0) return; // non-finite coordinates: the interpolation flags it
    int numqu = (nmin + 1) / 2;
    int io = (numqu - 1) / (nzt - 1), jo = numqu - io * (nzt - 1) - 1;
    auto dist = [&](int jj, int ii) {
        double dx = xx - old.X(jj, ii), dy = yy - old.Y(jj, ii);
        return sqrt(dx * dx + dy * dy);
    };
    double d1, d2, d3;
    if (nmin % 2 == 0) {
        d1 = dist(jo, io + 1); d2 = dist(jo + 1, io); d3 = dist(jo + 1, io + 1);
    } else {
        d1 = dist(jo, io); d2 = dist(jo + 1, io); d3 = dist(jo, io + 1);
    }
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    if (d1 > d2) {
        if (d2 > d3) {
            weights2(d2, d3, b1, b2);
        } else if (d1 > d3) {
            weights2(d2, d3, b1, b2);
        } else {
            weights2(d1, d2, b0, b1);
        }
    } else {
        if (d3 > d1) {
            if (d2 > d3)
                weights2(d1, d3, b0, b2);
            else
                weights2(d1, d2, b0, b1);
        } else {
            weights2(d1, d3, b0, b2);
        }
    }
    bc[p] = b0;
    bc[old.P + p] = b1;
    bc[2 * old.P + p] = b2;
}

// rem_interpolate (remesh.f90:445-491): new value of one field plane from
// the copy `src` of its old values; clamp0 applies remesh.f90:117-126 (aps >= 0)
template <class T>
__global__ void __launch_bounds__(GF_THREADS) k_interp(const T *__restrict__ src, T *__restrict__ dst, int nzt,
                                                       long long P, const int *__restrict__ numtr,
                                                       const double *__restrict__ bc, int clamp0, DevClock *C) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    int n = numtr[p];
    if (n <= 0) {
        set_status(C, GF_ERR_NONFINITE, (int)p);
        return;
    }
    int numq = (n + 1) / 2;
    int io = (numq - 1) / (nzt - 1), jo = numq - io * (nzt - 1) - 1;
    auto D = [&](int jj, int ii) { return (double)src[(long long)ii * nzt + jj]; };
    double f1, f2, f3;
    if (n % 2 == 0) {
        f1 = D(jo, io + 1); f2 = D(jo + 1, io); f3 = D(jo + 1, io + 1);
    } else {
        f1 = D(jo, io); f2 = D(jo + 1, io); f3 = D(jo, io + 1);
    }
    double v = bc[p] * f1 + bc[P + p] * f2 + bc[2 * P + p] * f3;
    if (clamp0 && v < 0.0) v = 0.0;
    dst[p] = T(v);
}

// ---------------------------------------------------------------- incoming material
// remesh.f90:129-194: layered phases of the first / last age zone on the
// three element columns next to an inflow wall (serial jl search by one
// thread, the element updates by the block), and aps reset there
template <class R>
__global__ void __launch_bounds__(GF_THREADS) k_incoming(DevClock *C, DevArrays A, GfDims d, GfRemeshArgs a) {
    __shared__ int r_j1[2][GF_MAXZONE_LAYER], r_j2[2][GF_MAXZONE_LAYER], r_ph[2][GF_MAXZONE_LAYER], r_n[2];
    const int nx = d.nx, nz = d.nz, idist = 2;
    const double *cord = A.cord;
    if (threadIdx.x == 0) {
        int ju = 1, jl = 1; // shared by both walls, as in the reference
        for (int side = 0; side < 2; ++side) {
            r_n[side] = 0;
            int on = side == 0 ? a.incoming_left : a.incoming_right;
            if (on != 1) continue;
            int nl = side == 0 ? a.nl_left : a.nl_right;
            const double *hc = side == 0 ? a.hc_left : a.hc_right;
            const int *iph = side == 0 ? a.iph_left : a.iph_right;
            int ic = side == 0 ? 0 : nx - 1; // node column of the wall (0-based)
            for (int m = 0; m < nl - 1; ++m) {
                ju = jl;
                for (int j = jl; j <= nz - 1; ++j)
                    if ((CY(cord, d, 0, ic) - 0.5 * (CY(cord, d, j - 1, ic) + CY(cord, d, j, ic))) > hc[m] * 1e3) {
                        jl = j;
                        break;
                    }
                r_j1[side][r_n[side]] = ju;
                r_j2[side][r_n[side]] = jl - 1;
                r_ph[side][r_n[side]] = iph[m];
                ++r_n[side];
            }
            r_j1[side][r_n[side]] = jl;
            r_j2[side][r_n[side]] = nz - 1;
            r_ph[side][r_n[side]] = iph[nl - 1];
            ++r_n[side];
        }
    }
    __syncthreads();
    R *aps = (R *)A.aps;
    for (int side = 0; side < 2; ++side) {
        int on = side == 0 ? a.incoming_left : a.incoming_right;
        if (on != 1) continue;
        // element columns i1..i2 (1-based)
        int i1 = side == 0 ? 1 : nx - 1 - idist, i2 = side == 0 ? 1 + idist : nx - 1;
        int ncol = i2 - i1 + 1;
        for (int t = threadIdx.x; t < ncol * (nz - 1); t += blockDim.x)
            aps[gf_elem(d, t % (nz - 1), i1 - 1 + t / (nz - 1))] = R(0.0);
        for (int r = 0; r < r_n[side]; ++r) {
            // newphase2marker (marker_data.f90:107-137) on rows j1..j2 (1-based)
            int j1 = r_j1[side][r], j2 = r_j2[side][r], iph = r_ph[side][r];
            int nj = j2 - j1 + 1;
            if (nj <= 0) continue;
            if (iph < 1 || iph > d.nphase) {
                if (threadIdx.x == 0) set_status(C, GF_ERR_ARG, iph);
                continue;
            }
            for (int t = threadIdx.x; t < nj * ncol; t += blockDim.x) {
                int j = j1 - 1 + t % nj, i = i1 - 1 + t / nj;
                long long e = gf_elem(d, j, i);
                int nm = A.nmark_elem[e];
                for (int n = 0; n < nm; ++n)
                    A.mark_phase[A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n] - 1] = (int8_t)iph;
                A.iphase[e] = iph;
                for (int k = 0; k < d.nphase; ++k) A.phase_ratio[gf_pr(d, e, k)] = 0.0;
                A.phase_ratio[gf_pr(d, e, iph - 1)] = 1.0;
            }
        }
        __syncthreads(); // the right wall's columns may overlap the left's on tiny meshes
    }
}

// init_areas (init_areas.f90): 1/det of the four triangles; stop 41 if negative
template <class R> __global__ void __launch_bounds__(GF_THREADS) k_init_areas(DevClock *C, DevArrays A, GfDims d) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
    const double *c = A.cord;
    double x1 = CX(c, d, j, i), y1 = CY(c, d, j, i), x2 = CX(c, d, j + 1, i), y2 = CY(c, d, j + 1, i);
    double x3 = CX(c, d, j, i + 1), y3 = CY(c, d, j, i + 1), x4 = CX(c, d, j + 1, i + 1), y4 = CY(c, d, j + 1, i + 1);
    double ar[4];
    ar[0] = 1.0 / (((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2));
    ar[1] = 1.0 / (((x2 * y4 - y2 * x4) - (x3 * y4 - y3 * x4)) + (x3 * y2 - y3 * x2));
    ar[2] = 1.0 / (((x2 * y4 - y2 * x4) - (x1 * y4 - y1 * x4)) + (x1 * y2 - y1 * x2));
    ar[3] = 1.0 / (((x4 * y3 - y4 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y4 - y1 * x4));
    R *area = (R *)A.area;
    bool neg = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        area[gf_ek(d, e, k)] = R(ar[k]);
        neg = neg || ar[k] < 0;
    }
    if (neg) set_status(C, 41, (int)e);
}

// ---------------------------------------------------------------- markers
// euler2bar (euler2bar.f90:1-98): own element, then rings of 2, 6 and 12
__device__ bool euler2bar(const double *cord, const GfDims &d, double x, double y, double &b1, double &b2, int &ntr,
                          int &ii, int &jj) {
    const int nx = d.nx, nz = d.nz;
    if (check_inside(cord, d, x, y, b1, b2, ntr, ii, jj)) return true;
    const int rings[3] = {2, 6, 12};
    for (int r = 0; r < 3; ++r) {
        int n = rings[r], prev = r == 0 ? 0 : rings[r - 1];
        for (int j = max(0, jj - n); j <= min(nz - 2, jj + n); ++j)
            for (int i = max(0, ii - n); i <= min(nx - 2, ii + n); ++i) {
                if (r == 0) {
                    if (i == ii && j == jj) continue;
                } else if (abs(i - ii) <= prev && abs(j - jj) <= prev) {
                    continue;
                }
                if (check_inside(cord, d, x, y, b1, b2, ntr, i, j)) {
                    ii = i;
                    jj = j;
                    return true;
                }
            }
    }
    return false;
}

// lpeuler2bar (lpeuler2bar.f90:1-62), step 1: locate each live marker
__global__ void __launch_bounds__(GF_THREADS) k_lp_locate(DevArrays A, GfDims d, int nmarkers, int *m_elem,
                                                          int *e_count) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmarkers) return;
    m_elem[m] = -1;
    if (A.mark_dead[m] == 0) return;
    const int nz = d.nz;
    int nt = A.mark_ntriag[m];
    int k = (nt - 1) % 2 + 1;
    int j = ((nt - k) / 2) % (nz - 1);
    int i = (nt - k) / 2 / (nz - 1);
    double b1, b2;
    int ntr;
    if (!euler2bar(A.cord, d, A.mark_a1[m], A.mark_a2[m], b1, b2, ntr, i, j)) {
        A.mark_dead[m] = 0;
        return;
    }
    A.mark_a1[m] = b1;
    A.mark_a2[m] = b2;
    A.mark_ntriag[m] = ntr;
    long long e = gf_elem(d, j, i);
    m_elem[m] = (int)e;
    atomicAdd(&e_count[e], 1);
}

// step 2: group marker indices by element (arbitrary order within a group)
__global__ void __launch_bounds__(GF_THREADS) k_lp_scatter(int nmarkers, const int *m_elem, const int *e_offset,
                                                           int *e_fill, int *m_slot) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmarkers) return;
    int e = m_elem[m];
    if (e < 0) return;
    m_slot[e_offset[e] + atomicAdd(&e_fill[e], 1)] = (int)m;
}

// step 3: the serial loop keeps, per element, the first 32 markers by index
// and kills the others; sort each group and write the element's list
__global__ void __launch_bounds__(GF_THREADS) k_lp_lists(DevArrays A, GfDims d, const int *e_count,
                                                         const int *e_offset, int *m_slot) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    int cnt = e_count[e];
    int *seg = m_slot + e_offset[e];
    for (int a = 1; a < cnt; ++a) {
        int v = seg[a], b = a - 1;
        while (b >= 0 && seg[b] > v) {
            seg[b + 1] = seg[b];
            --b;
        }
        seg[b + 1] = v;
    }
    int keep = cnt < GF_MAX_MARKERS_PER_ELEM ? cnt : GF_MAX_MARKERS_PER_ELEM;
    int *ids = A.mark_id_elem + e * GF_MAX_MARKERS_PER_ELEM;
    for (int n = 0; n < GF_MAX_MARKERS_PER_ELEM; ++n) ids[n] = n < keep ? seg[n] + 1 : 0;
    for (int n = keep; n < cnt; ++n) A.mark_dead[seg[n]] = 0;
    A.nmark_elem[e] = keep;
}

// marker2elem (marker2elem.f90:15-47): random candidates of an element with
// fewer than 5 markers, its own LCG stream (seed nloop + i + j, 1-based);
// count pass (write = 0) or write pass (markers numbered after `base`)
__global__ void __launch_bounds__(GF_THREADS) k_topup(DevClock *C, DevArrays A, GfDims d, int nloop, int write,
                                                      int *e_count, const int *e_offset, int base, const int *total,
                                                      int max_markers) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    if (write && (long long)base + *total > max_markers) {
        // the serial loop runs out of marker slots and stops with 133
        if (e == 0) set_status(C, 133, -1);
        return;
    }
    int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
    int iseed = nloop + (i + 1) + (j + 1);
    int nm0 = A.nmark_elem[e];
    int kinc = nm0, icount = 0, adds = 0;
    const double *c = A.cord;
    int iph = A.iphase[e];
    while (kinc <= 4) {
        double r1 = gf_myrandom(iseed), r2 = gf_myrandom(iseed);
        double x1 = CX(c, d, j, i) * (1 - r1) + CX(c, d, j, i + 1) * r1;
        double y1 = CY(c, d, j, i) * (1 - r1) + CY(c, d, j, i + 1) * r1;
        double x2 = CX(c, d, j + 1, i) * (1 - r1) + CX(c, d, j + 1, i + 1) * r1;
        double y2 = CY(c, d, j + 1, i) * (1 - r1) + CY(c, d, j + 1, i + 1) * r1;
        double xx = x1 * (1 - r2) + x2 * r2, yy = y1 * (1 - r2) + y2 * r2;
        double b1, b2;
        int ntr;
        bool in = check_inside(c, d, xx, yy, b1, b2, ntr, i, j);
        icount = icount + 1;
        if (icount > 100) {
            set_status(C, 133, (int)e);
            break;
        }
        if (!in) continue;
        if (write) {
            int kk = base + e_offset[e] + adds + 1; // 1-based marker number
            A.mark_dead[kk - 1] = 1;
            A.mark_a1[kk - 1] = b1;
            A.mark_a2[kk - 1] = b2;
            A.mark_age[kk - 1] = 0.0;
            A.mark_ntriag[kk - 1] = ntr;
            A.mark_phase[kk - 1] = (int8_t)iph;
            A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + nm0 + adds] = kk;
        }
        adds = adds + 1;
        kinc = kinc + 1;
    }
    if (write)
        A.nmark_elem[e] = nm0 + adds;
    else
        e_count[e] = adds;
}

// marker count after the top-up (device copy read by the host afterwards)
__global__ void k_add_markers(int *nmarkers, const int *total, int max_markers) {
    long long n = (long long)*nmarkers + *total;
    if (n <= max_markers) *nmarkers = (int)n;
}

// exclusive scan of n counts by one block; out has n + 1 entries (total last)
__global__ void __launch_bounds__(1024) k_scan(const int *in, int *out, long long n, int *total) {
    __shared__ int warp_sums[32];
    __shared__ int carry_s;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (long long base = 0; base < n; base += 1024) {
        long long t = base + threadIdx.x;
        int v = t < n ? in[t] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        if (w == 0) {
            int s = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        int carry = carry_s;
        int incl = x + (w > 0 ? warp_sums[w - 1] : 0) + carry;
        if (t < n) out[t] = incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[n] = carry_s;
        *total = carry_s;
    }
}

// jmoho (marker2elem.f90:66-77): first row whose mantle phases exceed 1/2,
// with the reference's flat-memory reads for phase ids above nphase
__global__ void k_jmoho(DevArrays A, GfDims d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nx - 1) return;
    const int mantle[5] = {4, 8, 9, 16, 18};
    long long total = (long long)d.E * d.nphase;
    int jm = d.nz - 1;
    for (int j = 0; j < d.nz - 1; ++j) {
        double sum = 0.0;
        for (int m = 0; m < 5; ++m) {
            long long off = (long long)(mantle[m] - 1) + (long long)d.nphase * gf_elem(d, j, i);
            if (off < total) sum += A.phase_ratio[off];
        }
        if (sum > 0.5) {
            jm = j + 1;
            break;
        }
    }
    A.jmoho[i] = jm;
}

// ---------------------------------------------------------------- surface processes
// diff_topo (fl_move.f90:138-315) on the moved surface, one CTA: the
// diffusion increment of every interior surface node from the positions
// before any of them changes, the edge copies, the limit to half the top
// element's thickness, the accumulators, then the new heights (and their
// hi/lo split in the mixed path).  The magma blocks add zero without melt.
__global__ void __launch_bounds__(1024) k_diff_topo(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A,
                                                    GfDims d) {
    const DevParams &P = *Pp;
    const int nx = d.nx;
    const double dt = C->dt;
    double *cord = A.cord, *dtopo = A.dtopo;
    for (int i = 1 + threadIdx.x; i < nx - 1; i += blockDim.x) {
        double snder = (P.topo_kappa * (CY(cord, d, 0, i + 1) - CY(cord, d, 0, i)) / (CX(cord, d, 0, i + 1) - CX(cord, d, 0, i)) -
                        P.topo_kappa * (CY(cord, d, 0, i) - CY(cord, d, 0, i - 1)) / (CX(cord, d, 0, i) - CX(cord, d, 0, i - 1))) /
                       (CX(cord, d, 0, i + 1) - CX(cord, d, 0, i - 1));
        if (snder < 0) {
            int iph = A.iphase[gf_elem(d, 0, i)];
            snder = snder * P.erodibility[iph - 1];
        }
        dtopo[i] = dt * snder;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        dtopo[0] = dtopo[1];
        dtopo[nx - 1] = dtopo[nx - 2];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        const double lim = 0.5 * (CY(cord, d, 0, i) - CY(cord, d, 1, i));
        const double v = lim < dtopo[i] ? lim : dtopo[i];
        dtopo[i] = v;
        A.dhacc_correction[i] = A.dhacc_correction[i] + v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nx - 1; i += blockDim.x) A.dhacc[i] = A.dhacc[i] + 0.5 * (dtopo[i] + dtopo[i + 1]);
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        const long long n = d.N + gf_node(d, 0, i);
        const double z = cord[n] + dtopo[i];
        cord[n] = z;
        if (A.cord_hi) {
            const float h = (float)z;
            A.cord_hi[n] = h;
            A.cord_lo[n] = (float)(z - (double)h);
        }
    }
}

// count_phase_ratio (marker_data.f90:140-172) of one element
__device__ void count_phase_ratio1(const DevParams &P, DevClock *C, DevArrays &A, const GfDims &d, long long e) {
    int nm = A.nmark_elem[e];
    if (nm == 0) {
        set_status(C, 134, (int)e);
        return;
    }
    int cnt[GF_MAXPH + 1];
    for (int k = 0; k <= GF_MAXPH; ++k) cnt[k] = 0;
    for (int m = 0; m < nm; ++m) {
        int iph = A.mark_phase[A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + m] - 1];
        if (iph >= 1 && iph <= GF_MAXPH) cnt[iph] += 1;
    }
    int best = 0, iph = 1;
    for (int k = 1; k <= P.nphase; ++k) {
        A.phase_ratio[gf_pr(d, e, k - 1)] = cnt[k] / (nm * 1.0);
        if (cnt[k] > best) {
            best = cnt[k];
            iph = k;
        }
    }
    A.iphase[e] = iph;
}

// add_marker (marker_data.f90:41-104) at (x, y) in element (j, i): 1 when
// added, 0 when outside the element, -1 when the element or the marker
// arrays are full
__device__ int add_marker1(DevArrays &A, const GfDims &d, double x, double y, int iph, double age, int j, int i,
                           int max_markers) {
    double b1, b2;
    int ntr;
    if (!check_inside(A.cord, d, x, y, b1, b2, ntr, i, j)) return 0;
    const long long e = gf_elem(d, j, i);
    const int kk = *A.nmarkers + 1, nm = A.nmark_elem[e] + 1;
    if (nm > GF_MAX_MARKERS_PER_ELEM || kk > max_markers) return -1;
    *A.nmarkers = kk;
    A.nmark_elem[e] = nm;
    A.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + nm - 1] = kk;
    A.mark_dead[kk - 1] = 1;
    A.mark_a1[kk - 1] = b1;
    A.mark_a2[kk - 1] = b2;
    A.mark_age[kk - 1] = age;
    A.mark_ntriag[kk - 1] = ntr;
    A.mark_phase[kk - 1] = (int8_t)iph;
    return 1;
}

// add_marker_at_top (fl_move.f90:429-472): a marker of phase kph at a random
// point in the upper dz_ratio of the top element of column i (seed loop +
// i + 1); false after 100 misses (stop 134)
__device__ bool add_marker_at_top1(DevArrays &A, const GfDims &d, int i, double dz_ratio, double time, int loop,
                                   int kph, int max_markers) {
    const double *c = A.cord;
    int iseed = loop + (i + 1), icount = 0;
    while (true) {
        double r1 = gf_myrandom(iseed), r2 = gf_myrandom(iseed);
        double x1 = CX(c, d, 0, i) * (1 - r1) + CX(c, d, 0, i + 1) * r1;
        double y1 = CY(c, d, 0, i) * (1 - r1) + CY(c, d, 0, i + 1) * r1;
        double x2 = CX(c, d, 1, i) * (1 - r1) + CX(c, d, 1, i + 1) * r1;
        double y2 = CY(c, d, 1, i) * (1 - r1) + CY(c, d, 1, i + 1) * r1;
        r2 = r2 * dz_ratio;
        double xx = x1 * (1 - r2) + x2 * r2, yy = y1 * (1 - r2) + y2 * r2;
        int inc = add_marker1(A, d, xx, yy, kph, time, 0, i, max_markers);
        if (inc == 1 || inc == -1) return true;
        if (++icount > 100) return false;
    }
}

// resurface (fl_move.f90:320-426), in two passes that give the serial
// loop's result.  Per surface element: an element whose accumulated erosion
// passes thickness / markers loses its topmost marker (its own marker list
// only, so all elements at once); then, in element order (the markers'
// numbering), deposition adds a sediment marker (ksed1) and accumulated
// extrusion arc markers (kocean1) by add_marker_at_top.  The conditions use
// the element's marker count from before its erosion, as the reference.
// Work flags and counts go to the flexure scratch (free after fl_flexure).
__global__ void __launch_bounds__(GF_THREADS) k_resurface_erode(const DevParams *__restrict__ Pp, DevClock *C,
                                                                DevArrays A, GfDims d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = d.nx, M = GF_MAX_MARKERS_PER_ELEM;
    if (i >= nx - 1) return;
    const double *c = A.cord;
    int *rs = (int *)A.flex;
    const double elz = 0.5 * (CY(c, d, 0, i) - CY(c, d, 1, i) + CY(c, d, 0, i + 1) - CY(c, d, 1, i + 1));
    const double chgtopo = A.dhacc[i];
    const long long e = gf_elem(d, 0, i);
    const int kinc = A.nmark_elem[e];
    int work = 0;
    if (-chgtopo * kinc >= elz && kinc > 1) {
        double ymax = -1e30;
        int kmax = 0;
        for (int k = 1; k <= kinc; ++k) {
            int n = A.mark_id_elem[e * M + k - 1];
            int m = A.mark_ntriag[n - 1];
            int kk = (m - 1) % 2 + 1;
            int jj = ((m - kk) / 2) % (d.nz - 1);
            int ii = (m - kk) / 2 / (d.nz - 1);
            double ba1 = A.mark_a1[n - 1], ba2 = A.mark_a2[n - 1];
            double ba3 = 1.0 - ba1 - ba2;
            int i1, i2, i3, j1, j2, j3;
            if (kk == 1) {
                i1 = ii; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj;
            } else {
                i1 = ii + 1; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj + 1;
            }
            double y = CY(c, d, j1, i1) * ba1 + CY(c, d, j2, i2) * ba2 + CY(c, d, j3, i3) * ba3;
            if (ymax < y) {
                ymax = y;
                kmax = k;
            }
        }
        if (kmax != 0) {
            int nmax = A.mark_id_elem[e * M + kmax - 1];
            A.mark_id_elem[e * M + kmax - 1] = A.mark_id_elem[e * M + kinc - 1];
            A.mark_id_elem[e * M + kinc - 1] = 0;
            A.mark_dead[nmax - 1] = 0;
            A.nmark_elem[e] = A.nmark_elem[e] - 1;
        }
        A.dhacc[i] = 0.0;
        work |= 4;
    }
    if (chgtopo * kinc >= elz && kinc != M) work |= 1;
    if (A.extr_acc[i] * kinc >= elz && kinc != M) work |= 2;
    rs[i] = work;
    rs[nx + i] = kinc;
    if (work == 4) count_phase_ratio1(*Pp, C, A, d, e);
}
// the additions, one warp: 32 columns' flags at a time, the first lane adds
// in column order
__global__ void k_resurface_add(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A, GfDims d, int nloop,
                                int max_markers) {
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const DevParams &P = *Pp;
    const int nx = d.nx, M = GF_MAX_MARKERS_PER_ELEM, lane = threadIdx.x;
    const int *rs = (const int *)A.flex;
    const double *c = A.cord;
    const double time = C->time;
    bool failed = false;
    for (int base = 0; base < nx - 1 && !failed; base += 32) {
        const int ii = base + lane;
        unsigned bal = __ballot_sync(0xffffffffu, ii < nx - 1 && (rs[ii] & 3));
        if (lane == 0)
            while (bal && !failed) {
                const int i = base + __ffs(bal) - 1;
                bal &= bal - 1;
                const int work = rs[i], kinc = rs[nx + i];
                const long long e = gf_elem(d, 0, i);
                const double elz = 0.5 * (CY(c, d, 0, i) - CY(c, d, 1, i) + CY(c, d, 0, i + 1) - CY(c, d, 1, i + 1));
                if (work & 1) { // sedimentation (ksed1)
                    if (!add_marker_at_top1(A, d, i, 0.1, time, nloop, 1, max_markers)) {
                        set_status(C, 134, (int)e);
                        failed = true;
                        break;
                    }
                    A.dhacc[i] = 0.0;
                }
                if (work & 2) { // volcanic extrusion: arc markers, seeds nloop + i + ii (fl_move.f90:403-416)
                    const double chgtopo2 = A.extr_acc[i];
                    const double q = ceil(chgtopo2 / elz * kinc);
                    const int n_to_add = q < (double)(M - kinc) ? (int)q : M - kinc;
                    const double dz_ratio = 1.0 < chgtopo2 / elz ? 1.0 : chgtopo2 / elz;
                    for (int k = 1; k <= n_to_add && !failed; ++k)
                        if (!add_marker_at_top1(A, d, i, dz_ratio, time, nloop + (i + 1) + k, 3, max_markers)) {
                            set_status(C, 134, (int)e);
                            failed = true;
                        }
                    if (failed) break;
                    A.extr_acc[i] = 0.0;
                }
                count_phase_ratio1(P, C, A, d, e);
            }
        failed = __shfl_sync(0xffffffffu, failed, 0);
    }
}

// fl_flexure (fl_flexure.f90:1-189), one CTA: column weights (with the last
// Eff_dens write of `frac` in the reference's serial order), q_init on the
// first call, the plate's rigidity, the block tridiagonal solve on one thread
// (the reference's forward sweep and back substitution), then the new bottom
// heights and the flexure velocity of every column.  Scratch: 12 nx doubles.
template <class R>
__global__ void __launch_bounds__(1024) k_flexure(const DevParams *__restrict__ Pp, DevClock *C, DevArrays A, GfDims d,
                                                  double Te, double rho_m) {
    const DevParams &P = *Pp;
    const int nx = d.nx, nz = d.nz;
    const long long N = d.N;
    const double g = P.g;
    double *q = A.flex, *Load = A.flex + nx, *dx = A.flex + 2 * nx, *D = A.flex + 3 * nx;
    double *cp = A.flex + 4 * nx, *rp = A.flex + 8 * nx, *u = A.flex + 10 * nx;
    __shared__ long long s_pos[1024];
    __shared__ double s_val[1024];
    long long mypos = -1;
    double myval = 0.0;
    bool zero = true;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        long long pos = (long long)i * (2 * nz + 4); // Eff_dens calls of column i, in order
        auto ED = [&](int j, int ie) {
            int w = 0;
            double f = 0.0;
            double r = gfk::eff_dens<R>(P, A, d, j, ie, gf_elem(d, j, ie), &w, &f);
            if (w) {
                mypos = pos;
                myval = f;
            }
            ++pos;
            return r;
        };
        double qi = 0.0;
        for (int j = 0; j < nz - 1; ++j) {
            double rho;
            if (i == 0) {
                rho = ED(j, 0);
            } else if (i == nx - 1) {
                rho = ED(j, nx - 2);
            } else {
                double r1 = ED(j, i - 1), r2 = ED(j, i);
                rho = 0.5 * (r1 + r2);
            }
            double dz = CY(A.cord, d, j, i) - CY(A.cord, d, j + 1, i);
            qi = qi + rho * g * dz;
        }
        double rho_b;
        if (i == 0) {
            rho_b = ED(nz - 2, 0);
        } else if (i == nx - 1) {
            rho_b = ED(nz - 2, nx - 2);
        } else {
            double r1 = ED(nz - 2, i - 1), r2 = ED(nz - 2, i);
            rho_b = 0.5 * (r1 + r2);
        }
        qi = qi - rho_b * g * (A.orig[N + gf_node(d, nz - 1, i)] - CY(A.cord, d, nz - 1, i));
        q[i] = qi;
        zero = zero && A.q_init[i] == 0.0;
    }
    s_pos[threadIdx.x] = mypos;
    s_val[threadIdx.x] = myval;
    const bool all_zero = __syncthreads_and(zero ? 1 : 0) != 0;
    if (threadIdx.x == 0) {
        long long best = -1;
        double v = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t)
            if (s_pos[t] > best) {
                best = s_pos[t];
                v = s_val[t];
            }
        if (best >= 0) C->frac = v;
    }
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        if (all_zero) A.q_init[i] = q[i];
        Load[i] = q[i] - A.q_init[i];
        if (i < nx - 1) {
            double v = CX(A.cord, d, nz - 1, i + 1) - CX(A.cord, d, nz - 1, i);
            dx[i] = v <= 0.0 ? 1.0 : v;
        }
        int iph = i < nx - 1 ? A.iphase[gf_elem(d, nz - 2, i)] : A.iphase[gf_elem(d, nz - 2, nx - 2)];
        if (iph < 1 || iph > P.nphase) iph = 1;
        double lambda = P.rl[iph - 1], mu = P.rm[iph - 1], E, nu;
        if (lambda + mu > 0.0) {
            E = mu * (3.0 * lambda + 2.0 * mu) / (lambda + mu);
            nu = lambda / (2.0 * (lambda + mu));
        } else {
            E = 1.0e11;
            nu = 0.25;
        }
        if (nu >= 1.0 || nu <= -1.0) nu = 0.25;
        double Di = (E * (Te * Te * Te)) / (12.0 * (1.0 - (nu * nu)));
        D[i] = Di <= 0.0 ? 1.0e15 : Di;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double rg = rho_m * g;
        cp[0] = cp[1] = cp[2] = cp[3] = 0.0;
        rp[0] = 0.0;
        rp[1] = rg > 0.0 ? Load[0] / rg : 0.0;
        for (int i = 1; i < nx - 1; ++i) {
            double a_i = 2.0 / (dx[i - 1] * (dx[i] + dx[i - 1]));
            double c_i = 2.0 / (dx[i] * (dx[i] + dx[i - 1]));
            double b_i = -(a_i + c_i);
            double d11 = b_i - a_i * cp[4 * (i - 1) + 0];
            double d12 = -rho_m * g - a_i * cp[4 * (i - 1) + 1];
            double d21 = 1.0 / D[i] - a_i * cp[4 * (i - 1) + 2];
            double d22 = b_i - a_i * cp[4 * (i - 1) + 3];
            double det = d11 * d22 - d12 * d21;
            if (fabs(det) < 1e-30) det = copysign(1e-30, det);
            double i11 = d22 / det, i12 = -d12 / det, i21 = -d21 / det, i22 = d11 / det;
            cp[4 * i + 0] = i11 * c_i;
            cp[4 * i + 1] = i12 * c_i;
            cp[4 * i + 2] = i21 * c_i;
            cp[4 * i + 3] = i22 * c_i;
            double t1 = -Load[i] - a_i * rp[2 * (i - 1)], t2 = 0.0 - a_i * rp[2 * (i - 1) + 1];
            rp[2 * i] = i11 * t1 + i12 * t2;
            rp[2 * i + 1] = i21 * t1 + i22 * t2;
        }
        u[2 * (nx - 1)] = 0.0;
        u[2 * (nx - 1) + 1] = rg > 0.0 ? Load[nx - 1] / rg : 0.0;
        for (int i = nx - 2; i >= 0; --i) {
            u[2 * i] = rp[2 * i] - (cp[4 * i + 0] * u[2 * (i + 1)] + cp[4 * i + 1] * u[2 * (i + 1) + 1]);
            u[2 * i + 1] = rp[2 * i + 1] - (cp[4 * i + 2] * u[2 * (i + 1)] + cp[4 * i + 3] * u[2 * (i + 1) + 1]);
        }
    }
    __syncthreads();
    const double dt = C->dt;
    double *vz = A.vel + N;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        const double vfo = A.vel_flex_old[i];
        for (int j = 0; j < nz - 1; ++j) vz[gf_node(d, j, i)] = vz[gf_node(d, j, i)] - vfo;
        const long long nb = N + gf_node(d, nz - 1, i);
        const double cord_old_z = A.cord[nb];
        A.cord[nb] = A.orig[nb] - u[2 * i + 1];
        double vel_flex = 0.0;
        if (dt > 0.0) vel_flex = (A.cord[nb] - cord_old_z) / dt;
        for (int j = 0; j < nz - 1; ++j) vz[gf_node(d, j, i)] = vz[gf_node(d, j, i)] + vel_flex;
        vz[gf_node(d, nz - 1, i)] = vel_flex;
        A.vel_flex_old[i] = vel_flex;
    }
}

// the surface accumulators length-weighted onto the new surface elements
// (remesh.f90:20-53), one thread, the reference's walk; cordo = the mesh
// before regridding, scratch = 2 (nx - 1) doubles
__global__ void k_surface_acc_remesh(DevArrays A, GfDims d, double *scratch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int nx = d.nx;
    const double *c = A.cord, *co = A.cord_old;
    double *dhnew = scratch, *extnew = scratch + (nx - 1);
    for (int k = 0; k < nx - 1; ++k) dhnew[k] = extnew[k] = 0.0;
    int i = 0, ii = 0;
    double xl = CX(c, d, 0, 0), xr;
    while ((i > ii ? i : ii) < nx - 1) {
        const double xo = CX(co, d, 0, ii + 1), xn = CX(c, d, 0, i + 1);
        xr = xo < xn ? xo : xn;
        if (xl < xr) {
            dhnew[i] = dhnew[i] + A.dhacc[ii] * (xr - xl);
            extnew[i] = extnew[i] + A.extr_acc[ii] * (xr - xl);
        }
        if (xr == xo)
            ii = ii + 1;
        else
            i = i + 1;
        if ((i > ii ? i : ii) < nx - 1) xl = xr;
    }
    for (int k = 0; k < nx - 1; ++k) {
        A.dhacc[k] = dhnew[k] / (CX(c, d, 0, k + 1) - CX(c, d, 0, k));
        A.extr_acc[k] = extnew[k] / (CX(c, d, 0, k + 1) - CX(c, d, 0, k));
    }
}

#include "gf_magma.cuh"

} // namespace gfr
} // namespace

// ---------------------------------------------------------------- launchers
#define GF_RLAUNCH(kern, n, ...)                                                                                       \
    do {                                                                                                               \
        if ((n) > 0) {                                                                                                 \
            kern<<<gfr::blocks_for(n), GF_THREADS, 0, g.s>>>(__VA_ARGS__);                                             \
            ++*g.launches;                                                                                             \
        }                                                                                                              \
    } while (0)

namespace {
// interpolate one field plane through the copy b.plane
template <class T>
void interp_plane(const GfLaunch &g, const GfRemeshBufs &b, T *field, int nzt, long long P, int clamp0) {
    cudaMemcpyAsync(b.plane, field, sizeof(T) * P, cudaMemcpyDeviceToDevice, g.s);
    GF_RLAUNCH(gfr::k_interp<T>, P, (const T *)b.plane, field, nzt, P, b.numtr, b.bc, clamp0, g.C);
}
} // namespace

template <class R> void GfRemesh<R>::regrid(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b) {
    using namespace gfr;
    const GfDims &d = g.d;
    const DevArrays &A = g.A;
    GF_RLAUNCH(k_bar2euler, (long long)a.nmarkers, A, d, a.nmarkers, a.has_dhacc);
    cudaMemcpyAsync(A.cord_old, A.cord, sizeof(double) * 2 * d.N, cudaMemcpyDeviceToDevice, g.s);
    GF_RLAUNCH(k_regrid_x, d.N, A, d, a, b.tx);
    GF_RLAUNCH(k_regrid_z, (long long)d.nx, A, d, a, b.tz);
    k_surface_acc_remesh<<<1, 1, 0, g.s>>>(A, d, b.plane);
    ++*g.launches;
    // element-wise fields on the element-centre grid (remesh.f90:57-127)
    int nzt = d.nz - 1, nxt = d.nx - 1;
    GF_RLAUNCH(k_centres, d.E, A, d, b.cold, b.cnew);
    PtGrid ge{b.cold, nzt, nxt, d.E};
    GF_RLAUNCH(k_trpars, 2LL * (nzt - 1) * (nxt - 1), ge, b.pt);
    GF_RLAUNCH(k_barcord, d.E, ge, (const double *)b.cnew, (const double *)b.pt, b.numtr, b.bc);
    R *st = (R *)A.stress0;
    for (int p = 0; p < 16; ++p) interp_plane<R>(g, b, st + p * d.E, nzt, d.E, 0);
    if (sizeof(R) == sizeof(float)) interp_plane<double>(g, b, A.p_ref, nzt, d.E, 0);
    for (int k = 0; k < 3; ++k) interp_plane<R>(g, b, (R *)A.strain + k * d.E, nzt, d.E, 0);
    interp_plane<R>(g, b, (R *)A.aps, nzt, d.E, 1);
    if (A.dike_backlog) // magma pools and dike / MOR accumulators (remesh.f90:106-115)
        for (double *f : {A.fmagma, A.fmagma2, A.dike_backlog, A.dike_marker_vol, A.mor_marker_vol})
            interp_plane<double>(g, b, f, nzt, d.E, 0);
    if (a.incoming_left == 1 || a.incoming_right == 1) {
        k_incoming<R><<<1, GF_THREADS, 0, g.s>>>(g.C, A, d, a);
        ++*g.launches;
    }
    interp_plane<double>(g, b, A.source, nzt, d.E, 0);
    // node-wise fields on the old node mesh (remesh.f90:200-235)
    cudaMemcpyAsync(A.temp0, A.temp, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, g.s);
    PtGrid gn{A.cord_old, d.nz, d.nx, d.N};
    GF_RLAUNCH(k_trpars, 2LL * (d.nz - 1) * (d.nx - 1), gn, b.pt);
    GF_RLAUNCH(k_barcord, d.N, gn, (const double *)A.cord, (const double *)b.pt, b.numtr, b.bc);
    for (int k = 0; k < 2; ++k) interp_plane<double>(g, b, A.vel + k * d.N, d.nz, d.N, 0);
    interp_plane<double>(g, b, A.temp, d.nz, d.N, 0);
    // xoriginal, zoriginal (remesh.f90:242-243)
    for (int k = 0; k < 2; ++k) interp_plane<double>(g, b, A.orig + k * d.N, d.nz, d.N, 0);
}

template <class R> void GfRemesh<R>::init_areas(const GfLaunch &g) {
    using namespace gfr;
    GF_RLAUNCH(k_init_areas<R>, g.d.E, g.C, g.A, g.d);
}

template <class R> void GfRemesh<R>::rebin_markers(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b) {
    using namespace gfr;
    const GfDims &d = g.d;
    cudaMemsetAsync(b.e_count, 0, sizeof(int) * d.E, g.s);
    cudaMemsetAsync(b.e_fill, 0, sizeof(int) * d.E, g.s);
    GF_RLAUNCH(k_lp_locate, (long long)a.nmarkers, g.A, d, a.nmarkers, b.m_elem, b.e_count);
    k_scan<<<1, 1024, 0, g.s>>>(b.e_count, b.e_offset, d.E, b.d_scalars);
    ++*g.launches;
    GF_RLAUNCH(k_lp_scatter, (long long)a.nmarkers, a.nmarkers, (const int *)b.m_elem, (const int *)b.e_offset,
               b.e_fill, b.m_slot);
    GF_RLAUNCH(k_lp_lists, d.E, g.A, d, (const int *)b.e_count, (const int *)b.e_offset, b.m_slot);
}

template <class R> void GfRemesh<R>::top_up_markers(const GfLaunch &g, const GfRemeshArgs &a, const GfRemeshBufs &b) {
    using namespace gfr;
    const GfDims &d = g.d;
    GF_RLAUNCH(k_topup, d.E, g.C, g.A, d, a.nloop, 0, b.e_count, (const int *)b.e_offset, a.nmarkers,
               (const int *)b.d_scalars, a.max_markers);
    k_scan<<<1, 1024, 0, g.s>>>(b.e_count, b.e_offset, d.E, b.d_scalars);
    ++*g.launches;
    GF_RLAUNCH(k_topup, d.E, g.C, g.A, d, a.nloop, 1, b.e_count, (const int *)b.e_offset, a.nmarkers,
               (const int *)b.d_scalars, a.max_markers);
    k_add_markers<<<1, 1, 0, g.s>>>(g.A.nmarkers, (const int *)b.d_scalars, a.max_markers);
    ++*g.launches;
}

template <class R> void GfRemesh<R>::jmoho(const GfLaunch &g) {
    using namespace gfr;
    if (g.A.jmoho) GF_RLAUNCH(k_jmoho, (long long)(g.d.nx - 1), g.A, g.d);
}

template <class R> void GfRemesh<R>::flexure(const GfLaunch &g, double Te, double rho_m) {
    using namespace gfr;
    k_flexure<R><<<1, 1024, 0, g.s>>>(g.P, g.C, g.A, g.d, Te, rho_m);
    ++*g.launches;
}

template <class R> void GfRemesh<R>::diff_topo(const GfLaunch &g, int resurface, int nloop, int max_markers) {
    using namespace gfr;
    k_diff_topo<<<1, 1024, 0, g.s>>>(g.P, g.C, g.A, g.d);
    ++*g.launches;
    if (g.A.dike_backlog && g.d.nx > 3) { // magma sub-model: arc extrusion and MOR crust
        const long long ncol = g.d.nx - 3;
        if (g.arc_rate > 0) {
            GF_RLAUNCH(k_arc_cols, 32 * ncol, g.P, g.C, g.A, g.d, g.arc_rate); // one warp per column
            GF_RLAUNCH(k_arc_nodes, (long long)g.d.nx, g.A, g.d);
        }
        GF_RLAUNCH(k_mor_cols, 32 * ncol, g.P, g.C, g.A, g.d);
        k_mor_chain<<<1, 32, 0, g.s>>>(g.A, g.d);
        ++*g.launches;
    }
    if (resurface) {
        GF_RLAUNCH(k_resurface_erode, (long long)(g.d.nx - 1), g.P, g.C, g.A, g.d);
        k_resurface_add<<<1, 32, 0, g.s>>>(g.P, g.C, g.A, g.d, nloop, max_markers);
        ++*g.launches;
    }
}

template struct GfRemesh<double>;
template struct GfRemesh<float>;

// ---------------------------------------------------------------- magma sub-model
namespace {
// the elements of `mode` in serial order into list, their number into *count
void mg_compact(const GfLaunch &g, int mode, int *list, int *count) {
    const unsigned nb = (unsigned)((g.d.E + gfr::MG_CB - 1) / gfr::MG_CB);
    gfr::k_mg_count<<<nb, gfr::MG_CB, 0, g.s>>>(g.A, g.d, mode);
    gfr::k_mg_write<<<nb, gfr::MG_CB, 0, g.s>>>(g.A, g.d, mode, list, count);
    *g.launches += 2;
}
} // namespace

void GfMagma::melting(const GfLaunch &g) {
    using namespace gfr;
    const DevArrays &A = g.A;
    GF_RLAUNCH(k_mg_cols, (long long)(g.d.nx - 1), A, g.d, 0);
    GF_RLAUNCH(k_melt_flags, g.d.E, g.P, A, g.d);
    mg_compact(g, MG_PRED_MASK, A.mg_list, A.mg_i + MI_COUNT);
    GF_RLAUNCH(k_melt_prep, g.d.E, g.P, A, g.d);
    k_melt_order<<<1, MG_CB, 0, g.s>>>(A, g.d);
    k_melt_serial<<<1, MG_CB, 0, g.s>>>(g.P, A, g.d);
    *g.launches += 2;
}

void GfMagma::therm(const GfLaunch &g, int max_markers) {
    using namespace gfr;
    const GfDims &d = g.d;
    const DevArrays &A = g.A;
    GF_RLAUNCH(k_mg_freeze, d.E, g.P, g.C, A, d);
    GF_RLAUNCH(k_mg_freeze_nodes, d.N, g.P, A, d);
    mg_compact(g, MG_PRED_W, A.mg_list, A.mg_i + MI_COUNT);
    k_mg_zone1<<<1, MG_CB, 0, g.s>>>(g.P, A, d);
    GF_RLAUNCH(k_mg_find, d.E, A, d);
    k_mg_zone2<<<1, MG_CB, 0, g.s>>>(g.P, A, d);
    *g.launches += 2;
    GF_RLAUNCH(k_mg_cols, (long long)(d.nx - 1), A, d, 1);
    // the MOR sources and the dike / mantle-cone sources, each in serial order
    mg_compact(g, MG_PRED_MOR, A.mg_list, A.mg_i + MI_COUNT);
    GF_RLAUNCH(k_mg_src, d.E, g.P, g.C, A, d, (const int *)A.mg_list, (const int *)(A.mg_i + MI_COUNT), A.mg_src);
    mg_compact(g, MG_PRED_ARC, A.mg_list2, A.mg_i + MI_COUNT2);
    GF_RLAUNCH(k_mg_src, d.E, g.P, g.C, A, d, (const int *)A.mg_list2, (const int *)(A.mg_i + MI_COUNT2), A.mg_src2);
    GF_RLAUNCH(k_mg_migrate, 4 * ((d.E + 31) / 32) * 32, g.P, A, d); // four threads per element
    GF_RLAUNCH(k_mg_release, d.E, g.P, A, d);
    mg_compact(g, MG_PRED_MASK, A.mg_list, A.mg_i + MI_COUNT);
    k_mg_markers<<<1, 1, 0, g.s>>>(g.P, g.C, A, d, max_markers);
    ++*g.launches;
}
