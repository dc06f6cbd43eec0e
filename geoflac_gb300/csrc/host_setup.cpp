// Host part of the reference's start-up (src/setflac.f90:4-66).
//
// One-time work, run on the host in FP64 in the reference's serial order so
// that the initial state (mesh, markers, phases, temperatures, stresses,
// boundary codes) is the one the reference builds.  rmasses, init_visc and
// dt_mass then run on the device (gf_finish_setflac).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/geoflac_gb300.h"
#include "gf_index.h"

namespace {

struct Stop {
    int code;
};

struct S {
    gf_params *p;
    gf_clock *c;
    gf_layout *L;
    GfDims d;
    double &cord(int j, int i, int k) { return L->cord[gf_n2(d, j, i, k)]; }
    double &temp(int j, int i) { return L->temp[gf_node(d, j, i)]; }
    double &bc(int j, int i, int k) { return L->bc[gf_n2(d, j, i, k)]; }
    int &ncod(int j, int i, int k) { return L->ncod[gf_n2(d, j, i, k)]; }
    long long e(int j, int i) { return gf_elem(d, j, i); }
};

// Square-and-multiply integer power (the evaluation of real**integer).
double ipow(double x, int m) {
    unsigned n = m < 0 ? (unsigned)(-m) : (unsigned)m;
    double y = (n % 2) ? x : 1.0;
    while (n >>= 1) {
        x = x * x;
        if (n % 2) y = y * x;
    }
    return m < 0 ? 1.0 / y : y;
}

// mesh1 (src/init_cord.f90:141-179): 1-D zoned mesh between x1 and x2.
void mesh1(double x1, double x2, double *xmesh, int n, int nzon, const int *nelz, const double *sizez) {
    double all_ratio = 0.0;
    int nel = 0;
    xmesh[0] = 0.0;
    for (int k = 0; k < nzon - 1; k += 2) {
        all_ratio = all_ratio + nelz[k] * sizez[k];
        for (int i = 0; i < nelz[k]; ++i) {
            nel = nel + 1;
            xmesh[nel] = xmesh[nel - 1] + sizez[k];
        }
        double ratio = std::pow(sizez[k + 2] / sizez[k], 1.0 / (double)(nelz[k + 1] + 1));
        for (int i = 1; i <= nelz[k + 1]; ++i) {
            nel = nel + 1;
            xmesh[nel] = xmesh[nel - 1] + sizez[k] * ipow(ratio, i);
            all_ratio = all_ratio + sizez[k] * ipow(ratio, i);
        }
    }
    for (int k = 0; k < nelz[nzon - 1]; ++k) {
        nel = nel + 1;
        xmesh[nel] = xmesh[nel - 1] + sizez[nzon - 1];
    }
    all_ratio = all_ratio + nelz[nzon - 1] * sizez[nzon - 1];
    double magnification = (x2 - x1) / all_ratio;
    for (int k = 0; k < n; ++k) xmesh[k] = x1 + xmesh[k] * magnification;
}

// init_cord (src/init_cord.f90:5-89) and test_grid (:97-134).
void init_cord(S &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    std::vector<double> rmesh(nx + nz + 2);
    if (p.ircoord > 0) {
        FILE *f = std::fopen(p.coordfile, "r");
        if (!f) throw Stop{21};
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < nz; ++j) {
                double x, y;
                if (std::fscanf(f, "%lf %lf", &x, &y) != 2) {
                    std::fclose(f);
                    throw Stop{21};
                }
                s.cord(j, i, 0) = x;
                s.cord(j, i, 1) = y;
            }
        std::fclose(f);
    } else {
        int nelsum = 0;
        for (int i = 0; i < p.nzonx; ++i) nelsum += p.nelz_x[i];
        if (p.nzonx != 0 && p.nzonx % 2 == 0) throw Stop{16};
        if (nelsum != nx - 1) throw Stop{17};
        nelsum = 0;
        for (int i = 0; i < p.nzony; ++i) nelsum += p.nelz_y[i];
        if (p.nzony != 0 && p.nzony % 2 == 0) throw Stop{18};
        if (nelsum != nz - 1) throw Stop{19};

        mesh1(p.x0, p.x0 + p.rxbo, rmesh.data(), nx, p.nzonx, p.nelz_x, p.sizez_x);
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < nz; ++j) s.cord(j, i, 0) = rmesh[i];
        mesh1(p.z0, p.z0 + p.rzbo, rmesh.data(), nz, p.nzony, p.nelz_y, p.sizez_y);
        for (int j = 0; j < nz; ++j)
            for (int i = 0; i < nx; ++i) s.cord(j, i, 1) = rmesh[j];
        // topography perturbations (init_cord.f90:49-66), 1-based node ranges
        for (int n = 0; n < p.inhom; ++n) {
            if (p.igeom[n] == 20) {
                double amp = p.xinitaps[n];
                for (int i = p.ix1[n]; i <= p.ix2[n]; ++i) s.cord(0, i - 1, 1) += amp;
            } else if (p.igeom[n] == 21) {
                double amp = p.xinitaps[n];
                for (int j = p.ix1[n]; j <= p.ix2[n] - 1; ++j)
                    s.cord(0, j - 1, 1) += amp * (double)(float)(j - p.ix1[n]) / (p.ix2[n] - p.ix1[n]);
                for (int i = p.ix2[n]; i <= p.iy1[n]; ++i) s.cord(0, i - 1, 1) += amp;
                for (int j = p.iy1[n] + 1; j <= p.iy2[n]; ++j)
                    s.cord(0, j - 1, 1) += amp * (double)(float)(p.iy2[n] - j) / (p.iy2[n] - p.iy1[n]);
            }
        }
        for (int i = 0; i < nx; ++i) {
            mesh1(s.cord(0, i, 1), s.cord(nz - 1, i, 1), rmesh.data(), nz, p.nzony, p.nelz_y, p.sizez_y);
            for (int j = 0; j < nz; ++j) s.cord(j, i, 1) = rmesh[j];
        }
    }
    double dxmin = 1e300, dzmin = 1e300;
    for (int i = 1; i < nx; ++i) dxmin = std::fmin(dxmin, s.cord(0, i, 0) - s.cord(0, i - 1, 0));
    for (int j = 0; j < nz - 1; ++j) dzmin = std::fmin(dzmin, s.cord(j, 0, 1) - s.cord(j + 1, 0, 1));
    p.dxmin = dxmin;
    p.dzmin = dzmin;
    if (s.L->dhacc_correction)
        for (int i = 0; i < nx; ++i) s.L->dhacc_correction[i] = 0.0;
    for (double *a : {s.L->dhacc, s.L->extr_acc, s.L->dtopo, s.L->q_init, s.L->vel_flex_old})
        if (a)
            for (int i = 0; i < nx; ++i) a[i] = 0.0;
}

// init_phase (src/init_phase.f90:5-53); element ranges are 1-based.
void init_phase(S &s) {
    gf_params &p = *s.p;
    if (p.irphase > 0) {
        FILE *f = std::fopen(p.phasefile, "r");
        if (!f) throw Stop{21};
        for (int i = 0; i < p.nx - 1; ++i)
            for (int j = 0; j < p.nz - 1; ++j) {
                int ii, jj, ph;
                if (std::fscanf(f, "%d %d %d", &ii, &jj, &ph) != 3) {
                    std::fclose(f);
                    throw Stop{21};
                }
                s.L->iphase[s.e(j, i)] = ph;
            }
        std::fclose(f);
    }
    for (int n = 0; n < p.inhom; ++n) {
        if (p.igeom[n] == 0) {
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j)
                for (int k = p.iy1[n]; k <= p.iy2[n]; ++k) {
                    if (p.inphase[n] > 0) s.L->iphase[s.e(k - 1, j - 1)] = p.inphase[n];
                    s.L->aps[s.e(k - 1, j - 1)] = p.xinitaps[n];
                }
        }
        if (p.igeom[n] == 3) {
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                float t = (float)(p.iy2[n] - p.iy1[n]) / (float)(p.ix2[n] - p.ix1[n]) * (float)(j - p.ix1[n]);
                int k = (int)std::lround(t) + p.iy1[n];
                if (p.inphase[n] > 0) s.L->iphase[s.e(k - 1, j - 1)] = p.inphase[n];
            }
        }
        if (p.igeom[n] == 4) {
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                float t = (float)(p.iy2[n] - p.iy1[n]) / (float)(p.ix2[n] - p.ix1[n]) * (float)(j - p.ix1[n]);
                int k1 = (int)std::floor(t) + p.iy1[n];
                int k2 = (int)std::ceil(t) + p.iy1[n];
                for (int k = k1; k <= k2; ++k) {
                    s.L->aps[s.e(k - 1, j - 1)] = p.xinitaps[n];
                    if (p.inphase[n] > 0) s.L->iphase[s.e(k - 1, j - 1)] = p.inphase[n];
                }
            }
        }
    }
}

// check_inside (src/euler2bar.f90:102-161): the two triangles of quad (j,i).
int check_inside(S &s, double x, double y, double &bar1, double &bar2, int &ntr, int i, int j) {
    for (int k = 0; k < 2; ++k) {
        double x1, x2, x3, y1, y2, y3;
        if (k == 0) {
            x1 = s.cord(j, i, 0); x2 = s.cord(j + 1, i, 0); x3 = s.cord(j, i + 1, 0);
            y1 = s.cord(j, i, 1); y2 = s.cord(j + 1, i, 1); y3 = s.cord(j, i + 1, 1);
        } else {
            x1 = s.cord(j, i + 1, 0); x2 = s.cord(j + 1, i, 0); x3 = s.cord(j + 1, i + 1, 0);
            y1 = s.cord(j, i + 1, 1); y2 = s.cord(j + 1, i, 1); y3 = s.cord(j + 1, i + 1, 1);
        }
        double det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
        double m11 = (x2 * y3 - y2 * x3) / det;
        double m12 = (y2 - y3) / det;
        double m13 = (x3 - x2) / det;
        double m21 = (x3 * y1 - y3 * x1) / det;
        double m22 = (y3 - y1) / det;
        double m23 = (x1 - x3) / det;
        bar1 = (m11 + m12 * x) + y * m13;
        bar2 = (m21 + m22 * x) + y * m23;
        if (bar1 >= 0.0 && bar2 >= 0.0 && bar1 + bar2 <= 1.0) {
            ntr = 2 * ((s.p->nz - 1) * i + j) + k + 1;
            return 1;
        }
    }
    return 0;
}

// add_marker (src/marker_data.f90:41-104), serial numbering.
int add_marker(S &s, double x, double y, int iph, double age, int j, int i) {
    double b1, b2;
    int ntr;
    if (!check_inside(s, x, y, b1, b2, ntr, i, j)) return 0;
    int kk = s.c->nmarkers + 1;
    long long e = s.e(j, i);
    int nm = s.L->nmark_elem[e] + 1;
    if (nm > GF_MAX_MARKERS_PER_ELEM || kk > s.L->max_markers) return -1;
    s.c->nmarkers = kk;
    s.L->nmark_elem[e] = nm;
    s.L->mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + (nm - 1)] = kk;
    s.L->mark_dead[kk - 1] = 1;
    s.L->mark_a1[kk - 1] = b1;
    s.L->mark_a2[kk - 1] = b2;
    s.L->mark_age[kk - 1] = age;
    s.L->mark_ntriag[kk - 1] = ntr;
    s.L->mark_phase[kk - 1] = (int8_t)iph;
    return 1;
}

// count_phase_ratio (src/marker_data.f90:140-172).
void count_phase_ratio(S &s, int j, int i) {
    long long e = s.e(j, i);
    int nm = s.L->nmark_elem[e];
    if (nm == 0) throw Stop{134};
    int cnt[GF_MAXPH + 1] = {0};
    for (int n = 0; n < nm; ++n) {
        int kk = s.L->mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n];
        int iph = s.L->mark_phase[kk - 1];
        if (iph >= 1 && iph <= GF_MAXPH) cnt[iph] += 1;
    }
    for (int k = 1; k <= s.p->nphase; ++k) s.L->phase_ratio[gf_pr(s.d, e, k - 1)] = cnt[k] / (nm * 1.0);
    int iph = 1, best = 0;
    for (int k = 1; k <= s.p->nphase; ++k)
        if (cnt[k] > best) {
            best = cnt[k];
            iph = k;
        }
    s.L->iphase[e] = iph;
}

// marker2elem (src/marker2elem.f90:1-81), serial order.
void marker2elem(S &s) {
    int nx = s.p->nx, nz = s.p->nz;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            int iseed = s.c->nloop + (i + 1) + (j + 1);
            int kinc = s.L->nmark_elem[s.e(j, i)];
            int icount = 0;
            while (kinc <= 4) {
                double r1 = gf_myrandom(iseed);
                double r2 = gf_myrandom(iseed);
                double x1 = s.cord(j, i, 0) * (1 - r1) + s.cord(j, i + 1, 0) * r1;
                double y1 = s.cord(j, i, 1) * (1 - r1) + s.cord(j, i + 1, 1) * r1;
                double x2 = s.cord(j + 1, i, 0) * (1 - r1) + s.cord(j + 1, i + 1, 0) * r1;
                double y2 = s.cord(j + 1, i, 1) * (1 - r1) + s.cord(j + 1, i + 1, 1) * r1;
                double xx = x1 * (1 - r2) + x2 * r2;
                double yy = y1 * (1 - r2) + y2 * r2;
                int inc = add_marker(s, xx, yy, s.L->iphase[s.e(j, i)], 0.0, j, i);
                icount = icount + 1;
                if (icount > 100) throw Stop{133};
                if (inc <= 0) continue;
                kinc = kinc + 1;
            }
            count_phase_ratio(s, j, i);
        }
    // Moho (marker2elem.f90:66-77).  The reference sums phase_ratio over the
    // mantle phase ids 4,8,9,16,18 even when nphase is smaller; the flat
    // offset then lands in a neighbouring element's entries, which is what
    // is reproduced here (entries past the end of the array count as 0).
    static const int mantle[5] = {4, 8, 9, 16, 18};
    long long total = (long long)s.d.E * s.p->nphase;
    if (s.L->jmoho) {
        for (int i = 0; i < nx - 1; ++i) {
            s.L->jmoho[i] = nz - 1;
            for (int j = 0; j < nz - 1; ++j) {
                double sum = 0.0;
                for (int m = 0; m < 5; ++m) {
                    long long off = (long long)(mantle[m] - 1) + (long long)s.p->nphase * s.e(j, i);
                    if (off < total) sum += s.L->phase_ratio[off];
                }
                if (sum > 0.5) {
                    s.L->jmoho[i] = j + 1;
                    break;
                }
            }
        }
    }
}

// newphase2marker (src/marker_data.f90:107-137), 1-based element ranges.
void newphase2marker(S &s, int j1, int j2, int i1, int i2, int iph) {
    for (int i = i1; i <= i2; ++i)
        for (int j = j1; j <= j2; ++j) {
            long long e = s.e(j - 1, i - 1);
            for (int n = 0; n < s.L->nmark_elem[e]; ++n) {
                int kk = s.L->mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + n];
                s.L->mark_phase[kk - 1] = (int8_t)iph;
            }
            s.L->iphase[e] = iph;
            for (int k = 0; k < s.p->nphase; ++k) s.L->phase_ratio[gf_pr(s.d, e, k)] = 0.0;
            s.L->phase_ratio[gf_pr(s.d, e, iph - 1)] = 1.0;
        }
}

// init_marker (src/init_marker.f90:1-164).  With markers_per_side = 3 this is
// the reference's 9-point pattern; other values place m x m points with the
// same construction (an extension with no reference counterpart).
void init_marker(S &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    int ms = p.markers_per_side > 0 ? p.markers_per_side : 3;
    const double half = 0.5;
    const double onesixth = 0.1666666666666666666666;
    const double fivesixth = 0.8333333333333333333333;
    std::memset(s.L->mark_id_elem, 0, sizeof(int) * (size_t)s.d.E * GF_MAX_MARKERS_PER_ELEM);
    std::memset(s.L->nmark_elem, 0, sizeof(int) * (size_t)s.d.E);
    s.c->nmarkers = 0;
    int iseed = 0;
    std::vector<double> w0(ms), w1(ms); // weights of the near / far node
    if (ms == 3) {
        w0[0] = fivesixth; w1[0] = onesixth;
        w0[1] = half;      w1[1] = half;
        w0[2] = onesixth;  w1[2] = fivesixth;
    } else {
        for (int m = 0; m < ms; ++m) {
            double t = (2.0 * m + 1.0) / (2.0 * ms);
            w0[m] = 1.0 - t;
            w1[m] = t;
        }
    }
    std::vector<double> ax(ms), ay(ms), bx(ms), by(ms), px(ms * ms), py(ms * ms);
    double hhc[GF_MAXZONE_LAYER];
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            for (int m = 0; m < ms; ++m) {
                ax[m] = s.cord(j, i, 0) * w0[m] + s.cord(j + 1, i, 0) * w1[m];
                ay[m] = s.cord(j, i, 1) * w0[m] + s.cord(j + 1, i, 1) * w1[m];
                bx[m] = s.cord(j, i + 1, 0) * w0[m] + s.cord(j + 1, i + 1, 0) * w1[m];
                by[m] = s.cord(j, i + 1, 1) * w0[m] + s.cord(j + 1, i + 1, 1) * w1[m];
            }
            for (int m = 0; m < ms; ++m)
                for (int q = 0; q < ms; ++q) {
                    px[m * ms + q] = ax[m] * w0[q] + bx[m] * w1[q];
                    py[m * ms + q] = ay[m] * w0[q] + by[m] * w1[q];
                }
            double dx = s.cord(j, i + 1, 0) - s.cord(j, i, 0);
            double dy = s.cord(j + 1, i, 1) - s.cord(j, i, 1);
            iseed = iseed + (i + 1) + (j + 1);
            int l = 0;
            int ii = i + 1; // 1-based column for the zone tests
            int guard = 0;
            while (l < ms * ms) {
                int kph = s.L->iphase[s.e(j, i)];
                double rx = gf_myrandom(iseed);
                double ry = gf_myrandom(iseed);
                rx = 0.5 - rx;
                ry = 0.5 - ry;
                // the reference's jitter is a third of the element (one
                // point spacing for its 3 x 3 pattern); m x m points keep it
                // at one spacing, dx / m
                double ddx = dx * rx / ms;
                double ddy = dy * ry / ms;
                double xx = px[l] + ddx;
                double yy = py[l] + ddy;
                for (int n = 0; n < p.nzone_age; ++n) {
                    if (ii < p.ixtb1[n] || ii > p.ixtb2[n]) continue;
                    if (n != 0 && p.iph_col_trans[n - 1] == 1) continue;
                    int nl = p.nph_layer[n];
                    for (int m = 0; m < nl - 1; ++m) hhc[m] = p.hc[n][m];
                    if (p.iph_col_trans[n] == 1) {
                        int i1 = p.ixtb1[n], i2 = p.ixtb2[n];
                        double r = (s.cord(0, i, 0) - s.cord(0, i1 - 1, 0)) / (s.cord(0, i2 - 1, 0) - s.cord(0, i1 - 1, 0));
                        for (int m = 0; m < nl - 1; ++m) hhc[m] = p.hc[n][m] + (p.hc[n + 1][m] - p.hc[n][m]) * r;
                    }
                    double yyy = yy * (-1e-3);
                    int m = 0;
                    for (; m < nl - 1; ++m)
                        if (yyy < hhc[m]) break;
                    kph = p.iph_col[n][m];
                }
                int inc = add_marker(s, xx, yy, kph, 0.0, j, i);
                if (++guard > 100000) throw Stop{133};
                if (inc <= 0) continue;
                l = l + 1;
            }
        }
    // initial heterogeneities (init_marker.f90:131-160)
    for (int n = 0; n < p.inhom; ++n) {
        if (p.inphase[n] < 0) continue;
        if (p.igeom[n] == 0) newphase2marker(s, p.iy1[n], p.iy2[n], p.ix1[n], p.ix2[n], p.inphase[n]);
        if (p.igeom[n] == 3) {
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                float t = (float)(p.iy2[n] - p.iy1[n]) / (float)(p.ix2[n] - p.ix1[n]) * (float)(j - p.ix1[n]);
                int k = (int)std::lround(t) + p.iy1[n];
                newphase2marker(s, k, k, j, j, p.inphase[n]);
            }
        }
        if (p.igeom[n] == 4) {
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                float t = (float)(p.iy2[n] - p.iy1[n]) / (float)(p.ix2[n] - p.ix1[n]) * (float)(j - p.ix1[n]);
                int k1 = (int)std::floor(t) + p.iy1[n];
                int k2 = (int)std::ceil(t) + p.iy1[n];
                if (p.inphase[n] >= 0) newphase2marker(s, k1, k2, j, j, p.inphase[n]);
            }
        }
    }
    marker2elem(s);
}

// init_areas (src/init_areas.f90:8-55): area = 1/det (inverse double area).
void init_areas(S &s) {
    int nx = s.p->nx, nz = s.p->nz;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < nz - 1; ++j) {
            double x1 = s.cord(j, i, 0), y1 = s.cord(j, i, 1);
            double x2 = s.cord(j + 1, i, 0), y2 = s.cord(j + 1, i, 1);
            double x3 = s.cord(j, i + 1, 0), y3 = s.cord(j, i + 1, 1);
            double x4 = s.cord(j + 1, i + 1, 0), y4 = s.cord(j + 1, i + 1, 1);
            long long e = s.e(j, i);
            double det;
            det = ((x2 * y3 - y2 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y2 - y1 * x2);
            s.L->area[gf_ek(s.d, e, 0)] = 1.0 / det;
            det = ((x2 * y4 - y2 * x4) - (x3 * y4 - y3 * x4)) + (x3 * y2 - y3 * x2);
            s.L->area[gf_ek(s.d, e, 1)] = 1.0 / det;
            det = ((x2 * y4 - y2 * x4) - (x1 * y4 - y1 * x4)) + (x1 * y2 - y1 * x2);
            s.L->area[gf_ek(s.d, e, 2)] = 1.0 / det;
            det = ((x4 * y3 - y4 * x3) - (x1 * y3 - y1 * x3)) + (x1 * y4 - y1 * x4);
            s.L->area[gf_ek(s.d, e, 3)] = 1.0 / det;
            for (int k = 0; k < 4; ++k)
                if (s.L->area[gf_ek(s.d, e, k)] < 0) throw Stop{41};
        }
}

// init_geotherm_profile (src/init_temp.f90:127-310) for column i (0-based).
void geotherm(S &s, int n, int i, double age_1n, double tp1n, double tp2n) {
    gf_params &p = *s.p;
    int nz = p.nz;
    const double pi = 3.14159265358979323846;
    double t_top = p.t_top, t_bot = p.t_bot;
    int ic = p.ictherm[n];
    if (ic == 1) {
        double diffusivity = 1e-6, age = age_1n;
        for (int j = 0; j < nz; ++j) {
            double f = (s.cord(0, i, 1) - s.cord(j, i, 1)) / std::sqrt(4 * diffusivity * age * 1e6 * GF_SEC_YEAR);
            s.temp(j, i) = t_top + (t_bot - t_top) * std::erf(f);
        }
    } else if (ic == 2) {
        double diffusivity = 1e-6, age = age_1n, yL0 = tp1n;
        double age_init = age * GF_SEC_YEAR * 1e6;
        double tau_d = yL0 * yL0 * 1e6 / (pi * pi * diffusivity);
        for (int j = 0; j < nz; ++j) {
            double y = (s.cord(0, i, 1) - s.cord(j, i, 1)) * 1e-3;
            double tss = t_top + (t_bot - t_top) * y / yL0;
            double tt = 0.0;
            for (int k = 1; k <= 100; ++k) tt = tt + 1.0 / k * std::exp(-k * k * age_init / tau_d) * std::sin(pi * k * y / yL0);
            s.temp(j, i) = tss + 2.0 / pi * (t_bot - t_top) * tt;
            if (s.temp(j, i) > t_bot || y > yL0) s.temp(j, i) = t_bot;
        }
    } else if (ic == 12) {
        double age = age_1n, yL0 = tp1n, ymoho = tp2n, cond = 3.3, dens_c = 2700.0, diffusivity = 1e-6;
        double age_init = age * GF_SEC_YEAR * 1e6;
        double tau_d = yL0 * yL0 * 1e6 / (pi * pi * diffusivity);
        double rr = ymoho / (yL0 - ymoho);
        double tm = (t_top + rr * t_bot + dens_c * p.hs * p.hr * p.hr * 1e6 / cond * (1.0 - std::exp(-ymoho / p.hr))) / (1 + rr);
        double qm = cond * (t_bot - tm) / (yL0 - ymoho);
        for (int j = 0; j < nz; ++j) {
            double y = (s.cord(0, i, 1) - s.cord(j, i, 1)) * 1e-3;
            double tss;
            if (y <= ymoho)
                tss = t_top + qm / cond * y + (dens_c * p.hs * p.hr * p.hr * 1e6 / cond) * (1.0 - std::exp(-y / p.hr));
            else if (y <= yL0)
                tss = tm + qm / cond * (y - ymoho);
            else
                tss = t_bot;
            double tt = 0.0;
            for (int k = 1; k <= 100; ++k) tt = tt + 1.0 / k * std::exp(-k * k * age_init / tau_d) * std::sin(pi * k * y / yL0);
            s.temp(j, i) = tss + 2.0 / pi * (t_bot - t_top) * tt;
            if (s.temp(j, i) > t_bot || y > yL0) s.temp(j, i) = t_bot;
        }
    } else if (ic == 21) {
        double bot_dep = age_1n;
        for (int j = 0; j < nz; ++j) {
            double y = (s.cord(0, i, 1) - s.cord(j, i, 1)) * 1e-3;
            s.temp(j, i) = y * (t_bot - t_top) / bot_dep;
            if (s.temp(j, i) > t_bot) s.temp(j, i) = t_bot;
        }
    } else if (ic == 22) {
        double temp1 = age_1n, ylayer1 = tp1n, ylayer2 = tp2n;
        for (int j = 0; j < nz; ++j) {
            double y = (s.cord(0, i, 1) - s.cord(j, i, 1)) * 1e-3;
            if (y <= ylayer1)
                s.temp(j, i) = t_top + (temp1 - t_top) * y / ylayer1;
            else
                s.temp(j, i) = temp1 + (t_bot - temp1) * (y - ylayer1) / (ylayer2 - ylayer1);
            if (s.temp(j, i) > t_bot) s.temp(j, i) = t_bot;
        }
    } else if (ic == 13) {
        double cond_c = 2.3, cond_m = 3.3, Fpart = 0.74, alc = 0.4e-6, am = 0.02e-6;
        double auc = (1.0 - Fpart) * age_1n * 1.0e-3 / (tp1n * 1000.0);
        std::vector<double> Q(nz + 1);
        Q[0] = age_1n * 1.0e-3;
        s.temp(0, i) = t_top;
        int kl = 0;
        int nx = p.nx;
        for (int j = 0; j < nz - 1; ++j) {
            double y = (s.cord(0, i, 1) - s.cord(j, i, 1)) * 1.0e-3;
            double xdz = std::fabs(s.cord(j + 1, i, 1) - s.cord(j, i, 1));
            double *src = (i < nx - 1) ? &s.L->source[s.e(j, i)] : nullptr;
            if (y < tp1n) {
                s.temp(j + 1, i) = s.temp(j, i) + (Q[j] / cond_c) * xdz - (auc) / (2.0 * cond_c) * (xdz * xdz);
                Q[j + 1] = Q[j] - auc * xdz;
                if (src) *src = auc * 1.0e-3;
            }
            if (y >= tp1n && y < (tp2n + tp1n)) {
                s.temp(j + 1, i) = s.temp(j, i) + (Q[j] / cond_c) * xdz - (alc) / (2.0 * cond_c) * (xdz * xdz);
                Q[j + 1] = Q[j] - alc * xdz;
                if (src) *src = alc * 1.0e-3;
            }
            if (y >= (tp2n + tp1n) && kl == 0) {
                s.temp(j + 1, i) = s.temp(j, i) + (Q[j] / cond_m) * xdz - (am) / (2.0 * cond_m) * (xdz * xdz);
                Q[j + 1] = Q[j] - am * xdz;
                if (src) *src = am * 1.0e-3;
                if (s.temp(j + 1, i) >= t_bot) kl = 1;
            }
            if (kl == 1) {
                s.temp(j + 1, i) = t_bot;
                if (src) *src = 0.0;
            }
        }
    } else {
        throw Stop{1};
    }
}

// init_temp (src/init_temp.f90:3-124).
void init_temp(S &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    if (p.irtemp > 0) {
        FILE *f = std::fopen(p.tempfile, "r");
        if (!f) throw Stop{21};
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < nz; ++j)
                if (std::fscanf(f, "%lf", &s.temp(j, i)) != 1) {
                    std::fclose(f);
                    throw Stop{21};
                }
        std::fclose(f);
    } else {
        for (int n = 0; n < p.nzone_age; ++n) {
            if (n != 0 && p.iph_col_trans[n - 1] == 1) continue;
            for (int i = p.ixtb1[n]; i <= p.ixtb2[n]; ++i) {
                double age_1n, tp1n, tp2n;
                if (p.iph_col_trans[n] == 1) {
                    int i1 = p.ixtb1[n], i2 = p.ixtb2[n];
                    double ratio = (s.cord(0, i - 1, 0) - s.cord(0, i1 - 1, 0)) / (s.cord(0, i2 - 1, 0) - s.cord(0, i1 - 1, 0));
                    age_1n = p.age_1[n] + (p.age_1[n + 1] - p.age_1[n]) * ratio;
                    tp1n = p.tp1[n] + (p.tp1[n + 1] - p.tp1[n]) * ratio;
                    tp2n = p.tp2[n] + (p.tp2[n + 1] - p.tp2[n]) * ratio;
                } else {
                    age_1n = p.age_1[n];
                    tp1n = p.tp1[n];
                    tp2n = p.tp2[n];
                }
                geotherm(s, n, i - 1, age_1n, tp1n, tp2n);
            }
        }
    }
    // radiogenic sources (init_temp.f90:54-58)
    for (int j = 0; j < nz - 1; ++j) {
        double y = -(s.cord(j + 1, 0, 1) + s.cord(j, 0, 1)) / 2 / 1000;
        double v = p.hs * std::exp(-y / p.hr);
        for (int i = 0; i < nx - 1; ++i) s.L->source[s.e(j, i)] = v;
    }
    for (int n = 0; n < p.inhom; ++n) {
        if (p.igeom[n] == 11) {
            int ixc = (p.ix1[n] + p.ix2[n]) / 2, iwidth = p.ix2[n] - p.ix1[n];
            double amp = p.xinitaps[n];
            for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                double q = (double)(float)(j - ixc) / (0.25 * (double)(float)iwidth);
                double pert = amp * std::exp(-(q * q));
                for (int k = p.iy1[n]; k <= p.iy2[n]; ++k) {
                    double pert2 = 1.0 * (k - p.iy1[n]) / (p.iy2[n] - p.iy1[n]);
                    s.temp(k - 1, j - 1) = std::fmin(p.t_bot, s.temp(k - 1, j - 1) + pert * pert2);
                }
            }
        }
        if (p.igeom[n] == 13 || p.igeom[n] == 14) {
            int ixc = (p.ix1[n] + p.ix2[n]) / 2, iwidth = p.ix2[n] - p.ix1[n];
            double amp = p.xinitaps[n];
            for (int k = p.iy1[n]; k <= p.iy2[n]; ++k) {
                int kk = k - p.iy1[n];
                for (int j = p.ix1[n]; j <= p.ix2[n]; ++j) {
                    double q = (double)(float)(j - ixc) / (0.25 * (double)(float)iwidth);
                    double pert = amp * std::exp(-(q * q));
                    int jj = p.igeom[n] == 13 ? j + kk : j - kk;
                    s.temp(k - 1, jj - 1) = std::fmax(p.t_top, std::fmin(p.t_bot, s.temp(k - 1, jj - 1) + pert));
                }
            }
        }
    }
}

// init_stress (src/init_stress.f90:5-60): lithostatic prestress, pisos.
void init_stress(S &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    p.pisos = 0.0;
    for (int i = 0; i < nx - 1; ++i) {
        double rogh;
        int iph0 = s.L->iphase[s.e(0, i)];
        if (iph0 == 3 || iph0 == 7)
            rogh = -1030.0 * p.g * 8.0e3;
        else
            rogh = 0.0;
        for (int j = 0; j < nz - 1; ++j) {
            long long e = s.e(j, i);
            int iph = s.L->iphase[e] - 1;
            double tmpr = 0.25 * (((s.temp(j, i) + s.temp(j + 1, i)) + s.temp(j, i + 1)) + s.temp(j + 1, i + 1));
            double densT = p.den[iph] * (1 - p.alfa[iph] * tmpr);
            double dh1 = s.cord(j, i, 1) - s.cord(j + 1, i, 1);
            double dh2 = s.cord(j, i + 1, 1) - s.cord(j + 1, i + 1, 1);
            double dh = 0.5 * (dh1 + dh2);
            double dPT = densT * p.g * dh;
            double dP = dPT * (1 - p.beta[iph] * rogh) / (1 + p.beta[iph] / 2 * dPT);
            double press = rogh + 0.5 * dP;
            for (int k = 0; k < 4; ++k) {
                s.L->stress0[gf_s(s.d, e, 0, k)] = -press;
                s.L->stress0[gf_s(s.d, e, 1, k)] = -press;
                s.L->stress0[gf_s(s.d, e, 2, k)] = 0.0;
                s.L->stress0[gf_s(s.d, e, 3, k)] = -press;
            }
            rogh = rogh + dP;
        }
        if (i == nx - 2 && p.nyhydro == 2) p.pisos = rogh + p.extra_pres;
    }
}

double bc_fun(const gf_params &p, int n, double x) {
    const double pi2 = 2.0 * 3.14159;
    double t = (x - p.bci[n]) * p.bch[n];
    return ((p.bca[n] + p.bcb[n] * x) + p.bcc[n] * x * x) +
           (p.bcd[n] * std::cos(pi2 * p.bce[n] * x) + p.bcf[n] * std::sin(pi2 * p.bcg[n] * x)) * std::exp(-(t * t));
}

// velbc (src/init_bc.f90:284-339); numbp and mid_j 1-based.
void velbc(S &s, int n, int numbp, double x, int mid_j) {
    gf_params &p = *s.p;
    double fun = bc_fun(p, n, x);
    int ii1 = 0, jj1 = 0;
    if (p.nofside[n] == 1) { ii1 = 1; jj1 = numbp; }
    if (p.nofside[n] == 2) { ii1 = numbp; jj1 = p.nz; }
    if (p.nofside[n] == 3) { ii1 = p.nx; jj1 = numbp; }
    if (p.nofside[n] == 4) { ii1 = numbp; jj1 = 1; }
    if (p.nofside[n] == 5) { ii1 = numbp; jj1 = mid_j; }
    if (ii1 < 1 || ii1 > p.nx || jj1 < 1 || jj1 > p.nz) return;
    if (p.nbc[n] == 10) {
        s.ncod(jj1 - 1, ii1 - 1, 0) = 1;
        if (std::fabs(s.bc(jj1 - 1, ii1 - 1, 0)) > 0.0) fun = s.bc(jj1 - 1, ii1 - 1, 0);
        s.bc(jj1 - 1, ii1 - 1, 0) = fun;
    }
    if (p.nbc[n] == 1 || p.nbc[n] == 200) {
        s.ncod(jj1 - 1, ii1 - 1, 1) = 1;
        s.bc(jj1 - 1, ii1 - 1, 1) = (p.nbc[n] == 200) ? 0.0 : fun;
    }
}

// init_bc (src/init_bc.f90:4-221) and vbcal (:385-409).  Stress boundary
// conditions (nbc 2/20/40) are counted but only used when nystressbc = 1,
// which the GPU path does not support (GF_ERR_UNSUPPORTED at gf_create).
void init_bc(S &s) {
    gf_params &p = *s.p;
    int nx = p.nx, nz = p.nz;
    std::memset(s.L->bc, 0, sizeof(double) * 2 * (size_t)s.d.N);
    std::memset(s.L->ncod, 0, sizeof(int) * 2 * (size_t)s.d.N);
    p.incoming_left = 0;
    p.incoming_right = 0;
    int nnop = 0;
    for (int n = 0; n < p.nofbc; ++n) {
        int ndbc = p.nbc2[n] - p.nbc1[n] + 1;
        bool stressbc = (p.nbc[n] == 2 || p.nbc[n] == 20 || p.nbc[n] == 40);
        if (stressbc) {
            ndbc = ndbc - 1;
            if (p.nbc2[n] < nz) ndbc = ndbc + 1;
        }
        bool vel = (p.nbc[n] == 1 || p.nbc[n] == 10 || p.nbc[n] == 30);
        if (p.nofside[n] == 1 || p.nofside[n] == 3) {
            int col = p.nofside[n] == 1 ? 0 : nx - 1;
            double x1 = s.cord(p.nbc1[n] - 1, col, 1), x2 = s.cord(p.nbc2[n] - 1, col, 1);
            for (int k = 1; k <= ndbc; ++k) {
                int numbp = k + p.nbc1[n] - 1;
                double x = (s.cord(numbp - 1, col, 1) - x1) / (x2 - x1);
                if (vel) velbc(s, n, numbp, x, 0);
                if (stressbc) nnop = nnop + 1;
                if ((p.nbc[n] == 1 || p.nbc[n] == 10) && p.nofside[n] == 1 && p.bca[n] > 0) p.incoming_left = 1;
                if ((p.nbc[n] == 1 || p.nbc[n] == 10) && p.nofside[n] == 3 && p.bca[n] < 0) p.incoming_right = 1;
            }
        }
        if (p.nofside[n] == 2 || p.nofside[n] == 4) {
            int row = p.nofside[n] == 2 ? nz - 1 : 0;
            double x1 = s.cord(row, p.nbc1[n] - 1, 0), x2 = s.cord(row, p.nbc2[n] - 1, 0);
            for (int k = 1; k <= ndbc; ++k) {
                int numbp = k + p.nbc1[n] - 1;
                double x = (s.cord(row, numbp - 1, 0) - x1) / (x2 - x1);
                if (vel || (p.nofside[n] == 2 && p.nbc[n] == 200)) velbc(s, n, numbp, x, 0);
                if (stressbc) nnop = nnop + 1;
            }
        }
        if (p.nofside[n] == 5) {
            if (p.nbc[n] != 10) throw Stop{55};
            for (int k = 1; k <= ndbc; ++k) {
                int numbp = k + p.nbc1[n] - 1;
                int jm = s.L->jmoho ? s.L->jmoho[n < nx - 1 ? n : nx - 2] : nz - 1;
                int top = std::min(jm * 2, nx);
                for (int mid_j = 1; mid_j <= top; ++mid_j) {
                    double x1 = s.cord(0, numbp - 1, 1);
                    double x2 = s.cord(top - 1, numbp - 1, 1);
                    double x = (s.cord(mid_j - 1, numbp - 1, 1) - x1) / (x2 - x1);
                    velbc(s, n, numbp, x, mid_j);
                }
            }
        }
    }
    p.nopbmax = nnop;
    // vbcal
    double vbc = 0.0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j)
            for (int k = 0; k < 2; ++k) {
                int c = s.ncod(j, i, k);
                if (c == 1 || c == 10 || c == 30) vbc = std::fmax(vbc, std::fabs(s.bc(j, i, k)));
            }
    if (vbc == 0.0) vbc = 1e-10;
    p.vbc = vbc;
}

} // namespace

extern "C" int gf_setflac_host(gf_params *p, gf_clock *c, gf_layout *L) {
    if (!p || !c || !L || !L->cord || !L->temp || !L->stress0 || !L->area || !L->iphase || !L->phase_ratio ||
        !L->mark_a1 || !L->nmark_elem || !L->mark_id_elem || !L->bc || !L->ncod || !L->source || !L->aps)
        return GF_ERR_ARG;
    if (L->nx != p->nx || L->nz != p->nz || L->nphase != p->nphase) return GF_ERR_ARG;
    S s{p, c, L, GfDims{p->nx, p->nz, p->nphase, (long long)p->nx * p->nz, (long long)(p->nx - 1) * (p->nz - 1)}};
    size_t N = (size_t)s.d.N, E = (size_t)s.d.E;
    try {
        std::memset(c, 0, sizeof *c);
        c->nloop = 0;
        c->time = 0.0;
        c->frac = p->frac;
        init_cord(s);
        for (size_t e = 0; e < E; ++e) L->aps[e] = 0.0;
        if (L->vel) std::memset(L->vel, 0, sizeof(double) * 2 * N);
        if (L->dvol) std::memset(L->dvol, 0, sizeof(double) * 4 * E);
        if (L->strain) std::memset(L->strain, 0, sizeof(double) * 3 * E);
        init_phase(s);
        init_marker(s);
        // check_visc_rheol (src/init_phase.f90:56-72)
        p->ivis_present = 0;
        for (size_t e = 0; e < E; ++e) {
            int irh = p->irheol[L->iphase[e] - 1];
            if (irh == 3 || irh >= 11) p->ivis_present = 1;
        }
        init_areas(s);
        // Amin (setflac.f90:42)
        double amin = 1e300;
        for (size_t e = 0; e < E; ++e) amin = std::fmin(amin, 0.5 / L->area[e] + 0.5 / L->area[E + e]);
        p->Amin = amin;
        init_temp(s);
        init_stress(s);
        init_bc(s);
        // field defaults (setflac.f90:53-66)
        if (L->temp0) std::memcpy(L->temp0, L->temp, sizeof(double) * N);
        if (L->xoriginal) std::memcpy(L->xoriginal, L->cord, sizeof(double) * N);
        if (L->zoriginal) std::memcpy(L->zoriginal, L->cord + N, sizeof(double) * N);
        for (size_t e = 0; e < E; ++e) {
            if (L->shrheat) L->shrheat[e] = 0.0;
            if (L->sshrheat) L->sshrheat[e] = 0.0;
            if (L->fmagma) L->fmagma[e] = 0.0;
            if (L->fmagma2) L->fmagma2[e] = 0.0;
            if (L->dike_released) L->dike_released[e] = 0.0;
            // melt fractions and dike / MOR accumulators (setflac.f90:60-63,
            // arrays.f90:124-128)
            for (double *f : {L->fmelt, L->fmelt2, L->dike_backlog, L->dike_marker_vol, L->mor_marker_vol})
                if (f) f[e] = 0.0;
            if (L->e2sr) L->e2sr[e] = 1e-16;
            if (L->visn) L->visn[e] = 0.0;
        }
        if (L->se2sr)
            for (size_t e = 0; e < 3 * E; ++e) L->se2sr[e] = 1e-16;
        if (L->extrusion) std::memset(L->extrusion, 0, sizeof(double) * p->nx);
        if (L->amass) std::memset(L->amass, 0, sizeof(double) * N);
        if (L->rmass) std::memset(L->rmass, 0, sizeof(double) * N);
        c->dtavg = 0.0;
        c->nsrate = -1;
    } catch (const Stop &st) {
        return st.code;
    }
    return GF_OK;
}

// The host part of a restart once the saved fields are in L and marker2elem
// has refreshed iphase and jmoho (rsflac.f90:109-116,217): check_visc_rheol
// and init_bc on the restored mesh (the boundary velocities are profiles
// along the restored side coordinates).
int gf_host_restart_bc(gf_params *p, gf_layout *L) {
    gf_clock c{};
    S s{p, &c, L, GfDims{p->nx, p->nz, p->nphase, (long long)p->nx * p->nz, (long long)(p->nx - 1) * (p->nz - 1)}};
    try {
        p->ivis_present = 0;
        for (long long e = 0; e < s.d.E; ++e) {
            int irh = p->irheol[L->iphase[e] - 1];
            if (irh == 3 || irh >= 11) p->ivis_present = 1;
        }
        init_bc(s);
    } catch (const Stop &st) {
        return st.code;
    }
    return GF_OK;
}

// Geotherm of node columns i_first..i_last (0-based) for age zone `zone`
// (init_geotherm_profile, src/init_temp.f90:127-310), on host arrays in the
// reference layout: used by the remesh event for material entering through a
// side wall (sidewalltemp, src/init_temp.f90:313-353).
int gf_host_geotherm_columns(gf_params *p, gf_layout *L, int zone, int i_first, int i_last) {
    gf_clock c{};
    S s{p, &c, L, GfDims{p->nx, p->nz, p->nphase, (long long)p->nx * p->nz, (long long)(p->nx - 1) * (p->nz - 1)}};
    try {
        for (int i = i_first; i <= i_last; ++i) geotherm(s, zone, i, p->age_1[zone], p->tp1[zone], p->tp2[zone]);
    } catch (const Stop &st) {
        return st.code;
    }
    return GF_OK;
}

// The zone pattern of mesh1 before scaling: x_k = x1 + t[k] * (x2 - x1) / all_ratio
// (src/init_cord.f90:141-179), so a device can regrid with the host's exact values.
void gf_host_mesh_template(int n, int nzon, const int *nelz, const double *sizez, double *t, double *all_ratio) {
    double ar = 0.0;
    for (int k = 0; k < nzon - 1; k += 2) {
        ar = ar + nelz[k] * sizez[k];
        double ratio = std::pow(sizez[k + 2] / sizez[k], 1.0 / (double)(nelz[k + 1] + 1));
        for (int i = 1; i <= nelz[k + 1]; ++i) ar = ar + sizez[k] * ipow(ratio, i);
    }
    ar = ar + nelz[nzon - 1] * sizez[nzon - 1];
    int nel = 0;
    t[0] = 0.0;
    for (int k = 0; k < nzon - 1; k += 2) {
        for (int i = 0; i < nelz[k]; ++i) {
            nel = nel + 1;
            t[nel] = t[nel - 1] + sizez[k];
        }
        double ratio = std::pow(sizez[k + 2] / sizez[k], 1.0 / (double)(nelz[k + 1] + 1));
        for (int i = 1; i <= nelz[k + 1]; ++i) {
            nel = nel + 1;
            t[nel] = t[nel - 1] + sizez[k] * ipow(ratio, i);
        }
    }
    for (int k = 0; k < nelz[nzon - 1]; ++k) {
        nel = nel + 1;
        t[nel] = t[nel - 1] + sizez[nzon - 1];
    }
    *all_ratio = ar;
    (void)n;
}
