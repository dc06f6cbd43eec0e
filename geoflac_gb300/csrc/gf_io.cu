// Output frames and restart files in the reference's binary layouts.
//
// outflac (src/outflac.f90) and outmarker (src/outmarker.f90): the derived
// float32 fields of one frame are computed on the device by three packing
// kernels (elements, nodes, the surface line) into one buffer, copied to the
// host once, and each field is written as record `nrec` of its direct-access
// file (`<name>.0`, fixed record length, no record markers), the record
// number kept in `_contents.0` / `_markers.0` as the reference does.
//
// saveflac / rsflac (src/saveflac.f90, src/rsflac.f90): the FP64 restart
// files `*.rs` written from the context's state and read back into it; the
// device then redoes what rsflac.f90 recomputes after reading (marker
// bins, marker2elem, areas, masses, viscosities, time step).

#include "gf_kernels.cuh"
#include "gf_internal.h"
#include "gf_member.h"

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// element fields of a frame, in file order
enum {
    EF_SRII, EF_SRXX, EF_SRZZ, EF_SRXZ, EF_EII, EF_EI, EF_EXX, EF_EZZ, EF_EXZ, EF_DENS, EF_AREA, EF_APS, EF_SII,
    EF_SXX, EF_SZZ, EF_SXZ, EF_SYY, EF_PRES, EF_TEMP, EF_VISC, EF_SRC, EF_FMELT, EF_FMELT2, EF_FMAGMA, EF_FMAGMA2,
    EF_DISS, EF_COUNT
};
// node fields: mesh (2N), vel (2N), temperature, cooling rate, xoriginal, zoriginal
enum { NF_MESH = 0, NF_VEL = 2, NF_TEMP = 4, NF_COOL = 5, NF_XORIG = 6, NF_ZORIG = 7, NF_COUNT = 8 };
// surface line: hfl (nx), topo (nx), dtopo (nx), extrusion (nx - 1)
enum { LF_HFL = 0, LF_TOPO = 1, LF_DTOPO = 2, LF_EXTR = 3, LF_COUNT = 4 };

struct FrameArgs {
    float *ef;  // [EF_COUNT][E]
    int *phase; // [E]
    float *nf;  // [NF_COUNT][N]
    float *lf;  // [LF_COUNT][nx]
    double dt, dtavg, hs;
};

template <class R>
__global__ void k_frame_elems(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, FrameArgs f) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    const DevParams &P = *Pp;
    int j = (int)(e % (d.nz - 1)), i = (int)(e / (d.nz - 1));
    const R *st = (const R *)A.stress0;
    const double pr = sizeof(R) == sizeof(float) ? A.p_ref[e] : 0.0;
    double s[4];
    for (int c = 0; c < 4; ++c) {
        double a = 0.25 * ((double)st[gf_s(d, e, c, 0)] + (double)st[gf_s(d, e, c, 1)] + (double)st[gf_s(d, e, c, 2)] +
                           (double)st[gf_s(d, e, c, 3)]);
        s[c] = c == 2 ? a : a - pr; // total stress (mixed storage is offset by p_ref)
    }
    const double sI = (s[0] + s[1] + s[3]) / 3.0;
    const double sII = 0.5 * sqrt((s[0] - s[1]) * (s[0] - s[1]) + 4.0 * s[2] * s[2]);
    const R *strain = (const R *)A.strain, *se2sr = (const R *)A.se2sr;
    const double e1 = strain[gf_ek(d, e, 0)], e2 = strain[gf_ek(d, e, 1)], e3 = strain[gf_ek(d, e, 2)];
    const double sr = (double)((const R *)A.e2sr)[e];
    auto put = [&](int k, double v) { f.ef[(long long)k * d.E + e] = (float)v; };
    put(EF_SRII, sr != 0.0 ? log10(sr) : 0.0);
    put(EF_SRXX, (double)se2sr[gf_ek(d, e, 0)] / f.dtavg);
    put(EF_SRZZ, (double)se2sr[gf_ek(d, e, 1)] / f.dtavg);
    put(EF_SRXZ, (double)se2sr[gf_ek(d, e, 2)] / f.dtavg);
    put(EF_EII, 0.5 * sqrt((e1 - e2) * (e1 - e2) + 4.0 * e3 * e3));
    put(EF_EI, 0.5 * (e1 + e2));
    put(EF_EXX, e1);
    put(EF_EZZ, e2);
    put(EF_EXZ, e3);
    int wrote = 0;
    double fv = 0.0;
    put(EF_DENS, gfk::eff_dens<R>(P, A, d, j, i, e, &wrote, &fv));
    const R *area = (const R *)A.area;
    put(EF_AREA, 0.5 / (double)area[gf_ek(d, e, 0)] + 0.5 / (double)area[gf_ek(d, e, 1)]);
    put(EF_APS, (double)((const R *)A.aps)[e]);
    put(EF_SII, sII);
    put(EF_SXX, s[0] - sI);
    put(EF_SZZ, s[1] - sI);
    put(EF_SXZ, s[2]);
    put(EF_SYY, s[3] - sI);
    put(EF_PRES, sI);
    const double *T = A.temp;
    put(EF_TEMP, 0.25 * (T[gf_node(d, j, i)] + T[gf_node(d, j + 1, i)] + T[gf_node(d, j, i + 1)] +
                         T[gf_node(d, j + 1, i + 1)]));
    put(EF_VISC, log10((double)((const R *)A.visn)[e]));
    put(EF_SRC, A.source[e]);
    put(EF_FMELT, A.fmelt ? A.fmelt[e] : 0.0);
    put(EF_FMELT2, A.fmelt2 ? A.fmelt2[e] : 0.0);
    put(EF_FMAGMA, A.fmagma ? A.fmagma[e] : 0.0);
    put(EF_FMAGMA2, A.fmagma2 ? A.fmagma2[e] : 0.0);
    const int iph = A.iphase[e];
    put(EF_DISS, P.ishearh != 0 ? (double)((const R *)A.shrheat)[e] / P.den[iph - 1] / f.hs : 0.0);
    f.phase[e] = iph;
}

__global__ void k_frame_nodes(DevArrays A, GfDims d, FrameArgs f) {
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.N) return;
    const long long N = d.N;
    f.nf[(NF_MESH)*N + n] = (float)(A.cord[n] / 1000);
    f.nf[(NF_MESH + 1) * N + n] = (float)(A.cord[N + n] / 1000);
    f.nf[(NF_VEL)*N + n] = (float)(A.vel[n] * GF_SEC_YEAR * 100);
    f.nf[(NF_VEL + 1) * N + n] = (float)(A.vel[N + n] * GF_SEC_YEAR * 100);
    f.nf[NF_TEMP * N + n] = (float)A.temp[n];
    f.nf[NF_COOL * N + n] = (float)((A.temp[n] - A.temp0[n]) / (f.dt / (GF_SEC_YEAR * 1.e6)));
    f.nf[NF_XORIG * N + n] = (float)A.orig[n];
    f.nf[NF_ZORIG * N + n] = (float)A.orig[N + n];
}

__global__ void k_frame_line(const DevParams *__restrict__ Pp, DevArrays A, GfDims d, FrameArgs f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nx) return;
    const int nx = d.nx;
    const long long N = d.N;
    int ii = min(i, nx - 2);
    double dtmpr = A.temp[gf_node(d, 1, i)] - A.temp[gf_node(d, 0, i)];
    double dl = -(A.cord[N + gf_node(d, 1, i)] - A.cord[N + gf_node(d, 0, i)]) / 1000;
    double cond = Pp->conduct[A.iphase[gf_elem(d, 0, ii)] - 1];
    f.lf[LF_HFL * nx + i] = (float)(cond * dtmpr / dl);
    f.lf[LF_TOPO * nx + i] = (float)(A.cord[N + gf_node(d, 0, i)] / 1000);
    // dtopo in mm/yr (outflac.f90:410-412); the last arc extrusion
    // (zero without the magma sub-model)
    f.lf[LF_DTOPO * nx + i] = (float)(A.dtopo[i] / f.dt * 1000 * GF_SEC_YEAR);
    f.lf[LF_EXTR * nx + i] = A.extrusion ? (float)A.extrusion[i] : 0.0f;
}

// marker positions (marker2xy, bar2euler.f90:73-117) and the output records
__global__ void k_frame_markers(DevArrays A, GfDims d, int nmarkers, float *fo, int *io) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmarkers) return;
    const int nz = d.nz;
    int n = A.mark_ntriag[m];
    double x = 0.0, y = 0.0;
    if (A.mark_dead[m] != 0 && n >= 1 && n <= 2 * d.E) { // dead markers: 0 (the reference leaves them unset)
        int k = (n - 1) % 2 + 1;
        int jj = ((n - k) / 2) % (nz - 1);
        int ii = (n - k) / 2 / (nz - 1);
        double ba1 = A.mark_a1[m], ba2 = A.mark_a2[m], ba3 = 1.0 - ba1 - ba2;
        int i1, i2, i3, j1, j2, j3;
        if (k == 1) {
            i1 = ii; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj;
        } else {
            i1 = ii + 1; i2 = ii; i3 = ii + 1; j1 = jj; j2 = jj + 1; j3 = jj + 1;
        }
        const double *c = A.cord;
        x = c[gf_node(d, j1, i1)] * ba1 + c[gf_node(d, j2, i2)] * ba2 + c[gf_node(d, j3, i3)] * ba3;
        y = c[d.N + gf_node(d, j1, i1)] * ba1 + c[d.N + gf_node(d, j2, i2)] * ba2 + c[d.N + gf_node(d, j3, i3)] * ba3;
        if (A.dhacc_correction) {
            if (j1 == 0) y = y - A.dhacc_correction[i1] * ba1;
            if (j2 == 0) y = y - A.dhacc_correction[i2] * ba2;
            if (j3 == 0) y = y - A.dhacc_correction[i3] * ba3;
        }
    }
    fo[0LL * nmarkers + m] = (float)(x * 1e-3);
    fo[1LL * nmarkers + m] = (float)(y * 1e-3);
    fo[2LL * nmarkers + m] = (float)(A.mark_age[m] / GF_SEC_YEAR / 1.e6);
    fo[3LL * nmarkers + m] = (float)A.mark_a1[m];
    fo[4LL * nmarkers + m] = (float)A.mark_a2[m];
    io[0LL * nmarkers + m] = A.mark_dead[m];
    io[1LL * nmarkers + m] = A.mark_phase[m];
    io[2LL * nmarkers + m] = A.mark_ntriag[m];
}

// ---------------------------------------------------------------- host files
std::string path_of(const char *dir, const std::string &name) {
    std::string d = dir && *dir ? dir : ".";
    return d + "/" + name;
}

// record `rec` (1-based) of a direct-access file with record length recl
int write_record(const char *dir, const std::string &name, long long rec, const void *data, size_t bytes,
                 size_t recl) {
    int fd = ::open(path_of(dir, name).c_str(), O_WRONLY | O_CREAT, 0644);
    if (fd < 0) return GF_ERR_IO;
    std::vector<char> buf;
    const char *src = static_cast<const char *>(data);
    if (bytes < recl) { // the rest of a longer record is zero-filled
        buf.assign(recl, 0);
        std::memcpy(buf.data(), data, bytes);
        src = buf.data();
    }
    off_t off = (off_t)(rec - 1) * (off_t)recl;
    size_t done = 0;
    while (done < recl) {
        ssize_t w = ::pwrite(fd, src + done, recl - done, off + (off_t)done);
        if (w <= 0) {
            ::close(fd);
            return GF_ERR_IO;
        }
        done += (size_t)w;
    }
    ::close(fd);
    return GF_OK;
}

int read_record(const char *dir, const std::string &name, long long rec, void *data, size_t bytes, size_t recl) {
    int fd = ::open(path_of(dir, name).c_str(), O_RDONLY);
    if (fd < 0) return GF_ERR_IO;
    std::vector<char> buf(recl);
    off_t off = (off_t)(rec - 1) * (off_t)recl;
    size_t done = 0;
    while (done < recl) {
        ssize_t r = ::pread(fd, buf.data() + done, recl - done, off + (off_t)done);
        if (r <= 0) {
            ::close(fd);
            return GF_ERR_IO;
        }
        done += (size_t)r;
    }
    ::close(fd);
    std::memcpy(data, buf.data(), bytes);
    return GF_OK;
}

// next record number of a contents file: 1 for a fresh series, else one more
// than the last record number listed (outflac.f90:17-33)
long long next_record(const char *dir, const char *contents, int fresh) {
    if (fresh) return 1;
    FILE *f = std::fopen(path_of(dir, contents).c_str(), "r");
    if (!f) return 1;
    long long last = 0, v;
    char line[512];
    while (std::fgets(line, sizeof line, f))
        if (std::sscanf(line, "%lld", &v) == 1) last = v;
    std::fclose(f);
    return last + 1;
}

int append_line(const char *dir, const char *contents, int fresh, const std::string &line) {
    FILE *f = std::fopen(path_of(dir, contents).c_str(), fresh ? "w" : "a");
    if (!f) return GF_ERR_IO;
    std::fputs(line.c_str(), f);
    std::fclose(f);
    return GF_OK;
}

#define IO_CK(call)                                                                                                    \
    do {                                                                                                               \
        int _rc = (call);                                                                                              \
        if (_rc) return _rc;                                                                                           \
    } while (0)
#define CU_CK(call)                                                                                                    \
    do {                                                                                                               \
        if ((call) != cudaSuccess) return GF_ERR_CUDA;                                                                 \
    } while (0)

// device buffer and pinned host copy of one output frame
struct Staging {
    void *dev = nullptr, *host = nullptr;
    ~Staging() {
        if (dev) cudaFree(dev);
        if (host) cudaFreeHost(host);
    }
    int alloc(size_t bytes) {
        if (cudaMalloc(&dev, bytes) != cudaSuccess) return GF_ERR_NOMEM;
        if (cudaMallocHost(&host, bytes) != cudaSuccess) return GF_ERR_NOMEM;
        return GF_OK;
    }
};

} // namespace

extern "C" {

int gf_outflac(gf_ctx *ctx, const char *dir, int fresh) {
    if (!ctx) return GF_ERR_ARG;
    GfMemberView v;
    IO_CK(gf_ctx_view(ctx, &v));
    gf_clock k;
    IO_CK(gf_get_clock(ctx, &k));
    const gf_params &p = *v.hp;
    const GfDims &d = v.d;
    const long long E = d.E, N = d.N, nx = d.nx;
    const size_t ebytes = (size_t)EF_COUNT * E * 4, pbytes = (size_t)E * 4, nbytes = (size_t)NF_COUNT * N * 4,
                 lbytes = (size_t)LF_COUNT * nx * 4;
    Staging sg;
    IO_CK(sg.alloc(ebytes + pbytes + nbytes + lbytes));
    FrameArgs f;
    char *base = static_cast<char *>(sg.dev);
    f.ef = reinterpret_cast<float *>(base);
    f.phase = reinterpret_cast<int *>(base + ebytes);
    f.nf = reinterpret_cast<float *>(base + ebytes + pbytes);
    f.lf = reinterpret_cast<float *>(base + ebytes + pbytes + nbytes);
    f.dt = k.dt;
    f.dtavg = k.dtavg;
    f.hs = p.hs;
    const unsigned T = 256;
    if (v.mode == GF_MODE_MIXED)
        k_frame_elems<float><<<(unsigned)((E + T - 1) / T), T, 0, v.s>>>(v.P, v.A, d, f);
    else
        k_frame_elems<double><<<(unsigned)((E + T - 1) / T), T, 0, v.s>>>(v.P, v.A, d, f);
    k_frame_nodes<<<(unsigned)((N + T - 1) / T), T, 0, v.s>>>(v.A, d, f);
    k_frame_line<<<(unsigned)((nx + T - 1) / T), T, 0, v.s>>>(v.P, v.A, d, f);
    CU_CK(cudaGetLastError());
    CU_CK(cudaMemcpyAsync(sg.host, sg.dev, ebytes + pbytes + nbytes + lbytes, cudaMemcpyDeviceToHost, v.s));
    CU_CK(cudaStreamSynchronize(v.s));
    const char *h = static_cast<const char *>(sg.host);
    const float *ef = reinterpret_cast<const float *>(h);
    const int *ph = reinterpret_cast<const int *>(h + ebytes);
    const float *nf = reinterpret_cast<const float *>(h + ebytes + pbytes);
    const float *lf = reinterpret_cast<const float *>(h + ebytes + pbytes + nbytes);

    const long long nrec = next_record(dir, "_contents.0", fresh);
    char line[128];
    std::snprintf(line, sizeof line, "%6lld %8d %10.6f\n", nrec, k.nloop, k.time / GF_SEC_YEAR / 1.e6);
    IO_CK(append_line(dir, "_contents.0", fresh, line));
    const float rtime = (float)k.time;
    IO_CK(write_record(dir, "time.0", nrec, &rtime, 4, 4));
    const int *io = p.io_flags; // vel srII eII aps sII sxx szz sxz pres temp phase visc - density src diss forc hfl topo
    auto el = [&](const char *name, int fld) { return write_record(dir, name, nrec, ef + (size_t)fld * E, E * 4, E * 4); };
    IO_CK(write_record(dir, "mesh.0", nrec, nf + (size_t)NF_MESH * N, 2 * N * 4, 2 * N * 4));
    if (io[0] == 1) IO_CK(write_record(dir, "vel.0", nrec, nf + (size_t)NF_VEL * N, 2 * N * 4, 2 * N * 4));
    if (io[9] == 1) IO_CK(write_record(dir, "temperature.0", nrec, nf + (size_t)NF_TEMP * N, N * 4, N * 4));
    IO_CK(write_record(dir, "coolingrate.0", nrec, nf + (size_t)NF_COOL * N, N * 4, N * 4));
    IO_CK(write_record(dir, "xoriginal.0", nrec, nf + (size_t)NF_XORIG * N, N * 4, N * 4));
    IO_CK(write_record(dir, "zoriginal.0", nrec, nf + (size_t)NF_ZORIG * N, N * 4, N * 4));
    if (io[1] == 1) {
        IO_CK(el("srII.0", EF_SRII));
        IO_CK(el("srxx.0", EF_SRXX));
        IO_CK(el("srzz.0", EF_SRZZ));
        IO_CK(el("srxz.0", EF_SRXZ));
    }
    if (io[2] == 1) {
        IO_CK(el("eII.0", EF_EII));
        IO_CK(el("eI.0", EF_EI));
        IO_CK(el("exx.0", EF_EXX));
        IO_CK(el("ezz.0", EF_EZZ));
        IO_CK(el("exz.0", EF_EXZ));
    }
    if (io[13] == 1) {
        IO_CK(el("density.0", EF_DENS));
        IO_CK(el("area.0", EF_AREA));
    }
    if (io[3] == 1) IO_CK(el("aps.0", EF_APS));
    if (io[4] == 1) IO_CK(el("sII.0", EF_SII));
    if (io[5] == 1) IO_CK(el("sxx.0", EF_SXX));
    if (io[6] == 1) IO_CK(el("szz.0", EF_SZZ));
    if (io[7] == 1) {
        IO_CK(el("sxz.0", EF_SXZ));
        IO_CK(el("syy.0", EF_SYY));
    }
    if (io[8] == 1) IO_CK(el("pres.0", EF_PRES));
    if (io[9] == 1) IO_CK(el("temp.0", EF_TEMP));
    if (io[10] == 1) IO_CK(write_record(dir, "phase.0", nrec, ph, E * 4, E * 4));
    if (io[11] == 1) IO_CK(el("visc.0", EF_VISC));
    if (io[14] == 1) {
        IO_CK(el("src.0", EF_SRC));
        IO_CK(el("fmelt.0", EF_FMELT));
        IO_CK(el("fmelt2.0", EF_FMELT2));
        IO_CK(el("fmagma.0", EF_FMAGMA));
        IO_CK(el("fmagma2.0", EF_FMAGMA2));
    }
    if (io[15] == 1) IO_CK(el("diss.0", EF_DISS));
    if (io[17] == 1) IO_CK(write_record(dir, "hfl.0", nrec, lf + (size_t)LF_HFL * nx, nx * 4, nx * 4));
    if (io[18] == 1) {
        IO_CK(write_record(dir, "topo.0", nrec, lf + (size_t)LF_TOPO * nx, nx * 4, nx * 4));
        IO_CK(write_record(dir, "dtopo.0", nrec, lf + (size_t)LF_DTOPO * nx, nx * 4, nx * 4));
        IO_CK(write_record(dir, "extrusion.0", nrec, lf + (size_t)LF_EXTR * nx, (nx - 1) * 4, (nx - 1) * 4));
    }
    return GF_OK;
}

int gf_outmarker(gf_ctx *ctx, const char *dir, int fresh) {
    if (!ctx) return GF_ERR_ARG;
    GfMemberView v;
    IO_CK(gf_ctx_view(ctx, &v));
    gf_clock k;
    IO_CK(gf_get_clock(ctx, &k));
    const int nm = k.nmarkers;
    const long long nrec = next_record(dir, "_markers.0", fresh);
    char line[128];
    std::snprintf(line, sizeof line, "%6lld %8d %8d %10.6f\n", nrec, k.nloop, nm, k.time / GF_SEC_YEAR / 1.e6);
    IO_CK(append_line(dir, "_markers.0", fresh, line));
    if (nm <= 0) return GF_OK;
    Staging sg;
    const size_t fb = (size_t)5 * nm * 4, ib = (size_t)3 * nm * 4;
    IO_CK(sg.alloc(fb + ib));
    float *fo = static_cast<float *>(sg.dev);
    int *io = reinterpret_cast<int *>(static_cast<char *>(sg.dev) + fb);
    k_frame_markers<<<(unsigned)((nm + 255) / 256), 256, 0, v.s>>>(v.A, v.d, nm, fo, io);
    CU_CK(cudaGetLastError());
    CU_CK(cudaMemcpyAsync(sg.host, sg.dev, fb + ib, cudaMemcpyDeviceToHost, v.s));
    CU_CK(cudaStreamSynchronize(v.s));
    const float *hf = static_cast<const float *>(sg.host);
    const int *hi = reinterpret_cast<const int *>(static_cast<const char *>(sg.host) + fb);
    char n1[64], n2[64];
    std::snprintf(n1, sizeof n1, "marker1.%06lld.0", nrec);
    std::snprintf(n2, sizeof n2, "marker2.%06lld.0", nrec);
    for (int r = 0; r < 5; ++r) IO_CK(write_record(dir, n1, r + 1, hf + (size_t)r * nm, nm * 4, nm * 4));
    for (int r = 0; r < 3; ++r) IO_CK(write_record(dir, n2, r + 1, hi + (size_t)r * nm, nm * 4, nm * 4));
    return GF_OK;
}

int gf_saveflac(gf_ctx *ctx, const char *dir) {
    if (!ctx) return GF_ERR_ARG;
    IO_CK(gf_download(ctx, GF_F_ALL));
    GfMemberView v;
    IO_CK(gf_ctx_view(ctx, &v));
    gf_clock k;
    IO_CK(gf_get_clock(ctx, &k));
    const gf_params &p = *v.hp;
    const gf_layout &L = *v.L;
    if (!L.cord || !L.vel || !L.strain || !L.stress0 || !L.temp || !L.iphase || !L.aps || !L.mark_a1 ||
        !L.mark_ntriag)
        return GF_ERR_ARG; // the host mirror must hold every saved field
    const long long E = v.d.E, N = v.d.N, nx = v.d.nx;
    const int nm = k.nmarkers;
    std::vector<double> orig((size_t)2 * N);
    CU_CK(cudaMemcpy(orig.data(), v.A.orig, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost));
    char line[160];
    std::snprintf(line, sizeof line, "%4d %8d %6.2f %9d %9d\n", 1, k.nloop, k.time / GF_SEC_YEAR / 1.e6, nm, 0);
    IO_CK(append_line(dir, "_contents.save", 1, line));
    double td[2] = {k.time, k.dt};
    IO_CK(write_record(dir, "time.rs", 1, td, 16, 16));
    std::vector<double> zeros((size_t)std::max(std::max(E, N), nx), 0.0);
    auto w8 = [&](const char *name, const double *a, long long n) {
        return write_record(dir, name, 1, a ? a : zeros.data(), (size_t)n * 8, (size_t)n * 8);
    };
    IO_CK(w8("cord.rs", L.cord, 2 * N));
    // surface and flexure accumulators
    IO_CK(w8("dhacc.rs", L.dhacc, nx - 1));
    IO_CK(w8("dhacc_corr.rs", L.dhacc_correction, nx));
    IO_CK(w8("extr_acc.rs", L.extr_acc, nx - 1));
    IO_CK(w8("q_init.rs", L.q_init, nx));
    IO_CK(w8("vel_flex_old.rs", L.vel_flex_old, nx));
    IO_CK(w8("vel.rs", L.vel, 2 * N));
    IO_CK(w8("strain.rs", L.strain, 3 * E));
    IO_CK(w8("stress.rs", L.stress0, 16 * E));
    IO_CK(w8("temp.rs", L.temp, N));
    IO_CK(w8("xoriginal.rs", orig.data(), N));
    IO_CK(w8("zoriginal.rs", orig.data() + N, N));
    // int32 phases in a record of 8 bytes per element (saveflac.f90:97-100)
    IO_CK(write_record(dir, "phase.rs", 1, L.iphase, (size_t)E * 4, (size_t)E * 8));
    IO_CK(w8("aps.rs", L.aps, E));
    IO_CK(w8("fmagma.rs", L.fmagma, E));
    IO_CK(w8("fmagma2.rs", L.fmagma2, E));
    IO_CK(w8("source.rs", L.source, E));
    IO_CK(w8("dike_backlog.rs", L.dike_backlog, E));
    IO_CK(w8("dike_marker_vol.rs", L.dike_marker_vol, E));
    IO_CK(w8("mor_marker_vol.rs", L.mor_marker_vol, E));
    std::snprintf(line, sizeof line, " %.17E\n", p.Amin);
    IO_CK(append_line(dir, "Amin.rs", 1, line));
    if (p.nyhydro == 2) { // read back by rsflac.f90:219-225
        std::snprintf(line, sizeof line, " %.17E\n", p.pisos);
        IO_CK(append_line(dir, "pisos.rs", 1, line));
    }
    if (nm > 0) {
        const size_t b8 = (size_t)nm * 8, b4 = (size_t)nm * 4;
        IO_CK(write_record(dir, "marker1.rs", 1, L.mark_a1, b8, b8));
        IO_CK(write_record(dir, "marker1.rs", 2, L.mark_a2, b8, b8));
        IO_CK(write_record(dir, "marker1.rs", 3, L.mark_age, b8, b8));
        // byte-sized fields widened to int32 records (saveflac.f90:155-169)
        std::vector<int> w((size_t)nm);
        for (int m = 0; m < nm; ++m) w[m] = L.mark_dead[m];
        IO_CK(write_record(dir, "marker2.rs", 1, w.data(), b4, b4));
        IO_CK(write_record(dir, "marker2.rs", 2, L.mark_ntriag, b4, b4));
        for (int m = 0; m < nm; ++m) w[m] = L.mark_phase[m];
        IO_CK(write_record(dir, "marker2.rs", 3, w.data(), b4, b4));
    }
    return GF_OK;
}

int gf_rsflac(gf_ctx *ctx, const char *dir) {
    if (!ctx) return GF_ERR_ARG;
    GfMemberView v;
    IO_CK(gf_ctx_view(ctx, &v));
    gf_params p = *v.hp;
    gf_layout &L = *v.L;
    if (!L.cord || !L.vel || !L.strain || !L.stress0 || !L.temp || !L.iphase || !L.aps || !L.mark_a1 ||
        !L.mark_ntriag || !L.mark_id_elem || !L.nmark_elem || !L.bc || !L.ncod || !L.jmoho)
        return GF_ERR_ARG;
    const long long E = v.d.E, N = v.d.N, nx = v.d.nx, nz = v.d.nz;
    // _contents.rs, or _contents.save as saveflac writes it
    FILE *f = std::fopen(path_of(dir, "_contents.rs").c_str(), "r");
    if (!f) f = std::fopen(path_of(dir, "_contents.save").c_str(), "r");
    if (!f) return GF_ERR_IO;
    long long nrec = 0, nmk = 0, unused = 0;
    int nloop = 0;
    double time_my = 0;
    int got = std::fscanf(f, "%lld %d %lf %lld %lld", &nrec, &nloop, &time_my, &nmk, &unused);
    std::fclose(f);
    if (got < 4 || nrec < 1 || nmk < 0 || nmk > (long long)L.max_markers) return GF_ERR_PARSE;
    const int nm = (int)nmk;
    double td[2];
    IO_CK(read_record(dir, "time.rs", nrec, td, 16, 16));
    auto r8 = [&](const char *name, double *a, long long n) {
        return a ? read_record(dir, name, nrec, a, (size_t)n * 8, (size_t)n * 8) : GF_OK;
    };
    std::vector<double> orig((size_t)2 * N);
    IO_CK(r8("cord.rs", L.cord, 2 * N));
    IO_CK(r8("dhacc.rs", L.dhacc, nx - 1));
    IO_CK(r8("dhacc_corr.rs", L.dhacc_correction, nx));
    IO_CK(r8("extr_acc.rs", L.extr_acc, nx - 1));
    IO_CK(r8("vel.rs", L.vel, 2 * N));
    IO_CK(r8("strain.rs", L.strain, 3 * E));
    IO_CK(r8("stress.rs", L.stress0, 16 * E));
    IO_CK(r8("temp.rs", L.temp, N));
    // both files are read into their own arrays (rsflac.f90:99-104 reads
    // zoriginal.rs into xoriginal)
    IO_CK(r8("xoriginal.rs", orig.data(), N));
    IO_CK(r8("zoriginal.rs", orig.data() + N, N));
    if (L.xoriginal) std::memcpy(L.xoriginal, orig.data(), sizeof(double) * N);
    if (L.zoriginal) std::memcpy(L.zoriginal, orig.data() + N, sizeof(double) * N);
    IO_CK(r8("q_init.rs", L.q_init, nx));
    IO_CK(r8("vel_flex_old.rs", L.vel_flex_old, nx));
    IO_CK(read_record(dir, "phase.rs", nrec, L.iphase, (size_t)E * 4, (size_t)E * 8));
    for (long long e = 0; e < E; ++e)
        if (L.iphase[e] < 1 || L.iphase[e] > p.nphase) return GF_ERR_PARSE;
    IO_CK(r8("aps.rs", L.aps, E));
    IO_CK(r8("fmagma.rs", L.fmagma, E));
    IO_CK(r8("fmagma2.rs", L.fmagma2, E));
    IO_CK(r8("source.rs", L.source, E));
    IO_CK(r8("dike_backlog.rs", L.dike_backlog, E));
    IO_CK(r8("dike_marker_vol.rs", L.dike_marker_vol, E));
    IO_CK(r8("mor_marker_vol.rs", L.mor_marker_vol, E));
    // melt fractions restart at zero (rsflac.f90:239-240)
    for (double *a : {L.fmelt, L.fmelt2})
        if (a) std::memset(a, 0, sizeof(double) * (size_t)E);
    f = std::fopen(path_of(dir, "Amin.rs").c_str(), "r");
    if (!f) return GF_ERR_IO;
    got = std::fscanf(f, "%lf", &p.Amin);
    std::fclose(f);
    if (got != 1) return GF_ERR_PARSE;
    if (p.nyhydro == 2) {
        f = std::fopen(path_of(dir, "pisos.rs").c_str(), "r");
        if (!f) return GF_ERR_IO;
        got = std::fscanf(f, "%lf", &p.pisos);
        std::fclose(f);
        if (got != 1) return GF_ERR_PARSE;
    }
    // smallest element width and thickness (rsflac.f90:38-39)
    double dxmin = 1e300, dzmin = 1e300;
    for (long long i = 1; i < nx; ++i) dxmin = std::fmin(dxmin, L.cord[i * nz] - L.cord[(i - 1) * nz]);
    for (long long j = 0; j < nz - 1; ++j) dzmin = std::fmin(dzmin, L.cord[N + j] - L.cord[N + j + 1]);
    p.dxmin = dxmin;
    p.dzmin = dzmin;
    if (nm > 0) {
        const size_t b8 = (size_t)nm * 8, b4 = (size_t)nm * 4;
        IO_CK(read_record(dir, "marker1.rs", 1, L.mark_a1, b8, b8));
        IO_CK(read_record(dir, "marker1.rs", 2, L.mark_a2, b8, b8));
        IO_CK(read_record(dir, "marker1.rs", 3, L.mark_age, b8, b8));
        std::vector<int> w((size_t)nm);
        IO_CK(read_record(dir, "marker2.rs", 1, w.data(), b4, b4));
        for (int m = 0; m < nm; ++m) L.mark_dead[m] = (int8_t)w[m];
        IO_CK(read_record(dir, "marker2.rs", 2, L.mark_ntriag, b4, b4));
        IO_CK(read_record(dir, "marker2.rs", 3, w.data(), b4, b4));
        for (int m = 0; m < nm; ++m) L.mark_phase[m] = (int8_t)w[m];
    }
    // element marker lists in marker order (rsflac.f90:146-172); a full
    // element skips the marker as the reference does
    std::memset(L.mark_id_elem, 0, sizeof(int) * (size_t)GF_MAX_MARKERS_PER_ELEM * E);
    std::memset(L.nmark_elem, 0, sizeof(int) * (size_t)E);
    for (int m = 0; m < nm; ++m) {
        if (L.mark_dead[m] == 0) continue;
        const long long nt = L.mark_ntriag[m];
        if (nt < 1 || nt > 2 * E) return 999; // stop 999
        const long long kk = (nt - 1) % 2 + 1;
        const long long j = ((nt - kk) / 2) % (nz - 1), i = (nt - kk) / 2 / (nz - 1);
        const long long e = i * (nz - 1) + j;
        if (L.nmark_elem[e] == GF_MAX_MARKERS_PER_ELEM) continue;
        L.nmark_elem[e] += 1;
        L.mark_id_elem[e * GF_MAX_MARKERS_PER_ELEM + L.nmark_elem[e] - 1] = m + 1;
    }
    IO_CK(gf_set_params(ctx, &p));
    gf_clock k;
    IO_CK(gf_get_clock(ctx, &k));
    k.nloop = nloop;
    k.time = td[0];
    k.dt = td[1];
    k.dtavg = 0.0;
    k.frac = p.frac;
    k.nmarkers = nm;
    k.nsrate = -1;
    k.need_remeshing = 0;
    IO_CK(gf_set_clock(ctx, &k));
    IO_CK(gf_upload(ctx, GF_F_CORD | GF_F_VEL | GF_F_TEMP | GF_F_STRESS | GF_F_STRAIN | GF_F_APS | GF_F_PHASE |
                             GF_F_RATE | GF_F_MARKERS));
    CU_CK(cudaMemcpy(v.A.orig, orig.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice));
    // marker2elem, then check_visc_rheol and init_bc on the host with the
    // phases and Moho rows it produced
    IO_CK(gf_marker2elem(ctx));
    IO_CK(gf_download(ctx, GF_F_PHASE));
    p = *v.hp;
    IO_CK(gf_host_restart_bc(&p, &L));
    IO_CK(gf_set_params(ctx, &p));
    IO_CK(gf_upload(ctx, GF_F_BC));
    return gf_ctx_restart_finish(ctx);
}

} // extern "C"
