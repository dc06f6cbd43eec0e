// Index helpers for the reference's column-major layout (0-based here).
//
// Node (j,i): j = 0..nz-1 (depth, fastest), i = 0..nx-1.
// Element (j,i): j = 0..nz-2, i = 0..nx-2.
// Triangle k = 0..3 is the reference's A,B,C,D (src/fl_node.f90:14-35).
#pragma once

#ifdef __CUDACC__
#define GF_HD __host__ __device__ __forceinline__
#else
#define GF_HD inline
#endif

struct GfDims {
    int nx, nz, nphase;
    long long N; // nodes
    long long E; // elements
};

GF_HD long long gf_node(const GfDims &d, int j, int i) { return (long long)i * d.nz + j; }
GF_HD long long gf_elem(const GfDims &d, int j, int i) { return (long long)i * (d.nz - 1) + j; }
// cord(j,i,k), vel(j,i,k), bc, ncod: k = 0 (x) or 1 (z)
GF_HD long long gf_n2(const GfDims &d, int j, int i, int k) { return k * d.N + gf_node(d, j, i); }
// stress0(j,i,c,k): c = component (0 sxx, 1 szz, 2 sxz, 3 syy), k = triangle
GF_HD long long gf_s(const GfDims &d, long long e, int c, int k) { return (long long)(c + 4 * k) * d.E + e; }
// area(j,i,k), dvol(j,i,k), strain(j,i,k), se2sr(j,i,k)
GF_HD long long gf_ek(const GfDims &d, long long e, int k) { return (long long)k * d.E + e; }
// phase_ratio(ph,j,i)
GF_HD long long gf_pr(const GfDims &d, long long e, int ph) { return e * d.nphase + ph; }

// LCG of src/myrandom_mod.f90:9-19 (returns r in [0,1), updates seed)
GF_HD double gf_myrandom(int &iseed) {
    iseed = iseed % 134456;
    iseed = (8121 * iseed + 28411) % 134456;
    return (iseed * 1.0) / 134456;
}
