// Index helpers for the reference's column-major layout (0-based here).
//
// Node (j,i): j = 0..nz-1 (depth, fastest), i = 0..nx-1.
// Element (j,i): j = 0..nz-2, i = 0..nx-2.
// Triangle k = 0..3 is the reference's A,B,C,D (src/fl_node.f90:14-35).
#pragma once

// static: each translation unit has its own copy (their index types may
// differ, see GF_IDX)
#ifdef __CUDACC__
#define GF_HD static __host__ __device__ __forceinline__
#else
#define GF_HD static inline
#endif

// Index type of the kernel code: 64-bit by default; a translation unit may
// define GF_IDX as int before its includes when every index of its arrays
// stays below 2^31 (the mixed-precision and ensemble units).
#ifndef GF_IDX
#define GF_IDX long long
#endif
struct GfDims {
    int nx, nz, nphase;
    long long N; // nodes
    long long E; // elements
};

GF_HD GF_IDX gf_node(const GfDims &d, int j, int i) { return (GF_IDX)i * (GF_IDX)d.nz + j; }
GF_HD GF_IDX gf_elem(const GfDims &d, int j, int i) { return (GF_IDX)i * (GF_IDX)(d.nz - 1) + j; }
// cord(j,i,k), vel(j,i,k), bc, ncod: k = 0 (x) or 1 (z)
GF_HD GF_IDX gf_n2(const GfDims &d, int j, int i, int k) { return (GF_IDX)k * (GF_IDX)d.N + gf_node(d, j, i); }
// stress0(j,i,c,k): c = component (0 sxx, 1 szz, 2 sxz, 3 syy), k = triangle
GF_HD GF_IDX gf_s(const GfDims &d, GF_IDX e, int c, int k) { return (GF_IDX)(c + 4 * k) * (GF_IDX)d.E + e; }
// area(j,i,k), dvol(j,i,k), strain(j,i,k), se2sr(j,i,k)
GF_HD GF_IDX gf_ek(const GfDims &d, GF_IDX e, int k) { return (GF_IDX)k * (GF_IDX)d.E + e; }
// phase_ratio(ph,j,i)
GF_HD GF_IDX gf_pr(const GfDims &d, GF_IDX e, int ph) { return e * (GF_IDX)d.nphase + ph; }

// LCG of src/myrandom_mod.f90:9-19 (returns r in [0,1), updates seed)
GF_HD double gf_myrandom(int &iseed) {
    iseed = iseed % 134456;
    iseed = (8121 * iseed + 28411) % 134456;
    return (iseed * 1.0) / 134456;
}
