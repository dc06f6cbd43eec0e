// Kernels of the explicit FLAC step, templated on the element-field type R
// (double for GF_MODE_FP64, float for GF_MODE_MIXED).  Each __device__
// routine restates one reference routine in the reference's evaluation order;
// the FP64 translation unit is compiled without FMA contraction so that its
// arithmetic is the serial Fortran's.
//
// Layout: element e = i*(nz-1)+j and node n = i*nz+j (j = depth, fastest), so
// consecutive threads touch consecutive addresses of every field.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gf_ctx.h"
#include "gf_math.h"

// internal linkage: each precision's translation unit has its own copy
namespace {
namespace gfk {

// ---------------------------------------------------------------- math
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sin(double x) { return gfm::sin(x); }
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ double m_tan(double x) { return gfm::tan(x); }
__device__ __forceinline__ float m_tan(float x) { return tanf(x); }
// sine and tangent of an angle in degrees: FP64 as the reference evaluates
// them (sin(phi * degrad)); FP32 through sinpi/cospi, whose argument
// reduction needs no local-memory slow path
__device__ __forceinline__ double m_sind(double deg) { return gfm::sin(deg * (3.14159265358979323846 / 180.0)); }
__device__ __forceinline__ float m_sind(float deg) { return sinpif(deg * (1.0f / 180.0f)); }
__device__ __forceinline__ double m_tand(double deg) { return gfm::tan(deg * (3.14159265358979323846 / 180.0)); }
__device__ __forceinline__ float m_tand(float deg) {
    const float x = deg * (1.0f / 180.0f);
    return sinpif(x) / cospif(x);
}
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }

// Programmatic dependent launch: the kernels of the step are launched with
// programmatic stream serialization, so that each one's CTAs can be placed on
// SMs while the kernel before it drains.  Every such kernel calls this
// first: it lets the next kernel launch early and waits until the kernel
// before it has finished and its writes are visible, before reading anything.
__device__ __forceinline__ void gf_pdl_entry() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void set_status(DevClock *C, int code, int where) {
    if (atomicCAS(&C->status, 0, code) == 0) C->status_aux = where;
}

// atomic min / max on non-negative doubles through their bit patterns
__device__ __forceinline__ void atomic_min_pos(unsigned long long *slot, double v) {
    atomicMin(slot, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_pos(unsigned long long *slot, double v) {
    atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

template <class T> __device__ __forceinline__ T warp_min(T v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <class T> __device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <class T> __device__ __forceinline__ T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

struct Quad {
    double x[4], y[4]; // nodes 1..4 = (j,i), (j+1,i), (j,i+1), (j+1,i+1)
};

__device__ __forceinline__ void load_quad(const double *__restrict__ cord, const GfDims &d, int j, int i, Quad &q) {
    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    q.x[0] = cord[n1];
    q.x[1] = cord[n1 + 1];
    q.x[2] = cord[n3];
    q.x[3] = cord[n3 + 1];
    q.y[0] = cord[d.N + n1];
    q.y[1] = cord[d.N + n1 + 1];
    q.y[2] = cord[d.N + n3];
    q.y[3] = cord[d.N + n3 + 1];
}

// Conversions between FP64 and FP32 on the integer pipe (mixed path).  On
// GB300 the FP64 pipe runs at 1/64 of the FP32 rate and the conversion
// instructions between the two formats issue to it; a mixed kernel that
// converts a few values per item is bound by that pipe.  These give the
// conversion instructions' results with integer operations:
//   gf_d2f: round to nearest even for finite values whose float is normal
//           (smaller magnitudes give a signed zero, larger an infinity);
//   gf_f2d: exact (float subnormals give a signed zero).
__device__ __forceinline__ float gf_d2f(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127; // float exponent
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    // mantissa bits 51..29 kept (20 from hi, 3 from lo), 28..0 dropped
    unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu, half = 0x10000000u;
    m += (rem > half || (rem == half && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(sign + ((unsigned)e << 23) + m); // a carry out of m raises the exponent
}
__device__ __forceinline__ double gf_f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    if (e == 0u) return __longlong_as_double((long long)((unsigned long long)sign << 32));
    const unsigned ed = (e == 255u) ? 0x7ffu : e - 127u + 1023u;
    const unsigned hi = sign | (ed << 20) | (m >> 3);
    return __longlong_as_double((long long)(((unsigned long long)hi << 32) | ((unsigned long long)(m & 7u) << 29)));
}
// The two 32-bit halves of a double's bit pattern and back, through an
// opaque move: the compiler would otherwise turn integer tests of the bits
// (a zero test, say) back into FP64 comparisons, which take a slot of the
// FP64 pipe.
__device__ __forceinline__ void gf_dsplit(double x, unsigned &lo, unsigned &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
__device__ __forceinline__ double gf_djoin(unsigned lo, unsigned hi) {
    double x;
    asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
    return x;
}
// Biased exponent field and zero test of a double, on the integer pipe.
__device__ __forceinline__ unsigned gf_dexp(double x) {
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    return (hi >> 20) & 0x7ffu;
}
__device__ __forceinline__ bool gf_dzero(double x) {
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    return ((hi << 1) | lo) == 0u;
}
// |x| in [2^-450, 2^451) (biased exponents 573 .. 1473): quotients and
// products of two such numbers are normal doubles
__device__ __forceinline__ bool gf_dmid(double x) { return gf_dexp(x) - 573u <= 900u; }

// FP64 multiplication on the integer pipes.  GB300 issues FP64 arithmetic
// at 1/64 of the FP32 rate, and the FP64 kernels wait on that pipe while
// the integer pipes idle, so a product of two doubles is formed here from
// their 53-bit significands with four 32x32->64-bit integer multiplies and
// rounded to nearest even: the bits of IEEE multiplication.  It covers
// operands that are zero or inside gf_dmid (the product is then a normal
// double or a signed zero); any other operand takes the FP64 multiply in a
// call that is not inlined, so that the common path issues no FP64
// instruction (a predicated-off FP64 multiply still takes its pipe slot).
// Restated with Python integers and checked against IEEE products, exact
// and near ties included, by tests/test_int_multiply.py.
__device__ __noinline__ double gf_mul_rare(double a, double b) { return a * b; }
__device__ __forceinline__ double gf_mul(double a, double b) {
    unsigned la, ha, lb, hb;
    gf_dsplit(a, la, ha);
    gf_dsplit(b, lb, hb);
    const bool za = ((ha << 1) | la) == 0u, zb = ((hb << 1) | lb) == 0u;
    const bool ia = ((ha >> 20) & 0x7ffu) - 573u <= 900u, ib = ((hb >> 20) & 0x7ffu) - 573u <= 900u;
    if (!((ia || za) && (ib || zb))) return gf_mul_rare(a, b);
    // significands with the hidden bit (21 high bits : 32 low bits) and
    // their 106-bit product w2:w1:w0:wm, w2 < 2^10
    const unsigned mh = (ha & 0xfffffu) | 0x100000u, nh = (hb & 0xfffffu) | 0x100000u;
    const unsigned long long p0 = (unsigned long long)la * lb;
    unsigned long long t = (unsigned long long)la * nh + (p0 >> 32);
    t += (unsigned long long)mh * lb;
    const unsigned long long u = (unsigned long long)mh * nh + (t >> 32);
    const unsigned w2 = (unsigned)(u >> 32), w1 = (unsigned)u, w0 = (unsigned)t, wm = (unsigned)p0;
    // product of the significands in [2, 4): keep bits 105..53, else 104..52
    const unsigned top = w2 >> 9, sh = 12u - top;
    const unsigned mhi = __funnelshift_l(w1, w2, sh), mlo = __funnelshift_l(w0, w1, sh);
    // the dropped bits of w0, left-aligned (round bit first; sh >= 11 low
    // zeros), and the sticky bit of wm or the kept value's parity: round up
    // iff rem > half, or rem == half and (sticky or odd)
    const unsigned rem = w0 << sh, x = min(wm, 1u) | (mlo & 1u);
    const unsigned up = (rem + x) > 0x80000000u ? 1u : 0u;
    // sign and biased exponent less one (mhi's hidden bit adds the one); the
    // sum of the sign bits wraps to their exclusive or, and the exponent sum
    // ea + eb - 1024 + top lies in [122, 1923]
    const unsigned S = (ha & 0xfff00000u) + (hb & 0xfff00000u) - (1024u << 20) + (top << 20);
    const unsigned long long r = ((unsigned long long)(mhi + S) << 32 | mlo) + up; // a carry out of the
                                                                                   // significand raises the exponent
    if (za || zb) return gf_djoin(0u, (ha ^ hb) & 0x80000000u);
    return gf_djoin((unsigned)r, (unsigned)(r >> 32));
}
__device__ __forceinline__ float gf_mul(float a, float b) { return a * b; }

// RN(1/b) without the FP64 pipe, for b inside gf_dmid (other b, and zero,
// take the IEEE division out of line).  With b = M 2^(E-1075), M in
// (2^52, 2^53), the significand of 1/b is q = RN(T), T = 2^105 / M in
// (2^52, 2^53):
//   1. float-float on the FP32 pipe: r = RN32(1/Mh) for the top 24 bits Mh
//      of M, corrected by the next 24 bits Ml (r + r (1 - (Mh + Ml) r)):
//      t1 = that times 2^53, within about 2^8 units of T;
//   2. one Newton-Raphson step for the reciprocal, t + t (1 - M t / 2^105),
//      in 64-bit integers: R = 2^105 - M t1 (below 2^62, so its low 64 bits
//      are exact), t = t1 + floor(R t1 / 2^105), within one unit of T;
//   3. the midpoint tests 2^106 - M (2t + 1) > 0 and 2^106 - M (2t - 1) < 0
//      (exact in 64 bits; never zero, as 2^106 / M is no half-integer for
//      M not a power of two) move t to RN(T).
// A power-of-two b has the exact reciprocal.  Restated on words and checked
// against IEEE division by tests/test_int_reciprocal.py.
__device__ __noinline__ double gf_rcp_rare(double b) { return 1.0 / b; }
// RN(2^105 / M) for the significand M = 2^52 + mhi:lo (steps 1-3 above)
__device__ __forceinline__ long long gf_rcp_sig(unsigned mhi, unsigned lo) {
    const float Mh = __uint_as_float(0x3f800000u | (((mhi << 3) | (lo >> 29)) & 0x7fffffu));
    const float Ml = __uint2float_rn((lo >> 5) & 0xffffffu) * 0x1p-47f; // exact
    const float r = __frcp_rn(Mh);
    const float e2 = fmaf(-Ml, r, fmaf(-Mh, r, 1.0f));
    const float rl = __fmul_rn(r, e2);
    // t1 = r 2^53 + trunc(rl 2^53) from the floats' bits (r in (0.5, 1],
    // |rl| < 2^-22)
    const unsigned ur = __float_as_uint(r), ul = __float_as_uint(rl);
    const int er = (int)((ur >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu), sh = el - 97;
    const unsigned Sl = (ul & 0x7fffffu) | 0x800000u;
    const unsigned v = el == 0 ? 0u : sh >= 0 ? Sl << sh : sh > -32 ? Sl >> -sh : 0u;
    long long t = ((long long)((ur & 0x7fffffu) | 0x800000u) << (er - 97)) + ((ul >> 31) ? -(long long)v : (long long)v);
    const unsigned long long M = ((unsigned long long)(mhi | 0x100000u) << 32) | lo;
    const long long R = -(long long)(M * (unsigned long long)t);
    t += __mul64hi(R, t) >> 41;
    const long long Dp = -(long long)(M * (unsigned long long)(2 * t + 1));
    return t + (Dp > 0 ? 1 : (Dp + (long long)(2 * M) < 0 ? -1 : 0));
}
__device__ __forceinline__ double gf_rcp(double b) {
    unsigned lo, hi;
    gf_dsplit(b, lo, hi);
    const unsigned E = (hi >> 20) & 0x7ffu;
    if (E - 573u > 900u) return gf_rcp_rare(b);
    const unsigned sign = hi & 0x80000000u, mhi = hi & 0xfffffu;
    if ((mhi | lo) == 0u) return gf_djoin(0u, sign | ((2046u - E) << 20));
    const unsigned long long bits = ((unsigned long long)(2044u - E) << 52) + (unsigned long long)gf_rcp_sig(mhi, lo);
    return gf_djoin((unsigned)bits, (unsigned)(bits >> 32) | sign);
}

// RN(a/b) without the FP64 pipe, for a zero or inside gf_dmid and b inside
// gf_dmid (others take the IEEE division out of line).  With significands
// Ma, Mb, the quotient's significand is RN(Q), Q = Ma 2^k / Mb in
// [2^52, 2^53) (k = 52 if Ma >= Mb, else 53): q = floor(Ma t / 2^(105-k))
// from t = RN(2^105 / Mb) lies within 2 of Q; the exact residual
// Ma 2^k - Mb q (below 2^55 in magnitude, so its low 64 bits are exact)
// brings q to floor(Q) with at most two steps each way, and 2 (residual) >
// Mb rounds it up (no ties: a quotient of two 53-bit significands is never
// halfway between two 53-bit values).  Restated on words and checked
// against IEEE division by tests/test_int_reciprocal.py.
__device__ __noinline__ double gf_ddiv_rare(double a, double b) { return a / b; }
__device__ __forceinline__ double gf_ddiv(double a, double b) {
    unsigned la, ha, lb, hb;
    gf_dsplit(a, la, ha);
    gf_dsplit(b, lb, hb);
    const unsigned Ea = (ha >> 20) & 0x7ffu, Eb = (hb >> 20) & 0x7ffu;
    const bool za = ((ha << 1) | la) == 0u;
    if (!((Ea - 573u <= 900u || za) && Eb - 573u <= 900u)) return gf_ddiv_rare(a, b);
    const unsigned sign = (ha ^ hb) & 0x80000000u;
    if (za) return gf_djoin(0u, sign);
    const unsigned long long Ma = ((unsigned long long)((ha & 0xfffffu) | 0x100000u) << 32) | la;
    const unsigned long long Mb = ((unsigned long long)((hb & 0xfffffu) | 0x100000u) << 32) | lb;
    const unsigned long long t = (unsigned long long)gf_rcp_sig(hb & 0xfffffu, lb);
    const int k = Ma >= Mb ? 52 : 53;
    unsigned long long q = (__umul64hi(Ma, t) << (k - 41)) | ((Ma * t) >> (105 - k));
    long long res = (long long)((Ma << k) - Mb * q);
    if (res < 0) { --q; res += (long long)Mb; }
    if (res < 0) { --q; res += (long long)Mb; }
    if (res >= (long long)Mb) { ++q; res -= (long long)Mb; }
    if (res >= (long long)Mb) { ++q; res -= (long long)Mb; }
    q += 2 * res > (long long)Mb ? 1u : 0u;
    const unsigned long long bits = ((unsigned long long)(1074 - k + (int)Ea - (int)Eb) << 52) + q;
    return gf_djoin((unsigned)bits, (unsigned)(bits >> 32) | sign);
}
__device__ __forceinline__ float gf_ddiv(float a, float b) { return a / b; }

// x * 2^K (K = -2 .. 2, the constant factors 0.25 .. 4 of the step): the
// exponent field moves by K while x and the result are normal doubles, a
// zero keeps its bits, and anything else takes the FP64 multiply out of line.
template <int K> __device__ __forceinline__ double gf_scale(double x) {
    static_assert(K >= -2 && K <= 2 && K != 0, "factor 0.25, 0.5, 2 or 4");
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    const unsigned e = (hi >> 20) & 0x7ffu;
    constexpr unsigned lo_e = (unsigned)(K < 0 ? 1 - K : 1), hi_e = (unsigned)(K < 0 ? 2046 : 2046 - K);
    if (e - lo_e <= hi_e - lo_e) return gf_djoin(lo, hi + (unsigned)(K * (1 << 20)));
    if (((hi << 1) | lo) == 0u) return x;
    return gf_mul_rare(x, K == -2 ? 0.25 : K == -1 ? 0.5 : K == 1 ? 2.0 : 4.0);
}
template <int K> __device__ __forceinline__ float gf_scale(float x) {
    return x * (K == -2 ? 0.25f : K == -1 ? 0.5f : K == 1 ? 2.0f : 4.0f);
}

// Additions and products with an operand that is +0 in the step's usual
// configuration (no thermal stress, no dike, plane strain), on the integer
// pipes: x + (+0) is x except that -0 gives +0, x - (+0) is x, +0 - x is -x
// except that +0 gives +0, and +0 * y is +0 for y in [+0, +max].  Any other
// operand takes the FP64 instruction out of line.  (A NaN x keeps its bits.)
__device__ __noinline__ double gf_add_rare(double a, double b) { return a + b; }
__device__ __forceinline__ bool gf_is_pzero(double z) {
    unsigned lo, hi;
    gf_dsplit(z, lo, hi);
    return (lo | hi) == 0u;
}
__device__ __forceinline__ double gf_plus_pzero(double x) {
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    return gf_djoin(lo, (lo == 0u && hi == 0x80000000u) ? 0u : hi);
}
__device__ __forceinline__ double gf_add_z(double x, double z) { // x + z
    return gf_is_pzero(z) ? gf_plus_pzero(x) : gf_add_rare(x, z);
}
__device__ __forceinline__ double gf_sub_z(double x, double z) { // x - z
    return gf_is_pzero(z) ? x : gf_add_rare(x, -z);
}
__device__ __forceinline__ double gf_zero_minus(double x) { // +0 - x
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    return gf_djoin(lo, (lo | hi) == 0u ? 0u : hi ^ 0x80000000u);
}
__device__ __forceinline__ double gf_mul_z(double z, double y) { // z * y
    unsigned zl, zh, yl, yh;
    gf_dsplit(z, zl, zh);
    gf_dsplit(y, yl, yh);
    if ((zl | zh) == 0u && yh < 0x7ff00000u) return 0.0;
    return gf_mul_rare(z, y);
}
// |x| > c for a positive finite constant c, on the bit patterns (a NaN x
// gives false, as the FP64 comparison does)
__device__ __forceinline__ bool gf_abs_gt(double x, double c) {
    unsigned lo, hi, cl, ch;
    gf_dsplit(x, lo, hi);
    gf_dsplit(c, cl, ch);
    const unsigned long long ax = (unsigned long long)(hi & 0x7fffffffu) << 32 | lo;
    const unsigned long long ac = (unsigned long long)ch << 32 | cl;
    return ax > ac && ax <= 0x7ff0000000000000ull;
}
// a == b (IEEE: +0 equals -0, a NaN equals nothing) on the bit patterns
__device__ __forceinline__ bool gf_deq(double a, double b) {
    unsigned al, ah, bl, bh;
    gf_dsplit(a, al, ah);
    gf_dsplit(b, bl, bh);
    const bool nan = ((ah & 0x7fffffffu) > 0x7ff00000u) || ((ah & 0x7fffffffu) == 0x7ff00000u && al != 0u);
    return (al == bl && ah == bh && !nan) || (((ah | bh) << 1) == 0u && (al | bl) == 0u);
}
__device__ __forceinline__ float gf_add_z(float x, float z) { return x + z; }
__device__ __forceinline__ float gf_sub_z(float x, float z) { return x - z; }
__device__ __forceinline__ float gf_zero_minus(float x) { return 0.0f - x; }
__device__ __forceinline__ float gf_mul_z(float z, float y) { return z * y; }

// r < 0.01 (pre_plast's phase-ratio cut-off, rh_plastic.f90:250) on the bit
// pattern: true for negative numbers and -0, false for NaNs, otherwise the
// order of the magnitudes
__device__ __forceinline__ bool gf_ratio_below_cut(double r) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(r);
    const unsigned long long cut = (unsigned long long)__double_as_longlong(0.01);
    if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return false;
    return (b >> 63) ? true : b < cut;
}

// Division by a shared denominator with the bits of IEEE division.  For a
// denominator b: y = RN(1/b) (one IEEE division) and yl = RN(RN(1 - b y) y),
// so that y + yl is 1/b to 2^-105 relative (1 - b y is exact in an FMA).
// Each quotient a / b then costs one multiply and three FMAs:
//   q = RN(a y + RN(a yl))   within 0.5 ulp + 2^-104 |a/b|: faithful,
//   r = a - b q              exact in an FMA because q is faithful,
//   RN(q + r y)              = RN(a/b) by Markstein's theorem (a faithful
//                            quotient and the correctly rounded reciprocal;
//                            P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119).
// Operands outside gf_dmid take an IEEE division; a zero numerator gives
// a * y, the signed zero of IEEE division.  Restated in exact arithmetic and
// checked against IEEE division (random and near-midpoint quotients) by
// tests/test_division.py.
struct GfRecip {
    double b, y, yl;
    bool ok;
};
__device__ __forceinline__ GfRecip gf_recip_y(double b, double y) { // y = 1.0 / b
    GfRecip r;
    r.b = b;
    r.y = y;
    r.yl = fma(-y, b, 1.0) * y;
    r.ok = gf_dmid(b);
    return r;
}
// a pair computed ahead (y = RN(1/b) exactly; yl need only be near (1 - b y) y)
__device__ __forceinline__ GfRecip gf_recip_pre(double b, double y, double yl) {
    GfRecip r;
    r.b = b;
    r.y = y;
    r.yl = yl;
    r.ok = gf_dmid(b);
    return r;
}
// (out of line, so that the common path issues none of its FP64 instructions)
__device__ __noinline__ double gf_div_rare(double a, double b, double y, bool ok) {
    return (ok && gf_dzero(a)) ? a * y : a / b;
}
// IMUL: the product a * yl on the integer pipes (gf_mul), for kernels small
// enough that its thirty instructions cost less than the FP64 slot
template <bool IMUL = false> __device__ __forceinline__ double gf_div(double a, const GfRecip &r) {
    if (!(r.ok && gf_dmid(a))) return gf_div_rare(a, r.b, r.y, r.ok);
    const double q = fma(a, r.y, IMUL ? gf_mul(a, r.yl) : a * r.yl);
    return fma(fma(-q, r.b, a), r.y, q);
}

// x = hi + lo with hi = float(x): the hi/lo split of the mixed path
__device__ __forceinline__ void gf_split(double x, float &h, float &l) {
    h = gf_d2f(x);
    l = gf_d2f(x - gf_f2d(h));
}
// an FP64 input in the kernel's precision R (FP64 kernels keep it as it is)
template <class R> __device__ __forceinline__ R gf_to(double x) {
    if constexpr (sizeof(R) == sizeof(float)) return gf_d2f(x);
    else return x;
}

// Mixed path: coordinates of a quad relative to its node 1, in FP32 from the
// hi/lo splits (the hi difference of neighbouring nodes is exact, the lo
// parts carry the rest), and velocities relative to node 1 the same way.
struct QuadF {
    float x[4], y[4];
};

__device__ __forceinline__ float hl_diff(const float *__restrict__ h, const float *__restrict__ l, GF_IDX a,
                                         GF_IDX b) {
    return (h[a] - h[b]) + (l[a] - l[b]);
}

__device__ __forceinline__ void quad_nodes(const GfDims &d, int j, int i, GF_IDX n[4]) {
    n[0] = gf_node(d, j, i);
    n[1] = n[0] + 1;
    n[2] = gf_node(d, j, i + 1);
    n[3] = n[2] + 1;
}

__device__ __forceinline__ void load_quad_rel(const DevArrays &A, const GfDims &d, int j, int i, QuadF &q) {
    GF_IDX n[4];
    quad_nodes(d, j, i, n);
    const float *xh = A.cord_hi, *xl = A.cord_lo, *yh = A.cord_hi + d.N, *yl = A.cord_lo + d.N;
    q.x[0] = 0.0f;
    q.y[0] = 0.0f;
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        q.x[k] = hl_diff(xh, xl, n[k], n[0]);
        q.y[k] = hl_diff(yh, yl, n[k], n[0]);
    }
}

__device__ __forceinline__ void load_vel_rel(const DevArrays &A, const GfDims &d, int j, int i, float vx[4],
                                             float vy[4]) {
    GF_IDX n[4];
    quad_nodes(d, j, i, n);
    const float *xh = A.vel_hi, *xl = A.vel_lo, *yh = A.vel_hi + d.N, *yl = A.vel_lo + d.N;
    vx[0] = 0.0f;
    vy[0] = 0.0f;
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        vx[k] = hl_diff(xh, xl, n[k], n[0]);
        vy[k] = hl_diff(yh, yl, n[k], n[0]);
    }
}

// Shape-function derivatives of the four triangles (fl_rheol.f90:98-132):
// dx[m][k], dz[m][k] for local vertex m of triangle k.  Coordinate
// differences are taken in FP64, then rounded to R.
template <class R>
__device__ __forceinline__ void shape_derivs(const Quad &q, const R ar[4], R dx[3][4], R dz[3][4]) {
    const double *x = q.x, *y = q.y;
    dx[0][0] = R(y[1] - y[2]) * ar[0]; dx[1][0] = R(y[2] - y[0]) * ar[0]; dx[2][0] = R(y[0] - y[1]) * ar[0];
    dz[0][0] = R(x[2] - x[1]) * ar[0]; dz[1][0] = R(x[0] - x[2]) * ar[0]; dz[2][0] = R(x[1] - x[0]) * ar[0];
    dx[0][1] = R(y[1] - y[3]) * ar[1]; dx[1][1] = R(y[3] - y[2]) * ar[1]; dx[2][1] = R(y[2] - y[1]) * ar[1];
    dz[0][1] = R(x[3] - x[1]) * ar[1]; dz[1][1] = R(x[2] - x[3]) * ar[1]; dz[2][1] = R(x[1] - x[2]) * ar[1];
    dx[0][2] = R(y[1] - y[3]) * ar[2]; dx[1][2] = R(y[3] - y[0]) * ar[2]; dx[2][2] = R(y[0] - y[1]) * ar[2];
    dz[0][2] = R(x[3] - x[1]) * ar[2]; dz[1][2] = R(x[0] - x[3]) * ar[2]; dz[2][2] = R(x[1] - x[0]) * ar[2];
    dx[0][3] = R(y[3] - y[2]) * ar[3]; dx[1][3] = R(y[2] - y[0]) * ar[3]; dx[2][3] = R(y[0] - y[3]) * ar[3];
    dz[0][3] = R(x[2] - x[3]) * ar[3]; dz[1][3] = R(x[0] - x[2]) * ar[3]; dz[2][3] = R(x[3] - x[0]) * ar[3];
}

// the same from relative FP32 coordinates (only differences enter)
__device__ __forceinline__ void shape_derivs_f(const QuadF &q, const float ar[4], float dx[3][4], float dz[3][4]) {
    const float *x = q.x, *y = q.y;
    dx[0][0] = (y[1] - y[2]) * ar[0]; dx[1][0] = (y[2] - y[0]) * ar[0]; dx[2][0] = (y[0] - y[1]) * ar[0];
    dz[0][0] = (x[2] - x[1]) * ar[0]; dz[1][0] = (x[0] - x[2]) * ar[0]; dz[2][0] = (x[1] - x[0]) * ar[0];
    dx[0][1] = (y[1] - y[3]) * ar[1]; dx[1][1] = (y[3] - y[2]) * ar[1]; dx[2][1] = (y[2] - y[1]) * ar[1];
    dz[0][1] = (x[3] - x[1]) * ar[1]; dz[1][1] = (x[2] - x[3]) * ar[1]; dz[2][1] = (x[1] - x[2]) * ar[1];
    dx[0][2] = (y[1] - y[3]) * ar[2]; dx[1][2] = (y[3] - y[0]) * ar[2]; dx[2][2] = (y[0] - y[1]) * ar[2];
    dz[0][2] = (x[3] - x[1]) * ar[2]; dz[1][2] = (x[0] - x[3]) * ar[2]; dz[2][2] = (x[1] - x[0]) * ar[2];
    dx[0][3] = (y[3] - y[2]) * ar[3]; dx[1][3] = (y[2] - y[0]) * ar[3]; dx[2][3] = (y[0] - y[3]) * ar[3];
    dz[0][3] = (x[2] - x[3]) * ar[3]; dz[1][3] = (x[0] - x[2]) * ar[3]; dz[2][3] = (x[3] - x[0]) * ar[3];
}

// ---------------------------------------------------------------- matprops

// Eff_visc (matprops.f90:136-215), always in FP64.
template <class R>
__device__ double eff_visc(const DevParams &P, const DevArrays &A, const GfDims &d, int j, int i, GF_IDX e,
                           const R *__restrict__ st) {
    for (int k = 0; k < P.ninh100; ++k)
        if (i + 1 >= P.w_ix1[k] && i + 1 <= P.w_ix2[k] && j + 1 >= P.w_iy1[k] && j + 1 <= P.w_iy2[k]) return P.v_min;
    const double adi_grad = 3e-1, r = 8.31448;
    const double *cord = A.cord, *temp = A.temp;
    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    double zcord = 0.25 * (cord[d.N + n1] + cord[d.N + n1 + 1] + cord[d.N + n3] + cord[d.N + n3 + 1]);
    double tmpr0 = 0.25 * (temp[n1] + temp[n1 + 1] + temp[n3] + temp[n3 + 1]);
    double zsurf = 0.50 * (cord[d.N + gf_node(d, 0, i)] + cord[d.N + gf_node(d, 0, i + 1)]);
    double tmpr = (zsurf - zcord) * 1e-3 * adi_grad + tmpr0;
    double s11 = 0.25 * ((double)st[gf_s(d, e, 0, 0)] + (double)st[gf_s(d, e, 0, 1)] + (double)st[gf_s(d, e, 0, 2)] +
                         (double)st[gf_s(d, e, 0, 3)]);
    double s22 = 0.25 * ((double)st[gf_s(d, e, 1, 0)] + (double)st[gf_s(d, e, 1, 1)] + (double)st[gf_s(d, e, 1, 2)] +
                         (double)st[gf_s(d, e, 1, 3)]);
    double s33 = 0.25 * ((double)st[gf_s(d, e, 3, 0)] + (double)st[gf_s(d, e, 3, 1)] + (double)st[gf_s(d, e, 3, 2)] +
                         (double)st[gf_s(d, e, 3, 3)]);
    double pres = -1 * (s11 + s22 + s33) / 3.0;
    double deptmpr410 = -101.58 * (tmpr + 273.0) - 216828.0;
    double deptmpr660 = 66.55 * (tmpr + 273.0) - 788494.0;
    double ev;
    if (zcord < deptmpr660) {
        ev = 1e22 * gfm::exp(-0.0115 * (tmpr - P.t_bot));
        return fmin(P.v_max, fmax(P.v_min, ev));
    } else if (zcord < deptmpr410) {
        ev = 1e21 * gfm::exp(-0.0115 * (tmpr - P.t_bot));
        return fmin(P.v_max, fmax(P.v_min, ev));
    }
    double srat = (double)((const R *)A.e2sr)[e];
    if (srat == 0) srat = P.vbc / P.rxbo;
    ev = 0.0;
    for (int k = 0; k < P.nphase; ++k) {
        double ratio = A.phase_ratio[gf_pr(d, e, k)];
        if (ratio < 0.01) continue;
        double pw = 1.0 / P.pln[k] - 1.0;
        double pw1 = -1.0 / P.pln[k];
        double vis = 0.25 * gfm::pow(srat, pw) * gfm::pow(0.75 * P.acoef[k], pw1) *
                     gfm::exp((P.eactiv[k] + P.vactiv[k] * pres) / (P.pln[k] * r * (tmpr + 273.0))) * 1e6;
        if (vis < P.v_min) vis = P.v_min;
        if (vis > P.v_max) vis = P.v_max;
        ev = ev + ratio / vis;
    }
    ev = 1 / ev;
    if (P.itype_melting == 1) {
        double fma = fmin(A.fmagma[e] + A.fmagma2[e], P.fmagma_max);
        ev = ev * gfm::exp(P.weaken_ratio_viscous * fma / P.fmagma_max);
    }
    return fmin(P.v_max, fmax(P.v_min, ev));
}

// Eff_visc in FP32 for the mixed-precision path: the power-law viscosity is
// evaluated as a sum of logarithms and clamped in log space, so no
// intermediate leaves the FP32 range (A^(-1/n) e^(E/nRT) alone can exceed it).
__device__ float eff_visc_f32(const DevParams &P, const DevArrays &A, const GfDims &d, int j, int i, GF_IDX e,
                              const float *__restrict__ st) {
    for (int k = 0; k < P.ninh100; ++k)
        if (i + 1 >= P.w_ix1[k] && i + 1 <= P.w_ix2[k] && j + 1 >= P.w_iy1[k] && j + 1 <= P.w_iy2[k])
            return (float)P.v_min;
    const float *zh = A.cord_hi + d.N;
    const double *temp = A.temp;
    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    float zcord = 0.25f * (zh[n1] + zh[n1 + 1] + zh[n3] + zh[n3 + 1]);
    float zsurf = 0.50f * (zh[gf_node(d, 0, i)] + zh[gf_node(d, 0, i + 1)]);
    float tmpr0 = 0.25f * ((float)temp[n1] + (float)temp[n1 + 1] + (float)temp[n3] + (float)temp[n3 + 1]);
    float tmpr = (zsurf - zcord) * 1e-3f * 0.3f + tmpr0;
    float s11 = 0.25f * (st[gf_s(d, e, 0, 0)] + st[gf_s(d, e, 0, 1)] + st[gf_s(d, e, 0, 2)] + st[gf_s(d, e, 0, 3)]);
    float s22 = 0.25f * (st[gf_s(d, e, 1, 0)] + st[gf_s(d, e, 1, 1)] + st[gf_s(d, e, 1, 2)] + st[gf_s(d, e, 1, 3)]);
    float s33 = 0.25f * (st[gf_s(d, e, 3, 0)] + st[gf_s(d, e, 3, 1)] + st[gf_s(d, e, 3, 2)] + st[gf_s(d, e, 3, 3)]);
    float pres = -(s11 + s22 + s33) / 3.0f + (float)A.p_ref[e]; // stored stresses are deviations from -p_ref
    float zc = zcord;
    float deptmpr410 = -101.58f * (tmpr + 273.0f) - 216828.0f;
    float deptmpr660 = 66.55f * (tmpr + 273.0f) - 788494.0f;
    float vmin = (float)P.v_min, vmax = (float)P.v_max;
    if (zc < deptmpr660 || zc < deptmpr410) {
        float ev = (zc < deptmpr660 ? 1e22f : 1e21f) * expf(-0.0115f * (tmpr - (float)P.t_bot));
        return fminf(vmax, fmaxf(vmin, ev));
    }
    float srat = ((const float *)A.e2sr)[e];
    if (srat == 0.0f) srat = float(P.vbc / P.rxbo);
    const float lmin = logf(vmin), lmax = logf(vmax);
    const float lsr = logf(srat), lbase = logf(0.25f * 1e6f);
    float ev = 0.0f;
    for (int k = 0; k < P.nphase; ++k) {
        float ratio = (float)A.phase_ratio[gf_pr(d, e, k)];
        if (ratio < 0.01f) continue;
        float n = P.f_pln[k];
        float lv = lbase + (1.0f / n - 1.0f) * lsr - (1.0f / n) * P.f_lacoef[k] +
                   (P.f_eactiv[k] + P.f_vactiv[k] * pres) / (n * 8.31448f * (tmpr + 273.0f));
        lv = fminf(lmax, fmaxf(lmin, lv));
        ev += ratio / expf(lv);
    }
    ev = 1.0f / ev;
    if (P.itype_melting == 1) {
        float fma = fminf(float(A.fmagma[e] + A.fmagma2[e]), (float)P.fmagma_max);
        ev *= expf((float)P.weaken_ratio_viscous * fma / (float)P.fmagma_max);
    }
    return fminf(vmax, fmaxf(vmin, ev));
}

template <class R>
__device__ __forceinline__ double visc_of(const DevParams &P, const DevArrays &A, const GfDims &d, int j, int i,
                                          GF_IDX e, const R *__restrict__ st) {
    if (sizeof(R) == sizeof(float)) return (double)eff_visc_f32(P, A, d, j, i, e, (const float *)st);
    return eff_visc<R>(P, A, d, j, i, e, st);
}

// Eff_dens (matprops.f90:3-83), FP64.  *wrote_frac/*frac_val report the
// write of the global frac the reference performs (matprops.f90:37,48).
template <class R>
__device__ double eff_dens(const DevParams &P, const DevArrays &A, const GfDims &d, int j, int i, GF_IDX e,
                           int *wrote_frac, double *frac_val) {
    const double adi_grad = 3e-1, den_ramp_dist = 30e3, amp410 = 0.05, amp660 = 0.085;
    const double *cord = A.cord, *temp = A.temp;
    const R *st = (const R *)A.stress0;
    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    double zcord = 0.25 * (cord[d.N + n1] + cord[d.N + n1 + 1] + cord[d.N + n3] + cord[d.N + n3 + 1]);
    double tmpr0 = 0.25 * (temp[n1] + temp[n1 + 1] + temp[n3] + temp[n3 + 1]);
    double zsurf = 0.50 * (cord[d.N + gf_node(d, 0, i)] + cord[d.N + gf_node(d, 0, i + 1)]);
    double tmpr = (zsurf - zcord) * 1e-3 * adi_grad + tmpr0;
    int iph = A.iphase[e];
    double deptmpr410 = -101.58 * (tmpr + 273.0) - 216828.0;
    double deptmpr420 = deptmpr410 - den_ramp_dist;
    double den_amp = 1.0;
    *wrote_frac = 0;
    if (deptmpr410 > zcord) {
        double f = (deptmpr410 - zcord) / (deptmpr410 - deptmpr420);
        if (f < 0.0) f = 0.0;
        if (f > 1.0) f = 1.0;
        *wrote_frac = 1;
        *frac_val = f;
        den_amp = 1.0 + amp410 * f;
    }
    double deptmpr660 = 66.55 * (tmpr + 273.0) - 788494.0;
    double deptmpr670 = deptmpr660 - den_ramp_dist;
    if (deptmpr660 > zcord) {
        double f = (deptmpr660 - zcord) / (deptmpr660 - deptmpr670);
        if (f < 0.0) f = 0.0;
        if (f > 1.0) f = 1.0;
        *wrote_frac = 1;
        *frac_val = f;
        den_amp = 1.05 + amp660 * f;
    }
    double press = 0;
    for (int k = 0; k < 4; ++k)
        press = press - ((double)st[gf_s(d, e, 0, k)] + (double)st[gf_s(d, e, 1, k)] + (double)st[gf_s(d, e, 3, k)]);
    press = press / 12;
    if (sizeof(R) == sizeof(float)) press = press + A.p_ref[e]; // mixed: stored stresses exclude -p_ref
    double ed = 0.0;
    for (int k = 0; k < P.nphase; ++k) {
        double ratio = A.phase_ratio[gf_pr(d, e, k)];
        if (ratio < 0.01) continue;
        double dens = P.den[k] * (1 - P.alfa[k] * tmpr + P.beta[k] * press);
        press = dens * P.g * zcord;
        dens = P.den[k] * (1 - P.alfa[k] * tmpr + P.beta[k] * press);
        ed = ed + ratio * dens;
    }
    if (iph == 4 || iph == 8 || iph == 9 || iph == 16 || iph == 18) ed = ed * den_amp;
    double fma = fmin(A.fmagma[e] + A.fmagma2[e], P.fmagma_max);
    ed = ed - fma * (ed - P.rho_magma);
    return ed;
}

// Eff_dens in FP32 for the mixed path (same formula as eff_dens; depths from
// the hi parts of the coordinates, the pressure from the stored deviations
// plus p_ref, temperatures from the hi/lo split).
__device__ float eff_dens_f32(const DevParams &P, const DevArrays &A, const GfDims &d, int j, int i, GF_IDX e,
                              int *wrote_frac, float *frac_val) {
    const float den_ramp_dist = 30e3f, amp410 = 0.05f, amp660 = 0.085f;
    const float *zh = A.cord_hi + d.N, *th = A.temp_hi;
    const float *st = (const float *)A.stress0;
    GF_IDX n1 = gf_node(d, j, i), n3 = gf_node(d, j, i + 1);
    float zcord = 0.25f * (zh[n1] + zh[n1 + 1] + zh[n3] + zh[n3 + 1]);
    float tmpr0 = 0.25f * (th[n1] + th[n1 + 1] + th[n3] + th[n3 + 1]);
    float zsurf = 0.50f * (zh[gf_node(d, 0, i)] + zh[gf_node(d, 0, i + 1)]);
    float tmpr = (zsurf - zcord) * 1e-3f * 0.3f + tmpr0;
    int iph = A.iphase[e];
    float deptmpr410 = -101.58f * (tmpr + 273.0f) - 216828.0f;
    float den_amp = 1.0f;
    *wrote_frac = 0;
    if (deptmpr410 > zcord) {
        float f = fminf(1.0f, fmaxf(0.0f, (deptmpr410 - zcord) / den_ramp_dist));
        *wrote_frac = 1;
        *frac_val = f;
        den_amp = 1.0f + amp410 * f;
    }
    float deptmpr660 = 66.55f * (tmpr + 273.0f) - 788494.0f;
    if (deptmpr660 > zcord) {
        float f = fminf(1.0f, fmaxf(0.0f, (deptmpr660 - zcord) / den_ramp_dist));
        *wrote_frac = 1;
        *frac_val = f;
        den_amp = 1.05f + amp660 * f;
    }
    float press = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) press = press - (st[gf_s(d, e, 0, k)] + st[gf_s(d, e, 1, k)] + st[gf_s(d, e, 3, k)]);
    press = press / 12.0f + A.pr_hi[e];
    float ed = 0.0f;
    for (int k = 0; k < P.nphase; ++k) {
        float ratio = (float)A.phase_ratio[gf_pr(d, e, k)];
        if (ratio < 0.01f) continue;
        float dens = P.f_den[k] * (1.0f - P.f_alfa[k] * tmpr + P.f_beta[k] * press);
        press = dens * P.f_g * zcord;
        dens = P.f_den[k] * (1.0f - P.f_alfa[k] * tmpr + P.f_beta[k] * press);
        ed = ed + ratio * dens;
    }
    if (iph == 4 || iph == 8 || iph == 9 || iph == 16 || iph == 18) ed = ed * den_amp;
    if (A.fmagma) {
        float fma = fminf((float)(A.fmagma[e] + A.fmagma2[e]), P.f_fmagma_max);
        ed = ed - fma * (ed - P.f_rho_magma);
    }
    return ed;
}

// ---------------------------------------------------------------- rheology

template <class R>
__device__ __forceinline__ void elastic(R bulkm, R rmu, R &s11, R &s22, R &s33, R &s12, R de11, R de22, R de12) {
    const R c4d3 = R(4.0 / 3.0), c2d3 = R(2.0 / 3.0);
    R a1 = bulkm + c4d3 * rmu;
    R a2 = bulkm - c2d3 * rmu;
    s11 = s11 + a1 * de11 + a2 * de22;
    s22 = s22 + a2 * de11 + a1 * de22;
    s12 = s12 + gf_scale<1>(rmu) * de12;
    s33 = s33 + a2 * (de11 + de22);
}

// The per-element factors of maxwell (rh_maxwell.f90:17-33): the reference
// evaluates them per triangle from the same element values.  ok is false
// where the reference stops with code 22.
template <class R> struct MaxwellConsts {
    R rmu, vic1, vic2;
    bool ok;
    bool pos; // vic1, 2 rmu and vic2 in [+0, +max] (FP64): +0 * each is +0
};
__device__ __forceinline__ bool gf_nonneg_finite(double x) {
    unsigned lo, hi;
    gf_dsplit(x, lo, hi);
    return hi < 0x7ff00000u;
}
// s33 of a triangle whose s33d, de33d are not known to be +0 (out of line)
__device__ __noinline__ double gf_maxwell_s33(double s33d, double vic1, double rmu2, double de33d, double vic2,
                                              double s0) {
    return (s33d * vic1 + rmu2 * de33d) * vic2 + s0;
}
template <class R> __device__ __forceinline__ MaxwellConsts<R> maxwell_consts(R rmu0, R viscosity, R dt) {
    const R visc_cut = R(1e19);
    MaxwellConsts<R> m;
    m.rmu = viscosity < visc_cut ? gf_ddiv(rmu0 * viscosity, visc_cut) : rmu0;
    R temp = gf_ddiv(m.rmu, gf_scale<1>(viscosity)) * dt;
    m.ok = !(temp > R(0.5));
    m.vic1 = R(1) - temp;
    if constexpr (sizeof(R) == sizeof(double)) m.vic2 = gf_rcp(R(1.0) + temp); // RN(1/(1 + temp))
    else m.vic2 = R(1.0) / (R(1.0) + temp);
    m.pos = false;
    if constexpr (sizeof(R) == sizeof(double))
        m.pos = gf_nonneg_finite(m.vic1) && gf_nonneg_finite(gf_scale<1>(m.rmu)) && gf_nonneg_finite(m.vic2);
    return m;
}

// maxwell (rh_maxwell.f90:2-76) of one triangle
template <class R>
__device__ __forceinline__ void maxwell(R bulkm, const MaxwellConsts<R> &m, R &s11, R &s22, R &s33, R &s12, R de11,
                                        R de22, R de33, R de12, R dv, int ndim) {
    const R c1d3 = R(1.0 / 3.0);
    const R rmu = m.rmu, vic1 = m.vic1, vic2 = m.vic2;
    R dev, de11d, de22d, de33d, s0, s11d, s22d, s33d;
    if (ndim == 2) {
        dev = de11 + de22;
        de11d = de11 - gf_scale<-1>(dev);
        de22d = de22 - gf_scale<-1>(dev);
        de33d = 0;
        s0 = gf_scale<-1>(s11 + s22);
        s11d = s11 - s0;
        s22d = s22 - s0;
        s33d = 0;
    } else {
        dev = de11 + de22 + de33;
        de11d = de11 - c1d3 * dev;
        de22d = de22 - c1d3 * dev;
        de33d = de33 - c1d3 * dev;
        s0 = c1d3 * (s11 + s22 + s33);
        s11d = s11 - s0;
        s22d = s22 - s0;
        s33d = s33 - s0;
    }
    const R rmu2 = gf_scale<1>(rmu);
    s11d = (s11d * vic1 + rmu2 * de11d) * vic2;
    s22d = (s22d * vic1 + rmu2 * de22d) * vic2;
    s12 = (s12 * vic1 + rmu2 * de12) * vic2;
    s0 = s0 + bulkm * dv;
    s11 = s11d + s0;
    s22 = s22d + s0;
    if constexpr (sizeof(R) == sizeof(double)) {
        // plane strain: s33d and de33d are +0, so (s33d vic1 + 2 rmu de33d)
        // vic2 is +0 for factors in [+0, +max], and s33 = +0 + s0
        s33 = (ndim == 2 && m.pos) ? gf_plus_pzero(s0) : gf_maxwell_s33(s33d, vic1, rmu2, de33d, vic2, s0);
    } else {
        s33d = (s33d * vic1 + rmu2 * de33d) * vic2;
        s33 = s33d + s0;
    }
}

// Per-element constants of the plastic return map (rh_plastic.f90:33-46).
// The reference evaluates them once per triangle with identical inputs; they
// are evaluated once per element here (same values, a quarter of the
// transcendental work).
template <class R> struct PlasticConsts {
    R anphi, anpsi, amc, e1, e2, x1, ten_max;
    float anphi_f, amc_f, ten_f; // FP64 path: FP32 copies for plastic_keeps_trial
};
// the FP32 copies of an FP64 element's constants (integer-pipe conversion)
__device__ __forceinline__ void plastic_consts_f32(PlasticConsts<double> &c) {
    c.anphi_f = gf_d2f(c.anphi);
    c.amc_f = gf_d2f(c.amc);
    c.ten_f = gf_d2f(c.ten_max);
}
__device__ __forceinline__ void plastic_consts_f32(PlasticConsts<float> &) {}

template <class R>
__device__ __forceinline__ PlasticConsts<R> plastic_consts(R bulkm, R rmu, R coh, R phi, R psi, R ten_off) {
    const R c4d3 = R(4.0 / 3.0), c2d3 = R(2.0 / 3.0);
    PlasticConsts<R> c;
    R sphi = m_sind(phi);
    R spsi = m_sind(psi);
    c.anphi = (R(1.0) + sphi) / (R(1.0) - sphi);
    c.anpsi = (R(1.0) + spsi) / (R(1.0) - spsi);
    c.amc = R(2.0) * coh * m_sqrt(c.anphi);
    c.e1 = bulkm + c4d3 * rmu;
    c.e2 = bulkm - c2d3 * rmu;
    c.x1 = (c.e1 - c.e2 * c.anpsi + c.e1 * c.anphi * c.anpsi - c.e2 * c.anphi);
    c.ten_max = (phi == R(0.0)) ? ten_off : fmin(ten_off, coh / m_tand(phi));
    plastic_consts_f32(c);
    return c;
}

// Whether plastic (FP64) keeps the elastic trial stress: no tension
// cut-off (s1 < ten_max, rh_plastic.f90:111) and no shear yield (fs >= 0,
// rh_plastic.f90:134-135).  Decided from an FP32 evaluation of s1 and fs with a
// bound on its distance to the FP64 evaluation; true only where the FP32
// margin exceeds that bound, false (take the FP64 path) otherwise.
//
// With A = max(|s11i|, |s22i|, |s12i|) and u = 2^-24 (the float inputs are
// within u A of the doubles; the FP32 steps round once each, the square root
// included, as this translation unit builds without contraction and with
// IEEE square roots), the FP32 values are within
//   s1:  12 u A                                       of the exact s1,
//   fs:  u (18 A + anphi (24 A + 5 |ten_max|) + 3 amc)  of the exact fs
// (|S0| <= A, rad <= 2 A, the square root of a sum of squares is
// 1-Lipschitz in its vector), and the FP64 values are within the same
// expressions in 2^-53.  The margins below exceed twice those sums and
// cover the FP32 copies of ten_max, anphi and amc and the rounding of the
// comparisons; the absolute 1e-30 covers inputs below the float range
// (flushed to zero), and any NaN or overflow fails the comparisons.
// tests/test_plastic_filter.py checks the bound on adversarial states.
__device__ __forceinline__ bool plastic_keeps_trial(const PlasticConsts<double> &c, double s11i, double s22i,
                                                    double s12i) {
    const float a = gf_d2f(s11i), b = gf_d2f(s22i), q = gf_d2f(s12i);
    const float A = fmaxf(fmaxf(fabsf(a), fabsf(b)), fabsf(q));
    const float d = a - b, s0 = 0.5f * (a + b);
    const float r = 0.5f * sqrtf(d * d + (4.0f * q) * q);
    const float s1 = s0 - r, sii = s0 + r;
    const float ten = c.ten_f, anphi = c.anphi_f, amc = c.amc_f, at = fabsf(ten);
    const float s3 = fminf(sii, ten);
    const float fs = (s1 - s3 * anphi) + amc;
    const float e_s1 = 3.4e-6f * A + 2.4e-7f * at + 1e-30f;
    const float e_fs = 1.2e-7f * (40.0f * A + anphi * (52.0f * A + 10.0f * at) + 4.0f * amc) + 1e-30f;
    return (s1 + e_s1 < ten) && (fs > e_fs);
}

// plastic (rh_plastic.f90:3-229), 2-D branch (icase = 1).
template <class R>
__device__ __forceinline__ void plastic(const PlasticConsts<R> &c, R rmu, R &depls, R hardn, R &s11, R &s22, R &s33,
                                        R &s12, R de11, R de22, R de33, R de12) {
    depls = R(0.0);
    R e1 = c.e1, e2 = c.e2, anphi = c.anphi, anpsi = c.anpsi, ten_max = c.ten_max;
    // (de33 is +0 in plane strain: gf_add_z / gf_mul_z take it on the
    // integer pipes)
    R s11i = s11 + gf_add_z(de22, de33) * e2 + de11 * e1;
    R s22i = s22 + gf_add_z(de11, de33) * e2 + de22 * e1;
    R s12i = s12 + gf_scale<1>(de12) * rmu;
    R s33i = gf_add_z(s33 + (de11 + de22) * e2, gf_mul_z(de33, e1));
    if constexpr (sizeof(R) == sizeof(double)) {
        if (plastic_keeps_trial(c, s11i, s22i, s12i)) {
            s11 = s11i; s22 = s22i; s33 = s33i; s12 = s12i;
            return;
        }
    }
    R sdif = s11i - s22i;
    R s0 = R(0.5) * (s11i + s22i);
    R rad = R(0.5) * m_sqrt(sdif * sdif + R(4.0) * s12i * s12i);
    R si = s0 - rad, sii = s0 + rad, psdif = si - sii;
    R s1 = si, s2 = s33i, s3 = sii;
    if (s1 >= ten_max) {
        s11 = ten_max; s22 = ten_max; s12 = R(0.0); s33 = ten_max;
        return;
    }
    if (s3 >= ten_max) s3 = ten_max;
    R fs = s1 - s3 * anphi + c.amc;
    if (fs < R(0.0)) {
        R alams = fs / (c.x1 + hardn);
        s1 = s1 - alams * (e1 - e2 * anpsi);
        s2 = s2 - alams * e2 * (R(1.0) - anpsi);
        s3 = s3 - alams * (e2 - e1 * anpsi);
        R dep1 = alams;
        R dep3 = -alams * anpsi;
        depls = R(0.5) * m_abs(dep1 - dep3);
    } else {
        s11 = s11i; s22 = s22i; s33 = s33i; s12 = s12i;
        return;
    }
    if (s1 >= ten_max) {
        s11 = ten_max; s22 = ten_max; s12 = R(0.0); s33 = ten_max;
        return;
    }
    if (s3 >= ten_max) s3 = ten_max;
    R cs2, si2;
    if (psdif == R(0.0)) {
        cs2 = R(1.0);
        si2 = R(0.0);
    } else {
        cs2 = sdif / psdif;
        si2 = R(2.0) * s12i / psdif;
    }
    R dc2 = (s1 - s3) * cs2;
    R dss = s1 + s3;
    s11 = R(0.5) * (dss + dc2);
    s22 = R(0.5) * (dss - dc2);
    s12 = R(0.5) * (s1 - s3) * si2;
    s33 = s2;
}

// plastic in the mixed path, where normal stresses are stored as deviations
// from the element's reference pressure p (total = stored - p): the same
// return map, with the tension cut-off and the yield function shifted by p so
// that no total stress (up to 1e10 Pa at depth) is formed in FP32.
__device__ __forceinline__ void plastic_dev(const PlasticConsts<float> &c, float rmu, float &depls, float hardn,
                                            float &s11, float &s22, float &s33, float &s12, float de11, float de22,
                                            float de33, float de12, float p, bool &mod) {
    depls = 0.0f;
    mod = true; // cleared below when the elastic trial stress is kept
    float e1 = c.e1, e2 = c.e2, anphi = c.anphi, anpsi = c.anpsi;
    float tm = c.ten_max + p; // tension cut-off in stored (deviation) units
    float s11i = s11 + (de22 + de33) * e2 + de11 * e1;
    float s22i = s22 + (de11 + de33) * e2 + de22 * e1;
    float s12i = s12 + de12 * 2.0f * rmu;
    float s33i = s33 + (de11 + de22) * e2 + de33 * e1;
    float sdif = s11i - s22i;
    float s0 = 0.5f * (s11i + s22i);
    float rad = 0.5f * sqrtf(sdif * sdif + 4.0f * s12i * s12i);
    float si = s0 - rad, sii = s0 + rad, psdif = si - sii;
    float s1 = si, s2 = s33i, s3 = sii;
    if (s1 >= tm) {
        s11 = tm; s22 = tm; s12 = 0.0f; s33 = tm;
        return;
    }
    if (s3 >= tm) s3 = tm;
    float fs = (s1 - s3 * anphi + c.amc) - p * (1.0f - anphi);
    if (fs < 0.0f) {
        float alams = fs / (c.x1 + hardn);
        s1 = s1 - alams * (e1 - e2 * anpsi);
        s2 = s2 - alams * e2 * (1.0f - anpsi);
        s3 = s3 - alams * (e2 - e1 * anpsi);
        depls = 0.5f * fabsf(alams + alams * anpsi);
    } else {
        s11 = s11i; s22 = s22i; s33 = s33i; s12 = s12i;
        mod = false; // the elastic trial stress is kept
        return;
    }
    if (s1 >= tm) {
        s11 = tm; s22 = tm; s12 = 0.0f; s33 = tm;
        return;
    }
    if (s3 >= tm) s3 = tm;
    float cs2 = 1.0f, si2 = 0.0f;
    if (psdif != 0.0f) {
        cs2 = sdif / psdif;
        si2 = 2.0f * s12i / psdif;
    }
    float dc2 = (s1 - s3) * cs2;
    float dss = s1 + s3;
    s11 = 0.5f * (dss + dc2);
    s22 = 0.5f * (dss - dc2);
    s12 = 0.5f * (s1 - s3) * si2;
    s33 = s2;
}

__device__ __forceinline__ void plastic_sel(const PlasticConsts<double> &c, double rmu, double &depls, double hardn,
                                            double &s11, double &s22, double &s33, double &s12, double de11,
                                            double de22, double de33, double de12, double, bool &mod) {
    plastic<double>(c, rmu, depls, hardn, s11, s22, s33, s12, de11, de22, de33, de12);
    mod = true;
}
__device__ __forceinline__ void plastic_sel(const PlasticConsts<float> &c, float rmu, float &depls, float hardn,
                                            float &s11, float &s22, float &s33, float &s12, float de11, float de22,
                                            float de33, float de12, float pref, bool &mod) {
    plastic_dev(c, rmu, depls, hardn, s11, s22, s33, s12, de11, de22, de33, de12, pref, mod);
}

// fl_rheol.f90:266-288 keeps the Maxwell stress unless the plastic one has
// the smaller second invariant.  When no triangle left its elastic trial
// stress, the two differ by the Maxwell relaxation alone, O(dt/tau) ~ 1e-8
// of the invariant for stiff lithosphere: below FP32 resolution, so the
// FP32 path decides with the difference written out analytically,
//   sv_a = (sp_a - t*S - 2*(mu - mu')*D) / (1 + t)   (and alike for s12),
//   use Maxwell  <=>  2*W + V - Q*t*(2 + t) <= 0,
// with S, B the start-of-step sums of s11-s22 and s12, D, D12 those of the
// strain increments, Q = sp_a^2 + 4 sp_b^2, W = sp_a*da + 4*sp_b*db,
// V = da^2 + 4*db^2 (da, db the bracketed corrections).
__device__ __forceinline__ bool maxwell_wins_unyielded(float sp_a, float sp_b, float S, float B, float D, float D12,
                                                       float rmu, float vis, float dt) {
    const float visc_cut = 1e19f;
    float rmu_m = vis < visc_cut ? rmu * vis / visc_cut : rmu;
    float t = rmu_m / (2.0f * vis) * dt;
    float da = -t * S - 2.0f * (rmu - rmu_m) * D;
    float db = -t * B - 2.0f * (rmu - rmu_m) * D12;
    float Q = sp_a * sp_a + 4.0f * sp_b * sp_b;
    float W = sp_a * da + 4.0f * sp_b * db;
    float V = da * da + 4.0f * db * db;
    return 2.0f * W + V - Q * t * (2.0f + t) <= 0.0f;
}

// One phase's terms of pre_plast in FP64 (rh_plastic.f90:249-280): the
// element path and the per-phase table of single-phase elements
// (k_plastic_table) both evaluate these operations.
__device__ __forceinline__ void pre_plast_phase(const DevParams &P, int k, double ratio, double pls_curr, double &phi,
                                                double &coh, double &psi, double &hardn) {
    const double pl1 = P.plstrain1[k], pl2 = P.plstrain2[k];
    const double f1 = P.fric1[k], f2 = P.fric2[k], c1 = P.cohesion1[k], c2 = P.cohesion2[k];
    const double d1 = P.dilat1[k], d2 = P.dilat2[k];
    double f, c, dd, h;
    if (pls_curr < pl1) {
        f = f1; c = c1; dd = d1; h = 0;
    } else if (pls_curr < pl2) {
        double dpl = (pls_curr - pl1) / (pl2 - pl1);
        f = f1 + (f2 - f1) * dpl;
        dd = d1 + (d2 - d1) * dpl;
        c = c1 + (c2 - c1) * dpl;
        h = P.hsoft[k];
    } else {
        f = f2; c = c2; dd = d2; h = 0;
    }
    phi = phi + ratio / f;
    coh = coh + ratio / c;
    psi = psi + ratio * dd;
    hardn = hardn + ratio * h;
}

// The same in FP32 with the mixed path's FP32 constants.
__device__ __forceinline__ void pre_plast_phase(const DevParams &P, int k, float ratio, float pls_curr, float &phi,
                                                float &coh, float &psi, float &hardn) {
    const float pl1 = P.f_pl1[k], pl2 = P.f_pl2[k];
    const float f1 = P.f_fric1[k], f2 = P.f_fric2[k], c1 = P.f_coh1[k], c2 = P.f_coh2[k];
    const float d1 = P.f_dil1[k], d2 = P.f_dil2[k];
    float f, c, dd, h;
    if (pls_curr < pl1) {
        f = f1; c = c1; dd = d1; h = 0;
    } else if (pls_curr < pl2) {
        float dpl = (pls_curr - pl1) / (pl2 - pl1);
        f = f1 + (f2 - f1) * dpl;
        dd = d1 + (d2 - d1) * dpl;
        c = c1 + (c2 - c1) * dpl;
        h = (c2 - c1) / (pl2 - pl1);
    } else {
        f = f2; c = c2; dd = d2; h = 0;
    }
    phi = phi + ratio / f;
    coh = coh + ratio / c;
    psi = psi + ratio * dd;
    hardn = hardn + ratio * h;
}

// pre_plast (rh_plastic.f90:231-291)
template <class R>
__device__ __forceinline__ void pre_plast(const DevParams &P, const DevArrays &A, const GfDims &d, GF_IDX e,
                                          R aps_e, R &coh, R &phi, R &psi, R &hardn) {
    R pls_curr = aps_e;
    phi = 0; coh = 0; psi = 0; hardn = 0;
    for (int k = 0; k < P.nphase; ++k) {
        if constexpr (sizeof(R) == sizeof(float)) {
            const double r = A.phase_ratio[gf_pr(d, e, k)];
            if (gf_ratio_below_cut(r)) continue;
            pre_plast_phase(P, k, gf_d2f(r), pls_curr, phi, coh, psi, hardn);
        } else {
            const double ratio = A.phase_ratio[gf_pr(d, e, k)];
            if (gf_ratio_below_cut(ratio)) continue;
            pre_plast_phase(P, k, ratio, pls_curr, phi, coh, psi, hardn);
        }
    }
    phi = R(1) / phi;
    coh = R(1) / coh;
    if (P.itype_melting == 1) {
        R fma = R(fmin(A.fmagma[e] + A.fmagma2[e], P.fmagma_max));
        R fm = R(P.fmagma_max), w = R(P.weaken_ratio_plastic);
        phi = phi * (R(1) - (R(1) - w) * fma / fm);
        coh = coh * (R(1) - (R(1) - w) * fma / fm);
    }
}

// Per-phase table of the plastic constants of single-phase elements, in the
// element fields' precision.
// pre_plast and plastic_consts of an element whose only phase present is
// k (phase ratio exactly 1, every other ratio below 0.01) depend on the
// element only through the branch its plastic strain takes: before
// softening (pls < plstrain1), at its start (pls == plstrain1, where the
// interpolation weight is +0) or after it (pls >= plstrain2).  For those
// the table holds the values the element path computes, from the same
// functions on the same inputs; other elements (mixed phases, strain
// inside the softening interval, melt weakening) take the element path.
template <class R>
__device__ __forceinline__ int plastic_table_state(const DevParams &P, const DevArrays &A, const GfDims &d, GF_IDX e,
                                                   int iph, R pls) {
    if (P.itype_melting == 1) return -1;
    for (int k = 0; k < P.nphase; ++k) {
        const double r = A.phase_ratio[gf_pr(d, e, k)];
        if (k == iph) {
            if (__double_as_longlong(r) != 0x3ff0000000000000ll) return -1; // exactly 1
        } else if (!gf_ratio_below_cut(r)) {
            return -1;
        }
    }
    R pl1, pl2;
    if constexpr (sizeof(R) == sizeof(float)) {
        pl1 = P.f_pl1[iph]; pl2 = P.f_pl2[iph];
        if (pls < pl1) return 0;
        if (pls < pl2) return __float_as_uint(pls) == __float_as_uint(pl1) ? 1 : -1;
    } else {
        pl1 = P.plstrain1[iph]; pl2 = P.plstrain2[iph];
        if (pls < pl1) return 0;
        if (pls < pl2) return __double_as_longlong(pls) == __double_as_longlong(pl1) ? 1 : -1;
    }
    return 2;
}

} // namespace gfk
} // namespace
