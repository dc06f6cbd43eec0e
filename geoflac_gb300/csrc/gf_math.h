// Deterministic FP64 elementary functions used by the FP64 step on both the
// host and the device, so that the two compute bit-identical results.
//
// Only IEEE-754 correctly rounded operations (+ - * / and exact scaling by
// powers of two) are used; built without FMA contraction (host:
// -ffp-contract=off, device: -fmad=false) they round identically everywhere.
// Methods:
//   exp  : Cody & Waite argument reduction x = k ln2 + r (ln2 split into a
//          32-bit head and a tail), |r| <= ln2/2, then the Taylor polynomial
//          of e^r to degree 14 (Horner).
//   log  : x = m 2^e with m in [sqrt(1/2), sqrt(2)), s = (m-1)/(m+1),
//          log m = 2 atanh s = 2 (s + s^3/3 + ... + s^23/23).
//   pow  : exp(y log x) for x > 0.
//   sin, cos, tan : Cody & Waite reduction by pi/2 (three-part constant),
//          |r| <= pi/4, Taylor series of sin r (to r^21) and cos r (to
//          r^22); tan = sin/cos with the quadrant swap.
// Accuracy: a few ulp of the correctly rounded value over the arguments the
// step uses (checked against the C library in the tests).
#pragma once

#ifdef __CUDACC__
#define GFM_HD __host__ __device__ __forceinline__
#else
#define GFM_HD inline
#endif

#include <math.h>

namespace gfm {

GFM_HD double round_half_up(double x) { return floor(x + 0.5); }

GFM_HD double exp(double x) {
    if (x != x) return x;
    if (x > 709.78) return HUGE_VAL;
    if (x < -745.2) return 0.0;
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
    const double inv_ln2 = 0x1.71547652b82fep+0;
    double kf = round_half_up(x * inv_ln2);
    double r = (x - kf * ln2_hi) - kf * ln2_lo;
    double p = 0x1.93974a8c07c9dp-37;     // 1/14!
    p = p * r + 0x1.6124613a86d09p-33;    // 1/13!
    p = p * r + 0x1.1eed8eff8d898p-29;    // 1/12!
    p = p * r + 0x1.ae64567f544e4p-26;    // 1/11!
    p = p * r + 0x1.27e4fb7789f5cp-22;    // 1/10!
    p = p * r + 0x1.71de3a556c734p-19;    // 1/9!
    p = p * r + 0x1.a01a01a01a01ap-16;    // 1/8!
    p = p * r + 0x1.a01a01a01a01ap-13;    // 1/7!
    p = p * r + 0x1.6c16c16c16c17p-10;    // 1/6!
    p = p * r + 0x1.1111111111111p-7;     // 1/5!
    p = p * r + 0x1.5555555555555p-5;     // 1/4!
    p = p * r + 0x1.5555555555555p-3;     // 1/3!
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    return ldexp(p, (int)kf);
}

GFM_HD double log(double x) {
    if (x != x) return x;
    if (x < 0.0) return NAN;
    if (x == 0.0) return -HUGE_VAL;
    if (x == HUGE_VAL) return x;
    int e;
    double m = frexp(x, &e); // x = m 2^e, m in [0.5, 1)
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = m * 2.0;
        e = e - 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double z = s * s;
    double t = 1.0 / 23.0;
    t = t * z + 1.0 / 21.0;
    t = t * z + 1.0 / 19.0;
    t = t * z + 1.0 / 17.0;
    t = t * z + 1.0 / 15.0;
    t = t * z + 1.0 / 13.0;
    t = t * z + 1.0 / 11.0;
    t = t * z + 1.0 / 9.0;
    t = t * z + 1.0 / 7.0;
    t = t * z + 1.0 / 5.0;
    t = t * z + 1.0 / 3.0;
    double logm = 2.0 * s + 2.0 * s * (z * t);
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
    double fe = (double)e;
    return fe * ln2_hi + (fe * ln2_lo + logm);
}

GFM_HD double pow(double x, double y) {
    if (y == 0.0) return 1.0;
    if (x == 1.0) return 1.0;
    if (x == 0.0) return y > 0.0 ? 0.0 : HUGE_VAL;
    if (x < 0.0) return NAN;
    return gfm::exp(y * gfm::log(x));
}

// sin r and cos r for |r| <= pi/4
GFM_HD void sincos_kernel(double r, double &s, double &c) {
    double z = r * r;
    // sin: r - r^3/3! + r^5/5! - ... - r^19/19! + r^21/21!
    double t = 0x1.71b8ef6dcf572p-66;      // 1/21!
    t = t * z - 0x1.2f49b46814157p-57;     // 1/19!
    t = t * z + 0x1.952c77030ad4ap-49;     // 1/17!
    t = t * z - 0x1.ae7f3e733b81fp-41;     // 1/15!
    t = t * z + 0x1.6124613a86d09p-33;     // 1/13!
    t = t * z - 0x1.ae64567f544e4p-26;     // 1/11!
    t = t * z + 0x1.71de3a556c734p-19;     // 1/9!
    t = t * z - 0x1.a01a01a01a01ap-13;     // 1/7!
    t = t * z + 0x1.1111111111111p-7;      // 1/5!
    t = t * z - 0x1.5555555555555p-3;      // 1/3!
    s = r + r * (z * t);
    // cos: 1 - r^2/2! + r^4/4! - ... + r^20/20! - r^22/22!
    double u = -0x1.0ce396db7f853p-70;     // 1/22!
    u = u * z + 0x1.e542ba4020225p-62;     // 1/20!
    u = u * z - 0x1.6827863b97d97p-53;     // 1/18!
    u = u * z + 0x1.ae7f3e733b81fp-45;     // 1/16!
    u = u * z - 0x1.93974a8c07c9dp-37;     // 1/14!
    u = u * z + 0x1.1eed8eff8d898p-29;     // 1/12!
    u = u * z - 0x1.27e4fb7789f5cp-22;     // 1/10!
    u = u * z + 0x1.a01a01a01a01ap-16;     // 1/8!
    u = u * z - 0x1.6c16c16c16c17p-10;     // 1/6!
    u = u * z + 0x1.5555555555555p-5;      // 1/4!
    u = u * z - 0.5;
    c = 1.0 + z * u;
}

GFM_HD double reduce_pio2(double x, int &q) {
    const double pio2_hi = 0x1.921fb54400000p+0;
    const double pio2_mid = 0x1.0b4611a600000p-34;
    const double pio2_lo = 0x1.3198a2e037073p-69;
    const double two_over_pi = 0x1.45f306dc9c883p-1;
    double kf = round_half_up(x * two_over_pi);
    q = (int)kf;
    return ((x - kf * pio2_hi) - kf * pio2_mid) - kf * pio2_lo;
}

GFM_HD double sin(double x) {
    int q;
    double r = reduce_pio2(x, q);
    double s, c;
    sincos_kernel(r, s, c);
    switch (q & 3) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
    }
}

GFM_HD double cos(double x) {
    int q;
    double r = reduce_pio2(x, q);
    double s, c;
    sincos_kernel(r, s, c);
    switch (q & 3) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
    }
}

GFM_HD double tan(double x) {
    int q;
    double r = reduce_pio2(x, q);
    double s, c;
    sincos_kernel(r, s, c);
    return (q & 1) ? -c / s : s / c;
}

} // namespace gfm
