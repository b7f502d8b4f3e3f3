/*
 * ft_fmath.h — project-written single-precision atan2 / sin used by the stroker's
 * join decisions (footile src/stroker.rs:354-356, 389-390).
 *
 * footile evaluates `angle_rel` (an atan2 difference) and `sin` with the host
 * libm.  Neither libm nor the CUDA math library promises the same last bit on a
 * CPU and on a GPU, so this header defines both functions from the mathematics
 * with IEEE-754 single-precision +, -, *, / and sqrt only (each correctly rounded
 * on both sides, no contraction).  The same source compiles for the host and for
 * sm_103a and gives identical bits on both.
 *
 * Method:
 *  - atan(z), 0 <= z <= 1: half-angle reduction atan(z) = 2*atan(z / (1 + sqrt(1+z^2)))
 *    to |t| <= tan(pi/8), then the Maclaurin series of atan to t^17
 *    (truncation error below 3e-9); z > 1 uses atan(z) = pi/2 - atan(1/z).
 *  - atan2(y, x): quadrant logic of the IEEE atan2 definition on top of atan.
 *  - sin(x): reduction by the nearest multiple of pi (pi split in two parts),
 *    then the Maclaurin series of sin to r^15 on |r| <= pi/2 (error below 1e-11).
 * Accuracy is a few ulp; only the branch decisions of the joins use these values.
 */
#ifndef FT_FMATH_H
#define FT_FMATH_H

#include <math.h>

#if defined(__CUDACC__)
#define FT_HD __host__ __device__ __forceinline__
#else
#define FT_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define FT_FADD(a, b) __fadd_rn((a), (b))
#define FT_FSUB(a, b) __fsub_rn((a), (b))
#define FT_FMUL(a, b) __fmul_rn((a), (b))
#define FT_FDIV(a, b) __fdiv_rn((a), (b))
#define FT_FSQRT(a) __fsqrt_rn((a))
#else
#define FT_FADD(a, b) ((a) + (b))
#define FT_FSUB(a, b) ((a) - (b))
#define FT_FMUL(a, b) ((a) * (b))
#define FT_FDIV(a, b) ((a) / (b))
#define FT_FSQRT(a) sqrtf((a))
#endif

#define FT_PI_F 3.14159265358979323846f
#define FT_PI_2_F 1.57079632679489661923f
#define FT_PI_4_F 0.78539816339744830962f

/* atan(t) for |t| <= tan(pi/8): Maclaurin series t - t^3/3 + t^5/5 - ... + t^17/17 */
FT_HD float ft_atan_series(float t) {
    float t2 = FT_FMUL(t, t);
    float p = 1.0f / 17.0f;
    p = FT_FSUB(1.0f / 15.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 13.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 11.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 9.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 7.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 5.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f / 3.0f, FT_FMUL(t2, p));
    p = FT_FSUB(1.0f, FT_FMUL(t2, p));
    return FT_FMUL(t, p);
}

/* atan(z) for 0 <= z <= 1 */
FT_HD float ft_atan_unit(float z) {
    float s = FT_FSQRT(FT_FADD(1.0f, FT_FMUL(z, z)));
    float t = FT_FDIV(z, FT_FADD(1.0f, s));
    return FT_FMUL(2.0f, ft_atan_series(t));
}

/* atan2(y, x) following the IEEE-754 quadrant rules. */
FT_HD float ft_atan2f(float y, float x) {
    if (x != x || y != y) return FT_FADD(x, y);
    float ax = fabsf(x), ay = fabsf(y);
    float base;
    if (ax == 0.0f && ay == 0.0f) {
        base = 0.0f;
    } else if (ax == INFINITY && ay == INFINITY) {
        base = FT_PI_4_F;
    } else if (ay <= ax) {
        base = ft_atan_unit(FT_FDIV(ay, ax));
    } else {
        base = FT_FSUB(FT_PI_2_F, ft_atan_unit(FT_FDIV(ax, ay)));
    }
    if (signbit(x)) base = FT_FSUB(FT_PI_F, base);
    return signbit(y) ? -base : base;
}

/* sin(x) */
FT_HD float ft_sinf(float x) {
    if (x != x || fabsf(x) == INFINITY) return FT_FSUB(x, x);
    /* nearest multiple of pi; pi = PI_HI + PI_LO with PI_HI exact in 12 bits */
    const float PI_HI = 3.140625f;
    const float PI_LO = 9.67653589793e-4f;
    float k = floorf(FT_FADD(FT_FMUL(x, 0.318309886183790672f), 0.5f));
    float r = FT_FSUB(FT_FSUB(x, FT_FMUL(k, PI_HI)), FT_FMUL(k, PI_LO));
    float r2 = FT_FMUL(r, r);
    /* r - r^3/3! + r^5/5! - ... - r^15/15! */
    float p = -1.0f / 1307674368000.0f;
    p = FT_FADD(1.0f / 6227020800.0f, FT_FMUL(r2, p));
    p = FT_FADD(-1.0f / 39916800.0f, FT_FMUL(r2, p));
    p = FT_FADD(1.0f / 362880.0f, FT_FMUL(r2, p));
    p = FT_FADD(-1.0f / 5040.0f, FT_FMUL(r2, p));
    p = FT_FADD(1.0f / 120.0f, FT_FMUL(r2, p));
    p = FT_FADD(-1.0f / 6.0f, FT_FMUL(r2, p));
    float s = FT_FADD(r, FT_FMUL(FT_FMUL(r, r2), p));
    /* odd multiples of pi flip the sign */
    float half = FT_FMUL(k, 0.5f);
    if (floorf(half) != half) s = -s;
    return s;
}

#endif /* FT_FMATH_H */
