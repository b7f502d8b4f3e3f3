/*
 * ft_fmath.h — the join decisions of footile's stroker (src/stroker.rs:340-396), taken
 * as a correctly rounded f32 libm takes them, identically on the host and on sm_103a.
 *
 * footile decides each join from `th = (a1 - a0).angle_rel(b0 - b1)` (pointy: the
 * difference of two f32 atan2, folded into [-pi, pi]) and `sm = |sin(th / 2)|` in f32,
 * with the platform libm.  The decisions are sharp thresholds on those f32 values:
 *   miter:  sm >= 1/ml and sm < 1        (stroker.rs:353-357)
 *   round:  th > 0                       (stroker.rs:389-391)
 * Near-straight joins of flattened curves sit right at `sm < 1` (sin(th/2) rounds to 1
 * for |th/2| above 1.5705521 rad), so a sine or an arctangent a few ulp away from the
 * correctly rounded value flips many of them.  This header therefore takes them as a
 * correctly rounded libm would:
 *  - `sm < 1` and `sm >= s` are decided on |th/2| against f32 thresholds:
 *    RN(sin x) < 1  <=>  x <= FT_SIN_BELOW_ONE (the largest float below asin(1 - 2^-25),
 *    computed once with 200-bit arithmetic), and RN(sin x) >= s  <=>  x >= G(s), G the
 *    smallest float at or above asin of the midpoint between s and its predecessor
 *    (ft_miter_angle, double precision).  No sine is evaluated.
 *  - th needs the correctly rounded f32 atan2 of both vectors.  A single-precision
 *    evaluation (ft_atan2f, error below 3.5e-7 rad, measured on 2e8 random pairs over
 *    40 binades) decides every join whose th lies farther than FT_TH_BAND from a
 *    threshold; the others are decided again with atan2 evaluated in double precision
 *    (ft_atan2_d: relative error near 1e-15) and rounded to f32.
 * Every operation is an IEEE-754 +, -, *, / or sqrt (correctly rounded on both sides,
 * no contraction), so the host and the device take identical decisions.
 *
 * Methods (the series of the mathematics, no library routine):
 *  - atan(z), 0 <= z <= 1: half-angle reduction atan(z) = 2*atan(z / (1 + sqrt(1+z^2)))
 *    (once in f32, to |t| <= tan(pi/8), Maclaurin series to t^17; twice in double, to
 *    |t| <= tan(pi/16), Maclaurin series to t^27); z > 1 uses pi/2 - atan(1/z).
 *  - atan2(y, x): quadrant logic of the IEEE atan2 definition on top of atan.
 *  - sin(x) (f32; used by the coverage adjoint's tests only): reduction by the nearest
 *    multiple of pi, Maclaurin series to r^15.
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

#if defined(__CUDA_ARCH__)
#define FT_DADD(a, b) __dadd_rn((a), (b))
#define FT_DSUB(a, b) __dsub_rn((a), (b))
#define FT_DMUL(a, b) __dmul_rn((a), (b))
#define FT_DDIV(a, b) __ddiv_rn((a), (b))
#define FT_DSQRT(a) __dsqrt_rn((a))
#define FT_D2F(a) __double2float_rn((a))
#else
#define FT_DADD(a, b) ((a) + (b))
#define FT_DSUB(a, b) ((a) - (b))
#define FT_DMUL(a, b) ((a) * (b))
#define FT_DDIV(a, b) ((a) / (b))
#define FT_DSQRT(a) sqrt((a))
#define FT_D2F(a) ((float)(a))
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

/* ------------------------------------------------------------ double precision */

/* atan(z) for 0 <= z <= 1: two half-angle steps to t <= tan(pi/16) < 0.199, then the
 * Maclaurin series to t^27 (truncation below 2e-22). */
FT_HD double ft_atan_unit_d(double z) {
    double t = z;
    for (int i = 0; i < 2; i++) t = FT_DDIV(t, FT_DADD(1.0, FT_DSQRT(FT_DADD(1.0, FT_DMUL(t, t)))));
    double t2 = FT_DMUL(t, t);
    double p = 1.0 / 27.0;
    p = FT_DSUB(1.0 / 25.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 23.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 21.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 19.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 17.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 15.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 13.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 11.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 9.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 7.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 5.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0 / 3.0, FT_DMUL(t2, p));
    p = FT_DSUB(1.0, FT_DMUL(t2, p));
    return FT_DMUL(4.0, FT_DMUL(t, p));
}

#define FT_PI_D 3.14159265358979323846
#define FT_PI_2_D 1.57079632679489661923
#define FT_PI_4_D 0.78539816339744830962

/* atan2(y, x) in double, IEEE-754 quadrant rules. */
FT_HD double ft_atan2_d(double y, double x) {
    if (x != x || y != y) return FT_DADD(x, y);
    double ax = fabs(x), ay = fabs(y);
    double base;
    if (ax == 0.0 && ay == 0.0) {
        base = 0.0;
    } else if (ax == INFINITY && ay == INFINITY) {
        base = FT_PI_4_D;
    } else if (ay <= ax) {
        base = ft_atan_unit_d(FT_DDIV(ay, ax));
    } else {
        base = FT_DSUB(FT_PI_2_D, ft_atan_unit_d(FT_DDIV(ax, ay)));
    }
    if (signbit(x)) base = FT_DSUB(FT_PI_D, base);
    return signbit(y) ? -base : base;
}

/* ------------------------------------------------------------ join decisions */

/* RN(sin x) < 1 exactly when |x| <= this float (the largest f32 below asin(1 - 2^-25) =
 * 1.5705521861692903, 0x3FC907DA; 200-bit arithmetic). */
#define FT_SIN_BELOW_ONE 1.570552110671997f
/* Half-width of the band around a decision threshold inside which th from the f32
 * arctangents (each within 3.5e-7 rad) is not trusted: 4e-6 rad. */
#define FT_TH_BAND 4e-6f

/* G(ml): RN(|sin x|) >= RN(1/ml) exactly when |x| >= G (x in [-pi_f/2, pi_f/2]): the
 * smallest float at or above asin(m), m the midpoint between s = RN(1/ml) and the float
 * below it.  +inf when s > 1 (no sine reaches it), 0 when s = 0; NaN for ml <= 0 or NaN
 * (footile's `ml > 0.0` fails: no miter). */
FT_HD float ft_miter_angle(float ml) {
    if (!(ml > 0.0f)) return NAN;
    const float s = FT_FDIV(1.0f, ml);
    if (s > 1.0f) return INFINITY;
    if (s == 0.0f) return 0.0f;
    const double m = FT_DMUL(0.5, FT_DADD((double)nextafterf(s, 0.0f), (double)s));
    /* asin(m) = atan2(m, sqrt((1 - m)(1 + m))), 1 - m exact */
    const double a = ft_atan2_d(m, FT_DSQRT(FT_DMUL(FT_DSUB(1.0, m), FT_DADD(1.0, m))));
    float g = FT_D2F(a);
    if ((double)g < a) g = nextafterf(g, INFINITY);
    return g;
}

/* pointy's angle_rel fold of d = atan2(u) - atan2(v) (f32, pi = the f32 PI constant). */
FT_HD float ft_fold_pi(float d) {
    const float PI = FT_PI_F;
    if (d < -PI) return FT_FADD(d, FT_FMUL(2.0f, PI));
    if (d > PI) return FT_FSUB(d, FT_FMUL(2.0f, PI));
    return d;
}

/* th = angle_rel(u, v) with correctly rounded f32 atan2 (double precision, rounded). */
FT_HD float ft_angle_rel_cr(float ux, float uy, float vx, float vy) {
    const float a = FT_D2F(ft_atan2_d((double)uy, (double)ux));
    const float b = FT_D2F(ft_atan2_d((double)vy, (double)vx));
    return ft_fold_pi(FT_FSUB(a, b));
}

/* The miter decision on an exact th: sm = |RN(sin(th/2))|, sm >= s && sm < 1 <=>
 * G <= |th/2| <= FT_SIN_BELOW_ONE (false for NaN th or G). */
FT_HD int ft_miter_from_th(float th, float g) {
    const float h = fabsf(FT_FDIV(th, 2.0f));
    return h <= FT_SIN_BELOW_ONE && h >= g;
}

/* footile's miter join (stroker.rs:350-357) for u = a1 - a0, v = b0 - b1 and
 * g = ft_miter_angle(ml): 1 when the miter point is drawn (the lines' intersection
 * still has to exist), 0 for a bevel. */
FT_HD int ft_miter_join(float ux, float uy, float vx, float vy, float g) {
    if (g != g) return 0;  /* ml <= 0: bevel */
    const float d = FT_FSUB(ft_atan2f(uy, ux), ft_atan2f(vy, vx));
    const float th = ft_fold_pi(d);
    const float h = fabsf(FT_FMUL(th, 0.5f));
    const float band = 0.5f * FT_TH_BAND;
    if (th == th && fabsf(h - FT_SIN_BELOW_ONE) > band && fabsf(h - g) > band)
        return h <= FT_SIN_BELOW_ONE && h >= g;
    return ft_miter_from_th(ft_angle_rel_cr(ux, uy, vx, vy), g);
}

/* footile's round join (stroker.rs:389-395): 1 when th > 0 draws the arc, 0 for the
 * bevel of th <= 0; a NaN th draws the arc (`th <= 0.0` is false). */
FT_HD int ft_round_join_arc(float ux, float uy, float vx, float vy) {
    const float d = FT_FSUB(ft_atan2f(uy, ux), ft_atan2f(vy, vx));
    const float th = ft_fold_pi(d);
    const float PI = FT_PI_F;
    if (th == th && fabsf(th) > FT_TH_BAND && fabsf(fabsf(d) - PI) > FT_TH_BAND) return th > 0.0f;
    return !(ft_angle_rel_cr(ux, uy, vx, vy) <= 0.0f);
}

#endif /* FT_FMATH_H */
