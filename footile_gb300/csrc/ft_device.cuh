// ft_device.cuh — device primitives of the GB300 fill/stroke path.
//
// Fixed 16.16 arithmetic with release-mode wrapping (footile src/fixed.rs:24-158),
// the f32 -> Fixed conversion of `Fixed::from(f32)` (fixed.rs:88-93, Rust `as`
// saturation), pointy 0.7 point operations as footile uses them (geom.rs:31-35,
// plotter.rs:170,275, stroker.rs:305-309,354-360) with every float operation
// rounded individually (no FMA contraction), and pix 0.14 Ch8 / SrcOver
// compositing (fig.rs:637-643).
#pragma once

#include <cstdint>
#include <climits>

#include "../../include/footile_gpu.h"
#include "../../include/ft_fmath.h"

namespace ftk {

// ------------------------------------------------------------------ Fixed
constexpr int FX_ONE = 1 << 16;
constexpr int FX_HALF = 1 << 15;
constexpr int FX_MASK = FX_ONE - 1;

__device__ __forceinline__ int wadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
__device__ __forceinline__ int wsub(int a, int b) { return (int)((unsigned)a - (unsigned)b); }
__device__ __forceinline__ int wmul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
// (a as i64 * b as i64) >> 16, as i32          fixed.rs:40-47
__device__ __forceinline__ int fxmul(int a, int b) {
    return (int)(unsigned)(((long long)a * (long long)b) >> 16);
}
// ((a as i64) << 16) / b as i64, as i32          fixed.rs:49-56
__device__ __forceinline__ int fxdiv(int a, int b) {
    return (int)(unsigned)(((long long)a * 65536LL) / (long long)b);
}
__device__ __forceinline__ int fxfloor(int v) { return v & ~FX_MASK; }
__device__ __forceinline__ int fxceil(int v) { return fxfloor(wadd(v, FX_ONE - 1)); }
__device__ __forceinline__ int fxround(int v) { return fxfloor(wadd(v, FX_HALF)); }
__device__ __forceinline__ int fxfract(int v) { return v & FX_MASK; }
__device__ __forceinline__ int fxavg(int a, int b) { return wadd(a, b) >> 1; }
__device__ __forceinline__ int fxabs(int v) { return v == INT_MIN ? INT_MIN : (v < 0 ? -v : v); }
__device__ __forceinline__ int fxint(int v) { return v >> 16; }
// pixel_cov (fig.rs:677-682): ((fcov << 8).round()) >> 16
__device__ __forceinline__ int pixel_cov(int fcov) {
    return (int)(short)fxint(fxround((int)((unsigned)fcov << 8)));
}
// Fixed::from(f32): (f * 65536.0) as i32 — truncation, saturation, NaN -> 0
__device__ __forceinline__ int f2fx(float f) {
    float m = __fmul_rn(f, 65536.0f);
    if (m != m) return 0;
    if (m >= 2147483648.0f) return INT_MAX;
    if (m <= -2147483648.0f) return INT_MIN;
    return __float2int_rz(m);
}

// ------------------------------------------------------- pointy 0.7 points
struct P2 {
    float x, y;
};
__device__ __forceinline__ P2 p2(float x, float y) { return P2{x, y}; }
__device__ __forceinline__ P2 padd(P2 a, P2 b) { return p2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ P2 psub(P2 a, P2 b) { return p2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ P2 pscale(P2 a, float s) { return p2(__fmul_rn(a.x, s), __fmul_rn(a.y, s)); }
// Pt::midpoint, (a + b) / 2: halving is an exact power-of-two scaling, so the product with 0.5
// rounds to the same bits as the IEEE quotient.
__device__ __forceinline__ float fmid(float a, float b) { return __fmul_rn(__fadd_rn(a, b), 0.5f); }
__device__ __forceinline__ P2 pmid(P2 a, P2 b) { return p2(fmid(a.x, b.x), fmid(a.y, b.y)); }
// Pt::distance_sq
__device__ __forceinline__ float pdist_sq(P2 a, P2 b) {
    float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y);
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}
// Pt::right (y, -x) and Pt::normalize (v / |v|)
__device__ __forceinline__ P2 pright(P2 v) { return p2(v.y, -v.x); }
__device__ __forceinline__ P2 pnormalize(P2 v) {
    float m = __fsqrt_rn(__fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)));
    return p2(__fdiv_rn(v.x, m), __fdiv_rn(v.y, m));
}
__device__ __forceinline__ bool pfinite(P2 p) { return isfinite(p.x) && isfinite(p.y); }
// Transform * Pt: x' = m0*x + m1*y + m2, y' = m3*x + m4*y + m5 (left to right)
__device__ __forceinline__ P2 xform(const float* m, P2 p) {
    float x = __fadd_rn(__fadd_rn(__fmul_rn(m[0], p.x), __fmul_rn(m[1], p.y)), m[2]);
    float y = __fadd_rn(__fadd_rn(__fmul_rn(m[3], p.x), __fmul_rn(m[4], p.y)), m[5]);
    return p2(x, y);
}
// Pt::angle_rel: atan2 difference folded into [-pi, pi]
__device__ __forceinline__ float pangle_rel(P2 a, P2 b) {
    float th = __fsub_rn(ft_atan2f(a.y, a.x), ft_atan2f(b.y, b.x));
    const float PI = 3.14159265358979323846f;
    if (th < -PI) return __fadd_rn(th, 2.0f * PI);
    if (th > PI) return __fsub_rn(th, 2.0f * PI);
    return th;
}
// Line::intersection of the lines through (a0,a1) and (b0,b1)
__device__ __forceinline__ bool pline_x(P2 a0, P2 a1, P2 b0, P2 b1, P2* out) {
    float x1 = a0.x, y1 = a0.y, x2 = a1.x, y2 = a1.y;
    float x3 = b0.x, y3 = b0.y, x4 = b1.x, y4 = b1.y;
    float den = __fsub_rn(__fmul_rn(__fsub_rn(x1, x2), __fsub_rn(y3, y4)),
                          __fmul_rn(__fsub_rn(y1, y2), __fsub_rn(x3, x4)));
    if (den == 0.0f) return false;
    float a = __fsub_rn(__fmul_rn(x1, y2), __fmul_rn(y1, x2));
    float b = __fsub_rn(__fmul_rn(x3, y4), __fmul_rn(y3, x4));
    float x = __fdiv_rn(__fsub_rn(__fmul_rn(a, __fsub_rn(x3, x4)), __fmul_rn(__fsub_rn(x1, x2), b)), den);
    float y = __fdiv_rn(__fsub_rn(__fmul_rn(a, __fsub_rn(y3, y4)), __fmul_rn(__fsub_rn(y1, y2), b)), den);
    *out = p2(x, y);
    return true;
}

// ------------------------------------------------------- pix 0.14 Ch8 / SrcOver
__device__ __forceinline__ unsigned ch8_mul(unsigned a, unsigned b) {
    unsigned l = (a << 4) | (a >> 4);
    unsigned r = (b << 4) | (b >> 4);
    return (l * r) >> 16;
}
__device__ __forceinline__ unsigned ch8_add(unsigned a, unsigned b) { return min(a + b, 255u); }
// composite_channels_alpha(&clr, SrcOver, &alpha) on one premultiplied RGBA pixel
__device__ __forceinline__ unsigned srcover_rgba(unsigned d, unsigned clr, unsigned alpha) {
    unsigned sa = ch8_mul(clr >> 24, alpha);
    unsigned inv = 255u - sa;
    unsigned out = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        unsigned dc = (d >> (8 * c)) & 0xFF;
        unsigned sc = (clr >> (8 * c)) & 0xFF;
        out |= ch8_add(ch8_mul(sc, alpha), ch8_mul(dc, inv)) << (8 * c);
    }
    return out;
}

// fill rule on the wrapped i16 running sum (imgbuf.rs:54-61, 157-167)
__device__ __forceinline__ unsigned resolve_cov(unsigned sum32, int rule) {
    int s = (int)(short)(sum32 & 0xFFFF);
    if (rule == FT_NONZERO) return (unsigned)min(max(s, 0), 255);
    int v = s & 0xFF;
    int odd = s & 0x100;
    int c = abs(v - odd);
    return (unsigned)min(c, 255);
}

}  // namespace ftk
