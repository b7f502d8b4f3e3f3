// ft_adjoint.cu — differentiable FP32 coverage of fills and its adjoint.
//
// The forward covers the flattened polygon of every path analytically: the path walk
// and De Casteljau subdivision of Plotter::fill (plotter.rs:175-332, same f32 tree as
// the integer rasteriser), sub-figures as Fig builds them (fig.rs:428-461), and the
// cell-area scheme of fig.rs:285-321 without its 16.16 / 1/256 quantisation: each edge
// adds, per raster row and cell, dir * h * (c + 1 - xmid) to cell c and the rest of h
// to cell c + 1 (all of h to cell 0 left of the raster); the row prefix sum
// (imgbuf.rs:38-51) times the figure's direction sign (fig_sign) is the winding area
// S; NonZero gives clamp(S, 0, 1), EvenOdd the period-2 triangle wave.  The integer rasteriser stays the shipped forward; this one
// exists to be differentiated.
//
// The backward recomputes the flattening and the edges (nothing but the winding area
// is kept from the forward) and takes, per edge P0->P1, the boundary integral
//   dS_p/dP0 = (-dy, dx) * int_{s in p} (1 - s) ds,  dS_p/dP1 = (-dy, dx) * int_{s in p} s ds
// weighted by g_p = dL/dcov_p * dcov/dS_p, then chains vertex gradients to the op
// floats through the Bernstein weights of each leaf's end parameter and the
// transpose of the transform's linear part.  The subdivision tree is held fixed
// (it is piecewise constant in the control points).
//
// One CTA per path: a 256-thread walk over the ops in chunks (block scans give each
// op its pen, vertex offset and sub-figure start), then bands of rows in a 64 KB
// shared buffer, (edge, row) items spread over the threads.
#include <climits>

#include "ft_adjoint.cuh"
#include "ft_device.cuh"

namespace fta {

using ftk::P2;
using ftk::p2;
using ftk::pdist_sq;
using ftk::pfinite;
using ftk::pmid;
using ftk::xform;

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NW = ABLOCK / 32;
constexpr int EPT = 4;                 // edges per thread per edge chunk
constexpr int ECHUNK = ABLOCK * EPT;

// The block's stroke point walk, carried from one chunk of ops (or window of points) to
// the next (stroke_points_block).
struct SPCarry {
    int pw;           // last PenWidth op so far, -1
    int pc, pc_pw;    // last Close/Move/Line/Quad/Cubic op so far and the PenWidth op before it
    int ce;           // last close event so far: 2 * op + (op is a Close), -1
    int kept;         // points kept so far (uncapped)
    int nsub;         // sub-strokes started after the first
    int have_prev;    // a point has been walked: its position and op follow
    float px, py;
    int pop;
    int last_op;      // op of the last stored point, -1
};

struct ASmem {
    int wsum[NW];
    int wmax[NW];
    int wmax2[NW];
    int wmax3[NW];
    int off[ECHUNK + 1];
    SPCarry spc;
    int carry_pen, carry_close, carry_base, carry_sub;
    int status;
    int total;
    unsigned long long top_key;
    int top, nxt, prv, sub_last;
    float sign;
};

__device__ __forceinline__ int warp_incl_sum(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}
__device__ __forceinline__ int warp_incl_max(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v = max(v, t);
    }
    return v;
}

// Block-wide exclusive sum; `total` gets the block's sum.  Every thread must call.
__device__ int block_excl_sum(int v, int* wsum, int& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_sum(v);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    int pre = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) {
        int x = wsum[i];
        pre += i < w ? x : 0;
        tot += x;
    }
    __syncthreads();
    total = tot;
    return pre + inc - v;
}

// Block-wide max scan: inclusive and exclusive (INT_MIN before the first thread).
__device__ void block_max_scan(int v, int* wmax, int& incl, int& excl) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = warp_incl_max(v);
    int ex = __shfl_up_sync(FULL, inc, 1);
    if (lane == 0) ex = INT_MIN;
    if (lane == 31) wmax[w] = inc;
    __syncthreads();
    int pre = INT_MIN;
#pragma unroll
    for (int i = 0; i < NW; i++) pre = i < w ? max(pre, wmax[i]) : pre;
    __syncthreads();
    incl = max(pre, inc);
    excl = max(pre, ex);
}

// What fixed.rs:88-93 makes of a coordinate, in pixels: NaN becomes 0 and values
// saturate at the ends of the 16.16 range.  Coordinates it changes take no gradient.
__device__ __forceinline__ float fx_range(float v) { return v != v ? 0.0f : fminf(fmaxf(v, -32768.0f), 32768.0f); }
__device__ __forceinline__ float2 fx_pass(P2 raw, float2 g) {
    return make_float2(fx_range(raw.x) == raw.x ? g.x : 0.0f, fx_range(raw.y) == raw.y ? g.y : 0.0f);
}

__device__ __forceinline__ float pow2neg(int d) { return __int_as_float((127 - d) << 23); }  // 2^-d, d <= 126

// Stack frames of the walks below: the right half of a subdivided curve without its
// start point, which is the end point of the left half's last leaf (the same value,
// carried down unchanged).  W: with pen widths.
template <bool CUBIC, bool W>
struct WalkFr {
    P2 b, c, d;
    float wb, wc, wd;
    int dep;
};
template <>
struct WalkFr<true, false> {
    P2 b, c, d;
    int dep;
};
template <>
struct WalkFr<false, true> {
    P2 b, c;
    float wb, wc;
    int dep;
};
template <>
struct WalkFr<false, false> {
    P2 b, c;
    int dep;
};

// De Casteljau walk of one quad (plotter.rs:248-265) or cubic (plotter.rs:311-332) in
// depth-first order; leaf(index, end point, end parameter t).  Returns the leaf count.
template <bool CUBIC, class Leaf>
__device__ int curve_walk(P2 a, P2 b, P2 c, P2 d, float tol_sq, int* depth_hit, Leaf leaf) {
    using Fr = WalkFr<CUBIC, false>;
    Fr st[FT_MAX_DEPTH + 1];
    int sp = 0, n = 0, dep = 0;
    float t = 0.0f;
    for (;;) {
        bool within;
        P2 l1, l2, m, r1, r2;
        if (CUBIC) {
            P2 ab = pmid(a, b), bc = pmid(b, c), cd = pmid(c, d);
            P2 abbc = pmid(ab, bc), bccd = pmid(bc, cd);
            m = pmid(abbc, bccd);
            within = pdist_sq(m, pmid(a, d)) <= tol_sq;
            l1 = ab;
            l2 = abbc;
            r1 = bccd;
            r2 = cd;
        } else {
            P2 ab = pmid(a, b), bc = pmid(b, c);
            m = pmid(ab, bc);
            within = pdist_sq(m, pmid(a, c)) <= tol_sq;
            l1 = ab;
            l2 = m;
            r1 = bc;
            r2 = c;
        }
        if (within || dep >= FT_MAX_DEPTH) {
            if (!within) *depth_hit = 1;
            t = __fadd_rn(t, pow2neg(dep));  // dyadic, exact
            leaf(n, CUBIC ? d : c, t);
            n++;
            if (sp == 0) break;
            --sp;
            a = CUBIC ? d : c;
            b = st[sp].b;
            c = st[sp].c;
            if constexpr (CUBIC) d = st[sp].d;
            dep = st[sp].dep;
        } else {
            if constexpr (CUBIC) {
                st[sp] = Fr{r1, r2, d, dep + 1};
                b = l1;
                c = l2;
                d = m;
            } else {
                st[sp] = Fr{r1, r2, dep + 1};
                b = l1;
                c = l2;
            }
            sp++;
            dep++;
        }
    }
    return n;
}

__device__ __forceinline__ int end_slot(int kind) { return kind == FT_OP_CUBIC ? 2 : (kind == FT_OP_QUAD ? 1 : 0); }

__device__ __forceinline__ P2 op_pt(const ft_op& o, int slot) { return p2(o.v[2 * slot], o.v[2 * slot + 1]); }

__device__ __forceinline__ ft_op load_op(const ft_op* ops, int i) {
    const float4* q = reinterpret_cast<const float4*>(ops + i);
    float4 x = __ldg(q), y = __ldg(q + 1);
    ft_op o;
    o.kind = __float_as_int(x.x);
    o.v[0] = x.y;
    o.v[1] = x.z;
    o.v[2] = x.w;
    o.v[3] = y.x;
    o.v[4] = y.y;
    o.v[5] = y.z;
    o.reserved = 0;
    return o;
}

enum { WALK_EMIT = 0, WALK_GRAD = 1 };

// The path walk of plotter.rs:175-224 over ops [0, n) in chunks of ABLOCK ops.
// WALK_EMIT writes vertex positions and sub-figure starts (and zeroes vertex gradients
// when `zero_grad`); WALK_GRAD chains vertex gradients to the op floats.  Returns the
// vertex count.
template <int MODE>
__device__ int path_walk(const AParams& p, ASmem& sm, const ft_op* ops, int n, float2* vpos, int* vsub,
                         float2* vgrad, bool zero_grad, float* gops) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        sm.carry_pen = -1;
        sm.carry_close = -1;
        sm.carry_base = 0;
        sm.carry_sub = -1;
    }
    __syncthreads();
    const float* m = p.xf;
    for (int c0 = 0; c0 < n; c0 += ABLOCK) {
        const int i = c0 + tid;
        ft_op o;
        o.kind = -1;
        if (i < n) o = load_op(ops, i);
        const int kind = o.kind;
        const bool pen_setting = kind == FT_OP_MOVE || kind == FT_OP_LINE || kind == FT_OP_QUAD || kind == FT_OP_CUBIC;
        int inc_pen, exc_pen, inc_close, exc_close;
        block_max_scan(pen_setting ? i : -1, sm.wmax, inc_pen, exc_pen);
        block_max_scan(kind == FT_OP_CLOSE ? i : -1, sm.wmax2, inc_close, exc_close);
        const int carry_pen = sm.carry_pen, carry_close = sm.carry_close;
        exc_pen = max(exc_pen, carry_pen);
        exc_close = max(exc_close, carry_close);
        const int prev_pen = exc_pen > exc_close ? exc_pen : -1;
        // curve geometry (transformed) and leaf count
        P2 A = p2(0.f, 0.f), B = A, C = A, D = A;
        int cnt = 0, depth_hit = 0;
        bool curve = false;
        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
            cnt = 1;
        } else if (kind == FT_OP_QUAD || kind == FT_OP_CUBIC) {
            P2 pen = p2(0.f, 0.f);
            if (prev_pen >= 0) {
                ft_op q = load_op(ops, prev_pen);
                pen = op_pt(q, end_slot(q.kind));
            }
            A = xform(m, pen);
            B = xform(m, op_pt(o, 0));
            C = xform(m, op_pt(o, 1));
            D = kind == FT_OP_CUBIC ? xform(m, op_pt(o, 2)) : C;
            if (!pfinite(A) || !pfinite(B) || !pfinite(C) || !pfinite(D)) {
                cnt = 1;
                atomicMax(&sm.status, (int)FT_ERR_ARG);
            } else {
                curve = true;
                auto none = [](int, P2, float) {};
                cnt = kind == FT_OP_CUBIC ? curve_walk<true>(A, B, C, D, p.tol_sq, &depth_hit, none)
                                          : curve_walk<false>(A, B, C, D, p.tol_sq, &depth_hit, none);
                if (depth_hit) atomicMax(&sm.status, (int)FT_ERR_DEPTH);
            }
        }
        int chunk_total;
        const int base = sm.carry_base + block_excl_sum(cnt, sm.wsum, chunk_total);
        const bool starts = cnt > 0 && (kind == FT_OP_MOVE || prev_pen < 0);
        int inc_sub, exc_sub;
        block_max_scan(starts ? base : -1, sm.wmax3, inc_sub, exc_sub);
        const int sub = max(inc_sub, sm.carry_sub);
        if (MODE == WALK_EMIT) {
            auto put = [&](int j, P2 q, float) {
                const int k = base + j;
                if (k < VCAP) {
                    vpos[k] = make_float2(fx_range(q.x), fx_range(q.y));
                    vsub[k] = sub;
                    if (zero_grad) vgrad[k] = make_float2(0.f, 0.f);
                }
            };
            if (curve) {
                if (kind == FT_OP_CUBIC)
                    curve_walk<true>(A, B, C, D, p.tol_sq, &depth_hit, put);
                else
                    curve_walk<false>(A, B, C, D, p.tol_sq, &depth_hit, put);
            } else if (cnt == 1) {
                put(0, xform(m, op_pt(o, end_slot(kind))), 1.0f);
            }
        } else if (cnt > 0) {
            // back through the transform: d(m*p)/dp = [[m0, m1], [m3, m4]]
            float* g = gops + (size_t)i * 6;
            if (!curve) {
                const float2 gv = fx_pass(xform(m, op_pt(o, end_slot(kind))), __ldcg(&vgrad[base]));  // L2 atomics
                const int s = end_slot(kind);
                atomicAdd(g + 2 * s, __fadd_rn(__fmul_rn(m[0], gv.x), __fmul_rn(m[3], gv.y)));
                atomicAdd(g + 2 * s + 1, __fadd_rn(__fmul_rn(m[1], gv.x), __fmul_rn(m[4], gv.y)));
            } else {
                float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // pen, b, c, d
                auto chain = [&](int j, P2 q, float t) {
                    const float2 gv = fx_pass(q, __ldcg(&vgrad[base + j]));
                    const float gx = __fadd_rn(__fmul_rn(m[0], gv.x), __fmul_rn(m[3], gv.y));
                    const float gy = __fadd_rn(__fmul_rn(m[1], gv.x), __fmul_rn(m[4], gv.y));
                    const float u = __fsub_rn(1.0f, t);
                    float w0, w1, w2, w3;
                    if (kind == FT_OP_CUBIC) {
                        w0 = __fmul_rn(__fmul_rn(u, u), u);
                        w1 = __fmul_rn(__fmul_rn(3.0f, t), __fmul_rn(u, u));
                        w2 = __fmul_rn(__fmul_rn(3.0f, t), __fmul_rn(t, u));
                        w3 = __fmul_rn(__fmul_rn(t, t), t);
                    } else {
                        w0 = __fmul_rn(u, u);
                        w1 = __fmul_rn(__fmul_rn(2.0f, t), u);
                        w2 = __fmul_rn(t, t);
                        w3 = 0.0f;
                    }
                    acc[0] = __fadd_rn(acc[0], __fmul_rn(w0, gx));
                    acc[1] = __fadd_rn(acc[1], __fmul_rn(w0, gy));
                    acc[2] = __fadd_rn(acc[2], __fmul_rn(w1, gx));
                    acc[3] = __fadd_rn(acc[3], __fmul_rn(w1, gy));
                    acc[4] = __fadd_rn(acc[4], __fmul_rn(w2, gx));
                    acc[5] = __fadd_rn(acc[5], __fmul_rn(w2, gy));
                    acc[6] = __fadd_rn(acc[6], __fmul_rn(w3, gx));
                    acc[7] = __fadd_rn(acc[7], __fmul_rn(w3, gy));
                };
                if (kind == FT_OP_CUBIC)
                    curve_walk<true>(A, B, C, D, p.tol_sq, &depth_hit, chain);
                else
                    curve_walk<false>(A, B, C, D, p.tol_sq, &depth_hit, chain);
                const int nslot = kind == FT_OP_CUBIC ? 3 : 2;
                for (int s = 0; s < nslot; s++) {
                    atomicAdd(g + 2 * s, acc[2 + 2 * s]);
                    atomicAdd(g + 2 * s + 1, acc[3 + 2 * s]);
                }
                if (prev_pen >= 0) {
                    const int s = end_slot(load_op(ops, prev_pen).kind);
                    float* gp = gops + (size_t)prev_pen * 6;
                    atomicAdd(gp + 2 * s, acc[0]);
                    atomicAdd(gp + 2 * s + 1, acc[1]);
                }
            }
        }
        __syncthreads();
        if (tid == ABLOCK - 1) {
            sm.carry_pen = max(inc_pen, carry_pen);
            sm.carry_close = max(inc_close, carry_close);
            sm.carry_base = base + cnt;
            sm.carry_sub = sub;
        }
        __syncthreads();
    }
    return sm.carry_base;
}

__device__ __forceinline__ int2 fxp(const float2* vpos, int k) {
    const float2 q = vpos[k];
    return make_int2(ftk::f2fx(q.x), ftk::f2fx(q.y));
}
__device__ __forceinline__ bool fx_ne(int2 a, int2 b) { return a.x != b.x || a.y != b.y; }

// The direction footile's Fig gives the figure (fig.rs:402-411, 493-494), as +1.0f
// (Forward) or -1.0f: the top vertex is the kept vertex with the least (y, x, id) in
// 16.16, where Fig::add_point drops a point equal to the previous one and Fig::close
// drops a last point equal to the sub-figure's first (fig.rs:373-383, 428-451), so the
// top is the first raw vertex with the least point outside sub-figures whose points
// all coincide; its neighbours in the kept sub-figure decide widdershins with
// wrapping Fixed products (fig.rs:116-119).  Edges count +1 in that direction, and
// NonZero clamps the signed row sum at 0 (imgbuf.rs:54-61).
__device__ float fig_sign(ASmem& sm, int V, const float2* vpos, const int* vsub, int* vflag) {
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) {
        sm.top_key = ~0ull;
        sm.top = INT_MAX;
        sm.nxt = INT_MAX;
        sm.prv = -1;
        sm.sub_last = -1;
    }
    for (int k = tid; k < V; k += ABLOCK) vflag[k] = 0;
    __syncthreads();
    for (int k = tid; k < V; k += ABLOCK) {
        const int s0 = vsub[k];
        if (fx_ne(fxp(vpos, k), fxp(vpos, s0))) vflag[s0] = 1;  // the sub-figure keeps a second point
    }
    __syncthreads();
    unsigned long long best = ~0ull;
    for (int k = tid; k < V; k += ABLOCK) {
        const int s0 = vsub[k];
        const int2 q = fxp(vpos, k);
        const bool kept = k == s0 || fx_ne(q, fxp(vpos, k - 1));
        if (!kept || !vflag[s0]) continue;
        const unsigned long long key = ((unsigned long long)((unsigned)q.y ^ 0x80000000u) << 32) |
                                       (unsigned long long)((unsigned)q.x ^ 0x80000000u);
        best = key < best ? key : best;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(FULL, best, o);
        best = t < best ? t : best;
    }
    if (lane == 0 && best != ~0ull) atomicMin(&sm.top_key, best);
    __syncthreads();
    const unsigned long long tk = sm.top_key;
    if (tk == ~0ull) return 1.0f;
    for (int k = tid; k < V; k += ABLOCK) {
        const int s0 = vsub[k];
        const int2 q = fxp(vpos, k);
        const unsigned long long key = ((unsigned long long)((unsigned)q.y ^ 0x80000000u) << 32) |
                                       (unsigned long long)((unsigned)q.x ^ 0x80000000u);
        const bool kept = k == s0 || fx_ne(q, fxp(vpos, k - 1));
        if (kept && vflag[s0] && key == tk) atomicMin(&sm.top, k);
    }
    __syncthreads();
    const int top = sm.top, s0 = vsub[top];
    const int2 qt = fxp(vpos, top), qs = fxp(vpos, s0);
    for (int k = s0 + 1 + tid; k < V && vsub[k] == s0; k += ABLOCK) {
        const int2 q = fxp(vpos, k);
        if (k > top && fx_ne(q, qt)) atomicMin(&sm.nxt, k);
        if (fx_ne(q, qs)) atomicMax(&sm.prv, k);
    }
    __syncthreads();
    float sign = 1.0f;
    if (tid == 0) {
        const int2 n = sm.nxt != INT_MAX ? fxp(vpos, sm.nxt) : qs;
        const int2 pv = top > s0 ? fxp(vpos, top - 1) : (sm.prv >= 0 ? fxp(vpos, sm.prv) : qt);
        const int ax = ftk::wsub(pv.x, qt.x), ay = ftk::wsub(pv.y, qt.y);
        const int bx = ftk::wsub(n.x, qt.x), by = ftk::wsub(n.y, qt.y);
        sm.sign = ftk::fxmul(ax, by) > ftk::fxmul(bx, ay) ? 1.0f : -1.0f;
    }
    __syncthreads();
    sign = sm.sign;
    __syncthreads();
    return sign;
}

// One edge, top end a, bottom end b (a.y < b.y).
struct EdgeG {
    P2 a, b;
    float dy, dxdy, xlo, xhi;
    float dir;   // +1 when the edge runs down (P0 on top), -1 up
    P2 perp;     // (-dy, dx) of P1 - P0
    int e, nxt;
    bool ok;
};

__device__ __forceinline__ int next_vertex(const int* vsub, int V, int k) {
    return (k + 1 < V && vsub[k + 1] == vsub[k]) ? k + 1 : vsub[k];
}

__device__ __forceinline__ EdgeG make_edge(const float2* vpos, const int* vsub, int V, int e) {
    EdgeG E;
    E.e = e;
    E.nxt = next_vertex(vsub, V, e);
    const float2 q0 = vpos[e], q1 = vpos[E.nxt];
    const P2 p0 = p2(q0.x, q0.y), p1 = p2(q1.x, q1.y);
    E.ok = pfinite(p0) && pfinite(p1) && p0.y != p1.y;
    const bool down = p1.y > p0.y;
    E.a = down ? p0 : p1;
    E.b = down ? p1 : p0;
    E.dir = down ? 1.0f : -1.0f;
    E.dy = __fsub_rn(E.b.y, E.a.y);
    E.dxdy = __fdiv_rn(__fsub_rn(E.b.x, E.a.x), E.dy);
    E.xlo = fminf(E.a.x, E.b.x);
    E.xhi = fmaxf(E.a.x, E.b.x);
    E.perp = p2(-__fsub_rn(p1.y, p0.y), __fsub_rn(p1.x, p0.x));
    return E;
}

// Rows of the edge inside rows [b0, b1]; first row in *r0.
__device__ __forceinline__ int edge_rows(const EdgeG& E, int b0, int b1, int* r0) {
    if (!E.ok) return 0;
    const float f0 = fmaxf(floorf(E.a.y), (float)b0);
    const float f1 = fminf(__fsub_rn(ceilf(E.b.y), 1.0f), (float)b1);
    if (!(f0 <= f1)) return 0;
    *r0 = (int)f0;
    return (int)f1 - (int)f0 + 1;
}

// Pieces of the edge in raster row r, cell by cell: cb(cell, h, xmid, u0, u1); cell -1
// is everything left of the raster; cells at or right of W are dropped.
template <class CB>
__device__ __forceinline__ void row_pieces(const EdgeG& E, int r, int W, CB cb) {
    const float yt = fmaxf(E.a.y, (float)r), yb = fminf(E.b.y, (float)(r + 1));
    if (!(yb > yt)) return;
    const float xt = yt == E.a.y ? E.a.x
                                 : fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(yt, E.a.y), E.dxdy)), E.xlo), E.xhi);
    const float xb = yb == E.b.y ? E.b.x
                                 : fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(yb, E.a.y), E.dxdy)), E.xlo), E.xhi);
    const float ut = __fdiv_rn(__fsub_rn(yt, E.a.y), E.dy), ub = __fdiv_rn(__fsub_rn(yb, E.a.y), E.dy);
    const float h = __fsub_rn(yb, yt);
    const float xl = fminf(xt, xb), xr = fmaxf(xt, xb);
    const bool rising = xt <= xb;
    const float cl = floorf(xl), cr = floorf(xr);
    if (cl == cr || xr == xl) {
        if (cl < (float)W) cb(cl < 0.0f ? -1 : (int)cl, h, __fmul_rn(__fadd_rn(xl, xr), 0.5f), ut, ub);
        return;
    }
    const float span = __fsub_rn(xr, xl), du = __fsub_rn(ub, ut);
    auto piece = [&](float x0, float x1, int c) {
        const float f0 = __fdiv_rn(__fsub_rn(x0, xl), span), f1 = __fdiv_rn(__fsub_rn(x1, xl), span);
        const float u0 = rising ? __fadd_rn(ut, __fmul_rn(f0, du)) : __fsub_rn(ub, __fmul_rn(f1, du));
        const float u1 = rising ? __fadd_rn(ut, __fmul_rn(f1, du)) : __fsub_rn(ub, __fmul_rn(f0, du));
        cb(c, __fmul_rn(__fsub_rn(f1, f0), h), __fmul_rn(__fadd_rn(x0, x1), 0.5f), u0, u1);
    };
    float c = cl;
    if (c < 0.0f) {
        const float x1 = fminf(xr, 0.0f);
        if (x1 > xl) piece(xl, x1, -1);
        c = 0.0f;
    }
    const float cend = fminf(cr, (float)(W - 1));
    for (; c <= cend; c = __fadd_rn(c, 1.0f)) {
        const float x0 = fmaxf(xl, c), x1 = fminf(xr, __fadd_rn(c, 1.0f));
        if (x1 > x0) piece(x0, x1, (int)c);
    }
}

// Forward pieces of the edge in raster row r: cb(cell, h, xmid) as row_pieces gives
// them, with one division per row (the height per unit of x) instead of two per piece.
template <class CB>
__device__ __forceinline__ void row_cells(const EdgeG& E, int r, int W, CB cb) {
    const float yt = fmaxf(E.a.y, (float)r), yb = fminf(E.b.y, (float)(r + 1));
    if (!(yb > yt)) return;
    const float xt = yt == E.a.y ? E.a.x
                                 : fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(yt, E.a.y), E.dxdy)), E.xlo), E.xhi);
    const float xb = yb == E.b.y ? E.b.x
                                 : fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(yb, E.a.y), E.dxdy)), E.xlo), E.xhi);
    const float h = __fsub_rn(yb, yt);
    const float xl = fminf(xt, xb), xr = fmaxf(xt, xb);
    const float cl = floorf(xl), cr = floorf(xr);
    if (cl == cr || xr == xl) {
        if (cl < (float)W) cb(cl < 0.0f ? -1 : (int)cl, h, __fmul_rn(__fadd_rn(xl, xr), 0.5f));
        return;
    }
    const float hs = __fdiv_rn(h, __fsub_rn(xr, xl));
    auto piece = [&](float x0, float x1, int c) {
        cb(c, __fmul_rn(__fsub_rn(x1, x0), hs), __fmul_rn(__fadd_rn(x0, x1), 0.5f));
    };
    float c = cl;
    if (c < 0.0f) {
        const float x1 = fminf(xr, 0.0f);
        if (x1 > xl) piece(xl, x1, -1);
        c = 0.0f;
    }
    const float cend = fminf(cr, (float)(W - 1));
    for (; c <= cend; c = __fadd_rn(c, 1.0f)) {
        const float x0 = fmaxf(xl, c), x1 = fminf(xr, __fadd_rn(c, 1.0f));
        if (x1 > x0) piece(x0, x1, (int)c);
    }
}

// All (edge, row) items of rows [b0, b0 + nb) of the path: forward adds cell areas to
// the band, backward accumulates the edge integrals against g = gv(row, cell) (the
// loss gradient times dcov/dS at that cell).  The edges visited are elist[0 .. n_e)
// (the band's binned edges), or 0 .. n_e - 1 when elist is null.
struct NoG {
    __device__ float operator()(int, int) const { return 0.0f; }
    __device__ void prefetch(int, int) const {}
};
template <bool BWD, class GV = NoG>
__device__ void band_edges(ASmem& sm, float* band, int W, int b0, int nb, int V, const float2* vpos,
                           const int* vsub, float2* vgrad, const int* elist, int n_e, GV gv = GV()) {
    const int tid = threadIdx.x;
    const int b1 = b0 + nb - 1;
    auto edge_at = [&](int i) { return elist ? elist[i] : i; };
    for (int e0 = 0; e0 < n_e; e0 += ECHUNK) {
        int cnt[EPT], sum = 0;
#pragma unroll
        for (int q = 0; q < EPT; q++) {
            const int i = e0 + tid * EPT + q;
            int r0;
            cnt[q] = i < n_e ? edge_rows(make_edge(vpos, vsub, V, edge_at(i)), b0, b1, &r0) : 0;
            sum += cnt[q];
        }
        int total;
        int pre = block_excl_sum(sum, sm.wsum, total);
#pragma unroll
        for (int q = 0; q < EPT; q++) {
            sm.off[tid * EPT + q] = pre;
            pre += cnt[q];
        }
        if (tid == 0) sm.off[ECHUNK] = total;
        __syncthreads();
        const int per = (total + ABLOCK - 1) / ABLOCK;
        const int beg = tid * per, end = min(total, beg + per);
        if (beg < end) {
            // last edge slot whose range starts at or before `beg`
            int lo = 0, hi = ECHUNK - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (sm.off[mid] <= beg)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            int slot = lo;
            EdgeG E = make_edge(vpos, vsub, V, edge_at(e0 + slot));
            int r0 = 0;
            edge_rows(E, b0, b1, &r0);
            float ga = 0.0f, gb = 0.0f;
            for (int it = beg; it < end; it++) {
                if (sm.off[slot + 1] <= it) {
                    if (BWD) {
                        atomicAdd(&vgrad[E.e].x, __fmul_rn(E.perp.x, ga));
                        atomicAdd(&vgrad[E.e].y, __fmul_rn(E.perp.y, ga));
                        atomicAdd(&vgrad[E.nxt].x, __fmul_rn(E.perp.x, gb));
                        atomicAdd(&vgrad[E.nxt].y, __fmul_rn(E.perp.y, gb));
                        ga = gb = 0.0f;
                    }
                    do {
                        slot++;
                    } while (sm.off[slot + 1] <= it);
                    E = make_edge(vpos, vsub, V, edge_at(e0 + slot));
                    edge_rows(E, b0, b1, &r0);
                }
                const int r = r0 + (it - sm.off[slot]);
                if (!BWD) {
                    float* row = band + (size_t)(r - b0) * W;
                    row_cells(E, r, W, [&](int c, float h, float xm) {
                        const float dh = __fmul_rn(E.dir, h);
                        if (c < 0) {
                            atomicAdd(row, dh);
                        } else {
                            atomicAdd(row + c, __fmul_rn(dh, __fsub_rn((float)(c + 1), xm)));
                            if (c + 1 < W) atomicAdd(row + c + 1, __fmul_rn(dh, __fsub_rn(xm, (float)c)));
                        }
                    });
                } else {
                    // the next item is usually this edge one row down: ask L1 for its cells now
                    if (r + 1 <= b1 && (float)(r + 1) < E.b.y) {
                        const float y0 = (float)(r + 1), y1 = fminf(E.b.y, (float)(r + 2));
                        const float xa = fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(y0, E.a.y), E.dxdy)), E.xlo), E.xhi);
                        const float xb = fminf(fmaxf(__fadd_rn(E.a.x, __fmul_rn(__fsub_rn(y1, E.a.y), E.dxdy)), E.xlo), E.xhi);
                        const float lo = fminf(xa, xb), hi = fmaxf(xa, xb);
                        if (hi >= 0.0f && lo < (float)W) {
                            const int c0 = max((int)floorf(lo), 0), c1 = min((int)floorf(hi), W - 1);
                            gv.prefetch(r + 1, c0);
                            if ((c1 >> 5) != (c0 >> 5)) gv.prefetch(r + 1, c1);
                        }
                    }
                    const bool down = E.dir > 0.0f;
                    row_pieces(E, r, W, [&](int c, float, float, float u0, float u1) {
                        if (c < 0) return;
                        const float g = gv(r, c);
                        const float i1 = __fsub_rn(u1, u0);
                        const float iu = __fmul_rn(__fmul_rn(0.5f, i1), __fadd_rn(u1, u0));
                        const float i0 = __fsub_rn(i1, iu);
                        ga = __fadd_rn(ga, __fmul_rn(g, down ? i0 : iu));
                        gb = __fadd_rn(gb, __fmul_rn(g, down ? iu : i0));
                    });
                }
            }
            if (BWD) {
                atomicAdd(&vgrad[E.e].x, __fmul_rn(E.perp.x, ga));
                atomicAdd(&vgrad[E.e].y, __fmul_rn(E.perp.y, ga));
                atomicAdd(&vgrad[E.nxt].x, __fmul_rn(E.perp.x, gb));
                atomicAdd(&vgrad[E.nxt].y, __fmul_rn(E.perp.y, gb));
            }
        }
        __syncthreads();
    }
}

// Bin the path's edges by row band (band k = rows [k * rpb, (k + 1) * rpb)) into the
// CSR list boff / blist: a count pass into the shared histogram `hist` (the band buffer,
// free before the band loop), a block scan, a fill pass.  The order of a band's edges is
// that of the atomics; every edge is visited once per band it reaches, as in the scan of
// all edges.  Returns false, uniformly, when the pairs exceed PAIR_CAP.
__device__ bool bin_edges(ASmem& sm, int* hist, int* boff, int* blist, int V, int H, int rpb, int nbands,
                          const float2* vpos, const int* vsub) {
    const int tid = threadIdx.x;
    for (int i = tid; i <= nbands; i += ABLOCK) hist[i] = 0;
    __syncthreads();
    for (int e = tid; e < V; e += ABLOCK) {
        int r0 = 0;
        const int n = edge_rows(make_edge(vpos, vsub, V, e), 0, H - 1, &r0);
        if (n > 0)
            for (int b = r0 / rpb, b1 = (r0 + n - 1) / rpb; b <= b1; b++) atomicAdd(&hist[b], 1);
    }
    __syncthreads();
    const int per = (nbands + ABLOCK - 1) / ABLOCK;
    const int lo = min(nbands, tid * per), hi = min(nbands, lo + per);
    int cnt = 0;
    for (int i = lo; i < hi; i++) cnt += hist[i];
    int total;
    int pre = block_excl_sum(cnt, sm.wsum, total);
    if (total > PAIR_CAP) return false;
    for (int i = lo; i < hi; i++) {
        const int c = hist[i];
        boff[i] = pre;
        hist[i] = pre;
        pre += c;
    }
    if (tid == 0) boff[nbands] = total;
    __syncthreads();
    for (int e = tid; e < V; e += ABLOCK) {
        int r0 = 0;
        const int n = edge_rows(make_edge(vpos, vsub, V, e), 0, H - 1, &r0);
        if (n > 0)
            for (int b = r0 / rpb, b1 = (r0 + n - 1) / rpb; b <= b1; b++) blist[atomicAdd(&hist[b], 1)] = e;
    }
    __syncthreads();
    return true;
}

// ------------------------------------------------------------------- strokes
// Plotter::stroke (plotter.rs:356-365): stroke points with widths from the pen walk
// (stroker.rs:204-236), the outline of every sub-stroke (stroker.rs:239-416) as
// footile emits it, then the fill of the outline transformed a second time.  Every
// outline point is recorded as a node over the stroke points: an offset point, a miter
// intersection or an arc point.  The backward
// reverses the nodes with their Jacobians (decisions held) and chains stroke points to
// the op floats (Bernstein weights of the transformed curve) and widths to the
// PenWidth ops (linear in t between the pen's width and the op's).

struct SPt {
    float x, y, w, t;
    int op, form, pen, w0, w1, pad;  // provenance; w0 / w1: PenWidth op of the start / end width (-1: the call's)
};
struct SNd {
    int kind, a, b, c, d;  // OFF: stroke points a -> b, c = 0 offsets a, 1 offsets b; MITER: nodes a0 a1 b0 b1;
                           // ARC: stroke point a (centre, width), nodes b (from) and c (to)
    float x, y;
    int pad;
};
struct SSub {
    int start, n, joined, done;
};
static_assert(sizeof(SPt) == SPT_BYTES && sizeof(SNd) == SND_BYTES && sizeof(SSub) == SSUB_BYTES, "layout");
enum { N_OFF = 0, N_MITER = 1, N_ARC = 2 };
enum { F_POINT = 0, F_QUAD = 1, F_CUBIC = 2 };

// The De Casteljau walk carrying widths (geom.rs:31-35): leaf(index, point, width, t).
template <bool CUBIC, class Leaf>
__device__ int curve_walk_w(P2 a, P2 b, P2 c, P2 d, float wa, float wb, float wc, float wd, float tol_sq,
                            int* depth_hit, Leaf leaf) {
    using Fr = WalkFr<CUBIC, true>;
    Fr st[FT_MAX_DEPTH + 1];
    int sp = 0, n = 0, dep = 0;
    float t = 0.0f;
    for (;;) {
        bool within;
        P2 l1, l2, m, r1, r2;
        float wl1, wl2, wm, wr1, wr2;
        if (CUBIC) {
            P2 ab = pmid(a, b), bc = pmid(b, c), cd = pmid(c, d);
            P2 abbc = pmid(ab, bc), bccd = pmid(bc, cd);
            m = pmid(abbc, bccd);
            float wab = ftk::fmid(wa, wb), wbc = ftk::fmid(wb, wc), wcd = ftk::fmid(wc, wd);
            float wabbc = ftk::fmid(wab, wbc), wbccd = ftk::fmid(wbc, wcd);
            wm = ftk::fmid(wabbc, wbccd);
            within = pdist_sq(m, pmid(a, d)) <= tol_sq;
            l1 = ab, l2 = abbc, r1 = bccd, r2 = cd;
            wl1 = wab, wl2 = wabbc, wr1 = wbccd, wr2 = wcd;
        } else {
            P2 ab = pmid(a, b), bc = pmid(b, c);
            m = pmid(ab, bc);
            float wab = ftk::fmid(wa, wb), wbc = ftk::fmid(wb, wc);
            wm = ftk::fmid(wab, wbc);
            within = pdist_sq(m, pmid(a, c)) <= tol_sq;
            l1 = ab, l2 = m, r1 = bc, r2 = c;
            wl1 = wab, wl2 = wm, wr1 = wbc, wr2 = wc;
        }
        if (within || dep >= FT_MAX_DEPTH) {
            if (!within) *depth_hit = 1;
            t = __fadd_rn(t, pow2neg(dep));
            if (CUBIC)
                leaf(n, d, wd, t);
            else
                leaf(n, c, wc, t);
            n++;
            if (sp == 0) break;
            --sp;
            a = CUBIC ? d : c, wa = CUBIC ? wd : wc;
            b = st[sp].b, c = st[sp].c, wb = st[sp].wb, wc = st[sp].wc;
            if constexpr (CUBIC) d = st[sp].d, wd = st[sp].wd;
            dep = st[sp].dep;
        } else {
            if constexpr (CUBIC) {
                st[sp] = Fr{r1, r2, d, wr1, wr2, wd, dep + 1};
                b = l1, c = l2, d = m;
                wb = wl1, wc = wl2, wd = wm;
            } else {
                st[sp] = Fr{r1, r2, wr1, wr2, dep + 1};
                b = l1, c = l2;
                wb = wl1, wc = wl2;
            }
            sp++;
            dep++;
        }
    }
    return n;
}

struct StrokeScr {
    SPt* sp;
    SSub* subs;
    SNd* nd;
    float2* ng;
    float4* spg;
    int* vnode;
    int* soff;  // per sub-stroke: first outline segment (both sides)
    int2* gst;  // per sub-stroke: first outline vertex of the forward / reverse side
};

__device__ __forceinline__ StrokeScr stroke_scr(unsigned char* scr) {
    StrokeScr S;
    S.sp = reinterpret_cast<SPt*>(scr + AS_SPT);
    S.subs = reinterpret_cast<SSub*>(scr + AS_SSUB);
    S.nd = reinterpret_cast<SNd*>(scr + AS_SND);
    S.ng = reinterpret_cast<float2*>(scr + AS_NG);
    S.spg = reinterpret_cast<float4*>(scr + AS_SPG);
    S.vnode = reinterpret_cast<int*>(scr + AS_VNODE);
    S.soff = reinterpret_cast<int*>(scr + AS_SOFF);
    S.gst = reinterpret_cast<int2*>(scr + AS_GST);
    return S;
}

// The stroke points and sub-strokes of the path (Plotter's pen walk into
// Stroke::add_point / close, plotter.rs:175-332, stroker.rs:204-236) with the whole
// block, the same as a walk of the ops one by one.  Ops go in chunks of ABLOCK: max scans give every op the PenWidth in effect and the pen before it (the last
// Close/Move/Line/Quad/Cubic before it, its end point and width), each op's points (curve
// leaves) are placed by a block scan into a raw window (the node area, unused until the
// outline), and the window is compacted in order.  The one-thread walk's rules, per raw
// point k after the first: a close event (a Close, or the Move's own close before its
// point) between the ops of points k - 1 and k ends the sub-stroke and keeps point k,
// the last such event giving the ended sub-stroke's `joined`; else k is dropped when it
// repeats point k - 1's position (the last kept point then has that position too).  The
// first VCAP kept points are stored; close events after the last stored point mark the
// last sub-stroke.  Returns the stored point count; *n_sub gets the sub-stroke count.
// Every thread must call.
constexpr int SP_RAW = 65536;  // raw points per window
static_assert((size_t)SP_RAW * SPT_BYTES <= (size_t)NODE_CAP * SND_BYTES, "raw window fits the node area");
__device__ int stroke_points_block(const AParams& p, ASmem& sm, const ft_op* ops, int n, float sw0,
                                   const StrokeScr& S, int* n_sub) {
    const int tid = threadIdx.x;
    const float* m = p.xf;
    SPCarry& C = sm.spc;
    SPt* raw = reinterpret_cast<SPt*>(S.nd);
    int* lpw_of = sm.off;  // per op of the chunk: the last PenWidth op before it
    if (tid == 0) {
        C.pw = C.pc = C.pc_pw = C.ce = -1;
        C.kept = C.nsub = C.have_prev = 0;
        C.px = C.py = 0.0f;
        C.pop = C.last_op = -1;
        S.subs[0].start = 0;
    }
    __syncthreads();
    auto sw_at = [&](int pw) { return pw >= 0 ? ops[pw].v[0] : sw0; };
    for (int c0 = 0; c0 < n; c0 += ABLOCK) {
        const int i = c0 + tid;
        ft_op o;
        o.kind = -1;
        if (i < n) o = load_op(ops, i);
        const int kind = o.kind;
        const bool pc = kind >= FT_OP_CLOSE && kind <= FT_OP_CUBIC;
        int inc, exc;
        block_max_scan(kind == FT_OP_PEN_WIDTH ? i : -1, sm.wmax, inc, exc);
        const int lpw = max(exc, C.pw);
        const int pw_last = max(inc, C.pw);
        lpw_of[tid] = lpw;
        int pc_inc, pc_exc;
        block_max_scan(pc ? i : -1, sm.wmax2, pc_inc, pc_exc);
        int ce_inc, ce_exc;
        block_max_scan(kind == FT_OP_CLOSE || kind == FT_OP_MOVE ? 2 * i + (kind == FT_OP_CLOSE) : -1, sm.wmax3,
                       ce_inc, ce_exc);
        const int ce = max(ce_inc, C.ce);  // close events up to and with this op
        // the pen before this op (plotter.rs:175-224; Close resets it to the origin)
        const int j = max(pc_exc, C.pc);
        const int j_pw = j < 0 ? -1 : (j >= c0 ? lpw_of[j - c0] : C.pc_pw);
        int pen = -1, pen_wsrc = -1;
        P2 penp = p2(0.0f, 0.0f);
        float penw = sw0;
        if (j >= 0) {
            const ft_op q = load_op(ops, j);
            pen_wsrc = j_pw;
            penw = sw_at(j_pw);
            if (q.kind != FT_OP_CLOSE) {
                pen = j;
                penp = op_pt(q, end_slot(q.kind));
            }
        }
        const float sw = sw_at(lpw);
        const int cur_pw = lpw;
        // this op's points
        const bool cubic = kind == FT_OP_CUBIC;
        P2 A = p2(0.0f, 0.0f), B = A, Cc = A, D = A;
        float wb = 0.0f, wc = 0.0f, wd = 0.0f;
        bool curve = false;
        int cnt = 0;
        if (kind == FT_OP_MOVE || kind == FT_OP_LINE) {
            cnt = 1;
        } else if (kind == FT_OP_QUAD || cubic) {
            A = xform(m, penp);
            B = xform(m, op_pt(o, 0));
            Cc = xform(m, op_pt(o, 1));
            D = cubic ? xform(m, op_pt(o, 2)) : Cc;
            if (cubic) {  // float_lerp (geom.rs:14-16)
                wb = __fadd_rn(sw, __fmul_rn(__fsub_rn(penw, sw), 1.0f / 3.0f));
                wc = __fadd_rn(sw, __fmul_rn(__fsub_rn(penw, sw), 2.0f / 3.0f));
                wd = sw;
            } else {
                wb = ftk::fmid(penw, sw);
                wc = sw;
                wd = sw;
            }
            cnt = 1;
            if (!pfinite(A) || !pfinite(B) || !pfinite(Cc) || !pfinite(D)) {
                atomicMax(&sm.status, (int)FT_ERR_ARG);
            } else {
                curve = true;
                int dh = 0;
                auto none = [](int, P2, float, float) {};
                cnt = cubic ? curve_walk_w<true>(A, B, Cc, D, penw, wb, wc, wd, p.tol_sq, &dh, none)
                            : curve_walk_w<false>(A, B, Cc, D, penw, wb, wc, wd, p.tol_sq, &dh, none);
                if (dh) atomicMax(&sm.status, (int)FT_ERR_DEPTH);
            }
        }
        int total;
        const int base = block_excl_sum(cnt, sm.wsum, total);
        for (int w0 = 0; w0 < total; w0 += SP_RAW) {
            const int w1 = min(w0 + SP_RAW, total);
            // ---- this window's raw points; `pad` holds the op's close events
            if (cnt > 0 && base < w1 && base + cnt > w0) {
                auto put = [&](int k, P2 q, float w, float t, int form, int pn, int ws0) {
                    const int r = base + k;
                    if (r >= w0 && r < w1) raw[r - w0] = SPt{q.x, q.y, w, t, i, form, pn, ws0, cur_pw, ce};
                };
                if (!curve) {
                    put(0, kind == FT_OP_MOVE || kind == FT_OP_LINE ? xform(m, op_pt(o, 0)) : D, sw, 1.0f, F_POINT,
                        -1, cur_pw);
                } else {
                    int dh = 0;
                    auto leaf = [&](int k, P2 q, float w, float t) {
                        put(k, q, w, t, cubic ? F_CUBIC : F_QUAD, pen, pen_wsrc);
                    };
                    if (cubic)
                        curve_walk_w<true>(A, B, Cc, D, penw, wb, wc, wd, p.tol_sq, &dh, leaf);
                    else
                        curve_walk_w<false>(A, B, Cc, D, penw, wb, wc, wd, p.tol_sq, &dh, leaf);
                }
            }
            __syncthreads();
            // ---- compact the window in order
            for (int r0 = 0; r0 < w1 - w0; r0 += ABLOCK) {
                const int r = r0 + tid;
                const bool valid = r < w1 - w0;
                SPt q{};
                bool have_prev = false, close_between = false, keep = false;
                if (valid) {
                    q = raw[r];
                    float px = C.px, py = C.py;
                    int pop = C.pop;
                    have_prev = C.have_prev != 0;
                    if (r > 0) {
                        const SPt pv = raw[r - 1];
                        px = pv.x;
                        py = pv.y;
                        pop = pv.op;
                        have_prev = true;
                    }
                    close_between = have_prev && (q.pad >> 1) > pop;
                    keep = !have_prev || close_between || !(q.x == px && q.y == py);
                }
                int ktot;
                const int K = C.kept + block_excl_sum(keep ? 1 : 0, sm.wsum, ktot);
                const bool stored = keep && K < VCAP;
                const bool starts = stored && close_between;
                int stot;
                const int J = C.nsub + 1 + block_excl_sum(starts ? 1 : 0, sm.wsum, stot);
                if (stored) {
                    const int joined = q.pad & 1;
                    q.pad = 0;
                    S.sp[K] = q;
                    if (starts) {
                        S.subs[J].start = K;
                        S.subs[J - 1].joined = joined;
                        S.subs[J - 1].done = 1;
                    }
                    atomicMax(&C.last_op, q.op);  // stored points come in op order
                }
                __syncthreads();
                if (valid && (r == w1 - w0 - 1 || tid == ABLOCK - 1)) {
                    C.have_prev = 1;
                    C.px = q.x;
                    C.py = q.y;
                    C.pop = q.op;
                }
                if (tid == 0) {
                    C.kept += ktot;
                    C.nsub += stot;
                }
                __syncthreads();
            }
        }
        if (tid == ABLOCK - 1) {
            C.pw = pw_last;
            const int pc_last = max(pc_inc, C.pc);
            if (pc_last >= c0) C.pc_pw = lpw_of[pc_last - c0];
            C.pc = pc_last;
            C.ce = ce;
        }
        __syncthreads();
    }
    const int ns = min(C.kept, VCAP), nsub = C.nsub + 1;
    for (int jj = tid; jj < nsub; jj += ABLOCK) {
        const int st = ns > 0 ? S.subs[jj].start : 0;
        S.subs[jj].n = (jj + 1 < nsub ? S.subs[jj + 1].start : ns) - st;
        if (jj == nsub - 1) {
            // close events after the last stored point end the last sub-stroke
            const bool closed = ns > 0 && (C.ce >> 1) > C.last_op;
            S.subs[jj].start = st;
            S.subs[jj].joined = closed ? (C.ce & 1) : 0;
            S.subs[jj].done = closed ? 1 : 0;
        }
    }
    __syncthreads();
    *n_sub = nsub;
    return ns;
}

// All threads: the outline of every sub-stroke (stroker.rs:239-416) and the polygon
// Plotter::stroke fills (the outline's Line points transformed again, sub-figures
// between its Closes).  Segments (sub-stroke, side, k) are independent: their offset
// points are nodes 2s and 2s + 1; the join at segment k (k >= 1) needs only segments
// k - 1 and k.  A pass counts each segment's vertices and extra nodes (a miter
// intersection, or the arc points of a round join), block scans place them, and each
// segment emits its vertices in footile's order: the open side's first offset point,
// the join, the open side's last offset point.  Arc points are numbered in the
// recursion's creation order within their segment, so a node's inputs are older nodes.
// Returns the vertex count (beyond VCAP nothing is written) and the node count.
__device__ void outline_block(const AParams& p, const StrokeScr& S, int nsub, ASmem& sm, float2* vpos, int* vsub,
                              int* out_v, int* out_n) {
    const int tid = threadIdx.x;
    const float* m = p.xf;
    const float tol_sq = p.tol_sq;
    if (tid == 0) {
        int t = 0;
        for (int si = 0; si < nsub; si++) {
            const SSub sb = S.subs[si];
            const int len = (sb.joined ? sb.n + 1 : (sb.n > 0 ? sb.n - 1 : 0)) & 0xFFFF;  // SubStroke::len (u16)
            S.soff[si] = t;
            t += 2 * len;
        }
        S.soff[nsub] = t;
        sm.total = t;
    }
    __syncthreads();
    const int T = sm.total;
    if (2LL * T > NODE_CAP) {
        if (tid == 0) atomicMax(&sm.status, (int)FT_ERR_CAP);
        *out_v = VCAP + 1;
        *out_n = 0;
        return;
    }
    struct Seg {
        int si, k, len, v0, v1;
        bool fwd, joined;
    };
    auto seg = [&](int s) {
        int lo = 0, hi = nsub - 1;  // the sub-stroke owning segment s
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.soff[mid] <= s)
                lo = mid;
            else
                hi = mid - 1;
        }
        const SSub sb = S.subs[lo];
        Seg g;
        g.si = lo;
        g.joined = sb.joined != 0;
        g.len = (S.soff[lo + 1] - S.soff[lo]) >> 1;
        const int u = s - S.soff[lo];
        g.fwd = u < g.len;
        g.k = g.fwd ? u : u - g.len;
        const int n = sb.n;
        if (g.fwd) {
            g.v0 = sb.start + g.k % n;
            g.v1 = sb.start + (g.k + 1) % n;
        } else {  // from the last point backwards (stroker.rs:244-246)
            g.v0 = sb.start + ((n - 1 - g.k) % n + n) % n;
            g.v1 = sb.start + ((n - 2 - g.k) % n + n) % n;
        }
        return g;
    };
    auto P = [&](int k) { return p2(S.sp[k].x, S.sp[k].y); };
    auto N = [&](int i) { return p2(S.nd[i].x, S.nd[i].y); };
    // offset points
    for (int s = tid; s < T; s += ABLOCK) {
        const Seg g = seg(s);
        const P2 vr = ftk::pnormalize(ftk::pright(ftk::psub(P(g.v1), P(g.v0))));
        const P2 a = ftk::padd(P(g.v0), ftk::pscale(vr, __fmul_rn(S.sp[g.v0].w, 0.5f)));
        const P2 b = ftk::padd(P(g.v1), ftk::pscale(vr, __fmul_rn(S.sp[g.v1].w, 0.5f)));
        S.nd[2 * s] = SNd{N_OFF, g.v0, g.v1, 0, 0, a.x, a.y, 0};
        S.nd[2 * s + 1] = SNd{N_OFF, g.v0, g.v1, 1, 0, b.x, b.y, 0};
    }
    __syncthreads();
    // arc recursion of a round join (stroker.rs:399-416); emit(node, value) per leaf,
    // node(c) creates an arc point
    struct Fr {
        int na, nb;
        P2 a, b;
        int dep;
    };
    auto arc_walk = [&](int k, int na0, int nb0, int* depth_hit, auto leaf, auto make) {
        Fr st[FT_MAX_DEPTH + 3];
        int sp = 0;
        st[sp++] = Fr{na0, nb0, N(na0), N(nb0), 0};
        const P2 pk = P(k);
        const float hw = __fmul_rn(S.sp[k].w, 0.5f);
        while (sp > 0) {
            const Fr f = st[--sp];
            const P2 vr = ftk::pnormalize(ftk::pright(ftk::psub(f.b, f.a)));
            const P2 c = ftk::padd(pk, ftk::pscale(vr, hw));
            if (!pfinite(c) || pdist_sq(c, pmid(f.a, f.b)) <= tol_sq) {
                leaf(f.nb, f.b);
            } else if (f.dep >= FT_MAX_DEPTH) {
                *depth_hit = 1;
                leaf(f.nb, f.b);
            } else {
                const int nc = make(k, f.na, f.nb, c);
                st[sp++] = Fr{nc, f.nb, c, f.b, f.dep + 1};  // right half after the left
                st[sp++] = Fr{f.na, nc, f.a, c, f.dep + 1};
            }
        }
    };
    enum { J_NONE = 0, J_MITER = 1, J_BEVEL = 2, J_ARC = 3 };
    int carry_v = 0, carry_n = 2 * T;
    for (int c0 = 0; c0 < T; c0 += ABLOCK) {
        const int s = c0 + tid;
        const bool valid = s < T;
        Seg g{};
        int jt = J_NONE, cnt_v = 0, cnt_n = 0, dh = 0;
        P2 xp = p2(0.0f, 0.0f);
        if (valid) {
            g = seg(s);
            if (g.k == 0 && !g.joined) cnt_v++;
            if (g.k >= 1) {
                const P2 A0 = N(2 * s - 2), A1 = N(2 * s - 1), B0 = N(2 * s), B1 = N(2 * s + 1);
                if (p.join == FT_JOIN_MITER) {
                    jt = J_BEVEL;
                    const ftk::P2 u = ftk::psub(A1, A0), v = ftk::psub(B0, B1);
                    if (ft_miter_join(u.x, u.y, v.x, v.y, p.miter_g) && ftk::pline_x(A0, A1, B0, B1, &xp))
                        jt = J_MITER;
                } else if (p.join == FT_JOIN_BEVEL) {
                    jt = J_BEVEL;
                } else {
                    const ftk::P2 u = ftk::psub(A1, A0), v = ftk::psub(B0, B1);
                    jt = ft_round_join_arc(u.x, u.y, v.x, v.y) ? J_ARC : J_BEVEL;
                }
                if (jt == J_MITER) {
                    cnt_v += 1;
                    cnt_n += 1;
                } else if (jt == J_BEVEL) {
                    cnt_v += 2;
                } else {
                    int leaves = 0, inner = 0;
                    arc_walk(g.v0, 2 * s - 1, 2 * s, &dh, [&](int, P2) { leaves++; },
                             [&](int, int, int, P2) { return -1 - (inner++); });
                    cnt_v += 1 + leaves;
                    cnt_n += inner;
                }
            }
            if (g.k == g.len - 1 && !g.joined) cnt_v++;
            if (dh) atomicMax(&sm.status, (int)FT_ERR_DEPTH);
        }
        int tot_v, tot_n;
        const int ov = carry_v + block_excl_sum(cnt_v, sm.wsum, tot_v);
        const int on = carry_n + block_excl_sum(cnt_n, sm.wsum, tot_n);
        if (valid && g.k == 0) {
            if (g.fwd)
                S.gst[g.si].x = ov;
            else
                S.gst[g.si].y = ov;
        }
        __syncthreads();
        if (valid) {
            const int sub_start = (g.fwd || !g.joined) ? S.gst[g.si].x : S.gst[g.si].y;
            int w = ov, nid = on;
            auto put = [&](int nd, P2 v) {
                if (w < VCAP) {
                    const P2 q = xform(m, v);
                    vpos[w] = make_float2(fx_range(q.x), fx_range(q.y));
                    vsub[w] = sub_start;
                    S.vnode[w] = nd;
                }
                w++;
            };
            auto make = [&](int kind, int a, int b, int c, int d, P2 v) {
                if (nid < NODE_CAP) S.nd[nid] = SNd{kind, a, b, c, d, v.x, v.y, 0};
                return nid++;
            };
            if (g.k == 0 && !g.joined) put(2 * s, N(2 * s));
            if (jt == J_MITER) {
                put(make(N_MITER, 2 * s - 2, 2 * s - 1, 2 * s, 2 * s + 1, xp), xp);
            } else if (jt == J_BEVEL) {
                put(2 * s - 1, N(2 * s - 1));
                put(2 * s, N(2 * s));
            } else if (jt == J_ARC) {
                put(2 * s - 1, N(2 * s - 1));
                int d2 = 0;
                arc_walk(g.v0, 2 * s - 1, 2 * s, &d2, [&](int nb, P2 b) { put(nb, b); },
                         [&](int k, int na, int nb, P2 c) { return make(N_ARC, k, na, nb, 0, c); });
            }
            if (g.k == g.len - 1 && !g.joined) put(2 * s + 1, N(2 * s + 1));
        }
        carry_v += tot_v;
        carry_n += tot_n;
        __syncthreads();
    }
    if (tid == 0 && (carry_v > VCAP || carry_n > NODE_CAP)) atomicMax(&sm.status, (int)FT_ERR_CAP);
    *out_v = carry_v;
    *out_n = min(carry_n, NODE_CAP);
}

// Backward of a stroke, all threads: outline vertex gradients (vgrad, fill space) ->
// nodes -> stroke points -> op floats and widths.  Offset nodes are [0, n_off), the
// others after them; a node's inputs are always older nodes: arcs (reverse creation
// order, one thread: an arc may feed another), then miter intersections and offset
// points in parallel, then stroke points.
__device__ void stroke_backward_block(const AParams& p, const ft_op* ops, float* gops, float* gwidth, int V, int nn,
                                      int ns, int n_off, const StrokeScr& S, const float2* vgrad) {
    const int tid = threadIdx.x;
    const float* m = p.xf;
    for (int i = tid; i < nn; i += ABLOCK) S.ng[i] = make_float2(0.0f, 0.0f);
    for (int k = tid; k < ns; k += ABLOCK) S.spg[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    __syncthreads();
    for (int j = tid; j < V; j += ABLOCK) {
        const int nd = S.vnode[j];
        const float2 g = fx_pass(xform(m, p2(S.nd[nd].x, S.nd[nd].y)), __ldcg(&vgrad[j]));
        atomicAdd(&S.ng[nd].x, m[0] * g.x + m[3] * g.y);
        atomicAdd(&S.ng[nd].y, m[1] * g.x + m[4] * g.y);
    }
    __syncthreads();
    // offset of stroke point ks along normalize(right(to - from)) * w / 2: gradients of
    // ks's position and width and of the direction's two ends
    auto offset_back = [&](float2 g, float fx, float fy, float tx, float ty, int ks, float2* gfrom, float2* gto) {
        const float ux = ty - fy, uy = -(tx - fx);
        const float len = sqrtf(ux * ux + uy * uy);
        const float vx = ux / len, vy = uy / len;
        const float w = S.sp[ks].w;
        atomicAdd(&S.spg[ks].x, g.x);
        atomicAdd(&S.spg[ks].y, g.y);
        atomicAdd(&S.spg[ks].z, 0.5f * (vx * g.x + vy * g.y));
        const float gvx = g.x * w * 0.5f, gvy = g.y * w * 0.5f;
        const float dv = vx * gvx + vy * gvy;
        const float gux = (gvx - vx * dv) / len, guy = (gvy - vy * dv) / len;
        *gto = make_float2(-guy, gux);  // u = (d.y, -d.x), d = to - from
        *gfrom = make_float2(guy, -gux);
    };
    // arc points exist only with round joins, after the offset nodes [0, n_off)
    if (tid == 0 && p.join == FT_JOIN_ROUND) {
        for (int i = nn - 1; i >= n_off; i--) {
            const SNd nd = S.nd[i];
            if (nd.kind != N_ARC) continue;
            const float2 g = __ldcg(&S.ng[i]);
            if (g.x == 0.0f && g.y == 0.0f) continue;
            float2 gf, gt;
            offset_back(g, S.nd[nd.b].x, S.nd[nd.b].y, S.nd[nd.c].x, S.nd[nd.c].y, nd.a, &gf, &gt);
            atomicAdd(&S.ng[nd.b].x, gf.x);
            atomicAdd(&S.ng[nd.b].y, gf.y);
            atomicAdd(&S.ng[nd.c].x, gt.x);
            atomicAdd(&S.ng[nd.c].y, gt.y);
        }
    }
    __syncthreads();
    // Miter intersections.  Their four offset points are recomputed from the stroke
    // points in double: between very short segments the float offsets' rounding is a
    // large part of the offset lines' directions, and the intersection's Jacobian
    // amplifies it.
    auto off64 = [&](int id, double& x, double& y) {
        const SNd o = S.nd[id];  // an offset node: stroke points a -> b
        const double fx = S.sp[o.a].x, fy = S.sp[o.a].y, tx = S.sp[o.b].x, ty = S.sp[o.b].y;
        const double ux = ty - fy, uy = -(tx - fx), len = sqrt(ux * ux + uy * uy);
        const int ks = o.c ? o.b : o.a;
        const double hw = 0.5 * (double)S.sp[ks].w;
        x = (double)S.sp[ks].x + ux / len * hw;
        y = (double)S.sp[ks].y + uy / len * hw;
    };
    for (int i = n_off + tid; i < nn; i += ABLOCK) {
        const SNd nd = S.nd[i];
        if (nd.kind != N_MITER) continue;
        const float2 gf = __ldcg(&S.ng[i]);
        if (gf.x == 0.0f && gf.y == 0.0f) continue;
        // intersection of lines a0-a1 and b0-b1 in coordinates relative to a1:
        // x = a1 + (B / D) * (a1 - a0), u = a0 - a1, v3 = b0 - a1, v4 = b1 - a1,
        // D = u x (v3 - v4), B = v3 x v4
        double a0x, a0y, ax, ay, b0x, b0y, b1x, b1y;
        off64(nd.a, a0x, a0y);
        off64(nd.b, ax, ay);
        off64(nd.c, b0x, b0y);
        off64(nd.d, b1x, b1y);
        const double gx = gf.x, gy = gf.y;
        const double ux = a0x - ax, uy = a0y - ay;
        const double v3x = b0x - ax, v3y = b0y - ay;
        const double v4x = b1x - ax, v4y = b1y - ay;
        const double den = ux * (v3y - v4y) - uy * (v3x - v4x);
        const double bb = v3x * v4y - v3y * v4x;
        const double q = bb / den;
        double gux = -q * gx, guy = -q * gy;
        const double gq = -(ux * gx + uy * gy);
        const double gb = gq / den, gden = -gq * q / den;
        double g3x = gb * v4y, g3y = -gb * v4x, g4x = -gb * v3y, g4y = gb * v3x;
        gux += gden * (v3y - v4y);
        guy -= gden * (v3x - v4x);
        g3y += gden * ux;
        g4y -= gden * ux;
        g3x -= gden * uy;
        g4x += gden * uy;
        atomicAdd(&S.ng[nd.a].x, (float)gux);
        atomicAdd(&S.ng[nd.a].y, (float)guy);
        atomicAdd(&S.ng[nd.c].x, (float)g3x);
        atomicAdd(&S.ng[nd.c].y, (float)g3y);
        atomicAdd(&S.ng[nd.d].x, (float)g4x);
        atomicAdd(&S.ng[nd.d].y, (float)g4y);
        atomicAdd(&S.ng[nd.b].x, (float)(gx - gux - g3x - g4x));
        atomicAdd(&S.ng[nd.b].y, (float)(gy - guy - g3y - g4y));
    }
    __syncthreads();
    for (int i = tid; i < min(nn, n_off); i += ABLOCK) {
        const SNd nd = S.nd[i];
        if (nd.kind != N_OFF) continue;
        const float2 g = __ldcg(&S.ng[i]);
        if (g.x == 0.0f && g.y == 0.0f) continue;
        float2 gf, gt;
        offset_back(g, S.sp[nd.a].x, S.sp[nd.a].y, S.sp[nd.b].x, S.sp[nd.b].y, nd.c ? nd.b : nd.a, &gf, &gt);
        atomicAdd(&S.spg[nd.a].x, gf.x);
        atomicAdd(&S.spg[nd.a].y, gf.y);
        atomicAdd(&S.spg[nd.b].x, gt.x);
        atomicAdd(&S.spg[nd.b].y, gt.y);
    }
    __syncthreads();
    auto gw = [&](int src, float v) {
        if (src < 0)
            atomicAdd(gwidth, v);
        else
            atomicAdd(gops + (size_t)src * 6, v);
    };
    for (int k = tid; k < ns; k += ABLOCK) {
        const SPt q = S.sp[k];
        const float4 g = __ldcg(&S.spg[k]);
        const float gx = m[0] * g.x + m[3] * g.y, gy = m[1] * g.x + m[4] * g.y;
        const int kind = load_op(ops, q.op).kind;
        auto add = [&](int j, int slot, float wgt) {
            atomicAdd(gops + (size_t)j * 6 + 2 * slot, wgt * gx);
            atomicAdd(gops + (size_t)j * 6 + 2 * slot + 1, wgt * gy);
        };
        if (q.form == F_POINT) {
            add(q.op, end_slot(kind), 1.0f);
            gw(q.w1, g.z);
            continue;
        }
        const float t = q.t, u = 1.0f - t;
        if (q.form == F_QUAD) {
            if (q.pen >= 0) add(q.pen, end_slot(load_op(ops, q.pen).kind), u * u);
            add(q.op, 0, 2.0f * t * u);
            add(q.op, 1, t * t);
        } else {
            if (q.pen >= 0) add(q.pen, end_slot(load_op(ops, q.pen).kind), u * u * u);
            add(q.op, 0, 3.0f * t * u * u);
            add(q.op, 1, 3.0f * t * t * u);
            add(q.op, 2, t * t * t);
        }
        gw(q.w0, u * g.z);
        gw(q.w1, t * g.z);
    }
}

__device__ __forceinline__ float cov_of(int rule, float s) {
    if (rule == FT_NONZERO) return fminf(fmaxf(s, 0.0f), 1.0f);
    const float m = __fsub_rn(s, __fmul_rn(2.0f, floorf(__fmul_rn(s, 0.5f))));
    return m <= 1.0f ? m : __fsub_rn(2.0f, m);
}
__device__ __forceinline__ float cov_d(int rule, float s) {
    if (rule == FT_NONZERO) return s > 0.0f && s < 1.0f ? 1.0f : 0.0f;
    const float m = __fsub_rn(s, __fmul_rn(2.0f, floorf(__fmul_rn(s, 0.5f))));
    return m < 1.0f ? 1.0f : -1.0f;
}

// g = sign * dLoss/dcov * dcov/dS at (row, cell) of one path's planes; dcov/dS from the
// winding area, or (no_area, NonZero) from the coverage: 1 exactly where 0 < cov < 1.
struct GradAt {
    const char* g;
    const char* cv;
    const char* ar;
    size_t off;
    uint32_t stride;
    float sign;
    int rule;
    bool no_area;
    __device__ size_t at(int r, int c) const { return off + (size_t)r * stride + 4 * (size_t)c; }
    __device__ float operator()(int r, int c) const;
    __device__ void prefetch(int r, int c) const {
        const size_t o = at(r, c);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(g + o));
        asm volatile("prefetch.global.L1 [%0];" ::"l"((no_area ? cv : ar) + o));
    }
};

__device__ __forceinline__ float* px_at(float* base, const ft_path_desc& d, int r) {
    return reinterpret_cast<float*>(reinterpret_cast<char*>(base) + d.raster_offset + (size_t)r * d.stride);
}

__device__ __forceinline__ float GradAt::operator()(int r, int c) const {
    const size_t o = at(r, c);
    const float gg = *reinterpret_cast<const float*>(g + o);
    if (no_area) {
        const float v = *reinterpret_cast<const float*>(cv + o);
        return v > 0.0f && v < 1.0f ? __fmul_rn(sign, gg) : 0.0f;
    }
    return __fmul_rn(__fmul_rn(sign, gg), cov_d(rule, *reinterpret_cast<const float*>(ar + o)));
}

template <bool BWD>
__global__ void __launch_bounds__(ABLOCK, 3) k_adjoint(AParams p) {
    extern __shared__ float band[];
    __shared__ ASmem sm;
    unsigned char* scr = p.scratch + (size_t)blockIdx.x * (p.stroke ? A_SCRATCH_STROKE : A_SCRATCH_PER_CTA);
    const StrokeScr S = stroke_scr(scr);
    __shared__ int s_counts[4];
    float2* vpos = reinterpret_cast<float2*>(scr + AS_POS);
    int* vsub = reinterpret_cast<int*>(scr + AS_SUB);
    float2* vgrad = reinterpret_cast<float2*>(scr + AS_GRAD);
    int* vflag = reinterpret_cast<int*>(scr + AS_FLAG);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (uint32_t path = blockIdx.x; path < p.n_paths; path += gridDim.x) {
        const ft_path_desc d = p.paths[path];
        const int W = (int)d.width, H = (int)d.height;
        const ft_op* ops = p.ops + d.op_begin;
        if (tid == 0) sm.status = FT_OK;
        __syncthreads();
        int V;
        if (p.stroke) {
            int nsub = 0;
            const int ns = stroke_points_block(p, sm, ops, (int)d.n_ops, d.s_width, S, &nsub);
            if (tid == 0) {
                s_counts[2] = ns;
                s_counts[0] = nsub;
            }
            __syncthreads();
            int nv = 0, nn = 0;
            outline_block(p, S, s_counts[0], sm, vpos, vsub, &nv, &nn);
            __syncthreads();
            if (tid == 0) {
                s_counts[0] = nv;
                s_counts[1] = nn;
                s_counts[3] = 2 * sm.total;  // offset nodes come first
            }
            __syncthreads();
            V = s_counts[0];
            if (BWD)
                for (int k = tid; k < min(V, VCAP); k += ABLOCK) vgrad[k] = make_float2(0.0f, 0.0f);
            __syncthreads();
        } else {
            V = path_walk<WALK_EMIT>(p, sm, ops, (int)d.n_ops, vpos, vsub, vgrad, BWD, nullptr);
        }
        const bool cap = V > VCAP || (p.stroke && sm.status == FT_ERR_CAP);
        if (cap && tid == 0) atomicMax(&sm.status, (int)FT_ERR_CAP);
        const float sign = cap ? 1.0f : fig_sign(sm, V, vpos, vsub, vflag);
        const int rows_per_band = W > 0 ? max(1, BAND_FLOATS / W) : 1;
        const int nbands = W > 0 ? (H + rows_per_band - 1) / rows_per_band : 0;
        int* boff = reinterpret_cast<int*>(scr + AS_BOFF);
        const int* blist = reinterpret_cast<const int*>(scr + AS_BLIST);
        if (BWD) {
            // every (edge, row) item of the path in one pass, g read at its own cell
            if (!cap && W > 0 && H > 0) {
                GradAt gv{reinterpret_cast<const char*>(p.grad_cov), reinterpret_cast<const char*>(p.cov),
                          reinterpret_cast<const char*>(p.area), d.raster_offset, d.stride, sign, p.rule,
                          p.no_area != 0};
                band_edges<true>(sm, nullptr, W, 0, H, V, vpos, vsub, vgrad, nullptr, V, gv);
            }
            __syncthreads();
        }
        bool binned = false;
        if (!BWD && !cap && nbands > 2 && nbands <= NB_CAP)
            binned = bin_edges(sm, reinterpret_cast<int*>(band), boff, reinterpret_cast<int*>(scr + AS_BLIST), V, H,
                               rows_per_band, nbands, vpos, vsub);
        __syncthreads();
        // forward: bands of rows accumulated in shared memory, resolved row by row
        for (int b0 = 0; b0 < H && W > 0 && !BWD; b0 += rows_per_band) {
            const int nb = min(rows_per_band, H - b0);
            const int nc = nb * W;
            int e_lo = 0, n_e = V;
            if (binned) {
                e_lo = boff[b0 / rows_per_band];
                n_e = boff[b0 / rows_per_band + 1] - e_lo;
            }
            if (binned && n_e == 0) {  // no edge reaches these rows: coverage and area 0
                for (int rr = warp; rr < nb; rr += NW) {
                    float* ar = px_at(p.area, d, b0 + rr);
                    float* cv = px_at(p.cov, d, b0 + rr);
                    for (int c = lane; c < W; c += 32) {
                        if (!p.no_area) ar[c] = 0.0f;
                        cv[c] = 0.0f;
                    }
                }
                continue;
            }
            for (int i = tid; i < nc; i += ABLOCK) band[i] = 0.0f;
            __syncthreads();
            if (!cap) band_edges<false>(sm, band, W, b0, nb, V, vpos, vsub, vgrad, binned ? blist + e_lo : nullptr, n_e);
            {
                __syncthreads();
                // row prefix sums, four 32-cell chunks scanned side by side; the float
                // additions are those of one chunk after the other
                for (int rr = warp; rr < nb; rr += NW) {
                    float* ar = px_at(p.area, d, b0 + rr);
                    float* cv = px_at(p.cov, d, b0 + rr);
                    const float* src = band + (size_t)rr * W;
                    float carry = 0.0f;
                    for (int c0 = 0; c0 < W; c0 += 128) {
                        float v[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const int c = c0 + 32 * u + lane;
                            v[u] = c < W ? src[c] : 0.0f;
                        }
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
                            for (int u = 0; u < 4; u++) {
                                const float t = __shfl_up_sync(FULL, v[u], o);
                                if (lane >= o) v[u] = __fadd_rn(v[u], t);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const int c = c0 + 32 * u + lane;
                            v[u] = __fadd_rn(v[u], carry);
                            carry = __shfl_sync(FULL, v[u], 31);
                            if (c < W) {
                                const float sv = __fmul_rn(sign, v[u]);
                                if (!p.no_area) ar[c] = sv;
                                cv[c] = cov_of(p.rule, sv);
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
        if (BWD && !cap) {
            if (p.stroke) {
                __syncthreads();
                stroke_backward_block(p, ops, p.grad_ops + (size_t)d.op_begin * 6, p.grad_width + path, V,
                                      s_counts[1], s_counts[2], s_counts[3], S, vgrad);
            } else {
                path_walk<WALK_GRAD>(p, sm, ops, (int)d.n_ops, vpos, vsub, vgrad, false,
                                     p.grad_ops + (size_t)d.op_begin * 6);
            }
        }
        if (tid == 0) p.status[path] = sm.status;
        __syncthreads();
    }
}

}  // namespace

// The backward reads g at each piece's own cell and needs no shared band.
int adjoint_blocks_per_sm(bool backward) {
    const int smem = BAND_FLOATS * (int)sizeof(float);
    int n = 0;
    if (backward) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adjoint<true>, ABLOCK, 0);
    } else {
        cudaFuncSetAttribute(k_adjoint<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adjoint<false>, ABLOCK, smem);
    }
    return n > 0 ? n : 1;
}

cudaError_t launch_adjoint(bool backward, const AParams& p, int grid, cudaStream_t s) {
    const int smem = BAND_FLOATS * (int)sizeof(float);
    if (backward) {
        k_adjoint<true><<<grid, ABLOCK, 0, s>>>(p);
    } else {
        cudaFuncSetAttribute(k_adjoint<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        k_adjoint<false><<<grid, ABLOCK, smem, s>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace fta
