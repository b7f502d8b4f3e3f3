// footile_oracle.cpp — TEST INFRASTRUCTURE ONLY (the test oracle).
//
// A sequential CPU restatement of footile's fill/stroke path.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it, as
// the oracle the CUDA path is compared against.  The shipped library never calls
// it, and nothing in it runs on the GPU.
//
// It follows the reference structure line by line (file:line of footile 0.7):
//   fixed.rs:24-158   Fixed 16.16 arithmetic, release-mode wrapping
//   vid.rs:9-70       Vid(u16) vertex ids and the 65,535-vertex cap
//   geom.rs:8-35      WidePt, float_lerp, midpoint
//   plotter.rs:96-365 Plotter state, add_ops/add_op, quad/cubic De Casteljau
//   stroker.rs:13-416 Stroke / SubStroke, stroke sides, offsets, joins, arcs
//   fig.rs:22-682     Fig, sub-figures, Edge cell-area math, Scanner sweep
//   imgbuf.rs:38-199  scalar NonZero / EvenOdd row resolve (the SSSE3 path computes
//                     the same values)
// The external crates are restated from their documented behaviour (not vendored
// in the reference): pointy 0.7 (Pt ops, Transform * Pt, Line::intersection) and
// pix 0.14 (Ch8 multiply / saturating add, SrcOver).  Those restatements are not
// pinned by any reference test except the full-coverage Rgba8p case (fig.rs:703).
//
// Two additions the reference lacks, identical in the CUDA path: recursion stops
// at FT_MAX_DEPTH levels (status FT_ERR_DEPTH), and a curve with a non-finite
// control point emits only its end point (status FT_ERR_ARG); footile would
// overflow its stack in both cases.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/footile_gpu.h"
#include "../include/ft_fmath.h"

namespace orc {

using i16 = int16_t;
using i32 = int32_t;
using i64 = int64_t;
using u16 = uint16_t;
using u32 = uint32_t;

// ---------------------------------------------------------------- Fixed (fixed.rs)
static const i32 FRACT_BITS = 16;
static const i32 FRACT_MASK = (1 << FRACT_BITS) - 1;
static const i32 FX_ONE = 1 << 16;
static const i32 FX_HALF = 1 << 15;
static const i32 FX_EPS = 1;

static inline i32 wadd(i32 a, i32 b) { return (i32)((u32)a + (u32)b); }
static inline i32 wsub(i32 a, i32 b) { return (i32)((u32)a - (u32)b); }
// fixed.rs:40-47  (a as i64 * b as i64) >> 16, as i32
static inline i32 fx_mul(i32 a, i32 b) { return (i32)(u32)(((i64)a * (i64)b) >> FRACT_BITS); }
// fixed.rs:49-56  ((a as i64) << 16) / b as i64, as i32
static inline i32 fx_div(i32 a, i32 b) { return (i32)(u32)(((i64)a * 65536) / (i64)b); }
static inline i32 fx_shl(i32 a, u32 s) { return (i32)((u32)a << s); }
static inline i32 fx_floor(i32 v) { return v & ~FRACT_MASK; }                 // fixed.rs:126-129
static inline i32 fx_ceil(i32 v) { return fx_floor(wsub(wadd(v, FX_ONE), FX_EPS)); }  // :131-134
static inline i32 fx_round(i32 v) { return fx_floor(wadd(v, FX_HALF)); }      // :136-139
static inline i32 fx_trunc(i32 v) { return v >= 0 ? fx_floor(v) : fx_ceil(v); }  // :141-148
static inline i32 fx_fract(i32 v) { return v & FRACT_MASK; }                  // :150-153
static inline i32 fx_avg(i32 a, i32 b) { return wadd(a, b) >> 1; }           // :155-158
static inline i32 fx_abs(i32 v) { return v == INT32_MIN ? INT32_MIN : (v < 0 ? -v : v); }  // :121-124 (wraps)
static inline i32 fx_to_int(i32 v) { return v >> FRACT_BITS; }                // :81-86
static inline i32 fx_from_int(i32 i) { return fx_shl(i, FRACT_BITS); }        // :74-79
// Rust `f32 as i32`: truncate toward zero, saturate, NaN -> 0.
static inline i32 rust_f32_as_i32(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (i32)f;
}
// fixed.rs:88-93  Fixed((f * 65536.0) as i32)
static inline i32 fx_from_f32(float f) {
    volatile float m = f * 65536.0f;
    return rust_f32_as_i32(m);
}
static inline float fx_to_f32(i32 v) { return (float)v / 65536.0f; }  // :136-141

// ------------------------------------------------------------ pointy 0.7 restated
struct Pt {
    float x, y;
};
static inline Pt pt(float x, float y) { return Pt{x, y}; }
static inline Pt padd(Pt a, Pt b) { return pt(a.x + b.x, a.y + b.y); }
static inline Pt psub(Pt a, Pt b) { return pt(a.x - b.x, a.y - b.y); }
static inline Pt pmul(Pt a, float s) { return pt(a.x * s, a.y * s); }
static inline Pt pmid(Pt a, Pt b) { return pt((a.x + b.x) / 2.0f, (a.y + b.y) / 2.0f); }
static inline float pdist_sq(Pt a, Pt b) {
    float dx = a.x - b.x, dy = a.y - b.y;
    return dx * dx + dy * dy;
}
static inline Pt pright(Pt v) { return pt(v.y, -v.x); }
static inline Pt pnormalize(Pt v) {
    float m = sqrtf(v.x * v.x + v.y * v.y);
    return pt(v.x / m, v.y / m);
}
// Trig of the join decisions: 0 = the shared ft_fmath.h functions (the ones the CUDA path
// uses), 1 = the C library's atan2f / sinf, for the test that counts the decisions the
// two would take differently (orc_join_decisions).  Recorded decisions go to the log.
static thread_local int g_trig_libm = 0;
static thread_local std::vector<int8_t>* g_join_log = nullptr;
static thread_local std::vector<float>* g_join_uv = nullptr;  // the vectors u = a1 - a0, v = b0 - b1 of each join
static inline float trig_atan2f(float y, float x) { return g_trig_libm ? atan2f(y, x) : ft_atan2f(y, x); }
static inline float trig_sinf(float x) { return g_trig_libm ? sinf(x) : ft_sinf(x); }
static inline void log_join(int d) {
    if (g_join_log) g_join_log->push_back((int8_t)d);
}
static inline void log_join_uv(float ux, float uy, float vx, float vy) {
    if (g_join_uv) g_join_uv->insert(g_join_uv->end(), {ux, uy, vx, vy});
}
static inline float pangle_rel(Pt a, Pt b) {
    float th = trig_atan2f(a.y, a.x) - trig_atan2f(b.y, b.x);
    const float PI = 3.14159265358979323846f;
    if (th < -PI) return th + 2.0f * PI;
    if (th > PI) return th - 2.0f * PI;
    return th;
}
// Line::intersection of the lines through (a0,a1) and (b0,b1); false when parallel.
static inline bool pline_intersection(Pt a0, Pt a1, Pt b0, Pt b1, Pt* out) {
    float x1 = a0.x, y1 = a0.y, x2 = a1.x, y2 = a1.y;
    float x3 = b0.x, y3 = b0.y, x4 = b1.x, y4 = b1.y;
    float den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
    if (den == 0.0f) return false;
    float a = x1 * y2 - y1 * x2;
    float b = x3 * y4 - y3 * x4;
    float x = (a * (x3 - x4) - (x1 - x2) * b) / den;
    float y = (a * (y3 - y4) - (y1 - y2) * b) / den;
    *out = pt(x, y);
    return true;
}
struct Xform {
    float m[6];
};
static inline Pt xform_apply(const Xform& t, Pt p) {
    float x = t.m[0] * p.x + t.m[1] * p.y + t.m[2];
    float y = t.m[3] * p.x + t.m[4] * p.y + t.m[5];
    return pt(x, y);
}
static inline bool pfinite(Pt p) { return std::isfinite(p.x) && std::isfinite(p.y); }

// ----------------------------------------------------------------- geom.rs
struct WidePt {
    Pt p;
    float w;
};
static inline WidePt wmid(WidePt a, WidePt b) { return WidePt{pmid(a.p, b.p), (a.w + b.w) / 2.0f}; }
static inline float float_lerp(float a, float b, float t) { return b + (a - b) * t; }  // geom.rs:14-16

// ----------------------------------------------------------- pix 0.14 restated
static inline uint8_t ch8_mul(uint8_t a, uint8_t b) {
    u32 l = a;
    l = (l << 4) | (l >> 4);
    u32 r = b;
    r = (r << 4) | (r >> 4);
    return (uint8_t)((l * r) >> 16);
}
static inline uint8_t ch8_add(uint8_t a, uint8_t b) {
    u32 s = (u32)a + b;
    return (uint8_t)(s > 255 ? 255 : s);
}
// composite_channels_alpha(&clr, SrcOver, &alpha) on premultiplied channels
static inline void srcover_rgba(uint8_t* d, const uint8_t* clr, uint8_t alpha) {
    uint8_t sa = ch8_mul(clr[3], alpha);
    uint8_t inv = (uint8_t)(255 - sa);
    for (int c = 0; c < 4; c++) d[c] = ch8_add(ch8_mul(clr[c], alpha), ch8_mul(d[c], inv));
}
static inline uint8_t sat_i16_u8(i16 v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

// ------------------------------------------------------------------ Raster
struct Raster {
    uint8_t* data;
    u32 w, h, stride;
    int fmt;
    uint8_t* row(u32 y) { return data + (size_t)y * stride; }
};

// ------------------------------------------------------------------- fig.rs
enum FigDir { Forward, Reverse };
static inline FigDir opposite(FigDir d) { return d == Forward ? Reverse : Forward; }

struct FxPt {
    i32 x, y;
    bool operator==(const FxPt& o) const { return x == o.x && y == o.y; }
};
// fig.rs:116-119  (self.x * rhs.y) > (rhs.x * self.y) with Fixed mul
static inline bool widdershins(FxPt a, FxPt b) { return fx_mul(a.x, b.y) > fx_mul(b.x, a.y); }
static inline FxPt fxsub(FxPt a, FxPt b) { return FxPt{wsub(a.x, b.x), wsub(a.y, b.y)}; }

static inline i32 row_of(i32 y) { return fx_to_int(y); }  // fig.rs:167-169

// fig.rs:677-682
static inline i16 pixel_cov(i32 fcov) { return (i16)fx_to_int(fx_round(fx_shl(fcov, 8))); }

// Vertex ids are V: footile's u16 (vid.rs:9-70), or u32 for the un-capped extension.
template <class V>
struct SubFigT {
    V start;
    size_t n_points;
    bool done;
    V next(V vid, FigDir dir) const {  // fig.rs:143-163
        if (dir == Forward) {
            V v = (V)(vid + 1);
            return v < (V)(start + n_points) ? v : start;
        }
        if (vid > start) return (V)(vid - 1);
        if (n_points > 0) return (V)(start + n_points - 1);
        return start;
    }
};

template <class V>
struct EdgeT {  // fig.rs:47-66
    V v1;
    i32 y_upper, y_lower;
    FigDir dir;
    i32 step_pix, inv_slope, x_bot, min_x, max_x;

    static i32 calculate_step(i32 dx, i32 dy) {  // fig.rs:204-210
        if (dx != 0) return std::min(fx_abs(fx_div(dy, dx)), FX_ONE);
        return 0;
    }
    static EdgeT make(V v0, V v1, FxPt p0, FxPt p1, FigDir dir) {  // fig.rs:179-201
        (void)v0;
        EdgeT e;
        i32 dx = wsub(p1.x, p0.x);
        i32 dy = wsub(p1.y, p0.y);
        e.step_pix = calculate_step(dx, dy);
        e.inv_slope = fx_div(dx, dy);
        e.y_upper = p0.y;
        e.y_lower = p1.y;
        i32 y_bot = wsub(fx_floor(wadd(e.y_upper, FX_ONE)), e.y_upper);
        e.x_bot = wadd(p0.x, fx_mul(e.inv_slope, y_bot));
        e.v1 = v1;
        e.dir = dir;
        e.min_x = 0;
        e.max_x = 0;
        return e;
    }
    i32 min_pix() const { return fx_to_int(min_x); }
    i32 max_pix() const { return fx_to_int(max_x); }
    i32 mid_x() const { return fx_avg(max_x, min_x); }
    bool is_ending(i32 y_row) const { return row_of(y_lower) == y_row; }
    i16 continuing_cov(i32 y_row) const { return is_ending(y_row) ? pixel_cov(fx_fract(y_lower)) : 256; }
    i16 starting_cov() const {  // fig.rs:238-241
        i32 y_row = row_of(y_upper);
        return (i16)(continuing_cov(y_row) - pixel_cov(fx_fract(y_upper)));
    }
    void set_x_limits(i32 x0, i32 y_row) {  // fig.rs:269-278
        i32 x1;
        if (is_ending(y_row)) {
            i32 y1 = wsub(fx_ceil(y_lower), y_lower);
            x1 = wsub(x_bot, fx_mul(inv_slope, y1));
        } else {
            x1 = x_bot;
        }
        min_x = std::min(x0, x1);
        max_x = std::max(x0, x1);
    }
    void calculate_x_limits_starting() {  // fig.rs:244-249
        i32 y_row = row_of(y_upper);
        i32 y0 = wsub(FX_ONE, fx_fract(y_upper));
        i32 x0 = wsub(x_bot, fx_mul(inv_slope, y0));
        set_x_limits(x0, y_row);
    }
    void calculate_x_limits_continuing(i32 y_row) {  // fig.rs:262-266
        i32 x0 = wsub(x_bot, inv_slope);
        set_x_limits(x0, y_row);
    }
    i32 step_cov(i32 r) const { return step_pix > 0 ? fx_mul(r, step_pix) : r; }  // :315-321
    i32 first_cov(i32 full_cov) const {                                          // :305-312
        i32 r;
        if (min_pix() == max_pix())
            r = fx_mul(wsub(FX_ONE, fx_fract(mid_x())), full_cov);
        else
            r = fx_mul(wsub(FX_ONE, fx_fract(min_x)), FX_HALF);
        return step_cov(r);
    }
    // fig.rs:285-302
    void scan_area(FigDir fdir, i16 cov, i16* area, size_t len) const {
        i16 ed = (dir == fdir) ? 1 : -1;
        i32 full_cov = fx_from_f32((float)cov / 256.0f);
        i32 x_cov = first_cov(full_cov);
        i32 step = step_cov(FX_ONE);
        i16 sum_pix = 0;
        for (i32 x = min_pix(); x < (i32)len; x++) {
            i16 x_pix = std::min(pixel_cov(x_cov), cov);
            i16 p = (i16)(x_pix - sum_pix);
            size_t xi = (size_t)std::max(x, 0);
            area[xi] = (i16)(area[xi] + (i16)(p * ed));
            sum_pix = (i16)(sum_pix + p);
            if (sum_pix >= cov) break;
            x_cov = std::min(wadd(x_cov, step), FX_ONE);
        }
    }
};

// imgbuf.rs:54-61 / 157-167 (scalar semantics; the SSSE3 path computes the same)
static void accumulate_non_zero(uint8_t* dst, i16* src, size_t n) {
    i16 sum = 0;
    for (size_t i = 0; i < n; i++) {
        sum = (i16)(sum + src[i]);
        src[i] = 0;
        dst[i] = sat_i16_u8(sum);
    }
}
static void accumulate_even_odd(uint8_t* dst, i16* src, size_t n) {
    i16 sum = 0;
    for (size_t i = 0; i < n; i++) {
        sum = (i16)(sum + src[i]);
        src[i] = 0;
        i16 v = (i16)(sum & 0xFF);
        i16 odd = (i16)(sum & 0x100);
        i16 c = (i16)std::abs(v - odd);
        dst[i] = sat_i16_u8(c);
    }
}

struct PlotDest {
    virtual void add_point(WidePt p) = 0;
    virtual void close(bool joined) = 0;
    virtual ~PlotDest() {}
};

// `cap`: footile's 65,535 vertices (Fig::add_point, fig.rs:430); larger only for the
// un-capped extension (u32 ids).
template <class V>
struct FigT : PlotDest {
    using SubFig = SubFigT<V>;
    std::vector<FxPt> points;
    std::vector<SubFig> subs;
    size_t cap = 65535;
    FigT() {
        points.reserve(1024);
        subs.push_back(SubFig{0, 0, false});
    }
    SubFig& sub_current() { return subs.back(); }
    void sub_add() { subs.push_back(SubFig{(V)points.size(), 0, false}); }
    bool is_coincident(FxPt p) const { return !points.empty() && points.back() == p; }
    void sub_set_done() {  // fig.rs:373-383
        SubFig& sub = sub_current();
        if (sub.n_points > 0) {
            FxPt p = points[sub.start];
            if (is_coincident(p)) {
                points.pop_back();
                sub.n_points -= 1;
            }
            sub.done = true;
        }
    }
    const SubFig& sub_at(V vid) const {  // fig.rs:386-394
        for (const SubFig& s : subs)
            if (vid < (V)(s.start + s.n_points)) return s;
        abort();  // unreachable!() in footile
    }
    V next(V vid, FigDir dir) const { return sub_at(vid).next(vid, dir); }
    FigDir get_dir(V vid) const {  // fig.rs:402-411
        FxPt p = points[vid];
        FxPt p0 = points[next(vid, Forward)];
        FxPt p1 = points[next(vid, Reverse)];
        return widdershins(fxsub(p1, p), fxsub(p0, p)) ? Forward : Reverse;
    }
    void add_point_pt(Pt pt) {  // fig.rs:428-442
        size_t n = points.size();
        if (n < cap) {
            bool done = sub_current().done;
            if (done) sub_add();
            FxPt p{fx_from_f32(pt.x), fx_from_f32(pt.y)};
            if (done || !is_coincident(p)) {
                points.push_back(p);
                sub_current().n_points += 1;
            }
        }
    }
    void close_fig() {  // fig.rs:457-461
        if (!points.empty()) sub_set_done();
    }
    void add_point(WidePt p) override { add_point_pt(p.p); }
    void close(bool) override { close_fig(); }
};

// fig.rs:505-666  Scanner
template <class V>
struct ScannerT {
    using Fig = FigT<V>;
    using Edge = EdgeT<V>;
    const Fig& fig;
    int rule;
    FigDir dir;
    Raster& r;
    u32 row_begin;
    const uint8_t* clr;
    std::vector<i16>& sgn_area;
    std::vector<Edge> edges;

    ScannerT(const Fig& f, int rule_, FigDir d, Raster& r_, u32 rb, const uint8_t* c, std::vector<i16>& sa)
        : fig(f), rule(rule_), dir(d), r(r_), row_begin(rb), clr(c), sgn_area(sa) {}

    void scan_vertices(const std::vector<V>& vids, i32 top_row) {
        size_t vi = 0;
        i32 y_row = top_row;
        for (u32 row = row_begin; row < r.h; row++) {
            scan_continuing_edges(y_row);
            while (vi < vids.size()) {
                V vid = vids[vi];
                if (row_of(fig.points[vid].y) > y_row) break;
                vi++;
                update_edges(vid, Forward);
                update_edges(vid, Reverse);
            }
            rasterize_row(r.row(row));
            advance_edges();
            y_row = wadd(y_row, 1);
        }
    }
    void scan_continuing_edges(i32 y_row) {
        for (Edge& e : edges) {
            i16 cov = e.continuing_cov(y_row);
            if (cov > 0) {
                e.calculate_x_limits_continuing(y_row);
                e.scan_area(dir, cov, sgn_area.data(), sgn_area.size());
            }
        }
    }
    void advance_edges() {
        for (Edge& e : edges) e.x_bot = wadd(e.x_bot, e.inv_slope);
    }
    void update_edges(V vid, FigDir d) {
        V v = fig.next(vid, d);
        if (v != vid) {
            i32 y = fig.points[vid].y;
            i32 yv = fig.points[v].y;
            if (yv > y)
                add_edge(vid, v, d);
            else if (yv < y)
                remove_edge(vid, opposite(d));
        }
    }
    void add_edge(V v0, V v1, FigDir d) {
        Edge e = Edge::make(v0, v1, fig.points[v0], fig.points[v1], d);
        i16 cov = e.starting_cov();
        if (cov > 0) {
            e.calculate_x_limits_starting();
            e.scan_area(dir, cov, sgn_area.data(), sgn_area.size());
        }
        edges.push_back(e);
    }
    void remove_edge(V v1, FigDir d) {
        for (size_t i = 0; i < edges.size(); i++) {
            if (edges[i].v1 == v1 && edges[i].dir == d) {
                edges[i] = edges.back();  // swap_remove
                edges.pop_back();
                return;
            }
        }
    }
    void rasterize_row(uint8_t* row) {
        size_t w = r.w;
        if (r.fmt == FT_MATTE8) {
            if (rule == FT_NONZERO)
                accumulate_non_zero(row, sgn_area.data(), w);
            else
                accumulate_even_odd(row, sgn_area.data(), w);
            return;
        }
        i16 sum = 0;
        for (size_t x = 0; x < w; x++) {
            sum = (i16)(sum + sgn_area[x]);
            sgn_area[x] = 0;
            uint8_t alpha;
            if (rule == FT_NONZERO) {
                alpha = sat_i16_u8(sum);
            } else {
                i16 v = (i16)(sum & 0xFF);
                i16 odd = (i16)(sum & 0x100);
                alpha = sat_i16_u8((i16)std::abs(v - odd));
            }
            srcover_rgba(row + 4 * x, clr, alpha);
        }
    }
};

using SubFig = SubFigT<u16>;
using Edge = EdgeT<u16>;
using Fig = FigT<u16>;
using Scanner = ScannerT<u16>;

// fig.rs:480-502
template <class V>
static void fig_fill(const FigT<V>& fig, int rule, Raster& r, const uint8_t* clr, std::vector<i16>& sgn_area) {
    size_t n = fig.points.size();
    if (n == 0) return;
    std::vector<V> vids(n);
    for (size_t i = 0; i < n; i++) vids[i] = (V)i;
    std::stable_sort(vids.begin(), vids.end(), [&](V a, V b) {
        const FxPt& p0 = fig.points[a];
        const FxPt& p1 = fig.points[b];
        if (p0.y != p1.y) return p0.y < p1.y;
        return p0.x < p1.x;
    });
    FigDir dir = fig.get_dir(vids[0]);
    i32 top_row = row_of(fig.points[vids[0]].y);
    u32 row_begin = (u32)std::max(top_row, 0);
    if (row_begin >= r.h) return;
    ScannerT<V> s(fig, rule, dir, r, row_begin, clr, sgn_area);
    s.scan_vertices(vids, top_row);
}

// -------------------------------------------------------------- stroker.rs
enum SDir { SFwd, SRev };
struct SubStroke {  // stroker.rs:31-97
    u16 start;
    u16 n_points;
    bool joined;
    bool done;
    u16 next(u16 vid, SDir dir) const {
        if (dir == SFwd) {
            u16 v = (u16)(vid + 1);
            return v < (u16)(start + n_points) ? v : start;
        }
        return vid > start ? (u16)(vid - 1) : (u16)(start + n_points - 1);
    }
    u16 len() const {
        if (joined) return (u16)(n_points + 1);
        if (n_points > 0) return (u16)(n_points - 1);
        return 0;
    }
};

struct Stroke : PlotDest {
    int join;
    float miter_limit;
    float miter_g;  // ft_miter_angle(miter_limit)
    float tol_sq;
    std::vector<WidePt> points;
    std::vector<SubStroke> subs;
    int* status;

    Stroke(int j, float ml, float tsq, int* st)
        : join(j), miter_limit(ml), miter_g(ft_miter_angle(ml)), tol_sq(tsq), status(st) {
        points.reserve(1024);
        subs.push_back(SubStroke{0, 0, false, false});
    }
    SubStroke& sub_current() { return subs.back(); }
    const SubStroke& sub_at(u16 vid) const {
        for (const SubStroke& s : subs)
            if (vid < (u16)(s.start + s.n_points)) return s;
        abort();
    }
    u16 next(u16 vid, SDir d) const { return sub_at(vid).next(vid, d); }
    void add_point(WidePt pt) override {  // stroker.rs:204-216
        size_t n = points.size();
        if (n < 65535) {
            bool done = sub_current().done;
            if (done) subs.push_back(SubStroke{(u16)points.size(), 0, false, false});
            bool coincident = !points.empty() && points.back().p.x == pt.p.x && points.back().p.y == pt.p.y;
            if (done || !coincident) {
                points.push_back(pt);
                sub_current().n_points = (u16)(sub_current().n_points + 1);
            }
        }
    }
    void close(bool joined) override {  // stroker.rs:230-236
        if (!points.empty()) {
            SubStroke& s = sub_current();
            s.joined = joined;
            s.done = true;
        }
    }
    // stroker.rs:239-262
    void path_ops(std::vector<ft_op>& ops) const {
        for (size_t i = 0; i < subs.size(); i++) {
            const SubStroke& s = subs[i];
            if (s.len() > 0) {
                u16 start = s.start;
                u16 end = s.next(s.start, SRev);
                stroke_side(ops, s, start, SFwd);
                if (s.joined) push_close(ops);
                stroke_side(ops, s, end, SRev);
                push_close(ops);
            }
        }
    }
    static void push_close(std::vector<ft_op>& ops) {
        ft_op o{};
        o.kind = FT_OP_CLOSE;
        ops.push_back(o);
    }
    static void stroke_point(std::vector<ft_op>& ops, Pt p) {
        ft_op o{};
        o.kind = FT_OP_LINE;
        o.v[0] = p.x;
        o.v[1] = p.y;
        ops.push_back(o);
    }
    // stroker.rs:265-295
    void stroke_side(std::vector<ft_op>& ops, const SubStroke& s, u16 start, SDir dir) const {
        bool have = false;
        Pt xr0{}, xr1{};
        u16 v0 = start;
        u16 v1 = next(v0, dir);
        bool joined = s.joined;
        u16 n = s.len();
        for (u16 k = 0; k < n; k++) {
            WidePt p0 = points[v0];
            WidePt p1 = points[v1];
            Pt pr0, pr1;
            stroke_offset(p0, p1, &pr0, &pr1);
            if (have)
                stroke_join(ops, p0, xr0, xr1, pr0, pr1);
            else if (!joined)
                stroke_point(ops, pr0);
            have = true;
            xr0 = pr0;
            xr1 = pr1;
            v0 = v1;
            v1 = next(v1, dir);
        }
        if (!joined && have) stroke_point(ops, xr1);
    }
    // stroker.rs:301-309
    static void stroke_offset(WidePt p0, WidePt p1, Pt* pr0, Pt* pr1) {
        Pt vr = pnormalize(pright(psub(p1.p, p0.p)));
        *pr0 = padd(p0.p, pmul(vr, p0.w / 2.0f));
        *pr1 = padd(p1.p, pmul(vr, p1.w / 2.0f));
    }
    void stroke_join(std::vector<ft_op>& ops, WidePt p, Pt a0, Pt a1, Pt b0, Pt b1) const {
        if (join == FT_JOIN_MITER)
            stroke_miter(ops, a0, a1, b0, b1, miter_limit);
        else if (join == FT_JOIN_BEVEL)
            stroke_bevel(ops, a1, b0);
        else
            stroke_round(ops, p, a0, a1, b0, b1);
    }
    // stroker.rs:340-367.  The decision sm >= 1/ml && sm < 1 is taken as a correctly
    // rounded f32 libm takes it (ft_fmath.h: the CUDA path's function); the test mode
    // g_trig_libm takes it with the C library's atan2f / sinf instead.
    bool miter_decision(Pt u, Pt v, float ml) const {
        if (!g_trig_libm) return ft_miter_join(u.x, u.y, v.x, v.y, miter_g);
        if (!(ml > 0.0f)) return false;
        float sm_min = 1.0f / ml;
        float th = pangle_rel(u, v);
        float sm = fabsf(trig_sinf(th / 2.0f));
        return sm >= sm_min && sm < 1.0f;
    }
    void stroke_miter(std::vector<ft_op>& ops, Pt a0, Pt a1, Pt b0, Pt b1, float ml) const {
        log_join_uv(a1.x - a0.x, a1.y - a0.y, b0.x - b1.x, b0.y - b1.y);
        if (miter_decision(psub(a1, a0), psub(b0, b1), ml)) {
            Pt xp;
            if (pline_intersection(a0, a1, b0, b1, &xp)) {
                log_join(1);
                stroke_point(ops, xp);
                return;
            }
        }
        log_join(0);
        stroke_bevel(ops, a1, b0);
    }
    static void stroke_bevel(std::vector<ft_op>& ops, Pt a1, Pt b0) {
        stroke_point(ops, a1);
        stroke_point(ops, b0);
    }
    // stroker.rs:380-396
    void stroke_round(std::vector<ft_op>& ops, WidePt p, Pt a0, Pt a1, Pt b0, Pt b1) const {
        const Pt u = psub(a1, a0), v = psub(b0, b1);
        log_join_uv(u.x, u.y, v.x, v.y);
        const bool arc = g_trig_libm ? !(pangle_rel(u, v) <= 0.0f) : ft_round_join_arc(u.x, u.y, v.x, v.y);
        log_join(arc ? 2 : 0);
        if (!arc) {
            stroke_bevel(ops, a1, b0);
        } else {
            stroke_point(ops, a1);
            stroke_arc(ops, p, a1, b0, 0);
        }
    }
    // stroker.rs:399-416 (+ depth cap; a non-finite arc point ends the recursion)
    void stroke_arc(std::vector<ft_op>& ops, WidePt p, Pt a, Pt b, int depth) const {
        Pt vr = pnormalize(pright(psub(b, a)));
        Pt c = padd(p.p, pmul(vr, p.w / 2.0f));
        Pt ab = pmid(a, b);
        if (!pfinite(c) || pdist_sq(c, ab) <= tol_sq) {
            stroke_point(ops, b);
        } else if (depth >= FT_MAX_DEPTH) {
            *status = std::max(*status, (int)FT_ERR_DEPTH);
            stroke_point(ops, b);
        } else {
            stroke_arc(ops, p, a, c, depth + 1);
            stroke_arc(ops, p, c, b, depth + 1);
        }
    }
};

// ---------------------------------------------------------------- plotter.rs
struct Plotter {
    Raster r;
    std::vector<i16> sgn_area;
    WidePt pen;
    Xform xf;
    float tol_sq;
    float s_width;
    int join;
    float miter_limit;
    int status;
    size_t fig_cap = 0;  // vertices per figure above footile's 65,535: the un-capped extension

    Plotter(Raster rr, float tol, const float* m, int j, float ml, float sw)
        : r(rr), sgn_area(rr.w, 0), xf(), join(j), miter_limit(ml), status(0) {
        float t = std::max(tol, 0.01f);  // set_tolerance, plotter.rs:133-137
        tol_sq = t * t;
        for (int i = 0; i < 6; i++) xf.m[i] = m[i];
        s_width = sw;
        pen = WidePt{pt(0, 0), s_width};
    }
    void reset() { pen = WidePt{pt(0, 0), s_width}; }
    WidePt transform_point(WidePt p) const { return WidePt{xform_apply(xf, p.p), p.w}; }
    void add_ops(const ft_op* ops, size_t n, PlotDest& dst) {  // plotter.rs:175-185
        reset();
        for (size_t i = 0; i < n; i++) add_op(dst, ops[i]);
    }
    void add_op(PlotDest& dst, const ft_op& op) {  // plotter.rs:188-197
        switch (op.kind) {
            case FT_OP_CLOSE:
                dst.close(true);
                reset();
                break;
            case FT_OP_MOVE: {
                WidePt p{pt(op.v[0], op.v[1]), s_width};
                dst.close(false);
                dst.add_point(transform_point(p));
                pen = p;
                break;
            }
            case FT_OP_LINE: {
                WidePt p{pt(op.v[0], op.v[1]), s_width};
                dst.add_point(transform_point(p));
                pen = p;
                break;
            }
            case FT_OP_QUAD: {  // plotter.rs:233-242
                WidePt bb{pt(op.v[0], op.v[1]), (pen.w + s_width) / 2.0f};
                WidePt cc{pt(op.v[2], op.v[3]), s_width};
                WidePt a = transform_point(pen), b = transform_point(bb), c = transform_point(cc);
                if (!pfinite(a.p) || !pfinite(b.p) || !pfinite(c.p)) {
                    status = std::max(status, (int)FT_ERR_ARG);
                    dst.add_point(c);
                } else {
                    quad_to_tran(dst, a, b, c, 0);
                }
                pen = cc;
                break;
            }
            case FT_OP_CUBIC: {  // plotter.rs:286-305
                float w0 = float_lerp(pen.w, s_width, 1.0f / 3.0f);
                float w1 = float_lerp(pen.w, s_width, 2.0f / 3.0f);
                WidePt bb{pt(op.v[0], op.v[1]), w0};
                WidePt cc{pt(op.v[2], op.v[3]), w1};
                WidePt dd{pt(op.v[4], op.v[5]), s_width};
                WidePt a = transform_point(pen), b = transform_point(bb), c = transform_point(cc),
                       d = transform_point(dd);
                if (!pfinite(a.p) || !pfinite(b.p) || !pfinite(c.p) || !pfinite(d.p)) {
                    status = std::max(status, (int)FT_ERR_ARG);
                    dst.add_point(d);
                } else {
                    cubic_to_tran(dst, a, b, c, d, 0);
                }
                pen = dd;
                break;
            }
            case FT_OP_PEN_WIDTH:
                s_width = op.v[0];
                break;
            default:
                break;
        }
    }
    bool within(Pt a, Pt b) const { return pdist_sq(a, b) <= tol_sq; }
    // plotter.rs:248-265
    void quad_to_tran(PlotDest& dst, WidePt a, WidePt b, WidePt c, int depth) {
        WidePt ab = wmid(a, b), bc = wmid(b, c), ab_bc = wmid(ab, bc), ac = wmid(a, c);
        if (within(ab_bc.p, ac.p)) {
            dst.add_point(c);
        } else if (depth >= FT_MAX_DEPTH) {
            status = std::max(status, (int)FT_ERR_DEPTH);
            dst.add_point(c);
        } else {
            quad_to_tran(dst, a, ab, ab_bc, depth + 1);
            quad_to_tran(dst, ab_bc, bc, c, depth + 1);
        }
    }
    // plotter.rs:311-332
    void cubic_to_tran(PlotDest& dst, WidePt pa, WidePt pb, WidePt pc, WidePt pd, int depth) {
        WidePt ab = wmid(pa, pb), bc = wmid(pb, pc), cd = wmid(pc, pd);
        WidePt ab_bc = wmid(ab, bc), bc_cd = wmid(bc, cd);
        WidePt pe = wmid(ab_bc, bc_cd);
        WidePt ad = wmid(pa, pd);
        if (within(pe.p, ad.p)) {
            dst.add_point(pd);
        } else if (depth >= FT_MAX_DEPTH) {
            status = std::max(status, (int)FT_ERR_DEPTH);
            dst.add_point(pd);
        } else {
            cubic_to_tran(dst, pa, ab, ab_bc, pe, depth + 1);
            cubic_to_tran(dst, pe, bc_cd, cd, pd, depth + 1);
        }
    }
    // plotter.rs:339-350
    void fill(int rule, const ft_op* ops, size_t n, const uint8_t* clr) {
        if (fig_cap > 65535) {  // un-capped extension: u32 vertex ids, `fig_cap` vertices
            FigT<u32> fig;
            fig.cap = fig_cap;
            add_ops(ops, n, fig);
            fig.close_fig();
            fig_fill(fig, rule, r, clr, sgn_area);
            return;
        }
        Fig fig;
        add_ops(ops, n, fig);
        fig.close_fig();
        fig_fill(fig, rule, r, clr, sgn_area);
    }
    // plotter.rs:356-365
    void stroke(const ft_op* ops, size_t n, const uint8_t* clr) {
        Stroke st(join, miter_limit, tol_sq, &status);
        add_ops(ops, n, st);
        std::vector<ft_op> outline;
        st.path_ops(outline);
        fill(FT_NONZERO, outline.data(), outline.size(), clr);
    }
};

}  // namespace orc

// ===================================================================== C ABI
extern "C" {

typedef struct orc_params {
    float tolerance;
    float transform[6];
    int32_t join;
    float miter_limit;
    uint32_t fig_cap;  // 0: footile's 65,535-vertex figures; larger: the un-capped extension (fills)
} orc_params;

static const float ORC_IDENTITY[6] = {1, 0, 0, 0, 1, 0};

static int orc_run(int stroke, int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt, const uint8_t clr[4],
                   uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride, const orc_params* prm,
                   float* s_width_inout) {
    orc::Raster r{raster, w, h, stride, fmt};
    float tol = prm ? prm->tolerance : 0.3f;
    const float* m = prm ? prm->transform : ORC_IDENTITY;
    int join = prm ? prm->join : FT_JOIN_MITER;
    float ml = prm ? prm->miter_limit : 4.0f;
    float sw = s_width_inout ? *s_width_inout : 1.0f;
    static const uint8_t zero_clr[4] = {0, 0, 0, 0};
    orc::Plotter p(r, tol, m, join, ml, sw);
    if (prm && !stroke) p.fig_cap = prm->fig_cap;
    if (stroke)
        p.stroke(ops, n_ops, clr ? clr : zero_clr);
    else
        p.fill(rule, ops, n_ops, clr ? clr : zero_clr);
    if (s_width_inout) *s_width_inout = p.s_width;
    return p.status;
}

__attribute__((visibility("default"))) int orc_fill(int32_t rule, const ft_op* ops, uint32_t n_ops, int32_t fmt,
                                                    const uint8_t clr[4], uint8_t* raster, uint32_t w, uint32_t h,
                                                    uint32_t stride, const orc_params* prm, float* s_width_inout) {
    return orc_run(0, rule, ops, n_ops, fmt, clr, raster, w, h, stride, prm, s_width_inout);
}

__attribute__((visibility("default"))) int orc_stroke(const ft_op* ops, uint32_t n_ops, int32_t fmt,
                                                      const uint8_t clr[4], uint8_t* raster, uint32_t w, uint32_t h,
                                                      uint32_t stride, const orc_params* prm, float* s_width_inout) {
    return orc_run(1, FT_NONZERO, ops, n_ops, fmt, clr, raster, w, h, stride, prm, s_width_inout);
}

// The stroke outline footile would fill (Stroke::path_ops, stroker.rs:239-247), for
// tests of the stroker alone.  Returns the number of ops (may exceed `cap`).
__attribute__((visibility("default"))) uint32_t orc_stroke_outline(const ft_op* ops, uint32_t n_ops,
                                                                   const orc_params* prm, float s_width,
                                                                   ft_op* out, uint32_t cap) {
    uint8_t dummy = 0;
    orc::Raster r{&dummy, 1, 1, 1, FT_MATTE8};
    float tol = prm ? prm->tolerance : 0.3f;
    const float* m = prm ? prm->transform : ORC_IDENTITY;
    orc::Plotter p(r, tol, m, prm ? prm->join : FT_JOIN_MITER, prm ? prm->miter_limit : 4.0f, s_width);
    orc::Stroke st(p.join, p.miter_limit, p.tol_sq, &p.status);
    p.add_ops(ops, n_ops, st);
    std::vector<ft_op> outline;
    st.path_ops(outline);
    for (uint32_t i = 0; i < outline.size() && i < cap; i++) out[i] = outline[i];
    return (uint32_t)outline.size();
}

// The stream the plotter hands the stroker (plotter.rs:175-224 into stroker.rs:204-236)
// and what the stroker keeps of it: `ev` gets 4 floats per event, (x, y, width, 0) for an
// add_point and (0, 0, 0, 1 + joined) for a close; `pts` 3 floats per kept stroke point;
// `subs` 4 ints per sub-stroke (start, points, joined, done).  Returns the event count;
// n_pts / n_subs get the other two counts.  Each array holds `cap` entries at most.
struct StrokeTee : orc::PlotDest {
    orc::Stroke& st;
    std::vector<float> ev;
    explicit StrokeTee(orc::Stroke& s) : st(s) {}
    void add_point(orc::WidePt p) override {
        ev.insert(ev.end(), {p.p.x, p.p.y, p.w, 0.0f});
        st.add_point(p);
    }
    void close(bool joined) override {
        ev.insert(ev.end(), {0.0f, 0.0f, 0.0f, joined ? 2.0f : 1.0f});
        st.close(joined);
    }
};

__attribute__((visibility("default"))) uint32_t orc_stroke_points(const ft_op* ops, uint32_t n_ops,
                                                                  const orc_params* prm, float s_width, float* ev,
                                                                  float* pts, uint32_t* n_pts, int32_t* subs,
                                                                  uint32_t* n_subs, uint32_t cap) {
    uint8_t dummy = 0;
    orc::Raster r{&dummy, 1, 1, 1, FT_MATTE8};
    float tol = prm ? prm->tolerance : 0.3f;
    const float* m = prm ? prm->transform : ORC_IDENTITY;
    orc::Plotter p(r, tol, m, prm ? prm->join : FT_JOIN_MITER, prm ? prm->miter_limit : 4.0f, s_width);
    orc::Stroke st(p.join, p.miter_limit, p.tol_sq, &p.status);
    StrokeTee tee(st);
    p.add_ops(ops, n_ops, tee);
    const uint32_t n_ev = (uint32_t)(tee.ev.size() / 4);
    for (uint32_t i = 0; i < n_ev && i < cap; i++)
        for (int k = 0; k < 4; k++) ev[4 * i + k] = tee.ev[4 * i + k];
    *n_pts = (uint32_t)st.points.size();
    for (uint32_t i = 0; i < *n_pts && i < cap; i++) {
        pts[3 * i] = st.points[i].p.x;
        pts[3 * i + 1] = st.points[i].p.y;
        pts[3 * i + 2] = st.points[i].w;
    }
    *n_subs = (uint32_t)st.subs.size();
    for (uint32_t i = 0; i < *n_subs && i < cap; i++) {
        subs[4 * i] = st.subs[i].start;
        subs[4 * i + 1] = st.subs[i].n_points;
        subs[4 * i + 2] = st.subs[i].joined;
        subs[4 * i + 3] = st.subs[i].done;
    }
    return n_ev;
}

// The join decisions of the stroke outline of `ops` (stroker.rs:340-396), one byte per
// join in outline order: 0 bevel, 1 miter, 2 round arc.  `libm` 0 takes the angle and
// the miter sine from ft_fmath.h (as the CUDA path does), 1 from the C library's
// atan2f / sinf — the functions Rust's f32::atan2 / f32::sin call — so a test can count
// the joins whose decision depends on which is used.  Returns the number of joins (may
// exceed `cap`).  With `uv` (4 floats per join, may be NULL), the join's vectors
// u = a1 - a0 and v = b0 - b1 (th = angle_rel(u, v)).
__attribute__((visibility("default"))) uint32_t orc_join_decisions(const ft_op* ops, uint32_t n_ops,
                                                                   const orc_params* prm, float s_width, int32_t libm,
                                                                   int8_t* out, float* uv, uint32_t cap) {
    uint8_t dummy = 0;
    orc::Raster r{&dummy, 1, 1, 1, FT_MATTE8};
    float tol = prm ? prm->tolerance : 0.3f;
    const float* m = prm ? prm->transform : ORC_IDENTITY;
    orc::Plotter p(r, tol, m, prm ? prm->join : FT_JOIN_MITER, prm ? prm->miter_limit : 4.0f, s_width);
    orc::Stroke st(p.join, p.miter_limit, p.tol_sq, &p.status);
    p.add_ops(ops, n_ops, st);
    std::vector<ft_op> outline;
    std::vector<int8_t> log;
    std::vector<float> uvs;
    orc::g_trig_libm = libm ? 1 : 0;
    orc::g_join_log = &log;
    orc::g_join_uv = uv ? &uvs : nullptr;
    st.path_ops(outline);
    orc::g_join_log = nullptr;
    orc::g_join_uv = nullptr;
    orc::g_trig_libm = 0;
    for (uint32_t i = 0; i < log.size() && i < cap; i++) {
        out[i] = log[i];
        if (uv)
            for (int k = 0; k < 4; k++) uv[4 * i + k] = uvs[4 * i + k];
    }
    return (uint32_t)log.size();
}

// Fixed vertices of the figure footile fills for `ops` (after Fig::close): for tests
// of the path walk, flattening and figure building alone.  Returns the vertex count.
__attribute__((visibility("default"))) uint32_t orc_fig_points(const ft_op* ops, uint32_t n_ops,
                                                               const orc_params* prm, int32_t* xy,
                                                               uint32_t cap) {
    uint8_t dummy = 0;
    orc::Raster r{&dummy, 1, 1, 1, FT_MATTE8};
    float tol = prm ? prm->tolerance : 0.3f;
    const float* m = prm ? prm->transform : ORC_IDENTITY;
    orc::Plotter p(r, tol, m, FT_JOIN_MITER, 4.0f, 1.0f);
    orc::Fig fig;
    p.add_ops(ops, n_ops, fig);
    fig.close_fig();
    for (uint32_t i = 0; i < fig.points.size() && i < cap; i++) {
        xy[2 * i] = fig.points[i].x;
        xy[2 * i + 1] = fig.points[i].y;
    }
    return (uint32_t)fig.points.size();
}

// imgbuf.rs accumulate_non_zero / accumulate_even_odd on one row.
__attribute__((visibility("default"))) void orc_accumulate(int32_t rule, int16_t* src, uint8_t* dst, uint32_t n) {
    if (rule == FT_NONZERO)
        orc::accumulate_non_zero(dst, src, n);
    else
        orc::accumulate_even_odd(dst, src, n);
}

// Fixed arithmetic (fixed.rs) for the known-answer tests.
__attribute__((visibility("default"))) int32_t orc_fx_from_f32(float f) { return orc::fx_from_f32(f); }
__attribute__((visibility("default"))) int32_t orc_fx_from_int(int32_t i) { return orc::fx_from_int(i); }
__attribute__((visibility("default"))) float orc_fx_to_f32(int32_t v) { return orc::fx_to_f32(v); }
__attribute__((visibility("default"))) int32_t orc_fx_to_int(int32_t v) { return orc::fx_to_int(v); }
__attribute__((visibility("default"))) int32_t orc_fx_op(int32_t op, int32_t a, int32_t b) {
    switch (op) {
        case 0: return orc::wadd(a, b);
        case 1: return orc::wsub(a, b);
        case 2: return orc::fx_mul(a, b);
        case 3: return orc::fx_div(a, b);
        case 4: return orc::fx_shl(a, (uint32_t)b);
        case 5: return a >> b;
        case 6: return orc::fx_abs(a);
        case 7: return orc::fx_floor(a);
        case 8: return orc::fx_ceil(a);
        case 9: return orc::fx_round(a);
        case 10: return orc::fx_trunc(a);
        case 11: return orc::fx_fract(a);
        case 12: return orc::fx_avg(a, b);
        case 13: return orc::widdershins(orc::FxPt{a, b}, orc::FxPt{0, 0}) ? 1 : 0;  // unused
        default: return 0;
    }
}
__attribute__((visibility("default"))) int32_t orc_widdershins(int32_t ax, int32_t ay, int32_t bx, int32_t by) {
    return orc::widdershins(orc::FxPt{ax, ay}, orc::FxPt{bx, by}) ? 1 : 0;
}
__attribute__((visibility("default"))) float orc_atan2f(float y, float x) { return ft_atan2f(y, x); }
__attribute__((visibility("default"))) float orc_sinf(float x) { return ft_sinf(x); }

// A sequence of Plotter calls on one raster (ft_composite_batch semantics): path i
// draws after paths 0..i-1 with its own colour; the pen width carries from call to
// call starting at *s_width_inout.
__attribute__((visibility("default"))) int orc_composite(int32_t stroke, int32_t rule, const ft_op* ops,
                                                         const ft_path_desc* paths, uint32_t n_paths, int32_t fmt,
                                                         uint8_t* raster, uint32_t w, uint32_t h, uint32_t stride,
                                                         const orc_params* prm, float* s_width_inout,
                                                         int32_t* status) {
    float sw = s_width_inout ? *s_width_inout : 1.0f;
    for (uint32_t i = 0; i < n_paths; i++) {
        const ft_path_desc& d = paths[i];
        int st = orc_run(stroke, rule, ops + d.op_begin, d.n_ops, fmt, d.clr, raster, w, h, stride, prm, &sw);
        if (status) status[i] = st;
    }
    if (s_width_inout) *s_width_inout = sw;
    return 0;
}

// A batch of independent Plotter calls (ft_fill_batch semantics) on `n_threads`
// host threads, one Plotter per path.  Statuses go to `status` (may be NULL).
__attribute__((visibility("default"))) int orc_fill_batch(int32_t stroke, int32_t rule, const ft_op* ops,
                                                          const ft_path_desc* paths, uint32_t n_paths, int32_t fmt,
                                                          uint8_t* rasters, const orc_params* prm, int32_t* status,
                                                          int32_t n_threads) {
    if (n_threads < 1) n_threads = 1;
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (;;) {
            uint32_t i = next.fetch_add(1);
            if (i >= n_paths) return;
            const ft_path_desc& d = paths[i];
            float sw = d.s_width;
            int st = orc_run(stroke, rule, ops + d.op_begin, d.n_ops, fmt, d.clr, rasters + d.raster_offset, d.width,
                             d.height, d.stride, prm, &sw);
            if (status) status[i] = st;
        }
    };
    if (n_threads == 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < n_threads; t++) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    return 0;
}

}  // extern "C"
