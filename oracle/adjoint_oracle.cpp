// adjoint_oracle.cpp — TEST INFRASTRUCTURE ONLY: the FP64 gradient oracle of the
// coverage adjoint (ft_adjoint_forward / ft_adjoint_backward).
//
// footile itself has no adjoint.  The differentiable quantity is defined here, in
// double precision, for the CUDA kernels (float) to be checked against:
//
//   * the polygon is the flattened path of Plotter::fill: the same pen walk
//     (plotter.rs:175-224) and the same De Casteljau subdivision tree
//     (plotter.rs:233-332), decided in f32 exactly as footile decides it; each
//     vertex is the Bernstein point B(t) of its segment at the leaf's end
//     parameter t (a dyadic rational), evaluated in f64.  The tree is piecewise
//     constant in the control points, so the gradient is taken with the tree held;
//   * sub-figures start at Move and at the first point after Close (fig.rs:428-461)
//     and close back to their first vertex;
//   * coverage is the analytic form of fig's cell-area scheme (fig.rs:285-321,
//     imgbuf.rs:38-51) without the 16.16 and 1/256 quantisation: every edge adds,
//     row by row and cell by cell, its signed area right of it to the row's
//     accumulation buffer (dir * h * (c + 1 - xmid) to cell c, the rest of h to
//     cell c + 1; all of h to cell 0 left of the raster); the row prefix sum times
//     the figure's direction sign (fig_sign) is the winding-weighted area S of each
//     pixel; NonZero maps S to clamp(S, 0, 1) like imgbuf.rs:54-61 clamps the signed
//     sum, EvenOdd to the triangle wave of period 2 (imgbuf.rs:157-167).
//
// The gradient of S over the edge P0->P1 is the boundary integral
//   dS_p/dP0 = (-dy, dx) * int_{s in p} (1 - s) ds,  dS_p/dP1 = (-dy, dx) * int_{s in p} s ds
// over the part of the edge inside pixel p (pixels off the raster take nothing),
// chained to control points by the Bernstein weights of each vertex and the
// transpose of the transform's linear part.
#include <algorithm>
#include <cmath>
#include <climits>
#include <functional>
#include <cstdint>
#include <vector>

#include "../include/footile_gpu.h"
#include "../include/ft_fmath.h"

namespace adj {

struct F2 {
    float x, y;
};
static inline F2 fmidp(F2 a, F2 b) { return F2{(a.x + b.x) / 2.0f, (a.y + b.y) / 2.0f}; }
static inline float fdist_sq(F2 a, F2 b) {
    float dx = a.x - b.x, dy = a.y - b.y;
    return dx * dx + dy * dy;
}
static inline F2 fxform(const float* m, F2 p) {
    return F2{m[0] * p.x + m[1] * p.y + m[2], m[3] * p.x + m[4] * p.y + m[5]};
}
static inline bool ffinite(F2 p) { return std::isfinite(p.x) && std::isfinite(p.y); }

// Leaf end parameters of the quad subdivision of plotter.rs:248-265, in DFS order.
static void quad_tree(F2 a, F2 b, F2 c, float tol_sq, int depth, double t0, std::vector<double>& ts,
                      std::vector<F2>& pts, int& st) {
    F2 ab = fmidp(a, b), bc = fmidp(b, c), abbc = fmidp(ab, bc), ac = fmidp(a, c);
    bool within = fdist_sq(abbc, ac) <= tol_sq;
    if (within || depth >= FT_MAX_DEPTH) {
        if (!within) st = std::max(st, (int)FT_ERR_DEPTH);
        ts.push_back(t0 + std::ldexp(1.0, -depth));
        pts.push_back(c);
        return;
    }
    quad_tree(a, ab, abbc, tol_sq, depth + 1, t0, ts, pts, st);
    quad_tree(abbc, bc, c, tol_sq, depth + 1, t0 + std::ldexp(1.0, -depth - 1), ts, pts, st);
}

// The same for the cubic of plotter.rs:311-332.
static void cubic_tree(F2 a, F2 b, F2 c, F2 d, float tol_sq, int depth, double t0, std::vector<double>& ts,
                       std::vector<F2>& pts, int& st) {
    F2 ab = fmidp(a, b), bc = fmidp(b, c), cd = fmidp(c, d);
    F2 abbc = fmidp(ab, bc), bccd = fmidp(bc, cd), pe = fmidp(abbc, bccd), ad = fmidp(a, d);
    bool within = fdist_sq(pe, ad) <= tol_sq;
    if (within || depth >= FT_MAX_DEPTH) {
        if (!within) st = std::max(st, (int)FT_ERR_DEPTH);
        ts.push_back(t0 + std::ldexp(1.0, -depth));
        pts.push_back(d);
        return;
    }
    cubic_tree(a, ab, abbc, pe, tol_sq, depth + 1, t0, ts, pts, st);
    cubic_tree(pe, bccd, cd, d, tol_sq, depth + 1, t0 + std::ldexp(1.0, -depth - 1), ts, pts, st);
}

enum { V_POINT = 0, V_QUAD = 1, V_CUBIC = 2 };

struct Vert {
    int op;    // op that emitted the vertex
    int form;  // V_POINT (Move/Line, or the end point of a non-finite curve), V_QUAD, V_CUBIC
    double t;  // Bernstein parameter of the vertex on its segment
};

struct Poly {
    std::vector<Vert> v;
    std::vector<F2> f;         // the f32 point footile's Fig receives for each vertex
    std::vector<int> sub;      // first vertex of the vertex's sub-figure
    std::vector<int> pen_src;  // per op: the op whose end point starts a curve (-1: the origin)
    int sign = 1;              // +1 when Fig's direction is Forward (fig.rs:402-411), -1 Reverse
    int status = 0;
};

// fixed.rs:88-93 (f32 -> Fixed, Rust's saturating `as i32`) and Fixed mul (wrapping)
static inline int32_t fx_of(float f) {
    float v = f * 65536.0f;
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v < -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
static inline int32_t fx_mul(int32_t a, int32_t b) { return (int32_t)(uint32_t)(((int64_t)a * (int64_t)b) >> 16); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

struct FxP {
    int32_t x, y;
    bool operator==(const FxP& o) const { return x == o.x && y == o.y; }
    bool operator!=(const FxP& o) const { return !(*this == o); }
};

struct Poly;
static int fig_sign(const Poly& P);

// End-point slot (pair of floats) of a pen-setting op.
static inline int end_slot(int kind) { return kind == FT_OP_CUBIC ? 2 : (kind == FT_OP_QUAD ? 1 : 0); }

// The pen walk of plotter.rs:175-224 with the subdivision decided in f32.
static Poly build(const ft_op* ops, uint32_t n, const float* m, float tol_sq) {
    Poly P;
    P.pen_src.assign(n, -1);
    int pen = -1;  // op holding the pen (-1: the origin, after the call start and after Close)
    bool fresh = true;
    int sub_start = 0;
    auto emit = [&](int op, int form, double t, F2 f) {
        if (fresh) {
            sub_start = (int)P.v.size();
            fresh = false;
        }
        P.v.push_back(Vert{op, form, t});
        P.f.push_back(f);
        P.sub.push_back(sub_start);
    };
    auto ptf = [&](int j, int slot) { return F2{ops[j].v[2 * slot], ops[j].v[2 * slot + 1]}; };
    std::vector<double> ts;
    std::vector<F2> pts;
    for (uint32_t i = 0; i < n; i++) {
        const ft_op& o = ops[i];
        switch (o.kind) {
            case FT_OP_CLOSE:
                fresh = true;
                pen = -1;
                break;
            case FT_OP_MOVE:
                fresh = true;
                emit((int)i, V_POINT, 1.0, fxform(m, ptf(i, 0)));
                pen = (int)i;
                break;
            case FT_OP_LINE:
                emit((int)i, V_POINT, 1.0, fxform(m, ptf(i, 0)));
                pen = (int)i;
                break;
            case FT_OP_QUAD:
            case FT_OP_CUBIC: {
                P.pen_src[i] = pen;
                F2 a = fxform(m, pen < 0 ? F2{0.0f, 0.0f} : ptf(pen, end_slot(ops[pen].kind)));
                F2 b = fxform(m, ptf(i, 0)), c = fxform(m, ptf(i, 1));
                bool cubic = o.kind == FT_OP_CUBIC;
                F2 d = cubic ? fxform(m, ptf(i, 2)) : c;
                if (!ffinite(a) || !ffinite(b) || !ffinite(c) || !ffinite(d)) {
                    P.status = std::max(P.status, (int)FT_ERR_ARG);
                    emit((int)i, V_POINT, 1.0, d);
                } else {
                    ts.clear();
                    pts.clear();
                    if (cubic)
                        cubic_tree(a, b, c, d, tol_sq, 0, 0.0, ts, pts, P.status);
                    else
                        quad_tree(a, b, c, tol_sq, 0, 0.0, ts, pts, P.status);
                    for (size_t j = 0; j < ts.size(); j++) emit((int)i, cubic ? V_CUBIC : V_QUAD, ts[j], pts[j]);
                }
                pen = (int)i;
                break;
            }
            default:
                break;
        }
    }
    if (P.v.size() > FT_MAX_POINTS) P.status = std::max(P.status, (int)FT_ERR_CAP);
    P.sign = fig_sign(P);
    return P;
}

struct D2 {
    double x, y;
};

// What fixed.rs:88-93 makes of a coordinate, in pixels: NaN becomes 0 and values
// saturate at the ends of the 16.16 range.  Coordinates it changes take no gradient.
static inline double fx_range(double v) { return std::isnan(v) ? 0.0 : std::clamp(v, -32768.0, 32768.0); }
static inline D2 fx_range(D2 p) { return D2{fx_range(p.x), fx_range(p.y)}; }
static inline D2 fx_pass(D2 raw, D2 g) {
    return D2{fx_range(raw.x) == raw.x ? g.x : 0.0, fx_range(raw.y) == raw.y ? g.y : 0.0};
}

// Vertex positions in f64.  Without `val`: the f32 points of the De Casteljau walk, the
// polygon footile's Fig receives (and the CUDA coverage covers), widened to double.
// With `val` (6 per op, the layout of ft_op.v): the Bernstein points B(t) of the same
// tree, continuous in the control values (for finite differences).
static std::vector<D2> positions(const Poly& P, const ft_op* ops, const double* val, const double* m) {
    std::vector<D2> out(P.v.size());
    if (!val) {
        for (size_t k = 0; k < P.v.size(); k++) out[k] = D2{(double)P.f[k].x, (double)P.f[k].y};
        return out;  // raw: callers apply fx_range
    }
    auto cp = [&](int j, int slot) { return D2{val[6 * j + 2 * slot], val[6 * j + 2 * slot + 1]}; };
    for (size_t k = 0; k < P.v.size(); k++) {
        const Vert& v = P.v[k];
        int kind = ops[v.op].kind;
        D2 p;
        if (v.form == V_POINT) {
            p = cp(v.op, end_slot(kind));
        } else {
            int ps = P.pen_src[v.op];
            D2 a = ps < 0 ? D2{0.0, 0.0} : cp(ps, end_slot(ops[ps].kind));
            double t = v.t, u = 1.0 - t;
            if (v.form == V_QUAD) {
                D2 b = cp(v.op, 0), c = cp(v.op, 1);
                double w0 = u * u, w1 = 2 * t * u, w2 = t * t;
                p = D2{w0 * a.x + w1 * b.x + w2 * c.x, w0 * a.y + w1 * b.y + w2 * c.y};
            } else {
                D2 b = cp(v.op, 0), c = cp(v.op, 1), d = cp(v.op, 2);
                double w0 = u * u * u, w1 = 3 * t * u * u, w2 = 3 * t * t * u, w3 = t * t * t;
                p = D2{w0 * a.x + w1 * b.x + w2 * c.x + w3 * d.x, w0 * a.y + w1 * b.y + w2 * c.y + w3 * d.y};
            }
        }
        out[k] = D2{m[0] * p.x + m[1] * p.y + m[2], m[3] * p.x + m[4] * p.y + m[5]};
    }
    return out;
}

// The direction footile's Fig gives the figure (fig.rs:402-411, 493-494): the top vertex
// is the kept vertex with the least (y, x, id) in 16.16 after Fig::add_point drops
// points equal to the previous one and Fig::close drops a last point equal to its
// sub-figure's first (fig.rs:373-383, 428-451); its neighbours in the sub-figure
// decide widdershins with wrapping Fixed products.  Edges add +1 in that direction,
// and NonZero clamps the signed sum at 0 (imgbuf.rs:54-61), so the coverage of the
// analytic fill is clamp(sign * S, 0, 1).
static int fig_sign(const Poly& P) {
    const int n = (int)P.v.size();
    std::vector<FxP> q(n);
    for (int k = 0; k < n; k++) q[k] = FxP{fx_of(P.f[k].x), fx_of(P.f[k].y)};
    std::vector<int> sub_end(n, -1);  // last raw vertex of each sub-figure, at its first vertex
    std::vector<char> single(n, 1);   // every raw vertex of the sub-figure equals its first
    for (int k = 0; k < n; k++) {
        sub_end[P.sub[k]] = k;
        if (q[k] != q[P.sub[k]]) single[P.sub[k]] = 0;
    }
    int top = -1;
    for (int k = 0; k < n; k++) {
        const int s0 = P.sub[k];
        const bool kept = k == s0 || q[k] != q[k - 1];
        if (!kept || single[s0]) continue;
        if (top < 0 || q[k].y < q[top].y || (q[k].y == q[top].y && q[k].x < q[top].x)) top = k;
    }
    if (top < 0) return 1;
    const int s0 = P.sub[top], e = sub_end[s0];
    FxP nxt = q[s0];
    for (int j = top + 1; j <= e; j++)
        if (q[j] != q[top]) {
            nxt = q[j];
            break;
        }
    FxP prv = q[top];
    if (top > s0) {
        prv = q[top - 1];
    } else {
        for (int j = e; j > s0; j--)
            if (q[j] != q[s0]) {
                prv = q[j];
                break;
            }
    }
    const FxP t = q[top];
    const int32_t ax = wsub(prv.x, t.x), ay = wsub(prv.y, t.y);  // p1 - p (Reverse neighbour)
    const int32_t bx = wsub(nxt.x, t.x), by = wsub(nxt.y, t.y);  // p0 - p (Forward neighbour)
    return fx_mul(ax, by) > fx_mul(bx, ay) ? 1 : -1;
}

static inline int next_vertex(const Poly& P, int k) {
    int n = (int)P.v.size();
    return (k + 1 < n && P.sub[k + 1] == P.sub[k]) ? k + 1 : P.sub[k];
}

// Pieces of the edge P0->P1 per raster row and cell column.  cb(row, cell, h, xmid, u0, u1):
// the piece of height h (> 0) in the cell, with mean x xmid and parameter range [u0, u1]
// along the edge taken top to bottom; cell -1 stands for everything left of the raster.
template <class CB>
static void edge_pieces(D2 p0, D2 p1, int W, int H, CB cb) {
    if (p0.y == p1.y) return;
    D2 a = p0.y < p1.y ? p0 : p1, b = p0.y < p1.y ? p1 : p0;
    double dy = b.y - a.y, dxdy = (b.x - a.x) / dy;
    double xlo = std::min(a.x, b.x), xhi = std::max(a.x, b.x);
    double r0d = std::max(0.0, std::floor(a.y)), r1d = std::min((double)H - 1, std::ceil(b.y) - 1);
    if (!(r0d <= r1d)) return;
    for (int r = (int)r0d; r <= (int)r1d; r++) {
        double yt = std::max(a.y, (double)r), yb = std::min(b.y, (double)r + 1);
        if (yb <= yt) continue;
        double xt = yt == a.y ? a.x : std::clamp(a.x + (yt - a.y) * dxdy, xlo, xhi);
        double xb = yb == b.y ? b.x : std::clamp(a.x + (yb - a.y) * dxdy, xlo, xhi);
        double ut = (yt - a.y) / dy, ub = (yb - a.y) / dy, h = yb - yt;
        double xl = std::min(xt, xb), xr = std::max(xt, xb);
        bool rising = xt <= xb;  // x grows with u
        double cl = std::floor(xl), cr = std::floor(xr);
        if (cl == cr || xr == xl) {
            cb(r, cl < 0 ? -1 : (int)std::min(cl, (double)W), h, 0.5 * (xl + xr), ut, ub);
            continue;
        }
        double span = xr - xl;
        auto piece = [&](double x0, double x1, int c) {
            double f0 = (x0 - xl) / span, f1 = (x1 - xl) / span;
            double u0 = rising ? ut + f0 * (ub - ut) : ub - f1 * (ub - ut);
            double u1 = rising ? ut + f1 * (ub - ut) : ub - f0 * (ub - ut);
            cb(r, c, (f1 - f0) * h, 0.5 * (x0 + x1), u0, u1);
        };
        double c = cl;
        if (c < 0) {
            double x1 = std::min(xr, 0.0);
            if (x1 > xl) piece(xl, x1, -1);
            c = 0;
        }
        for (; c <= cr && c < W; c += 1) {
            double x0 = std::max(xl, c), x1 = std::min(xr, c + 1);
            if (x1 > x0) piece(x0, x1, (int)c);
        }
    }
}

static inline double coverage(int rule, double s) {
    if (rule == FT_NONZERO) return std::clamp(s, 0.0, 1.0);
    double m = s - 2.0 * std::floor(s / 2.0);
    return m <= 1.0 ? m : 2.0 - m;
}
static inline double coverage_d(int rule, double s) {
    if (rule == FT_NONZERO) return s > 0.0 && s < 1.0 ? 1.0 : 0.0;
    double m = s - 2.0 * std::floor(s / 2.0);
    return m < 1.0 ? 1.0 : -1.0;
}

// Coverage of a polygon (positions `pos`, sub-figures and sign of P): area and cov.
static void cover(const Poly& P, const std::vector<D2>& pos, int rule, uint32_t w, uint32_t h, double* cov,
                  double* area) {
    std::vector<double> acc((size_t)w * h, 0.0);
    for (int k = 0; k < (int)pos.size(); k++) {
        D2 p0 = pos[k], p1 = pos[next_vertex(P, k)];
        double dir = p1.y > p0.y ? 1.0 : -1.0;
        edge_pieces(p0, p1, (int)w, (int)h, [&](int r, int c, double hh, double xm, double, double) {
            double* row = &acc[(size_t)r * w];
            if (c < 0) {
                row[0] += dir * hh;
            } else if (c < (int)w) {
                row[c] += dir * hh * (c + 1 - xm);
                if (c + 1 < (int)w) row[c + 1] += dir * hh * (xm - c);
            }
        });
    }
    const double sg = P.sign;
    for (uint32_t r = 0; r < h; r++) {
        double s = 0.0;
        for (uint32_t c = 0; c < w; c++) {
            s += sg * acc[(size_t)r * w + c];
            if (area) area[(size_t)r * w + c] = s;
            cov[(size_t)r * w + c] = coverage(rule, s);
        }
    }
}

// Gradient of sum(grad_cov * cov) with respect to the polygon's vertex positions.
static std::vector<D2> vertex_grads(const Poly& P, const std::vector<D2>& pos, int rule, uint32_t w, uint32_t h,
                                    const double* area, const double* grad_cov) {
    std::vector<double> gs((size_t)w * h);
    for (size_t i = 0; i < gs.size(); i++) gs[i] = P.sign * grad_cov[i] * coverage_d(rule, area[i]);
    std::vector<D2> gp(pos.size(), D2{0.0, 0.0});
    for (int k = 0; k < (int)pos.size(); k++) {
        int nk = next_vertex(P, k);
        D2 p0 = pos[k], p1 = pos[nk];
        bool down = p1.y > p0.y;  // P0 is the top end: s = u
        double ga = 0.0, gb = 0.0;
        edge_pieces(p0, p1, (int)w, (int)h, [&](int r, int c, double, double, double u0, double u1) {
            if (c < 0 || c >= (int)w) return;
            double g = gs[(size_t)r * w + c];
            double i1 = u1 - u0, iu = 0.5 * (u1 * u1 - u0 * u0);
            if (down) {
                ga += g * (i1 - iu);
                gb += g * iu;
            } else {
                ga += g * iu;
                gb += g * (i1 - iu);
            }
        });
        double px = -(p1.y - p0.y), py = p1.x - p0.x;
        gp[k].x += px * ga;
        gp[k].y += py * ga;
        gp[nk].x += px * gb;
        gp[nk].y += py * gb;
    }
    return gp;
}

struct Setup {
    Poly P;
    std::vector<double> val;
    bool bernstein = false;
    double m[6];
};

static Setup setup(const ft_op* ops, uint32_t n, const double* val, const float* xf, float tol) {
    Setup S;
    float t = std::max(tol, 0.01f);
    S.P = build(ops, n, xf, t * t);
    S.bernstein = val != nullptr;
    S.val.resize(6 * (size_t)n);
    for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < 6; k++) S.val[6 * i + k] = val ? val[6 * i + k] : (double)ops[i].v[k];
    for (int k = 0; k < 6; k++) S.m[k] = xf[k];
    return S;
}


// ===================================================================== strokes
// The stroke of Plotter::stroke (plotter.rs:356-365): stroke points from the pen walk
// with widths (stroker.rs:204-236), the outline of each sub-stroke (stroker.rs:239-416)
// and the fill of that outline, NonZero, transformed a second time.  The f32 pass
// makes footile's decisions (coincident points, joins, miter limit, arc subdivision)
// and records each outline point as a node over the stroke points: an offset point,
// a miter intersection or an arc point.  The nodes are then evaluated and
// differentiated in double with the decisions held.

static inline F2 f2sub(F2 a, F2 b) { return F2{a.x - b.x, a.y - b.y}; }
static inline F2 f2add(F2 a, F2 b) { return F2{a.x + b.x, a.y + b.y}; }
static inline F2 f2mul(F2 a, float s) { return F2{a.x * s, a.y * s}; }
static inline F2 f2right(F2 v) { return F2{v.y, -v.x}; }
static inline F2 f2norm(F2 v) {
    float m = sqrtf(v.x * v.x + v.y * v.y);
    return F2{v.x / m, v.y / m};
}
static inline bool f2line_x(F2 a0, F2 a1, F2 b0, F2 b1, F2* out) {
    float x1 = a0.x, y1 = a0.y, x2 = a1.x, y2 = a1.y, x3 = b0.x, y3 = b0.y, x4 = b1.x, y4 = b1.y;
    float den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
    if (den == 0.0f) return false;
    float a = x1 * y2 - y1 * x2, b = x3 * y4 - y3 * x4;
    *out = F2{(a * (x3 - x4) - (x1 - x2) * b) / den, (a * (y3 - y4) - (y1 - y2) * b) / den};
    return true;
}

struct WP {
    F2 p;
    float w;
};
static inline WP wpmid(WP a, WP b) { return WP{fmidp(a.p, b.p), (a.w + b.w) / 2.0f}; }

// Leaves of the width-carrying subdivision (the same tree as quad_tree / cubic_tree).
static void quad_wtree(WP a, WP b, WP c, float tol_sq, int depth, double t0, std::vector<double>& ts,
                       std::vector<WP>& pts, int& st) {
    WP ab = wpmid(a, b), bc = wpmid(b, c), abbc = wpmid(ab, bc), ac = wpmid(a, c);
    bool within = fdist_sq(abbc.p, ac.p) <= tol_sq;
    if (within || depth >= FT_MAX_DEPTH) {
        if (!within) st = std::max(st, (int)FT_ERR_DEPTH);
        ts.push_back(t0 + std::ldexp(1.0, -depth));
        pts.push_back(c);
        return;
    }
    quad_wtree(a, ab, abbc, tol_sq, depth + 1, t0, ts, pts, st);
    quad_wtree(abbc, bc, c, tol_sq, depth + 1, t0 + std::ldexp(1.0, -depth - 1), ts, pts, st);
}
static void cubic_wtree(WP a, WP b, WP c, WP d, float tol_sq, int depth, double t0, std::vector<double>& ts,
                        std::vector<WP>& pts, int& st) {
    WP ab = wpmid(a, b), bc = wpmid(b, c), cd = wpmid(c, d);
    WP abbc = wpmid(ab, bc), bccd = wpmid(bc, cd), pe = wpmid(abbc, bccd), ad = wpmid(a, d);
    bool within = fdist_sq(pe.p, ad.p) <= tol_sq;
    if (within || depth >= FT_MAX_DEPTH) {
        if (!within) st = std::max(st, (int)FT_ERR_DEPTH);
        ts.push_back(t0 + std::ldexp(1.0, -depth));
        pts.push_back(d);
        return;
    }
    cubic_wtree(a, ab, abbc, pe, tol_sq, depth + 1, t0, ts, pts, st);
    cubic_wtree(pe, bccd, cd, d, tol_sq, depth + 1, t0 + std::ldexp(1.0, -depth - 1), ts, pts, st);
}

enum { N_OFF = 0, N_MITER = 1, N_ARC = 2 };
struct SNode {
    int kind;
    int a, b, c, d;  // OFF: stroke points a -> b, c = 0 offsets a, 1 offsets b; MITER: nodes a0 a1 b0 b1;
                     // ARC: stroke point a (centre, width), nodes b (from) and c (to)
    F2 f;            // f32 value (footile's outline point)
};

struct StrokeFig {
    Poly cl;                  // stroke points (provenance, f32 points in cl.f)
    std::vector<float> wf;    // f32 widths of the stroke points
    std::vector<int> wsrc0;   // width source of the curve start (PenWidth op, -1: the call's width)
    std::vector<int> wsrc1;   // width source of the op's own width
    std::vector<SNode> nodes;
    std::vector<int> verts;   // outline vertex -> node
    Poly fig;                 // the outline polygon as the fill sees it (f32, transformed again)
    int status = 0;
};

static StrokeFig build_stroke(const ft_op* ops, uint32_t n, const float* m, float tol_sq, int join, float ml,
                              float sw0) {
    StrokeFig S;
    Poly& P = S.cl;
    P.pen_src.assign(n, -1);
    float sw = sw0;
    int cur_pw = -1;                // PenWidth op in force
    int pen = -1, pen_wsrc = -1;    // op holding the pen, width source of the pen
    WP penp{F2{0.0f, 0.0f}, sw0};
    struct Sub {
        int start, n;
        bool joined, done;
    };
    std::vector<Sub> subs{Sub{0, 0, false, false}};
    auto close = [&](bool joined) {
        if (!P.v.empty()) {
            subs.back().joined = joined;
            subs.back().done = true;
        }
    };
    auto add = [&](WP q, int op, int form, double t, int w0, int w1) {  // Stroke::add_point
        if (P.v.size() >= FT_MAX_POINTS) return;
        bool done = subs.back().done;
        if (done) subs.push_back(Sub{(int)P.v.size(), 0, false, false});
        bool coincident = !P.f.empty() && P.f.back().x == q.p.x && P.f.back().y == q.p.y;
        if (done || !coincident) {
            P.v.push_back(Vert{op, form, t});
            P.f.push_back(q.p);
            P.sub.push_back(subs.back().start);
            S.wf.push_back(q.w);
            S.wsrc0.push_back(w0);
            S.wsrc1.push_back(w1);
            subs.back().n++;
        }
    };
    auto ptf = [&](int j, int slot) { return F2{ops[j].v[2 * slot], ops[j].v[2 * slot + 1]}; };
    std::vector<double> ts;
    std::vector<WP> pts;
    for (uint32_t i = 0; i < n; i++) {
        const ft_op& o = ops[i];
        switch (o.kind) {
            case FT_OP_CLOSE:
                close(true);
                pen = -1;
                pen_wsrc = cur_pw;
                penp = WP{F2{0.0f, 0.0f}, sw};
                break;
            case FT_OP_MOVE:
            case FT_OP_LINE: {
                WP q{ptf(i, 0), sw};
                if (o.kind == FT_OP_MOVE) close(false);
                add(WP{fxform(m, q.p), q.w}, (int)i, V_POINT, 1.0, cur_pw, cur_pw);
                pen = (int)i;
                pen_wsrc = cur_pw;
                penp = q;
                break;
            }
            case FT_OP_QUAD:
            case FT_OP_CUBIC: {
                P.pen_src[i] = pen;
                const bool cubic = o.kind == FT_OP_CUBIC;
                WP a{fxform(m, penp.p), penp.w}, b, c, d;
                if (cubic) {
                    float w0 = sw + (penp.w - sw) * (1.0f / 3.0f);  // float_lerp, geom.rs:14-16
                    float w1 = sw + (penp.w - sw) * (2.0f / 3.0f);
                    b = WP{fxform(m, ptf(i, 0)), w0};
                    c = WP{fxform(m, ptf(i, 1)), w1};
                    d = WP{fxform(m, ptf(i, 2)), sw};
                } else {
                    b = WP{fxform(m, ptf(i, 0)), (penp.w + sw) / 2.0f};
                    c = WP{fxform(m, ptf(i, 1)), sw};
                    d = c;
                }
                if (!ffinite(a.p) || !ffinite(b.p) || !ffinite(c.p) || !ffinite(d.p)) {
                    S.status = std::max(S.status, (int)FT_ERR_ARG);
                    add(d, (int)i, V_POINT, 1.0, cur_pw, cur_pw);
                } else {
                    ts.clear();
                    pts.clear();
                    if (cubic)
                        cubic_wtree(a, b, c, d, tol_sq, 0, 0.0, ts, pts, S.status);
                    else
                        quad_wtree(a, b, c, tol_sq, 0, 0.0, ts, pts, S.status);
                    for (size_t j = 0; j < ts.size(); j++)
                        add(pts[j], (int)i, cubic ? V_CUBIC : V_QUAD, ts[j], pen_wsrc, cur_pw);
                }
                pen = (int)i;
                pen_wsrc = cur_pw;
                penp = WP{cubic ? ptf(i, 2) : ptf(i, 1), sw};
                break;
            }
            case FT_OP_PEN_WIDTH:
                sw = o.v[0];
                cur_pw = (int)i;
                break;
            default:
                break;
        }
    }
    // outline (stroker.rs:239-295)
    std::vector<char> is_close;  // per outline op: 1 = Close
    auto emit = [&](int node) {
        S.verts.push_back(node);
        is_close.push_back(0);
    };
    auto emit_close = [&]() {
        S.verts.push_back(-1);
        is_close.push_back(1);
    };
    auto off = [&](int k0, int k1, int which) {
        F2 vr = f2norm(f2right(f2sub(P.f[k1], P.f[k0])));
        int ks = which ? k1 : k0;
        F2 v = f2add(P.f[ks], f2mul(vr, S.wf[ks] / 2.0f));
        S.nodes.push_back(SNode{N_OFF, k0, k1, which, 0, v});
        return (int)S.nodes.size() - 1;
    };
    std::function<void(int, int, int, int)> arc = [&](int k, int na, int nb, int depth) {
        F2 a = S.nodes[na].f, b = S.nodes[nb].f;
        F2 vr = f2norm(f2right(f2sub(b, a)));
        F2 c = f2add(P.f[k], f2mul(vr, S.wf[k] / 2.0f));
        F2 ab = fmidp(a, b);
        if (!ffinite(c) || fdist_sq(c, ab) <= tol_sq) {
            emit(nb);
        } else if (depth >= FT_MAX_DEPTH) {
            S.status = std::max(S.status, (int)FT_ERR_DEPTH);
            emit(nb);
        } else {
            S.nodes.push_back(SNode{N_ARC, k, na, nb, 0, c});
            int nc = (int)S.nodes.size() - 1;
            arc(k, na, nc, depth + 1);
            arc(k, nc, nb, depth + 1);
        }
    };
    auto do_join = [&](int k, int a0, int a1, int b0, int b1) {
        F2 A0 = S.nodes[a0].f, A1 = S.nodes[a1].f, B0 = S.nodes[b0].f, B1 = S.nodes[b1].f;
        if (join == FT_JOIN_MITER) {
            // footile's decision as a correctly rounded f32 libm takes it (ft_fmath.h)
            const F2 u = f2sub(A1, A0), v = f2sub(B0, B1);
            {
                F2 xp;
                if (ft_miter_join(u.x, u.y, v.x, v.y, ft_miter_angle(ml)) && f2line_x(A0, A1, B0, B1, &xp)) {
                    S.nodes.push_back(SNode{N_MITER, a0, a1, b0, b1, xp});
                    emit((int)S.nodes.size() - 1);
                    return;
                }
            }
            emit(a1);
            emit(b0);
        } else if (join == FT_JOIN_BEVEL) {
            emit(a1);
            emit(b0);
        } else {
            const F2 u = f2sub(A1, A0), v = f2sub(B0, B1);
            if (!ft_round_join_arc(u.x, u.y, v.x, v.y)) {
                emit(a1);
                emit(b0);
            } else {
                emit(a1);
                arc(k, a1, b0, 0);
            }
        }
    };
    for (const Sub& sb : subs) {
        const int len = sb.joined ? sb.n + 1 : (sb.n > 0 ? sb.n - 1 : 0);  // SubStroke::len (u16)
        const int lenw = len & 0xFFFF;
        if (lenw == 0) continue;
        auto nextv = [&](int v, bool fwd) {
            if (fwd) return v + 1 < sb.start + sb.n ? v + 1 : sb.start;
            return v > sb.start ? v - 1 : sb.start + sb.n - 1;
        };
        for (int side = 0; side < 2; side++) {
            const bool fwd = side == 0;
            int v0 = fwd ? sb.start : nextv(sb.start, false);
            int v1 = nextv(v0, fwd);
            bool have = false;
            int x0 = -1, x1 = -1;
            for (int k = 0; k < lenw; k++) {
                int o0 = off(v0, v1, 0), o1 = off(v0, v1, 1);
                if (have)
                    do_join(v0, x0, x1, o0, o1);
                else if (!sb.joined)
                    emit(o0);
                have = true;
                x0 = o0;
                x1 = o1;
                v0 = v1;
                v1 = nextv(v1, fwd);
            }
            if (!sb.joined && have) emit(x1);
            if (fwd && sb.joined) emit_close();
        }
        emit_close();
    }
    // the fill of the outline: Line points transformed again, sub-figures between Closes
    Poly& F = S.fig;
    bool fresh = true;
    int sub_start = 0;
    std::vector<int> vmap;
    for (size_t j = 0; j < S.verts.size(); j++) {
        if (is_close[j]) {
            fresh = true;
            continue;
        }
        if (fresh) {
            sub_start = (int)F.v.size();
            fresh = false;
        }
        F.v.push_back(Vert{S.verts[j], V_POINT, 1.0});
        F.f.push_back(fxform(m, S.nodes[S.verts[j]].f));
        F.sub.push_back(sub_start);
    }
    if (F.v.size() > FT_MAX_POINTS) S.status = std::max(S.status, (int)FT_ERR_CAP);
    F.sign = fig_sign(F);
    return S;
}

struct StrokeEval {
    std::vector<D2> P;   // stroke points (transformed once)
    std::vector<double> W;
    std::vector<D2> N;   // node values
    std::vector<D2> V;   // outline vertices (transformed again)
};

static inline D2 d2right(D2 v) { return D2{v.y, -v.x}; }

// Node values in double from stroke points (P, W).
static void eval_nodes(const StrokeFig& S, StrokeEval& E) {
    E.N.resize(S.nodes.size());
    for (size_t i = 0; i < S.nodes.size(); i++) {
        const SNode& nd = S.nodes[i];
        if (nd.kind == N_OFF || nd.kind == N_ARC) {
            D2 from = nd.kind == N_OFF ? E.P[nd.a] : E.N[nd.b];
            D2 to = nd.kind == N_OFF ? E.P[nd.b] : E.N[nd.c];
            D2 u = d2right(D2{to.x - from.x, to.y - from.y});
            double len = std::sqrt(u.x * u.x + u.y * u.y);
            D2 vr{u.x / len, u.y / len};
            int ks = nd.kind == N_OFF ? (nd.c ? nd.b : nd.a) : nd.a;
            E.N[i] = D2{E.P[ks].x + vr.x * E.W[ks] / 2, E.P[ks].y + vr.y * E.W[ks] / 2};
        } else {
            D2 a0 = E.N[nd.a], a1 = E.N[nd.b], b0 = E.N[nd.c], b1 = E.N[nd.d];
            double x1 = a0.x, y1 = a0.y, x2 = a1.x, y2 = a1.y, x3 = b0.x, y3 = b0.y, x4 = b1.x, y4 = b1.y;
            double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
            double a = x1 * y2 - y1 * x2, b = x3 * y4 - y3 * x4;
            E.N[i] = D2{(a * (x3 - x4) - (x1 - x2) * b) / den, (a * (y3 - y4) - (y1 - y2) * b) / den};
        }
    }
}

// Stroke points, nodes and outline in double.  Without `val`: footile's f32 stroke
// points and outline widened (the polygon the CUDA path covers); with `val` (6 per
// op) and `sw0`: Bernstein points and linear widths of the held tree.
static StrokeEval evaluate(const StrokeFig& S, const ft_op* ops, const double* val, double sw0, const double* m) {
    StrokeEval E;
    const size_t ns = S.cl.v.size();
    E.P.resize(ns);
    E.W.resize(ns);
    if (!val) {
        for (size_t k = 0; k < ns; k++) {
            E.P[k] = D2{(double)S.cl.f[k].x, (double)S.cl.f[k].y};
            E.W[k] = S.wf[k];
        }
    } else {
        E.P = positions(S.cl, ops, val, m);
        auto wv = [&](int src) { return src < 0 ? sw0 : val[6 * src]; };
        for (size_t k = 0; k < ns; k++) {
            const Vert& v = S.cl.v[k];
            E.W[k] = v.form == V_POINT ? wv(S.wsrc1[k]) : (1.0 - v.t) * wv(S.wsrc0[k]) + v.t * wv(S.wsrc1[k]);
        }
    }
    eval_nodes(S, E);
    E.V.resize(S.fig.v.size());
    for (size_t j = 0; j < S.fig.v.size(); j++) {
        if (!val) {
            E.V[j] = D2{(double)S.fig.f[j].x, (double)S.fig.f[j].y};
        } else {
            D2 q = E.N[S.fig.v[j].op];
            E.V[j] = D2{m[0] * q.x + m[1] * q.y + m[2], m[3] * q.x + m[4] * q.y + m[5]};
        }
    }
    return E;
}

// Reverse pass over the nodes: outline vertex gradients gV -> stroke point position
// and width gradients (gP, gW).
static void backprop_nodes(const StrokeFig& S, const StrokeEval& E, const std::vector<D2>& gV, const double* m,
                           std::vector<D2>& gP, std::vector<double>& gW) {
    std::vector<D2> gN(S.nodes.size(), D2{0.0, 0.0});
    for (size_t j = 0; j < gV.size(); j++) {
        D2& g = gN[S.fig.v[j].op];
        g.x += m[0] * gV[j].x + m[3] * gV[j].y;
        g.y += m[1] * gV[j].x + m[4] * gV[j].y;
    }
    gP.assign(E.P.size(), D2{0.0, 0.0});
    gW.assign(E.P.size(), 0.0);
    for (int i = (int)S.nodes.size() - 1; i >= 0; i--) {
        const SNode& nd = S.nodes[i];
        const D2 g = gN[i];
        if (g.x == 0.0 && g.y == 0.0) continue;
        if (nd.kind == N_OFF || nd.kind == N_ARC) {
            D2 from = nd.kind == N_OFF ? E.P[nd.a] : E.N[nd.b];
            D2 to = nd.kind == N_OFF ? E.P[nd.b] : E.N[nd.c];
            D2 u = d2right(D2{to.x - from.x, to.y - from.y});
            double len = std::sqrt(u.x * u.x + u.y * u.y);
            D2 vr{u.x / len, u.y / len};
            int ks = nd.kind == N_OFF ? (nd.c ? nd.b : nd.a) : nd.a;
            gP[ks].x += g.x;
            gP[ks].y += g.y;
            gW[ks] += 0.5 * (vr.x * g.x + vr.y * g.y);
            D2 gvr{g.x * E.W[ks] / 2, g.y * E.W[ks] / 2};
            double dv = vr.x * gvr.x + vr.y * gvr.y;
            D2 gu{(gvr.x - vr.x * dv) / len, (gvr.y - vr.y * dv) / len};
            D2 gd{-gu.y, gu.x};  // u = (d.y, -d.x)
            if (nd.kind == N_OFF) {
                gP[nd.b].x += gd.x;
                gP[nd.b].y += gd.y;
                gP[nd.a].x -= gd.x;
                gP[nd.a].y -= gd.y;
            } else {
                gN[nd.c].x += gd.x;
                gN[nd.c].y += gd.y;
                gN[nd.b].x -= gd.x;
                gN[nd.b].y -= gd.y;
            }
        } else {
            D2 a0 = E.N[nd.a], a1 = E.N[nd.b], b0 = E.N[nd.c], b1 = E.N[nd.d];
            double x1 = a0.x, y1 = a0.y, x2 = a1.x, y2 = a1.y, x3 = b0.x, y3 = b0.y, x4 = b1.x, y4 = b1.y;
            double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
            double a = x1 * y2 - y1 * x2, b = x3 * y4 - y3 * x4;
            double x = (a * (x3 - x4) - (x1 - x2) * b) / den, y = (a * (y3 - y4) - (y1 - y2) * b) / den;
            double gNx = g.x / den, gNy = g.y / den, gden = -(g.x * x + g.y * y) / den;
            double ga = gNx * (x3 - x4) + gNy * (y3 - y4), gb = -gNx * (x1 - x2) - gNy * (y1 - y2);
            double gx1 = -gNx * b + ga * y2 + gden * (y3 - y4);
            double gx2 = gNx * b - ga * y1 - gden * (y3 - y4);
            double gy1 = -gNy * b - ga * x2 - gden * (x3 - x4);
            double gy2 = gNy * b + ga * x1 + gden * (x3 - x4);
            double gx3 = gNx * a + gb * y4 - gden * (y1 - y2);
            double gx4 = -gNx * a - gb * y3 + gden * (y1 - y2);
            double gy3 = gNy * a - gb * x4 + gden * (x1 - x2);
            double gy4 = -gNy * a + gb * x3 - gden * (x1 - x2);
            gN[nd.a].x += gx1;
            gN[nd.a].y += gy1;
            gN[nd.b].x += gx2;
            gN[nd.b].y += gy2;
            gN[nd.c].x += gx3;
            gN[nd.c].y += gy3;
            gN[nd.d].x += gx4;
            gN[nd.d].y += gy4;
        }
    }
}

}  // namespace adj

extern "C" {

// Forward: winding area S and coverage of every pixel (row-major w x h doubles).
// Without `val` the polygon is footile's f32 flattened polygon; with `val` (6 doubles
// per op) its vertices are the Bernstein points of `val` on the subdivision tree the
// op floats decide.  Returns the status
// (FT_ERR_CAP: more than 65,535 vertices, coverage left zero).
__attribute__((visibility("default"))) int orc_adj_forward(int32_t rule, const ft_op* ops, uint32_t n_ops,
                                                           const double* val, uint32_t w, uint32_t h, float tol,
                                                           const float* xf, double* cov, double* area) {
    adj::Setup S = adj::setup(ops, n_ops, val, xf, tol);
    std::vector<adj::D2> pos;
    if (S.P.status != FT_ERR_CAP) pos = adj::positions(S.P, ops, S.bernstein ? S.val.data() : nullptr, S.m);
    for (adj::D2& q : pos) q = adj::fx_range(q);
    adj::cover(S.P, pos, rule, w, h, cov, area);
    return S.P.status;
}

// Backward: gradient of sum(grad_cov * cov) with respect to the control values
// (6 per op, accumulated into grad_val), given the forward's winding area.
__attribute__((visibility("default"))) int orc_adj_backward(int32_t rule, const ft_op* ops, uint32_t n_ops,
                                                            const double* val, uint32_t w, uint32_t h, float tol,
                                                            const float* xf, const double* area,
                                                            const double* grad_cov, double* grad_val) {
    adj::Setup S = adj::setup(ops, n_ops, val, xf, tol);
    if (S.P.status == FT_ERR_CAP) return S.P.status;
    std::vector<adj::D2> raw = adj::positions(S.P, ops, S.bernstein ? S.val.data() : nullptr, S.m), pos = raw;
    for (adj::D2& q : pos) q = adj::fx_range(q);
    std::vector<adj::D2> gp = adj::vertex_grads(S.P, pos, rule, w, h, area, grad_cov);
    for (size_t k = 0; k < gp.size(); k++) gp[k] = adj::fx_pass(raw[k], gp[k]);
    for (size_t k = 0; k < pos.size(); k++) {
        const adj::Vert& v = S.P.v[k];
        // back through the transform's linear part
        double gx = S.m[0] * gp[k].x + S.m[3] * gp[k].y, gy = S.m[1] * gp[k].x + S.m[4] * gp[k].y;
        auto add = [&](int j, int slot, double wgt) {
            grad_val[6 * j + 2 * slot] += wgt * gx;
            grad_val[6 * j + 2 * slot + 1] += wgt * gy;
        };
        int kind = ops[v.op].kind;
        if (v.form == adj::V_POINT) {
            add(v.op, adj::end_slot(kind), 1.0);
            continue;
        }
        double t = v.t, u = 1.0 - t;
        int ps = S.P.pen_src[v.op];
        if (v.form == adj::V_QUAD) {
            if (ps >= 0) add(ps, adj::end_slot(ops[ps].kind), u * u);
            add(v.op, 0, 2 * t * u);
            add(v.op, 1, t * t);
        } else {
            if (ps >= 0) add(ps, adj::end_slot(ops[ps].kind), u * u * u);
            add(v.op, 0, 3 * t * u * u);
            add(v.op, 1, 3 * t * t * u);
            add(v.op, 2, t * t * t);
        }
    }
    return S.P.status;
}

}  // extern "C"

extern "C" {

// Stroke forward: coverage of Plotter::stroke's outline (the same as orc_adj_forward
// for fills).  `sw0` is the pen width at the call's start.  `val` (6 per op, may be
// NULL): Bernstein stroke points and linear widths of the held tree, the PenWidth
// widths taken from val[6 * op].
__attribute__((visibility("default"))) int orc_adj_stroke_forward(const ft_op* ops, uint32_t n_ops, const double* val,
                                                                  double sw0, uint32_t w, uint32_t h, float tol,
                                                                  const float* xf, int32_t join, float ml,
                                                                  double* cov, double* area) {
    const float t = std::max(tol, 0.01f);
    adj::StrokeFig S = adj::build_stroke(ops, n_ops, xf, t * t, join, ml, (float)sw0);
    double m[6];
    for (int k = 0; k < 6; k++) m[k] = xf[k];
    std::vector<adj::D2> pos;
    if (S.status != FT_ERR_CAP) pos = adj::evaluate(S, ops, val, sw0, m).V;
    for (adj::D2& q : pos) q = adj::fx_range(q);
    adj::cover(S.fig, pos, FT_NONZERO, w, h, cov, area);
    return S.status;
}

// Stroke backward: d(sum(grad_cov * cov)) / d(op floats) into grad_val (6 per op;
// PenWidth ops in slot 0) and / d(sw0) into *grad_sw0.
__attribute__((visibility("default"))) int orc_adj_stroke_backward(const ft_op* ops, uint32_t n_ops, const double* val,
                                                                   double sw0, uint32_t w, uint32_t h, float tol,
                                                                   const float* xf, int32_t join, float ml,
                                                                   const double* area, const double* grad_cov,
                                                                   double* grad_val, double* grad_sw0) {
    const float t = std::max(tol, 0.01f);
    adj::StrokeFig S = adj::build_stroke(ops, n_ops, xf, t * t, join, ml, (float)sw0);
    if (S.status == FT_ERR_CAP) return S.status;
    double m[6];
    for (int k = 0; k < 6; k++) m[k] = xf[k];
    adj::StrokeEval E = adj::evaluate(S, ops, val, sw0, m);
    std::vector<adj::D2> pos = E.V;
    for (adj::D2& q : pos) q = adj::fx_range(q);
    std::vector<adj::D2> gV = adj::vertex_grads(S.fig, pos, FT_NONZERO, w, h, area, grad_cov);
    for (size_t j = 0; j < gV.size(); j++) gV[j] = adj::fx_pass(E.V[j], gV[j]);
    std::vector<adj::D2> gP;
    std::vector<double> gW;
    adj::backprop_nodes(S, E, gV, m, gP, gW);
    auto gw = [&](int src, double g) {
        if (src < 0) {
            if (grad_sw0) *grad_sw0 += g;
        } else {
            grad_val[6 * src] += g;
        }
    };
    for (size_t k = 0; k < gP.size(); k++) {
        const adj::Vert& v = S.cl.v[k];
        double gx = m[0] * gP[k].x + m[3] * gP[k].y, gy = m[1] * gP[k].x + m[4] * gP[k].y;
        auto add = [&](int j, int slot, double wgt) {
            grad_val[6 * j + 2 * slot] += wgt * gx;
            grad_val[6 * j + 2 * slot + 1] += wgt * gy;
        };
        int kind = ops[v.op].kind;
        if (v.form == adj::V_POINT) {
            add(v.op, adj::end_slot(kind), 1.0);
            gw(S.wsrc1[k], gW[k]);
            continue;
        }
        double tt = v.t, u = 1.0 - tt;
        int ps = S.cl.pen_src[v.op];
        if (v.form == adj::V_QUAD) {
            if (ps >= 0) add(ps, adj::end_slot(ops[ps].kind), u * u);
            add(v.op, 0, 2 * tt * u);
            add(v.op, 1, tt * tt);
        } else {
            if (ps >= 0) add(ps, adj::end_slot(ops[ps].kind), u * u * u);
            add(v.op, 0, 3 * tt * u * u);
            add(v.op, 1, 3 * tt * tt * u);
            add(v.op, 2, tt * tt * tt);
        }
        gw(S.wsrc0[k], u * gW[k]);
        gw(S.wsrc1[k], tt * gW[k]);
    }
    return S.status;
}

// The f32 outline of the stroke (Line / Close ops as footile's Stroke::path_ops emits
// them, before the second transform), for checking the node pass against the
// stroker.  Returns the op count (may exceed cap).
__attribute__((visibility("default"))) uint32_t orc_adj_stroke_outline(const ft_op* ops, uint32_t n_ops, float tol,
                                                                       const float* xf, int32_t join, float ml,
                                                                       float sw0, ft_op* out, uint32_t cap) {
    const float t = std::max(tol, 0.01f);
    adj::StrokeFig S = adj::build_stroke(ops, n_ops, xf, t * t, join, ml, sw0);
    uint32_t k = 0;
    for (int v : S.verts) {
        if (k < cap) {
            ft_op o{};
            if (v < 0) {
                o.kind = FT_OP_CLOSE;
            } else {
                o.kind = FT_OP_LINE;
                o.v[0] = S.nodes[v].f.x;
                o.v[1] = S.nodes[v].f.y;
            }
            out[k] = o;
        }
        k++;
    }
    return k;
}

}  // extern "C"
