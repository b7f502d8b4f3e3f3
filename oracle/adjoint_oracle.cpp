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
#include <cstdint>
#include <vector>

#include "../include/footile_gpu.h"

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

// Vertex positions in f64.  Without `val`: the f32 points of the De Casteljau walk, the
// polygon footile's Fig receives (and the CUDA coverage covers), widened to double.
// With `val` (6 per op, the layout of ft_op.v): the Bernstein points B(t) of the same
// tree, continuous in the control values (for finite differences).
static std::vector<D2> positions(const Poly& P, const ft_op* ops, const double* val, const double* m) {
    std::vector<D2> out(P.v.size());
    if (!val) {
        for (size_t k = 0; k < P.v.size(); k++) out[k] = D2{(double)P.f[k].x, (double)P.f[k].y};
        return out;
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
    std::vector<double> acc((size_t)w * h, 0.0);
    if (S.P.status != FT_ERR_CAP) {
        std::vector<adj::D2> pos = adj::positions(S.P, ops, S.bernstein ? S.val.data() : nullptr, S.m);
        for (int k = 0; k < (int)pos.size(); k++) {
            adj::D2 p0 = pos[k], p1 = pos[adj::next_vertex(S.P, k)];
            double dir = p1.y > p0.y ? 1.0 : -1.0;
            adj::edge_pieces(p0, p1, (int)w, (int)h, [&](int r, int c, double hh, double xm, double, double) {
                double* row = &acc[(size_t)r * w];
                if (c < 0) {
                    row[0] += dir * hh;
                } else if (c < (int)w) {
                    row[c] += dir * hh * (c + 1 - xm);
                    if (c + 1 < (int)w) row[c + 1] += dir * hh * (xm - c);
                }
            });
        }
    }
    const double sg = S.P.sign;
    for (uint32_t r = 0; r < h; r++) {
        double s = 0.0;
        for (uint32_t c = 0; c < w; c++) {
            s += sg * acc[(size_t)r * w + c];
            if (area) area[(size_t)r * w + c] = s;
            cov[(size_t)r * w + c] = adj::coverage(rule, s);
        }
    }
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
    std::vector<double> gs((size_t)w * h);
    for (size_t i = 0; i < gs.size(); i++) gs[i] = S.P.sign * grad_cov[i] * adj::coverage_d(rule, area[i]);
    std::vector<adj::D2> pos = adj::positions(S.P, ops, S.bernstein ? S.val.data() : nullptr, S.m);
    std::vector<adj::D2> gp(pos.size(), adj::D2{0.0, 0.0});
    for (int k = 0; k < (int)pos.size(); k++) {
        int nk = adj::next_vertex(S.P, k);
        adj::D2 p0 = pos[k], p1 = pos[nk];
        bool down = p1.y > p0.y;  // P0 is the top end: s = u
        double ga = 0.0, gb = 0.0;
        adj::edge_pieces(p0, p1, (int)w, (int)h, [&](int r, int c, double, double, double u0, double u1) {
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
