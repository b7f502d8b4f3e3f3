// footile.hpp — C++ host side of the GB300 path, mirroring footile's Rust API
// (src/lib.rs:39-41): Path2D, PathOp, FillRule, JoinStyle and Plotter<P> over the
// C ABI of footile_gpu.h.  Header-only; link with libfootile_gpu.so.
//
//   footile::Path2D pb;
//   auto fish = pb.relative().pen_width(3.0f).move_to(112, 24).line_to(-32, 24)
//                  .cubic_to(-96, -48, -96, 80, 0, 32).close().finish();
//   footile::Plotter<footile::Matte8> p(footile::Raster<footile::Matte8>(128, 128));
//   p.fill(footile::FillRule::NonZero, fish, footile::Matte8{255});
//
// Errors: footile panics; this binding throws footile::Error carrying the FT_ERR_*
// status and the library's message.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "footile_gpu.h"

namespace footile {

// src/path.rs:8-14
enum class FillRule : int32_t { NonZero = FT_NONZERO, EvenOdd = FT_EVENODD };

// src/stroker.rs:13-20
struct JoinStyle {
    int32_t kind;
    float limit;
    static JoinStyle Miter(float limit) { return JoinStyle{FT_JOIN_MITER, limit}; }
    static JoinStyle Bevel() { return JoinStyle{FT_JOIN_BEVEL, 0.0f}; }
    static JoinStyle Round() { return JoinStyle{FT_JOIN_ROUND, 0.0f}; }
};

class Error : public std::runtime_error {
   public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

   private:
    int code_;
};

// src/path.rs:18-31: one `ft_op` record per PathOp.
struct PathOp {
    static ft_op make(int32_t kind, float a = 0, float b = 0, float c = 0, float d = 0, float e = 0, float f = 0) {
        ft_op o{};
        o.kind = kind;
        o.v[0] = a;
        o.v[1] = b;
        o.v[2] = c;
        o.v[3] = d;
        o.v[4] = e;
        o.v[5] = f;
        return o;
    }
    static ft_op Close() { return make(FT_OP_CLOSE); }
    static ft_op Move(float x, float y) { return make(FT_OP_MOVE, x, y); }
    static ft_op Line(float x, float y) { return make(FT_OP_LINE, x, y); }
    static ft_op Quad(float bx, float by, float cx, float cy) { return make(FT_OP_QUAD, bx, by, cx, cy); }
    static ft_op Cubic(float bx, float by, float cx, float cy, float dx, float dy) {
        return make(FT_OP_CUBIC, bx, by, cx, cy, dx, dy);
    }
    static ft_op PenWidth(float w) { return make(FT_OP_PEN_WIDTH, w); }
};

// src/path.rs:44-171: relative coordinates by default, resolved in f32 while building.
class Path2D {
   public:
    Path2D& absolute() {
        absolute_ = true;
        return *this;
    }
    Path2D& relative() {
        absolute_ = false;
        return *this;
    }
    Path2D& close() {
        ops_.push_back(PathOp::Close());
        pen_x_ = pen_y_ = 0.0f;
        return *this;
    }
    Path2D& move_to(float x, float y) {
        pt(x, y);
        ops_.push_back(PathOp::Move(x, y));
        pen_x_ = x;
        pen_y_ = y;
        return *this;
    }
    Path2D& line_to(float x, float y) {
        pt(x, y);
        ops_.push_back(PathOp::Line(x, y));
        pen_x_ = x;
        pen_y_ = y;
        return *this;
    }
    Path2D& quad_to(float bx, float by, float cx, float cy) {
        pt(bx, by);
        pt(cx, cy);
        ops_.push_back(PathOp::Quad(bx, by, cx, cy));
        pen_x_ = cx;
        pen_y_ = cy;
        return *this;
    }
    Path2D& cubic_to(float bx, float by, float cx, float cy, float dx, float dy) {
        pt(bx, by);
        pt(cx, cy);
        pt(dx, dy);
        ops_.push_back(PathOp::Cubic(bx, by, cx, cy, dx, dy));
        pen_x_ = dx;
        pen_y_ = dy;
        return *this;
    }
    Path2D& pen_width(float w) {
        ops_.push_back(PathOp::PenWidth(w));
        return *this;
    }
    std::vector<ft_op> finish() { return std::move(ops_); }

   private:
    void pt(float& x, float& y) const {
        if (!absolute_) {
            x = pen_x_ + x;
            y = pen_y_ + y;
        }
    }
    std::vector<ft_op> ops_;
    bool absolute_ = false;
    float pen_x_ = 0.0f, pen_y_ = 0.0f;
};

// Pixel formats the plotter accepts (Ch8, premultiplied, linear, src/plotter.rs:38-41).
struct Matte8 {
    uint8_t value;
    static constexpr int32_t format = FT_MATTE8;
};
struct Rgba8p {
    uint8_t r, g, b, a;
    static constexpr int32_t format = FT_RGBA8P;
};

template <class P>
class Raster {
   public:
    Raster(uint32_t w, uint32_t h) : w_(w), h_(h), px_((size_t)w * h, P{}) {}
    Raster(uint32_t w, uint32_t h, P fill) : w_(w), h_(h), px_((size_t)w * h, fill) {}
    uint32_t width() const { return w_; }
    uint32_t height() const { return h_; }
    const std::vector<P>& pixels() const { return px_; }
    std::vector<P>& pixels() { return px_; }
    uint8_t* bytes() { return reinterpret_cast<uint8_t*>(px_.data()); }

   private:
    uint32_t w_, h_;
    std::vector<P> px_;
};

// src/plotter.rs:38-381
template <class P>
class Plotter {
   public:
    explicit Plotter(Raster<P> raster, int device = 0) : raster_(std::move(raster)) {
        int rc = ft_ctx_create(device, &ctx_);
        if (rc != FT_OK) throw Error(rc, "ft_ctx_create failed");
    }
    ~Plotter() {
        if (ctx_) ft_ctx_destroy(ctx_);
    }
    Plotter(const Plotter&) = delete;
    Plotter& operator=(const Plotter&) = delete;

    uint32_t width() const { return raster_.width(); }
    uint32_t height() const { return raster_.height(); }

    Plotter& set_tolerance(float t) {
        check(ft_set_tolerance(ctx_, t));
        return *this;
    }
    Plotter& set_transform(const float m[6]) {
        check(ft_set_transform(ctx_, m));
        return *this;
    }
    Plotter& set_join(JoinStyle js) {
        check(ft_set_join(ctx_, js.kind, js.limit));
        return *this;
    }
    float pen_width() {
        float w = 0.0f;
        check(ft_get_pen_width(ctx_, &w));
        return w;
    }

    Raster<P>& fill(FillRule rule, const std::vector<ft_op>& ops, P clr) {
        uint8_t c[4];
        color(clr, c);
        check(ft_fill(ctx_, static_cast<int32_t>(rule), ops.data(), (uint32_t)ops.size(), P::format, c,
                      raster_.bytes(), raster_.width(), raster_.height(), raster_.width() * (uint32_t)sizeof(P),
                      FT_HOST));
        return raster_;
    }
    Raster<P>& stroke(const std::vector<ft_op>& ops, P clr) {
        uint8_t c[4];
        color(clr, c);
        check(ft_stroke(ctx_, ops.data(), (uint32_t)ops.size(), P::format, c, raster_.bytes(), raster_.width(),
                        raster_.height(), raster_.width() * (uint32_t)sizeof(P), FT_HOST));
        return raster_;
    }

    const Raster<P>& raster() const { return raster_; }
    Raster<P>& raster_mut() { return raster_; }
    Raster<P> into_raster() { return std::move(raster_); }

   private:
    static void color(Matte8 m, uint8_t* c) { c[0] = c[1] = c[2] = c[3] = m.value; }
    static void color(Rgba8p p, uint8_t* c) {
        c[0] = p.r;
        c[1] = p.g;
        c[2] = p.b;
        c[3] = p.a;
    }
    void check(int rc) {
        if (rc != FT_OK) throw Error(rc, ft_last_error(ctx_));
    }

    ft_ctx* ctx_ = nullptr;
    Raster<P> raster_;
};

}  // namespace footile
