// The fishy example of footile (examples/fishy.rs) through the C++ host mirror
// include/footile.hpp: fill, then two strokes, on one Rgba8p Plotter; plus the
// Matte8 fill of the crate's doc example (src/lib.rs:14-26).  Writes the raw raster
// bytes to argv[1] (Rgba8p 128x128) and argv[2] (Matte8 128x128).
#include <cstdio>

#include "footile.hpp"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    using namespace footile;
    try {
        auto fish = Path2D()
                        .relative()
                        .pen_width(3.0f)
                        .move_to(112.0f, 24.0f)
                        .line_to(-32.0f, 24.0f)
                        .cubic_to(-96.0f, -48.0f, -96.0f, 80.0f, 0.0f, 32.0f)
                        .line_to(32.0f, 24.0f)
                        .line_to(-16.0f, -40.0f)
                        .close()
                        .finish();
        auto eye = Path2D()
                       .relative()
                       .pen_width(2.0f)
                       .move_to(24.0f, 48.0f)
                       .line_to(8.0f, 8.0f)
                       .move_to(0.0f, -8.0f)
                       .line_to(-8.0f, 8.0f)
                       .finish();
        Plotter<Rgba8p> p(Raster<Rgba8p>(128, 128));
        p.fill(FillRule::NonZero, fish, Rgba8p{127, 96, 96, 255});
        p.stroke(fish, Rgba8p{255, 208, 208, 255});
        p.stroke(eye, Rgba8p{0, 0, 0, 255});
        FILE* f = fopen(argv[1], "wb");
        fwrite(p.raster().pixels().data(), 4, 128 * 128, f);
        fclose(f);

        Plotter<Matte8> m(Raster<Matte8>(128, 128));
        m.fill(FillRule::NonZero, fish, Matte8{255});
        f = fopen(argv[2], "wb");
        fwrite(m.raster().pixels().data(), 1, 128 * 128, f);
        fclose(f);
        printf("pen width %.1f\n", p.pen_width());
    } catch (const footile::Error& e) {
        fprintf(stderr, "footile error %d: %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
