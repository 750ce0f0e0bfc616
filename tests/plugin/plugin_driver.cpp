// Builds a scene through the reference's own API (Path2d, Paint, Scene::push_draw_path), packs
// it with the drop-in SceneBuilderCuda, and tiles the packed scene with both the reference's
// d3d9 tiler (through the harness) and the restated oracle.  Prints "OK <fills>" when the two
// agree and the packed colours / fill rules are the ones the scene holds.
#include <cstdio>
#include <cstring>

#include "core/path2d.h"
#include "core/scene.h"
#include "pf_oracle.h"
#include "renderer_cuda.h"

using namespace Pathfinder;

int main() {
    Scene scene(0, RectF({0.f, 0.f}, {300.f, 200.f}));
    for (int i = 0; i < 8; i++) {
        Path2d p;
        const float o = 7.f * i;
        p.move_to(10.f + o, 20.f + o);
        p.cubic_to(120.f - o, -10.f + o, 200.f + o, 150.f, 90.f, 180.f - o);
        p.quadratic_to(40.f + o, 120.f, 30.f + 2 * o, 60.f);
        p.line_to(60.f, 40.f + o);
        p.close_path();
        if (i % 3 == 0) {  // a second contour (hole) on some paths
            p.move_to(50.f + o, 60.f);
            p.line_to(50.f + o, 90.f);
            p.line_to(80.f + o, 90.f);
            p.close_path();
        }
        DrawPath dp;
        dp.outline = p.into_outline();
        dp.paint = scene.push_paint(Paint::from_color(ColorU(20 * i, 255 - 20 * i, 100, i % 2 ? 160 : 255)));
        dp.fill_rule = i % 2 ? FillRule::EvenOdd : FillRule::Winding;
        scene.push_draw_path(dp);
    }
    SceneBuilderCuda builder;
    builder.build(&scene, nullptr);
    const pf_scene_view &v = builder.view();
    if (v.n_paths != 8) return std::printf("FAIL paths %u\n", v.n_paths), 1;
    for (uint32_t i = 0; i < v.n_paths; i++) {
        const uint32_t want = uint32_t(20 * i) | uint32_t(255 - 20 * i) << 8 | 100u << 16 | uint32_t(i % 2 ? 160 : 255) << 24;
        if (v.color[i] != want || v.fill_rule[i] != (i % 2)) return std::printf("FAIL paint %u\n", i), 1;
    }
    pfo_result a{}, b{};
    if (pfref_tile_scene(&v, &a) || pfo_tile_scene(&v, PFO_Z_D3D9, &b)) return std::printf("FAIL tile\n"), 1;
    bool same = a.n_tiles == b.n_tiles && a.n_fills == b.n_fills && a.n_list == b.n_list &&
                !std::memcmp(a.tile_backdrop, b.tile_backdrop, a.n_tiles) &&
                !std::memcmp(a.tile_alpha, b.tile_alpha, a.n_tiles) &&
                !std::memcmp(a.fills, b.fills, a.n_fills * 8) && !std::memcmp(a.fb_list, b.fb_list, a.n_list * 4);
    std::printf("%s %llu\n", same ? "OK" : "FAIL", (unsigned long long)a.n_fills);
    return same ? 0 : 1;
}
