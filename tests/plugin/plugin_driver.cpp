// Builds a scene through the reference's own API (Path2d, Paint, Scene::push_draw_path and
// push_clip_path, a view box with an origin), packs it with the drop-in SceneBuilderCuda, and
// tiles the packed scene with both the reference's d3d9 tiler (through the harness) and the
// restated oracle.  Prints "OK <fills>" when the two
// agree and the packed colours / fill rules / clip assignments are the ones the scene holds.
#include <cstdio>
#include <cstring>

#include "core/path2d.h"
#include "core/scene.h"
#include "device_cuda.h"
#include "pf_oracle.h"
#include "renderer_cuda.h"

using namespace Pathfinder;

// The headless device: transfers through staging buffers round-trip, the Renderer base class
// and the palette's metadata upload run on it, and RendererCuda::draw without a CUDA device
// logs an error and leaves the destination as it was (the reference logs and continues).
static int check_headless_device(Scene &scene) {
    auto device = DeviceCuda::create(0);
    auto queue = std::make_shared<QueueCuda>();
    auto tex = device->create_texture({{7, 5}, TextureFormat::Rgba8Unorm}, "t");
    std::vector<uint8_t> in(7 * 5 * 4), out(7 * 5 * 4, 0), part(3 * 2 * 4, 0);
    for (size_t i = 0; i < in.size(); i++) in[i] = uint8_t(i * 7 + 3);
    auto enc = device->create_command_encoder("transfers");
    enc->write_texture(tex, {}, in.data());
    enc->read_texture(tex, {}, out.data());
    enc->read_texture(tex, RectI({2, 1}, {5, 3}), part.data());
    auto buf = device->create_buffer({BufferType::Storage, 64, MemoryProperty::DeviceLocal}, "b");
    std::vector<uint8_t> bin(40), bout(40, 0);
    for (size_t i = 0; i < bin.size(); i++) bin[i] = uint8_t(255 - i);
    enc->write_buffer(buf, 16, 40, bin.data());
    enc->read_buffer(buf, 16, 40, bout.data());
    queue->submit(enc, device->create_fence("f"));
    if (out != in || bout != bin) return std::printf("FAIL transfers\n"), 1;
    for (int y = 0; y < 2; y++)
        if (std::memcmp(&part[y * 12], &in[((1 + y) * 7 + 2) * 4], 12)) return std::printf("FAIL region\n"), 1;
    auto renderer = std::make_shared<RendererCuda>(device, queue);  // Renderer::Renderer on DeviceCuda
    auto dest = device->create_texture({{300, 200}, TextureFormat::Rgba8Unorm}, "dest");
    renderer->set_dest_texture(dest);
    auto meta = scene.palette.build_paint_info(renderer.get());  // the metadata upload
    if (meta.size() != 8) return std::printf("FAIL palette %zu\n", meta.size()), 1;
    auto builder = std::make_shared<SceneBuilderCuda>();
    builder->build(&scene, renderer.get());
    if (builder->view().width != 300.f || builder->view().height != 200.f) return std::printf("FAIL dest size\n"), 1;
    auto &px = static_cast<TextureCuda *>(dest.get())->pixels();
    std::fill(px.begin(), px.end(), uint8_t(9));
    renderer->draw(builder, true);  // no CUDA device in this process: logged, destination untouched
    for (uint8_t v : px)
        if (v != 9) return std::printf("FAIL draw without a device touched the destination\n"), 1;
    return 0;
}

int main() {
    // a view box with an origin: tiles and lines are clipped to it (Scene::set_view_box rounds
    // its right edge up to 304)
    Scene scene(0, RectF({12.5f, 7.0f}, {300.f, 200.f}));
    // two clip paths (Scene::push_clip_path): a diamond and an even-odd ring
    uint32_t clip_ids[2];
    {
        Path2d c;
        c.move_to(150.f, 5.f);
        c.line_to(290.f, 100.f);
        c.line_to(150.f, 195.f);
        c.line_to(10.f, 100.f);
        c.close_path();
        ClipPath cp;
        cp.outline = c.into_outline();
        clip_ids[0] = scene.push_clip_path(cp);
        Path2d r;
        r.move_to(40.f, 30.f);
        r.cubic_to(260.f, 10.f, 280.f, 190.f, 60.f, 170.f);
        r.close_path();
        r.move_to(90.f, 70.f);
        r.line_to(180.f, 75.f);
        r.line_to(150.f, 130.f);
        r.close_path();
        ClipPath cr;
        cr.outline = r.into_outline();
        cr.fill_rule = FillRule::EvenOdd;
        clip_ids[1] = scene.push_clip_path(cr);
    }
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
        if (i % 4 != 3) dp.clip_path = std::make_shared<uint32_t>(clip_ids[i % 2]);
        scene.push_draw_path(dp);
    }
    SceneBuilderCuda builder;
    builder.build(&scene, nullptr);
    const pf_scene_view &v = builder.view();
    if (v.n_paths != 10 || !v.path_clip || !v.path_is_clip) return std::printf("FAIL paths %u\n", v.n_paths), 1;
    if (!v.view_box || v.view_box[0] != 12.5f || v.view_box[1] != 7.0f || v.view_box[2] != 304.f ||
        v.view_box[3] != 200.f || v.load_action != PF_LOAD_CLEAR)
        return std::printf("FAIL view box\n"), 1;
    for (uint32_t i = 0; i < 10; i++) {
        const uint32_t want = i >= 8 ? PF_NO_CLIP : i % 4 == 3 ? PF_NO_CLIP : 8 + clip_ids[i % 2];
        if (v.path_clip[i] != want || v.path_is_clip[i] != (i >= 8)) return std::printf("FAIL clip %u\n", i), 1;
    }
    for (uint32_t i = 0; i < 8; i++) {
        const uint32_t want = uint32_t(20 * i) | uint32_t(255 - 20 * i) << 8 | 100u << 16 | uint32_t(i % 2 ? 160 : 255) << 24;
        if (v.color[i] != want || v.fill_rule[i] != (i % 2)) return std::printf("FAIL paint %u\n", i), 1;
    }
    pfo_result a{}, b{};
    if (pfref_tile_scene(&v, &a) || pfo_tile_scene(&v, PFO_Z_D3D9, &b)) return std::printf("FAIL tile\n"), 1;
    bool same = a.n_tiles == b.n_tiles && a.n_fills == b.n_fills && a.n_list == b.n_list &&
                !std::memcmp(a.tile_backdrop, b.tile_backdrop, a.n_tiles) &&
                !std::memcmp(a.tile_alpha, b.tile_alpha, a.n_tiles) &&
                !std::memcmp(a.fills, b.fills, a.n_fills * 8) && !std::memcmp(a.fb_list, b.fb_list, a.n_list * 4) &&
                !std::memcmp(a.tile_mask, b.tile_mask, a.n_tiles) &&
                !std::memcmp(a.tile_clip, b.tile_clip, a.n_tiles * 8);
    uint64_t clipped = 0;
    for (uint64_t t = 0; t < a.n_tiles; t++) clipped += a.tile_mask[t] != 0;
    same = same && clipped > 0;
    if (!same) return std::printf("FAIL %llu\n", (unsigned long long)a.n_fills), 1;
    if (check_headless_device(scene)) return 1;
    std::printf("OK %llu\n", (unsigned long long)a.n_fills);
    return 0;
}
