// ref_harness.cpp - drives the reference's own d3d9 CPU tiler over a pf_scene_view.
//
// TEST INFRASTRUCTURE ONLY (see pf_oracle.h).  Compiled together with the
// reference's sources where they lie (oracle/Makefile); the result goes to
// oracle/_ref/ and is never shipped.
//
// What it runs, in the reference's own code:
//   Tiler::Tiler / Tiler::generate_tiles   pathfinder/core/d3d9/tiler.cpp:317-343
//     (generate_fills -> process_segment -> process_line_segment -> ObjectBuilder::add_fill /
//      adjust_alpha_tile_backdrop; prepare_tiles), one path at a time in path order, single
//      threaded so alpha-tile ids come out in a fixed order;
//   build_tile_batches_for_draw_path_display_item  pathfinder/core/d3d9/scene_builder.cpp:18-95
//     (visible tiles in path order and the z-buffer).
// SceneBuilderD3D9::build itself is bypassed because it needs a GPU Renderer for the palette.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "core/d3d9/scene_builder.h"
#include "core/d3d9/tiler.h"
#include "core/scene.h"

#include "pf_oracle.h"

namespace Pathfinder {
std::vector<DrawTileBatchD3D9> build_tile_batches_for_draw_path_display_item(const Scene &scene,
                                                                             const std::vector<BuiltDrawPath> &built_paths,
                                                                             Range draw_path_range);
}

using namespace Pathfinder;

namespace {

struct HarnessBuilder : public SceneBuilderD3D9 {
    void attach(Scene *s) {
        scene = s;
        for (auto &n : next_alpha_tile_indices) n = 0;
    }
};

template <typename T>
T *dup(const std::vector<T> &v) {
    T *p = static_cast<T *>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
    if (!v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
    return p;
}

}  // namespace

extern "C" int pfref_tile_scene(const pf_scene_view *sv, pfo_result *out) {
    if (!sv || !out) return 1;
    std::memset(out, 0, sizeof(*out));

    Scene scene(0, RectF(Vec2F(0.0f, 0.0f), Vec2F(sv->width, sv->height)));
    const RectF view_box = scene.get_view_box();

    HarnessBuilder builder;
    builder.attach(&scene);

    const uint32_t n_paths = sv->n_paths;
    std::vector<BuiltDrawPath> built(n_paths);
    std::vector<int32_t> rect(4 * n_paths);
    std::vector<uint64_t> tile_first(n_paths + 1, 0), col_first(n_paths + 1, 0);
    std::vector<uint8_t> tile_alpha;
    std::vector<int8_t> tile_backdrop;
    std::vector<uint32_t> tile_fill_count;
    std::vector<uint16_t> fills;
    std::vector<int32_t> col_backdrop;
    std::vector<uint32_t> path_fills(n_paths, 0);

    for (uint32_t p = 0; p < n_paths; p++) {
        Outline outline;
        for (uint32_t c = sv->path_start[p]; c < sv->path_start[p + 1]; c++) {
            Contour contour;
            for (uint32_t i = sv->contour_start[c]; i < sv->contour_start[c + 1]; i++) {
                contour.push_point(Vec2F(sv->points[2 * i], sv->points[2 * i + 1]),
                                   static_cast<PointFlag>(sv->point_flags[i]), true);
            }
            contour.closed = true;
            outline.push_contour(contour);
        }

        const FillRule rule = sv->fill_rule[p] ? FillRule::EvenOdd : FillRule::Winding;
        TilingPathInfo info{};
        info.type = TilingPathInfo::Type::Draw;
        info.info.paint_id = 0;
        info.info.blend_mode = BlendMode::SrcOver;
        info.info.fill_rule = rule;

        Tiler tiler(builder, p, outline, rule, view_box, nullptr, {}, info);
        tiler.generate_tiles();

        const BuiltPath &bp = tiler.object_builder.built_path;
        const RectI tb = bp.tile_bounds;
        rect[4 * p + 0] = tb.left;
        rect[4 * p + 1] = tb.top;
        rect[4 * p + 2] = tb.right;
        rect[4 * p + 3] = tb.bottom;
        const uint64_t base = tile_first[p];
        const uint64_t ntiles = bp.data.tiles.data.size();
        tile_first[p + 1] = base + ntiles;
        col_first[p + 1] = col_first[p] + bp.data.backdrops.size();

        std::map<uint32_t, uint64_t> alpha_to_tile;
        for (uint64_t t = 0; t < ntiles; t++) {
            const auto &tile = bp.data.tiles.data[t];
            tile_alpha.push_back(tile.alpha_tile_id.is_valid() ? 1 : 0);
            tile_backdrop.push_back(tile.backdrop);
            tile_fill_count.push_back(0);
            if (tile.alpha_tile_id.is_valid()) alpha_to_tile[tile.alpha_tile_id.value] = t;
        }
        for (int32_t b : bp.data.backdrops) col_backdrop.push_back(b);

        // group this path's fills by tile, canonical order inside a tile
        std::vector<std::vector<uint64_t>> per_tile(ntiles);
        for (const Fill &f : tiler.object_builder.fills) {
            auto it = alpha_to_tile.find(f.link);
            if (it == alpha_to_tile.end()) return 2;  // fill without its alpha tile: should not happen
            const uint64_t key = (uint64_t(f.line_segment.from_x) << 48) | (uint64_t(f.line_segment.from_y) << 32) |
                                 (uint64_t(f.line_segment.to_x) << 16) | uint64_t(f.line_segment.to_y);
            per_tile[it->second].push_back(key);
        }
        path_fills[p] = tiler.object_builder.fills.size();
        for (uint64_t t = 0; t < ntiles; t++) {
            auto &v = per_tile[t];
            std::sort(v.begin(), v.end());
            tile_fill_count[base + t] = v.size();
            for (uint64_t k : v) {
                fills.push_back(uint16_t(k >> 48));
                fills.push_back(uint16_t(k >> 32));
                fills.push_back(uint16_t(k >> 16));
                fills.push_back(uint16_t(k));
            }
        }

        BuiltDrawPath bdp;
        bdp.path = bp;
        bdp.occludes = ((sv->color[p] >> 24) & 0xffu) == 0xffu;
        bdp.color_texture_info = nullptr;
        built[p] = bdp;
    }

    auto batches = build_tile_batches_for_draw_path_display_item(scene, built, Range(0, n_paths));
    const RectI fb_rect = round_rect_out_to_tile_bounds(view_box);
    const uint32_t fbw = fb_rect.width(), fbh = fb_rect.height();
    std::vector<int32_t> z(size_t(fbw) * fbh, -1);
    std::vector<std::vector<uint32_t>> lists(size_t(fbw) * fbh);
    if (batches.size() > 1) return 3;  // solid colours never split a batch
    if (!batches.empty()) {
        const auto &batch = batches[0];
        // the reference z-buffer starts at 0 and takes max(path id); -1 marks "no occluder" here
        std::vector<uint8_t> occluded(size_t(fbw) * fbh, 0);
        for (uint32_t p = 0; p < n_paths; p++) {
            if (!built[p].occludes) continue;
            for (const auto &tile : built[p].path.data.tiles.data) {
                if (tile.alpha_tile_id.is_valid() || tile.backdrop == 0) continue;
                occluded[size_t(tile.tile_y - fb_rect.min_y()) * fbw + (tile.tile_x - fb_rect.min_x())] = 1;
            }
        }
        for (size_t i = 0; i < z.size(); i++) {
            if (occluded[i]) z[i] = int32_t(batch.z_buffer_data.data[i]);
        }
        for (const auto &tile : batch.tiles) {
            const size_t fb = size_t(tile.tile_y - fb_rect.min_y()) * fbw + (tile.tile_x - fb_rect.min_x());
            const uint32_t p = tile.path_id;
            if (int64_t(p) < int64_t(z[fb])) continue;  // culled as in tile.vert:114
            const RectI tb = built[p].path.tile_bounds;
            const uint64_t gt = tile_first[p] + uint64_t(tile.tile_y - tb.top) * tb.width() + (tile.tile_x - tb.left);
            lists[fb].push_back(uint32_t(gt));
        }
    }
    std::vector<uint64_t> list_first(lists.size() + 1, 0);
    std::vector<uint32_t> flat;
    for (size_t i = 0; i < lists.size(); i++) {
        list_first[i + 1] = list_first[i] + lists[i].size();
        flat.insert(flat.end(), lists[i].begin(), lists[i].end());
    }

    out->n_paths = n_paths;
    out->path_rect = dup(rect);
    out->path_tile_first = dup(tile_first);
    out->path_column_first = dup(col_first);
    out->n_tiles = tile_alpha.size();
    out->tile_alpha = dup(tile_alpha);
    out->tile_backdrop = dup(tile_backdrop);
    out->tile_fill_count = dup(tile_fill_count);
    out->n_fills = fills.size() / 4;
    out->fills = dup(fills);
    out->n_columns = col_backdrop.size();
    out->column_backdrop = dup(col_backdrop);
    out->fb_tiles_x = fbw;
    out->fb_tiles_y = fbh;
    out->z = dup(z);
    out->fb_list_first = dup(list_first);
    out->n_list = flat.size();
    out->fb_list = dup(flat);
    out->path_fills = dup(path_fills);
    out->path_microlines = nullptr;
    return 0;
}

extern "C" void pfref_free(pfo_result *r) {
    if (!r) return;
    std::free(r->path_rect);
    std::free(r->path_tile_first);
    std::free(r->path_column_first);
    std::free(r->tile_alpha);
    std::free(r->tile_backdrop);
    std::free(r->tile_fill_count);
    std::free(r->fills);
    std::free(r->column_backdrop);
    std::free(r->z);
    std::free(r->fb_list_first);
    std::free(r->fb_list);
    std::free(r->path_fills);
    std::free(r->path_microlines);
    std::memset(r, 0, sizeof(*r));
}
