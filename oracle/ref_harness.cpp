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
//   nsvgParse (third_party/nanosvg.h) with SvgScene's replay through Path2d and Paint
//     (pathfinder/core/svg.cpp:63-205), for the SVG ingestion's pin.
// SceneBuilderD3D9::build itself is bypassed because it needs a GPU Renderer for the palette.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "core/d3d9/scene_builder.h"
#include "core/d3d9/tiler.h"
#include "core/dash.h"
#include "core/paint/gradient.h"
#include "core/paint/paint.h"
#include "core/scene.h"
#include "core/stroke.h"
#include <umHalf.h>

#include <string>
#include "core/path2d.h"
#define NANOSVG_IMPLEMENTATION
#include <nanosvg.h>

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

    const RectF given = sv->view_box ? RectF(Vec2F(sv->view_box[0], sv->view_box[1]),
                                             Vec2F(sv->view_box[2], sv->view_box[3]))
                                     : RectF(Vec2F(0.0f, 0.0f), Vec2F(sv->width, sv->height));
    Scene scene(0, given);
    const RectF view_box = scene.get_view_box();

    HarnessBuilder builder;
    builder.attach(&scene);

    const uint32_t n_paths = sv->n_paths;
    // clip paths follow the draw paths; each is tiled on its own (build_clip_path_on_cpu,
    // pathfinder/core/d3d9/scene_builder.cpp:200-223) before the draw paths that use it
    uint32_t n_draw = n_paths;
    std::vector<uint32_t> clip_index(n_paths, 0xffffffffu);  // path -> index among the clip paths
    std::vector<BuiltPath> built_clips;
    if (sv->path_is_clip) {
        for (uint32_t p = 0; p < n_paths; p++)
            if (sv->path_is_clip[p]) {
                if (n_draw == n_paths) n_draw = p;
                clip_index[p] = uint32_t(built_clips.size());
                built_clips.emplace_back();
            } else if (n_draw != n_paths) {
                return 4;  // a draw path after a clip path
            }
    }
    std::vector<BuiltDrawPath> built(n_draw);
    // clip paths' alpha tile ids -> (clip path, tile in its rect); draw tiles that name one are
    // resolved to global tile indices once every path's first tile is known
    std::map<uint32_t, std::pair<uint32_t, uint64_t>> alpha_clip;
    struct ClipRef {
        uint64_t g;           // draw tile (global)
        uint32_t clip_path;
        uint64_t clip_tile;   // in the clip path's rect
        int src_backdrop;     // clip job's source backdrop, or INT32_MIN
    };
    std::vector<ClipRef> clip_refs;
    std::vector<uint8_t> tile_mask;
    std::vector<uint64_t> tile_clip;
    std::vector<int8_t> tile_dest_backdrop;
    std::vector<int32_t> rect(4 * n_paths);
    std::vector<uint64_t> tile_first(n_paths + 1, 0), col_first(n_paths + 1, 0);
    std::vector<uint8_t> tile_alpha;
    std::vector<int8_t> tile_backdrop;
    std::vector<uint32_t> tile_fill_count;
    std::vector<uint16_t> fills;
    std::vector<int32_t> col_backdrop;
    std::vector<uint32_t> path_fills(n_paths, 0);

    auto make_outline = [&](uint32_t p) {
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
        return outline;
    };
    std::vector<std::vector<Fill>> clip_fills(built_clips.size());
    for (uint32_t p = n_draw; p < n_paths; p++) {
        const FillRule rule = sv->fill_rule[p] ? FillRule::EvenOdd : FillRule::Winding;
        TilingPathInfo info{};
        info.type = TilingPathInfo::Type::Clip;
        Tiler tiler(builder, clip_index[p], make_outline(p), rule, view_box, nullptr, {}, info);
        tiler.generate_tiles();
        built_clips[clip_index[p]] = tiler.object_builder.built_path;
        clip_fills[clip_index[p]] = tiler.object_builder.fills;
        const auto &tiles = built_clips[clip_index[p]].data.tiles.data;
        for (uint64_t t = 0; t < tiles.size(); t++)
            if (tiles[t].alpha_tile_id.is_valid()) alpha_clip[tiles[t].alpha_tile_id.value] = {p, t};
    }

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
        const bool is_clip = p >= n_draw;
        BuiltPath bp;
        std::vector<Fill> own_fills;
        std::vector<uint64_t> fill_tile;  // clipped draw paths: the tile of each fill
        if (is_clip) {
            bp = built_clips[clip_index[p]];
            own_fills = clip_fills[clip_index[p]];
        } else {
            TilingPathInfo info{};
            info.type = TilingPathInfo::Type::Draw;
            info.info.paint_id = 0;
            info.info.blend_mode = BlendMode::SrcOver;
            info.info.fill_rule = rule;
            std::shared_ptr<uint32_t> clip_id;
            if (sv->path_clip && sv->path_clip[p] != PF_NO_CLIP) {
                const uint32_t c = sv->path_clip[p];
                if (c >= n_paths || clip_index[c] == 0xffffffffu) return 5;
                clip_id = std::make_shared<uint32_t>(clip_index[c]);
            }
            Tiler tiler(builder, p, outline, rule, view_box, clip_id, built_clips, info);
            tiler.generate_tiles();
            bp = tiler.object_builder.built_path;
            own_fills = tiler.object_builder.fills;
            if (clip_id) {
                // prepare_tiles takes the alpha tile id off a culled tile, while its fills keep
                // linking to it: the fills' tiles come from the same path tiled without the clip,
                // whose fills are the same sequence
                Tiler plain(builder, p, outline, rule, view_box, nullptr, {}, info);
                plain.generate_tiles();
                const auto &ptiles = plain.object_builder.built_path.data.tiles.data;
                std::map<uint32_t, uint64_t> plain_tile;
                for (uint64_t t = 0; t < ptiles.size(); t++)
                    if (ptiles[t].alpha_tile_id.is_valid()) plain_tile[ptiles[t].alpha_tile_id.value] = t;
                const auto &pf = plain.object_builder.fills;
                if (pf.size() != own_fills.size()) return 9;
                fill_tile.assign(pf.size(), 0);
                for (size_t k = 0; k < pf.size(); k++) {
                    auto it = plain_tile.find(pf[k].link);
                    if (it == plain_tile.end()) return 9;
                    fill_tile[k] = it->second;
                }
            }
        }
        const RectI tb = bp.tile_bounds;
        rect[4 * p + 0] = tb.left;
        rect[4 * p + 1] = tb.top;
        rect[4 * p + 2] = tb.right;
        rect[4 * p + 3] = tb.bottom;
        const uint64_t base = tile_first[p];
        const uint64_t ntiles = bp.data.tiles.data.size();
        tile_first[p + 1] = base + ntiles;
        col_first[p + 1] = col_first[p] + bp.data.backdrops.size();

        // the path's own fills link to its own alpha tiles; a clipped solid tile may now name the
        // clip's alpha tile (mask 1), found through the clip paths' ids
        std::map<uint32_t, uint64_t> alpha_to_tile;
        if (fill_tile.empty())
            for (const Fill &f : own_fills) alpha_to_tile[f.link] = UINT64_MAX;
        for (uint64_t t = 0; t < ntiles; t++) {
            const auto &tile = bp.data.tiles.data[t];
            tile_alpha.push_back(tile.alpha_tile_id.is_valid() ? 1 : 0);
            tile_backdrop.push_back(tile.backdrop);
            tile_fill_count.push_back(0);
            tile_mask.push_back(0);
            tile_clip.push_back(UINT64_MAX);
            tile_dest_backdrop.push_back(0);
            if (!tile.alpha_tile_id.is_valid()) continue;
            auto own = alpha_to_tile.find(tile.alpha_tile_id.value);
            if (own != alpha_to_tile.end()) {
                own->second = t;
            } else if (!fill_tile.empty() && alpha_clip.find(tile.alpha_tile_id.value) == alpha_clip.end()) {
                alpha_to_tile[tile.alpha_tile_id.value] = t;  // a clipped path's own alpha tile
            } else {
                auto ct = alpha_clip.find(tile.alpha_tile_id.value);
                if (ct == alpha_clip.end()) return 6;  // an alpha tile with neither own fills nor a clip's
                tile_mask.back() = 1;
                clip_refs.push_back({base + t, ct->second.first, ct->second.second, INT32_MIN});
            }
        }
        if (bp.data.clip_tiles) {
            for (const auto &job : bp.data.clip_tiles->data) {
                if (!(job.dest_tile_id.is_valid() && job.src_tile_id.is_valid())) continue;
                auto d = alpha_to_tile.find(job.dest_tile_id.value);
                auto c = alpha_clip.find(job.src_tile_id.value);
                if (d == alpha_to_tile.end() || d->second == UINT64_MAX || c == alpha_clip.end()) return 7;
                tile_mask[base + d->second] = 2;
                tile_dest_backdrop[base + d->second] = int8_t(job.dest_backdrop);
                clip_refs.push_back({base + d->second, c->second.first, c->second.second, int(job.src_backdrop)});
            }
        }
        for (int32_t b : bp.data.backdrops) col_backdrop.push_back(b);

        // group this path's fills by tile, canonical order inside a tile
        std::vector<std::vector<uint64_t>> per_tile(ntiles);
        for (size_t k = 0; k < own_fills.size(); k++) {
            const Fill &f = own_fills[k];
            uint64_t tile = 0;
            if (!fill_tile.empty()) {
                tile = fill_tile[k];
            } else {
                auto it = alpha_to_tile.find(f.link);
                if (it == alpha_to_tile.end() || it->second == UINT64_MAX) return 2;  // fill without its alpha tile
                tile = it->second;
            }
            const uint64_t key = (uint64_t(f.line_segment.from_x) << 48) | (uint64_t(f.line_segment.from_y) << 32) |
                                 (uint64_t(f.line_segment.to_x) << 16) | uint64_t(f.line_segment.to_y);
            per_tile[tile].push_back(key);
        }
        path_fills[p] = own_fills.size();
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

        if (is_clip) continue;
        BuiltDrawPath bdp;
        bdp.path = bp;
        bdp.occludes = ((sv->color[p] >> 24) & 0xffu) == 0xffu;
        if (sv->path_paint && sv->path_paint[p].type != PF_PAINT_SOLID) {
            // PaintMetadata::is_opaque of a gradient paint (Paint::is_opaque, paint.cpp:9-19)
            const pf_paint &pp = sv->path_paint[p];
            const LineSegmentF line(pp.line[0], pp.line[1], pp.line[2], pp.line[3]);
            Gradient g = pp.type == PF_PAINT_LINEAR ? Gradient::linear(line)
                                                    : Gradient::radial(line, Vec2F(pp.radii[0], pp.radii[1]));
            for (uint32_t i = 0; i < pp.stop_count; i++)
                g.add_color_stop(ColorU(sv->stops[pp.stop_first + i].color), sv->stops[pp.stop_first + i].offset);
            bdp.occludes = Paint::from_gradient(g).is_opaque();
        }
        bdp.color_texture_info = nullptr;
        built[p] = bdp;
    }

    for (const ClipRef &c : clip_refs) {
        const uint64_t gc = tile_first[c.clip_path] + c.clip_tile;
        tile_clip[c.g] = gc;
        if (c.src_backdrop != INT32_MIN && int8_t(c.src_backdrop) != tile_backdrop[gc]) return 8;
    }

    auto batches = build_tile_batches_for_draw_path_display_item(scene, built, Range(0, n_draw));
    const RectI fb_rect = round_rect_out_to_tile_bounds(view_box);
    const uint32_t fbw = fb_rect.width(), fbh = fb_rect.height();
    std::vector<int32_t> z(size_t(fbw) * fbh, -1);
    std::vector<std::vector<uint32_t>> lists(size_t(fbw) * fbh);
    if (batches.size() > 1) return 3;  // solid colours never split a batch
    if (!batches.empty()) {
        const auto &batch = batches[0];
        // the reference z-buffer starts at 0 and takes max(path id); -1 marks "no occluder" here
        std::vector<uint8_t> occluded(size_t(fbw) * fbh, 0);
        for (uint32_t p = 0; p < n_draw; p++) {
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
    out->tile_mask = dup(tile_mask);
    out->tile_clip = dup(tile_clip);
    out->tile_dest_backdrop = dup(tile_dest_backdrop);
    return 0;
}

// Canvas::stroke_path (pathfinder/core/canvas.cpp:270-300) minus the canvas: each stroked
// path's outline (contours as Path2d::into_outline makes them: empty ones dropped) is dashed
// with OutlineDash when it has a pattern, then converted with OutlineStrokeToFill; other paths
// are copied.
extern "C" int pfref_stroke_scene(const pf_scene_view *sv, pfo_outline *out) {
    std::memset(out, 0, sizeof(*out));
    // the reference loops forever on an all-zero dash pattern: only well-formed patterns
    for (uint32_t p = 0; sv->path_stroke && p < sv->n_paths; p++) {
        const pf_stroke &st = sv->path_stroke[p];
        if (!(st.line_width > 0.0f) || !st.dash_count) continue;
        if (uint64_t(st.dash_first) + st.dash_count > sv->n_dashes) return 1;
        float total = 0;
        for (uint32_t i = 0; i < st.dash_count; i++) total += sv->dashes[st.dash_first + i];
        if (!(total > 0.0f)) return 1;
    }
    std::vector<float> pts;
    std::vector<uint8_t> flags, rule(sv->n_paths);
    std::vector<uint32_t> cstart{0}, pstart{0};
    auto emit = [&](const Contour &c) {
        for (size_t i = 0; i < c.points.size(); i++) {
            pts.push_back(c.points[i].x);
            pts.push_back(c.points[i].y);
            flags.push_back(static_cast<uint8_t>(c.flags[i]));
        }
        cstart.push_back(static_cast<uint32_t>(flags.size()));
    };
    for (uint32_t p = 0; p < sv->n_paths; p++) {
        const pf_stroke *st = sv->path_stroke ? &sv->path_stroke[p] : nullptr;
        rule[p] = sv->fill_rule[p];
        if (!st || !(st->line_width > 0.0f)) {
            for (uint32_t k = sv->path_start[p]; k < sv->path_start[p + 1]; k++) {
                Contour c;
                for (uint32_t i = sv->contour_start[k]; i < sv->contour_start[k + 1]; i++)
                    c.push_point(Vec2F(sv->points[2 * i], sv->points[2 * i + 1]),
                                 static_cast<PointFlag>(sv->point_flags[i]), false);
                emit(c);
            }
        } else {
            rule[p] = PF_FILL_NONZERO;
            Outline outline;
            for (uint32_t k = sv->path_start[p]; k < sv->path_start[p + 1]; k++) {
                Contour c;
                for (uint32_t i = sv->contour_start[k]; i < sv->contour_start[k + 1]; i++)
                    c.push_point(Vec2F(sv->points[2 * i], sv->points[2 * i + 1]),
                                 static_cast<PointFlag>(sv->point_flags[i]), true);
                c.closed = sv->contour_closed && sv->contour_closed[k];
                outline.push_contour(c);
            }
            if (st->dash_count) {
                std::vector<float> dashes(sv->dashes + st->dash_first, sv->dashes + st->dash_first + st->dash_count);
                OutlineDash dasher(outline, dashes, st->dash_offset);
                dasher.dash();
                outline = dasher.into_outline();
            }
            StrokeStyle style;
            style.line_width = st->line_width;
            style.miter_limit = st->miter_limit;
            style.line_cap = static_cast<LineCap>(st->line_cap);
            style.line_join = static_cast<LineJoin>(st->line_join);
            OutlineStrokeToFill stroker(outline, style);
            stroker.offset();
            for (const Contour &c : stroker.into_outline().contours) emit(c);
        }
        pstart.push_back(static_cast<uint32_t>(cstart.size() - 1));
    }
    out->n_points = static_cast<uint32_t>(flags.size());
    out->n_contours = static_cast<uint32_t>(cstart.size() - 1);
    out->n_paths = sv->n_paths;
    out->points = dup(pts);
    out->point_flags = dup(flags);
    out->contour_start = dup(cstart);
    out->path_start = dup(pstart);
    out->fill_rule = dup(rule);
    return 0;
}

// The reference's Gradient over the stops in order, sampled the way GradientTileBuilder::
// allocate fills a ramp row (pathfinder/core/paint/gradient.cpp:61-110).
extern "C" void pfref_gradient_ramp(const pf_color_stop *stops, uint32_t n, uint32_t *ramp) {
    Gradient g = Gradient::linear(LineSegmentF());
    for (uint32_t i = 0; i < n; i++) g.add_color_stop(ColorU(stops[i].color), stops[i].offset);
    for (uint32_t x = 0; x < GRADIENT_TILE_LENGTH; x++) {
        const ColorU c = g.sample(((float)x + 0.5f) / GRADIENT_TILE_LENGTH);
        ramp[x] = uint32_t(c.r_) | uint32_t(c.g_) << 8 | uint32_t(c.b_) << 16 | uint32_t(c.a_) << 24;
    }
}

// umHalf's float -> half -> float, as the metadata texture stores values.
extern "C" float pfref_half(float f) { return float(half(f)); }

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
    std::free(r->tile_mask);
    std::free(r->tile_clip);
    std::free(r->tile_dest_backdrop);
    std::memset(r, 0, sizeof(*r));
}

// SvgScene::SvgScene (pathfinder/core/svg.cpp:135-205) up to the canvas: the Path2d of each
// shape, its fill and stroke paints from convert_nsvg_paint (svg.cpp:63-133), and the canvas's
// own tests (Canvas::fill_path / stroke_path / push_path, canvas.cpp:180-300) of which paths
// are drawn.  The canvas itself is not linked (it pulls in the GPU renderers).
namespace {
Paint harness_paint(const NSVGpaint &np) {
    Paint paint;
    if (np.type == NSVG_PAINT_COLOR) {
        paint = Paint::from_color(ColorU(np.color));
    } else if (np.type == NSVG_PAINT_LINEAR_GRADIENT || np.type == NSVG_PAINT_RADIAL_GRADIENT) {
        NSVGgradient *g = np.gradient;
        Transform2 gradient_xform(g->xform2), path_xform(g->xform3);
        Gradient gradient;
        if (np.type == NSVG_PAINT_LINEAR_GRADIENT) {
            Vec2F from = {g->x1, g->y1}, to = {g->x2, g->y2};
            from = path_xform * gradient_xform * from;
            to = path_xform * gradient_xform * to;
            gradient = Gradient::linear(LineSegmentF(from, to));
        } else {
            gradient = Gradient::radial(LineSegmentF(Vec2F(g->cx, g->cy), Vec2F(g->fx, g->fy)), Vec2F(0.0, g->r));
            std::get<GradientRadial>(gradient.geometry).transform = path_xform * gradient_xform;
        }
        if (g->spread == NSVG_SPREAD_REPEAT) gradient.wrap = GradientWrap::Repeat;
        for (int i = 0; i < g->nstops; i++) gradient.add_color_stop(ColorU(g->stops[i].color), g->stops[i].offset);
        paint = Paint::from_gradient(gradient);
    }
    return paint;
}
}  // namespace

extern "C" int pfref_svg_scene(const char *text, size_t length, float dpi, pfo_svg *out) {
    std::memset(out, 0, sizeof(*out));
    std::string copy(text, length);
    NSVGimage *image = nsvgParse(&copy[0], "px", dpi);
    if (!image) return 1;
    std::vector<float> pts, dashes;
    std::vector<uint8_t> flags, closed, rule;
    std::vector<uint32_t> cstart{0}, pstart{0}, color, ramps;
    std::vector<pf_stroke> strokes;
    std::vector<pf_paint> paints;
    std::vector<pf_color_stop> stops;
    auto push = [&](const Outline &outline, const Paint &paint, const NSVGpaint &np, uint8_t fill_rule,
                    const pf_stroke &st) {
        for (const Contour &c : outline.contours) {
            for (size_t i = 0; i < c.points.size(); i++) {
                pts.push_back(c.points[i].x);
                pts.push_back(c.points[i].y);
                flags.push_back(static_cast<uint8_t>(c.flags[i]));
            }
            cstart.push_back(static_cast<uint32_t>(flags.size()));
            closed.push_back(c.closed ? 1 : 0);
        }
        pstart.push_back(static_cast<uint32_t>(cstart.size() - 1));
        rule.push_back(fill_rule);
        strokes.push_back(st);
        const ColorU base = paint.get_base_color();
        color.push_back(uint32_t(base.r_) | uint32_t(base.g_) << 8 | uint32_t(base.b_) << 16 | uint32_t(base.a_) << 24);
        pf_paint pp;
        std::memset(&pp, 0, sizeof pp);
        pp.transform[0] = pp.transform[3] = 1.0f;
        uint32_t ramp[GRADIENT_TILE_LENGTH] = {0};
        if (const auto overlay = paint.get_overlay()) {
            const Gradient &g = std::get<Gradient>(overlay->contents);
            if (const auto *lin = std::get_if<GradientLinear>(&g.geometry)) {
                pp.type = PF_PAINT_LINEAR;
                pp.line[0] = lin->line.from().x, pp.line[1] = lin->line.from().y;
                pp.line[2] = lin->line.to().x, pp.line[3] = lin->line.to().y;
            } else {
                const auto &rad = std::get<GradientRadial>(g.geometry);
                pp.type = PF_PAINT_RADIAL;
                pp.line[0] = rad.line.from().x, pp.line[1] = rad.line.from().y;
                pp.line[2] = rad.line.to().x, pp.line[3] = rad.line.to().y;
                pp.radii[0] = rad.radii.x, pp.radii[1] = rad.radii.y;
                pp.transform[0] = rad.transform.m11(), pp.transform[1] = rad.transform.m21();
                pp.transform[2] = rad.transform.m12(), pp.transform[3] = rad.transform.m22();
                pp.transform[4] = rad.transform.m13(), pp.transform[5] = rad.transform.m23();
            }
            pp.wrap = g.wrap == GradientWrap::Repeat ? PF_WRAP_REPEAT : PF_WRAP_CLAMP;
            pp.stop_first = static_cast<uint32_t>(stops.size());
            pp.stop_count = static_cast<uint32_t>(np.gradient->nstops);
            for (int i = 0; i < np.gradient->nstops; i++)
                stops.push_back(pf_color_stop{np.gradient->stops[i].offset, np.gradient->stops[i].color});
            for (uint32_t x = 0; x < GRADIENT_TILE_LENGTH; x++) {
                const ColorU c = g.sample(((float)x + 0.5f) / GRADIENT_TILE_LENGTH);
                ramp[x] = uint32_t(c.r_) | uint32_t(c.g_) << 8 | uint32_t(c.b_) << 16 | uint32_t(c.a_) << 24;
            }
        }
        paints.push_back(pp);
        ramps.insert(ramps.end(), ramp, ramp + GRADIENT_TILE_LENGTH);
    };
    for (NSVGshape *shape = image->shapes; shape; shape = shape->next) {
        Path2d path;
        for (NSVGpath *np = shape->paths; np; np = np->next) {
            path.move_to(np->pts[0], np->pts[1]);
            for (int i = 0; i < np->npts - 3; i += 3) {
                const float *q = &np->pts[i * 2];
                path.cubic_to(q[2], q[3], q[4], q[5], q[6], q[7]);
            }
            if (np->closed) path.close_path();
        }
        const Paint fill = harness_paint(shape->fill);
        if (fill.is_visible() && fill.get_base_color().is_visible()) {
            pf_stroke none;
            std::memset(&none, 0, sizeof none);
            push(path.into_outline(), fill, shape->fill,
                 shape->fillRule == NSVG_FILLRULE_EVENODD ? PF_FILL_EVEN_ODD : PF_FILL_NONZERO, none);
        }
        const Paint stroke = harness_paint(shape->stroke);
        if (stroke.is_visible() && shape->strokeWidth > 0 && stroke.get_base_color().is_visible()) {
            pf_stroke st;
            std::memset(&st, 0, sizeof st);
            st.line_width = shape->strokeWidth;
            st.miter_limit = shape->miterLimit;
            st.line_cap = shape->strokeLineCap == NSVG_CAP_ROUND    ? PF_CAP_ROUND
                          : shape->strokeLineCap == NSVG_CAP_SQUARE ? PF_CAP_SQUARE
                                                                    : PF_CAP_BUTT;
            st.line_join = shape->strokeLineJoin == NSVG_JOIN_ROUND   ? PF_JOIN_ROUND
                           : shape->strokeLineJoin == NSVG_JOIN_BEVEL ? PF_JOIN_BEVEL
                                                                      : PF_JOIN_MITER;
            if (shape->strokeDashCount > 0) {
                st.dash_first = static_cast<uint32_t>(dashes.size());
                st.dash_count = static_cast<uint32_t>(shape->strokeDashCount);
                dashes.insert(dashes.end(), shape->strokeDashArray, shape->strokeDashArray + shape->strokeDashCount);
            }
            push(path.into_outline(), stroke, shape->stroke, PF_FILL_NONZERO, st);
        }
    }
    out->width = image->width;
    out->height = image->height;
    nsvgDelete(image);
    out->n_points = static_cast<uint32_t>(flags.size());
    out->n_contours = static_cast<uint32_t>(cstart.size() - 1);
    out->n_paths = static_cast<uint32_t>(color.size());
    out->n_dashes = static_cast<uint32_t>(dashes.size());
    out->n_stops = static_cast<uint32_t>(stops.size());
    out->points = dup(pts);
    out->point_flags = dup(flags);
    out->contour_start = dup(cstart);
    out->contour_closed = dup(closed);
    out->path_start = dup(pstart);
    out->fill_rule = dup(rule);
    out->color = dup(color);
    out->path_stroke = dup(strokes);
    out->dashes = dup(dashes);
    out->path_paint = dup(paints);
    out->stops = dup(stops);
    out->ramps = dup(ramps);
    return 0;
}

extern "C" void pfref_svg_free(pfo_svg *s) {
    if (!s) return;
    std::free(s->points);
    std::free(s->point_flags);
    std::free(s->contour_start);
    std::free(s->contour_closed);
    std::free(s->path_start);
    std::free(s->fill_rule);
    std::free(s->color);
    std::free(s->path_stroke);
    std::free(s->dashes);
    std::free(s->path_paint);
    std::free(s->stops);
    std::free(s->ramps);
    std::memset(s, 0, sizeof(*s));
}
