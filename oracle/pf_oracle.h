/*
 * pf_oracle.h - CPU oracle for the GPU-driven fill pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing on the product path links, loads or
 * calls this code; only tests/, the smoke check and bench.py's CPU-baseline
 * leg use it, and only as the checker or the timed CPU baseline.
 *
 * Two implementations fill the same pfo_result:
 *   - pf_oracle.c    : a plain-C restatement of the reference's d3d9 CPU tiler
 *                      (libpforacle.so, built everywhere);
 *   - ref_harness.cpp: the reference's own Tiler/ObjectBuilder/SceneBuilderD3D9
 *                      compiled from its sources (oracle/_ref/libpfref.so, built
 *                      only where the reference tree is present).
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#include <stdint.h>

#include "../include/pfcuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* z-buffer rule.  D3D9: every solid tile of an opaque path occludes
 * (pathfinder/core/d3d9/scene_builder.cpp:57-78).  D3D11: solid tiles that the
 * even-odd rule leaves empty (even backdrop) do not occlude
 * (pathfinder/shaders/d3d11/propagate.comp:190-198). */
#define PFO_Z_D3D9 0
#define PFO_Z_D3D11 1

typedef struct pfo_result {
    uint32_t n_paths;
    int32_t *path_rect;          /* [n_paths][4] */
    uint64_t *path_tile_first;   /* [n_paths + 1] */
    uint64_t *path_column_first; /* [n_paths + 1] */
    uint64_t n_tiles;
    uint8_t *tile_alpha;
    int8_t *tile_backdrop;
    uint32_t *tile_fill_count;
    uint64_t n_fills;
    uint16_t *fills;             /* [n_fills][4], grouped by tile, sorted inside a tile */
    uint64_t n_columns;
    int32_t *column_backdrop;
    uint32_t fb_tiles_x, fb_tiles_y;
    int32_t *z;                  /* [fb tiles], -1 = no occluder */
    uint64_t *fb_list_first;     /* [fb tiles + 1] */
    uint64_t n_list;
    uint32_t *fb_list;
    uint64_t n_microlines;       /* flattened leaf lines that reached the tile walk */
    uint32_t *path_microlines;   /* [n_paths] leaf lines per path */
    uint32_t *path_fills;        /* [n_paths] fills per path */
    /* clipped draw tiles (Tiler::prepare_tiles, tiler.cpp:386-431): 0 own mask, 1 the clip
     * tile's mask, 2 own mask combined with the clip tile's; the clip tile (global index or
     * UINT64_MAX); for 2, the draw tile's backdrop before it was zeroed */
    uint8_t *tile_mask;
    uint64_t *tile_clip;
    int8_t *tile_dest_backdrop;
} pfo_result;

/* Restated tiler: flatten, bin, propagate, z-buffer, composite lists.  The _mt
 * variant tiles paths on `threads` worker threads (same output). */
int pfo_tile_scene(const pf_scene_view *scene, int z_rule, pfo_result *out);
int pfo_tile_scene_mt(const pf_scene_view *scene, int z_rule, int threads, pfo_result *out);

/*
 * FP64 analytic-area coverage and src-over composite of a tiled scene.
 * rgba: width_px*height_px*4 bytes (RGBA8); with load_action PF_LOAD_LOAD it holds
 * the destination to composite over on entry.  The tiled result must use the d3d11
 * framebuffer grid (PFO_Z_D3D11: tiles from (0, 0) over the image).  coverage_f (optional, may be
 * NULL): [n_tiles*256] float coverage of every alpha tile after the fill
 * rule, row-major 16x16 (solid and empty tiles are left untouched).
 * first_tile/n_tiles_limit restrict the coverage pass to a tile range (use
 * 0 and UINT64_MAX for all).  threads: worker threads (>= 1).
 */
int pfo_render(const pf_scene_view *scene, const pfo_result *tiled, uint8_t *rgba,
               float *coverage_f, int threads);

void pfo_free(pfo_result *r);

/*
 * Stroke-to-fill and dashing (pf_stroke.c): the scene's fill outline, every stroked path
 * (pf_stroke::line_width > 0) replaced by its stroke outline (OutlineDash, then
 * OutlineStrokeToFill, as Canvas::stroke_path does) and filled nonzero; other paths copied.
 */
typedef struct pfo_outline {
    uint32_t n_points, n_contours, n_paths;
    float *points;           /* [n_points][2] */
    uint8_t *point_flags;    /* [n_points] */
    uint32_t *contour_start; /* [n_contours + 1] */
    uint32_t *path_start;    /* [n_paths + 1] */
    uint8_t *fill_rule;      /* [n_paths] */
} pfo_outline;

/* 0 ok; 1 invalid stroke data; 3 out of memory; 4 too large; 5 a dash pattern needs more than
 * 2^22 steps on one path */
int pfo_stroke_scene(const pf_scene_view *scene, pfo_outline *out);
int pfo_stroke_check(const pf_scene_view *scene);
void pfo_outline_free(pfo_outline *o);

/*
 * Gradient paints (pf_paint.c): umHalf's truncating float -> half -> float round trip, the
 * 256-texel ramp of a gradient's stops (bit-exact), whether a path's paint is opaque, the
 * half-float metadata the shader reads and the straight-alpha colour at a pixel centre.
 */
float pfo_half_trunc(float f);
void pfo_gradient_ramp(const pf_color_stop *stops, uint32_t n, uint32_t *ramp);
int pfo_paint_is_opaque(const pf_scene_view *s, uint32_t p);
void pfo_paint_meta(const pf_paint *pp, float meta[12]);
void pfo_paint_color(const pf_paint *pp, const float meta[12], const uint32_t *ramp, double x, double y,
                     double out[4]);

/* Reference harness (oracle/_ref/libpfref.so): same output, z rule D3D9. */
int pfref_tile_scene(const pf_scene_view *scene, pfo_result *out);
/* The reference's own OutlineDash + OutlineStrokeToFill over the same scene. */
int pfref_stroke_scene(const pf_scene_view *scene, pfo_outline *out);
/* The reference's Gradient (add_color_stop, sample) for a ramp, and umHalf's round trip. */
void pfref_gradient_ramp(const pf_color_stop *stops, uint32_t n, uint32_t *ramp);
float pfref_half(float f);
void pfref_free(pfo_result *r);

/*
 * SVG: the reference's nanosvg (nsvgParse(text, "px", dpi), third_party/nanosvg.h) replayed as
 * SvgScene::SvgScene does (core/svg.cpp:135-205) through the reference's own Path2d and Paint,
 * written as a scene in pf_scene_view's layout: per shape a fill path when Canvas::fill_path
 * would draw one, then a stroke path (its contours plus a pf_stroke, dash phase 0) when
 * Canvas::stroke_path would.  stops are nanosvg's, in the order add_color_stop receives them;
 * ramps holds, per path, the 256 texels of the reference Gradient's ramp (zero for colour paints).
 */
typedef struct pfo_svg {
    uint32_t n_points, n_contours, n_paths, n_dashes, n_stops;
    float width, height;
    float *points;             /* [n_points][2] */
    uint8_t *point_flags;      /* [n_points] */
    uint32_t *contour_start;   /* [n_contours + 1] */
    uint8_t *contour_closed;   /* [n_contours] */
    uint32_t *path_start;      /* [n_paths + 1] */
    uint8_t *fill_rule;        /* [n_paths] */
    uint32_t *color;           /* [n_paths] */
    pf_stroke *path_stroke;    /* [n_paths] */
    float *dashes;             /* [n_dashes] */
    pf_paint *path_paint;      /* [n_paths] */
    pf_color_stop *stops;      /* [n_stops] */
    uint32_t *ramps;           /* [n_paths][256] */
} pfo_svg;
/* 0 ok; 1 nanosvg returned no image */
int pfref_svg_scene(const char *text, size_t length, float dpi, pfo_svg *out);
void pfref_svg_free(pfo_svg *s);

#ifdef __cplusplus
}
#endif

#endif
