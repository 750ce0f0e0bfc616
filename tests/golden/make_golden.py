"""Generate the golden fixtures from the reference's own d3d9 tiler.

Run in a checkout next to the reference sources (the reference tree is the one
oracle.REF_ROOT names: PF_REFERENCE_ROOT, else the oracle Makefile's default):

    python tests/golden/make_golden.py [fixture names]   # all fixtures when no name is given

For every scene below it builds oracle/_ref/libpfref.so (the reference's Tiler,
ObjectBuilder and SceneBuilderD3D9 compiled from their sources, driven by
oracle/ref_harness.cpp), runs it, and stores the scene together with the
reference's canonical integer output:

* ``<name>.npz``   - inputs and every canonical array (small scenes), and
* ``digests.json`` - SHA-256 of every canonical array of the full-size scenes,
                     plus a digest of their inputs so a test can tell that the
                     generator still produces the same scene.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "pathfinder-cpp_gb300"))

import oracle  # noqa: E402
import scenes as S  # noqa: E402
import svg_docs  # noqa: E402

CANON_KEYS = ["path_rect", "path_tile_first", "path_column_first", "tile_alpha", "tile_backdrop",
              "tile_fill_count", "fills", "column_backdrop", "fb_tiles", "z", "fb_list_first", "fb_list",
              "tile_mask", "tile_clip", "tile_dest_backdrop"]
INPUT_KEYS = ["points", "flags", "contour_start", "path_start", "fill_rule", "color"]
CLIP_KEYS = ["path_clip", "path_is_clip"]  # stored when the scene has clip paths
STROKE_KEYS = ["path_stroke", "contour_closed", "dashes"]  # stored when the scene has strokes
PAINT_KEYS = ["path_paint", "stops"]  # stored when the scene has gradient paints (with ref_ramps)
# the reference's stroke outline (OutlineDash + OutlineStrokeToFill), stored as out_<key>
OUTLINE_KEYS = ["points", "flags", "contour_start", "path_start", "fill_rule"]


def build_scene(paths, width, height, clear=0) -> S.Scene:
    """paths: list of (contours, rule, rgba); contours: list of (points[N,2], flags[N])."""
    pts, fl, cstart, pstart, rules, colors = [], [], [0], [0], [], []
    for contours, rule, rgba in paths:
        for p, f in contours:
            p = np.asarray(p, np.float32).reshape(-1, 2)
            f = np.asarray(f, np.uint8)
            assert len(p) == len(f)
            pts.append(p)
            fl.append(f)
            cstart.append(cstart[-1] + len(p))
        pstart.append(pstart[-1] + len(contours))
        rules.append(rule)
        colors.append(int(S.pack_rgba(*rgba)))
    return S.Scene(points=np.concatenate(pts) if pts else np.zeros((0, 2), np.float32),
                   flags=np.concatenate(fl) if fl else np.zeros(0, np.uint8),
                   contour_start=np.asarray(cstart, np.uint32), path_start=np.asarray(pstart, np.uint32),
                   fill_rule=np.asarray(rules, np.uint8), color=np.asarray(colors, np.uint32),
                   width=float(width), height=float(height), clear=int(clear))


def poly(*xy):
    p = np.asarray(xy, np.float32).reshape(-1, 2)
    return p, np.zeros(len(p), np.uint8)


def edge_scenes():
    red, green, blue = (255, 0, 0, 255), (0, 160, 0, 255), (0, 0, 255, 255)
    half = (20, 40, 200, 128)
    out = {}
    # 16x16-aligned square: exact backdrops, no fills inside
    out["aligned_square"] = build_scene([([poly(16, 16, 48, 16, 48, 48, 16, 48)], 0, red)], 64, 64)
    # half-pixel offset rectangle: coverage 0.5 on its edges
    out["half_pixel_rect"] = build_scene([([poly(10.5, 7.5, 37.5, 7.5, 37.5, 40.5, 10.5, 40.5)], 0, blue)], 48, 48)
    # self-overlapping pentagram, even-odd (hole) and nonzero (filled)
    star = poly(50, 5, 79, 95, 2, 40, 98, 40, 21, 95)
    out["star_even_odd"] = build_scene([([star], 1, red), ([poly(*(np.asarray(star[0]).ravel() + 3))], 0, half)],
                                       100, 100)
    # crossing the left, right and bottom edges; partly above the top edge (top is never clipped)
    out["view_box_edges"] = build_scene([
        ([poly(-30, 20, 90, -40, 130, 60, 40, 140)], 0, green),
        ([poly(-10, -50, 60, -30, 20, 30)], 1, half),
        ([poly(70, 70, 140, 75, 75, 160)], 0, blue)], 100, 90)
    # canvas width not a multiple of 16, tiny shapes, a point exactly on the right edge
    out["odd_canvas"] = build_scene([
        ([poly(0, 0, 100, 0, 100, 75, 0, 75)], 0, (255, 255, 255, 255)),
        ([poly(96, 10, 112, 20, 96, 40)], 0, red),
        ([poly(3.25, 3.75, 5.5, 3.75, 4.0, 6.0)], 0, blue)], 100, 75, clear=int(S.pack_rgba(10, 20, 30, 255)))
    # lines through tile corners (the walk's tie rule) and exact tile boundaries
    out["tile_corners"] = build_scene([
        ([poly(0, 0, 64, 64, 0, 64)], 0, red),
        ([poly(64, 0, 0, 64, 64, 64)], 1, half),
        ([poly(16, 48, 48, 16, 48, 48)], 0, green)], 64, 64)
    # closing line skipped when first ~= last (1e-4), kept when they differ by more
    out["closing_line"] = build_scene([
        ([poly(10, 10, 50, 12, 30, 50, 10.00005, 10.00003)], 0, red),
        ([poly(16.00001, 20, 40, 30, 15.99, 60.2)], 0, blue)], 64, 64)
    # malformed point patterns stop the contour; single-point and empty contours; empty path
    q_bad = (np.asarray([[5, 5], [30, 5], [40, 20], [30, 40], [5, 40]], np.float32),
             np.asarray([0, 1, 1, 0, 0], np.uint8))
    c_ok = (np.asarray([[5, 50], [20, 45], [40, 45], [55, 60], [30, 62]], np.float32),
            np.asarray([0, 1, 2, 0, 0], np.uint8))
    one = (np.asarray([[60, 60]], np.float32), np.asarray([0], np.uint8))
    ctl_first = (np.asarray([[10, 10], [20, 20], [30, 10]], np.float32), np.asarray([1, 0, 0], np.uint8))
    empty = (np.zeros((0, 2), np.float32), np.zeros(0, np.uint8))
    out["malformed"] = build_scene([([q_bad], 0, red), ([c_ok, one, empty], 0, green), ([], 0, blue),
                                    ([ctl_first], 0, half)], 64, 64)
    # quadratics and cubics with coincident control points; degenerate and vertical lines
    quad = (np.asarray([[4, 30], [32, -10], [60, 30], [32, 62], [4, 30]], np.float32),
            np.asarray([0, 1, 0, 1, 0], np.uint8))
    cub = (np.asarray([[8, 8], [8, 8], [56, 56], [56, 8], [56, 8], [56, 8], [8, 56]], np.float32),
           np.asarray([0, 1, 2, 0, 1, 2, 0], np.uint8))
    vert = poly(20, 5, 20, 60, 20, 60, 40, 60, 40, 5)
    out["curves_degenerate"] = build_scene([([quad], 0, red), ([cub], 1, half), ([vert], 0, green)], 64, 64)
    # a long line from far above the view box into it (walks many tiles above the rect)
    out["from_far_above"] = build_scene([([poly(30, -900, 50, 40, 10, 50)], 0, red),
                                         ([poly(5, 20, 60, -3000, 60, 60)], 1, blue)], 64, 64)
    # entirely outside the view box (left, right, below, above): empty tile rects
    out["outside"] = build_scene([([poly(-50, 10, -10, 10, -30, 40)], 0, red),
                                  ([poly(80, 10, 120, 10, 100, 40)], 0, red),
                                  ([poly(10, 80, 40, 80, 30, 120)], 0, red),
                                  ([poly(10, -80, 40, -80, 30, -20)], 0, red)], 64, 64)
    # glyph with holes (inner contour reversed), nonzero
    outer = poly(8, 8, 56, 8, 56, 56, 8, 56)
    inner = poly(20, 20, 20, 44, 44, 44, 44, 20)
    out["hole"] = build_scene([([outer, inner], 0, (0, 0, 0, 255))], 64, 64,
                              clear=int(S.pack_rgba(255, 255, 255, 255)))
    # translucent stack over an opaque base (z-buffer must not cull what shows through)
    out["translucent_stack"] = build_scene([
        ([poly(0, 0, 64, 0, 64, 64, 0, 64)], 0, (200, 200, 200, 255)),
        ([poly(4, 4, 60, 10, 30, 60)], 0, (255, 0, 0, 100)),
        ([poly(10, 50, 60, 50, 35, 2)], 1, (0, 0, 255, 160)),
        ([poly(20, 20, 40, 20, 40, 40, 20, 40)], 0, (0, 255, 0, 255)),
        ([poly(0, 30, 64, 34, 64, 36, 0, 40)], 0, (255, 255, 0, 60))], 64, 64)
    # winding beyond int8: 200 nested copies of one square (backdrop wraps)
    sq = poly(8, 8, 40, 8, 40, 40, 8, 40)
    out["int8_wrap"] = build_scene([([sq] * 200, 0, red), ([sq] * 130, 1, half)], 48, 48)
    return out


def clip_scenes():
    """Clip paths: every case of Tiler::prepare_tiles (tiler.cpp:386-431)."""
    red, blue, half = (255, 0, 0, 255), (0, 0, 255, 255), (20, 40, 200, 128)
    white = (255, 255, 255, 255)
    out = {}
    # a square clipped by a smaller diamond: alpha over alpha (combined masks), solid inside
    # (unchanged), solid over the diamond's edge tiles (the clip's mask), outside its rect (culled)
    diamond = poly(48, 8, 88, 48, 48, 88, 8, 48)
    sq = poly(2, 2, 94, 2, 94, 94, 2, 94)
    out["clip_diamond"] = S.with_clips(
        build_scene([([sq], 0, red), ([poly(30, 30, 66, 30, 66, 66, 30, 66)], 0, half)], 96, 96),
        build_scene([([diamond], 0, white)], 96, 96), np.array([0, -1]))
    # a clip with a hole: blank clip tiles inside its rect cull the draw path's solid tiles there
    outer = poly(4, 4, 92, 4, 92, 92, 4, 92)
    inner = poly(28, 28, 28, 68, 68, 68, 68, 28)
    out["clip_hole"] = S.with_clips(
        build_scene([([poly(0, 0, 96, 0, 96, 96, 0, 96)], 0, blue), ([poly(10, 40, 86, 44, 48, 90)], 1, half)],
                    96, 96),
        build_scene([([outer, inner], 0, white)], 96, 96), np.array([0, 0]))
    # an even-odd star as the clip of an even-odd star and of a translucent quadratic blob
    star = poly(50, 5, 79, 95, 2, 40, 98, 40, 21, 95)
    blob = (np.asarray([[10, 50], [50, -10], [90, 50], [50, 110], [10, 50]], np.float32),
            np.asarray([0, 1, 0, 1, 0], np.uint8))
    out["clip_even_odd"] = S.with_clips(
        build_scene([([poly(*(np.asarray(star[0]).ravel() + 2))], 1, red), ([blob], 0, half)], 100, 100),
        build_scene([([star], 1, white)], 100, 100), np.array([0, 0]))
    # two clips, one partly outside the view box, one path clipped by a clip of an empty rect
    out["clip_two"] = S.with_clips(
        build_scene([([poly(0, 0, 80, 0, 80, 80, 0, 80)], 0, red), ([poly(20, 10, 70, 60, 5, 70)], 0, blue),
                     ([poly(40, 40, 60, 40, 50, 60)], 0, half)], 80, 80),
        build_scene([([poly(-20, 30, 50, -10, 70, 70)], 0, white), ([poly(200, 200, 240, 200, 220, 240)], 0, white)],
                    80, 80), np.array([0, 0, 1]))
    return out


def stroke(width, cap=S.CAP_BUTT, join=S.JOIN_MITER, miter=10.0, dash=None, offset=0.0):
    return (width, cap, join, miter, dash, offset)


def with_strokes(sc: S.Scene, styles, closed) -> S.Scene:
    """styles: per path a stroke(...) tuple or None (filled); closed: per contour 0/1."""
    st = np.zeros(sc.n_paths, S.STROKE_DTYPE)
    dashes = []
    for p, style in enumerate(styles):
        if style is None:
            continue
        width, cap, join, miter, dash, offset = style
        st[p] = (width, miter, cap, join, 0, len(dashes), len(dash) if dash else 0, offset)
        if dash:
            dashes.extend(dash)
    sc.path_stroke = st
    sc.contour_closed = np.asarray(closed, np.uint8)
    sc.dashes = np.asarray(dashes if dashes else [1.0], np.float32)
    return sc


def curve(*items):
    """A contour from (x, y, flag) triples."""
    a = np.asarray(items, np.float32).reshape(-1, 3)
    return a[:, :2].copy(), a[:, 2].astype(np.uint8)


def stroke_scenes():
    """Stroke-to-fill and dashing (core/stroke.cpp, core/dash.cpp): caps, joins, curves,
    degenerate input and dash patterns."""
    red, green, blue = (255, 0, 0, 255), (0, 160, 0, 255), (0, 0, 255, 255)
    half = (20, 40, 200, 128)
    out = {}
    v = poly(10, 80, 40, 20, 70, 80)
    out["stroke_caps"] = with_strokes(build_scene(
        [([v], 0, red), ([poly(10, 100, 40, 40, 70, 100)], 0, half), ([poly(10, 60, 40, 5, 70, 60)], 0, blue),
         ([poly(85, 10, 85, 110)], 0, green)], 100, 120),
        [stroke(6, S.CAP_BUTT), stroke(10, S.CAP_SQUARE, S.JOIN_BEVEL), stroke(14, S.CAP_ROUND, S.JOIN_ROUND),
         stroke(5, S.CAP_ROUND)], [0, 0, 0, 0])
    tri = poly(20, 20, 100, 30, 40, 90)
    sharp = poly(10, 110, 118, 100, 10, 104)
    ring = poly(70, 70, 110, 70, 110, 110, 70, 110, 70, 70)   # last point repeats the first
    out["stroke_joins"] = with_strokes(build_scene(
        [([tri], 0, red), ([poly(60, 10, 120, 50, 80, 60)], 0, half), ([sharp], 0, blue), ([ring], 0, green),
         ([poly(5, 60, 30, 40, 55, 60)], 0, half)], 128, 128),
        [stroke(8, join=S.JOIN_MITER), stroke(6, join=S.JOIN_BEVEL), stroke(4, join=S.JOIN_MITER, miter=1.5),
         stroke(7, join=S.JOIN_ROUND), stroke(9, S.CAP_SQUARE, S.JOIN_ROUND)], [1, 1, 1, 1, 0])
    quad = curve(10, 100, 0, 50, -20, 1, 90, 100, 0)
    cub = curve(10, 20, 0, 10, 20, 1, 60, 90, 2, 110, 20, 0)             # ctrl0 == from
    cub2 = curve(10, 60, 0, 50, 0, 1, 110, 60, 2, 110, 60, 0)            # ctrl1 == to
    loop = curve(20, 110, 0, 120, 40, 1, 0, 40, 2, 100, 110, 0)          # a cubic with a loop
    tight = curve(60, 60, 0, 64, 50, 1, 68, 50, 2, 72, 60, 0)            # wide stroke, tight curve
    out["stroke_curves"] = with_strokes(build_scene(
        [([quad], 0, red), ([cub], 0, half), ([cub2], 0, blue), ([loop], 0, green), ([tight], 0, half)],
        128, 128),
        [stroke(5, S.CAP_ROUND, S.JOIN_ROUND), stroke(3), stroke(4, S.CAP_SQUARE, S.JOIN_BEVEL),
         stroke(6, S.CAP_BUTT, S.JOIN_MITER, 4.0), stroke(30, S.CAP_ROUND, S.JOIN_ROUND)], [0, 1, 0, 0, 0])
    out["stroke_degenerate"] = with_strokes(build_scene(
        [([poly(30, 30)], 0, red),                                   # one point
         ([poly(50, 50, 50, 50)], 0, red),                           # two equal points
         ([poly(10, 80, 40, 80, 40, 80, 70, 60)], 0, blue),          # a zero-length line inside
         ([poly(80, 10, 80.05, 10.02, 80.09, 10.01, 110, 40)], 0, half),  # segments under 0.1 px
         ([poly(20, 110, 100, 110, 40, 110)], 0, green),             # a 180-degree turn
         ([poly(60, 60, 70, 65)], 0, half),                          # a huge width
         ([poly(5, 5, 20, 5, 20, 20)], 0, red)],                     # width under a pixel
        128, 128),
        [stroke(6, S.CAP_ROUND, S.JOIN_ROUND), stroke(6, S.CAP_SQUARE), stroke(5, S.CAP_SQUARE, S.JOIN_MITER),
         stroke(4, S.CAP_ROUND, S.JOIN_ROUND), stroke(6, S.CAP_BUTT, S.JOIN_MITER), stroke(200, S.CAP_ROUND),
         stroke(0.5, S.CAP_BUTT, S.JOIN_BEVEL)], [0, 1, 0, 0, 0, 0, 1])
    wave = curve(10, 40, 0, 40, 0, 1, 60, 80, 2, 90, 40, 0, 100, 30, 0)
    out["stroke_dashes"] = with_strokes(build_scene(
        [([poly(10, 10, 110, 10), poly(10, 20, 110, 20)], 0, red),   # the pattern runs on across contours
         ([wave], 0, blue),
         ([poly(20, 60, 100, 60, 100, 110, 20, 110)], 0, half),     # a closed contour dashed
         ([poly(10, 120, 118, 120)], 0, green)],                     # a zero entry in the pattern
        128, 128),
        [stroke(4, S.CAP_BUTT, dash=[7, 5]), stroke(5, S.CAP_ROUND, S.JOIN_ROUND, dash=[12, 4, 3, 4], offset=9.5),
         stroke(6, S.CAP_SQUARE, S.JOIN_MITER, dash=[20, 10], offset=25.0),
         stroke(3, S.CAP_ROUND, dash=[0, 8, 6, 4])], [0, 0, 0, 1, 0])
    return out


def with_paints(sc: S.Scene, paints) -> S.Scene:
    """paints: per path None (solid) or (type, wrap, stops [(offset, rgba)], line, radii, transform)."""
    pp = np.zeros(sc.n_paths, S.PAINT_DTYPE)
    pp["transform"] = [1, 0, 0, 1, 0, 0]
    stops = []
    for p, paint in enumerate(paints):
        if paint is None:
            continue
        kind, wrap, st, line, radii, xf = paint
        pp[p]["type"], pp[p]["wrap"] = kind, wrap
        pp[p]["stop_first"], pp[p]["stop_count"] = len(stops), len(st)
        pp[p]["line"], pp[p]["radii"] = line, radii
        if xf is not None:
            pp[p]["transform"] = xf
        stops.extend((o, int(S.pack_rgba(*c))) for o, c in st)
    sc.path_paint = pp
    sc.stops = np.asarray(stops if stops else [(0.0, 0)], S.STOP_DTYPE)
    return sc


def gradient_scenes():
    """Gradient paints (Paint::from_gradient): linear and radial, clamped and repeated, opaque
    and translucent stops, unsorted and repeated offsets, a transformed radial gradient."""
    L, R, C, P = S.PAINT_LINEAR, S.PAINT_RADIAL, S.WRAP_CLAMP, S.WRAP_REPEAT
    red, green, blue, white = (255, 0, 0, 255), (0, 160, 0, 255), (0, 0, 255, 255), (255, 255, 255, 255)
    half = (20, 40, 200, 128)
    out = {}
    rects = [poly(4, 4, 60, 4, 60, 60, 4, 60), poly(68, 4, 124, 4, 124, 60, 68, 60),
             poly(4, 68, 60, 68, 60, 124, 4, 124), poly(68, 68, 124, 68, 124, 124, 68, 124),
             poly(30, 30, 98, 40, 64, 100)]
    out["grad_linear"] = with_paints(build_scene([([r], 0, white) for r in rects], 128, 128, clear=0xff202020), [
        (L, C, [(0.0, red), (1.0, blue)], [4, 0, 60, 0], [0, 0], None),
        (L, P, [(0.5, green), (0.0, red), (1.0, blue)], [70, 6, 90, 30], [0, 0], None),
        (L, C, [(0.2, half), (0.8, (200, 200, 0, 60))], [4, 124, 60, 68], [0, 0], None),
        (L, C, [(0.3, red), (0.3, green), (0.7, blue)], [68, 68, 124, 124], [0, 0], None),
        (L, C, [(0.5, (255, 128, 0, 200))], [30, 30, 98, 100], [0, 0], None)])
    out["grad_radial"] = with_paints(build_scene([([r], 0, white) for r in rects], 128, 128, clear=0xff000000), [
        (R, C, [(0.0, white), (1.0, blue)], [32, 32, 32, 32], [0, 28], None),
        (R, P, [(0.0, red), (0.5, green), (1.0, red)], [96, 32, 100, 28], [0, 12], None),
        (R, C, [(0.0, half), (1.0, (250, 250, 250, 40))], [20, 100, 44, 90], [6, 30], None),
        (R, C, [(0.0, green), (1.0, red)], [96, 96, 96, 96], [0, 24], [0.8, 0.45, -0.45, 0.8, 60.0, -24.0]),
        (R, P, [(0.0, blue), (1.0, white)], [64, 64, 70, 60], [10, 40], None)])
    return out


def generator_scenes():
    return {
        "gen_plain_small_s1": S.plain_small(seed=1, n_paths=24, side=256),
        "gen_large_mixed_s2": S.large_single(seed=2, n_paths=120, side=512),
        "gen_glyphs_s3": S.glyphs(seed=3, n_paths=400, side=256),
        "gen_mixed_s4": S.mixed(seed=4, n_paths=96, side=512),
        "gen_batched_scene_s5": S.batched(n_scenes=3, first_seed=5, hi_paths=64)[2],
        "gen_clipped_s6": S.clipped(seed=6, n_paths=60, side=256, n_clips=4),
        "gen_stroked_s7": S.stroked(seed=7, n_paths=40, side=256, dash_share=0.4, fill_share=0.2),
        "gen_gradient_s8": S.gradient_scene(seed=8, n_paths=60, side=256),
    }


def with_view_box(sc: S.Scene, box) -> S.Scene:
    sc.view_box = np.asarray(box, np.float32)
    return sc


def view_box_scenes():
    """Scenes whose view box (Scene::set_view_box) is not the canvas: an inner box with a
    fractional origin, a box reaching above and left of the canvas (negative tile coordinates)
    and past its right and bottom edges, and a clipped scene inside a box."""
    wide = S.large_single(seed=12, n_paths=60, side=640)
    wide.points = (wide.points.astype(np.float64) * 1.25 - 96.0).astype(np.float32)  # some paths off canvas
    return {
        "view_box_inner": with_view_box(S.plain_small(seed=9, n_paths=40, side=512), [37.5, 21.25, 401.7, 389.0]),
        "view_box_outside": with_view_box(S.Scene(**{**wide.__dict__, "width": 480.0, "height": 400.0}),
                                          [-70.3, -33.0, 530.0, 470.5]),
        "view_box_clipped": with_view_box(S.clipped(seed=13, n_paths=50, side=256, n_clips=3), [64.0, 40.0, 200.0, 230.0]),
    }


def svg_scenes():
    """SVG documents through the reference's nanosvg + SvgScene replay (the harness): the scene
    the reference's canvas builds, stored with the document's text (svg_text) so the parser can be
    checked against it where the reference is absent.  Paint arrays are kept only when the
    document has a gradient."""
    docs = {k: v for k, v in svg_docs.HAND.items() if k != "svg_empty"}
    docs.update({f"svg_random_s{seed}": svg_docs.random_document(seed) for seed in (101, 102, 103)})
    out = {}
    for name, text in docs.items():
        r = oracle.reference_svg_scene(text)
        sc = S.Scene(points=r["points"], flags=r["flags"], contour_start=r["contour_start"],
                     path_start=r["path_start"], fill_rule=r["fill_rule"], color=r["color"],
                     width=float(r["width"]), height=float(r["height"]))
        sc.path_stroke = r["path_stroke"].view(S.STROKE_DTYPE)
        sc.contour_closed, sc.dashes = r["contour_closed"], r["dashes"]
        paint = r["path_paint"].view(S.PAINT_DTYPE)
        if np.any(paint["type"] != S.PAINT_SOLID):
            sc.path_paint, sc.stops = paint, r["stops"].view(S.STOP_DTYPE)
        out[name] = (sc, text)
    return out


def full_scenes():
    return {"plain_small_1024": S.plain_small()}


def digest(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


def scene_digest(sc: S.Scene) -> str:
    h = hashlib.sha256()
    for k in INPUT_KEYS:
        h.update(digest(getattr(sc, k)).encode())
    h.update(np.asarray([sc.width, sc.height, sc.clear], np.float64).tobytes())
    return h.hexdigest()


def main() -> None:
    oracle.build(reference=True)
    if not oracle.have_reference():
        raise SystemExit("the reference tiler could not be built (is the reference tree present?)")
    small = dict(edge_scenes())
    small.update(clip_scenes())
    small.update(stroke_scenes())
    small.update(gradient_scenes())
    small.update(generator_scenes())
    small.update(view_box_scenes())
    texts = {}
    for name, (sc, text) in svg_scenes().items():
        small[name], texts[name] = sc, text
    only = set(sys.argv[1:])  # names to (re)write; all when none are given
    for name, sc in small.items():
        if only and name not in only:
            continue
        ref = oracle.reference_tile_scene(sc)
        arrays = {k: getattr(sc, k) for k in INPUT_KEYS}
        if sc.path_clip is not None:
            arrays.update({k: getattr(sc, k) for k in CLIP_KEYS})
        if sc.path_stroke is not None:
            arrays.update({k: getattr(sc, k) for k in STROKE_KEYS})
            outline = oracle.stroke_scene(sc, reference=True)
            arrays.update({"out_" + k: getattr(outline, k) for k in OUTLINE_KEYS})
        if sc.path_paint is not None:
            arrays.update({k: getattr(sc, k) for k in PAINT_KEYS})
            arrays["ref_ramps"] = oracle.reference_ramps(sc)
        if sc.view_box is not None:
            arrays["view_box"] = sc.view_box
        arrays["meta"] = np.asarray([sc.width, sc.height, sc.clear], np.float64)
        if name in texts:
            arrays["svg_text"] = np.frombuffer(texts[name].encode(), np.uint8)
        for k in CANON_KEYS:
            arrays["ref_" + k] = ref[k]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        print(f"{name}: {sc.n_paths} paths, {len(ref['fills'])} fills, {int(ref['tile_alpha'].sum())} alpha tiles")
    if only:
        return
    digests = {}
    for name, sc in full_scenes().items():
        ref = oracle.reference_tile_scene(sc)
        digests[name] = {"scene": scene_digest(sc), "canon": {k: digest(ref[k]) for k in CANON_KEYS},
                         "fills": int(len(ref["fills"])), "alpha_tiles": int(ref["tile_alpha"].sum())}
        print(f"{name}: {digests[name]['fills']} fills")
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
