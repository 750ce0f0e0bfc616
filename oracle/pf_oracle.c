/*
 * pf_oracle.c - CPU restatement of the reference's d3d9 tiler, and an FP64
 * analytic-area coverage + src-over composite oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see pf_oracle.h).  Parity of this restatement is
 * pinned against the reference's own tiler (ref_harness.cpp) through the
 * committed golden fixtures in tests/golden/.
 *
 * Float arithmetic follows the reference operation by operation (the reference
 * runs it in SSE lanes, pathfinder/common/f32x4.h, with no FMA contraction); this
 * file must be compiled with -ffp-contract=off so the same holds on Arm.
 */
#include "pf_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define TILE 16
#define FLATTENING_TOLERANCE 1.0f   /* pathfinder/core/d3d9/tiler.cpp:15 */
#define FLOAT_EPSILON 0.0001f       /* pathfinder/common/math/basic.h:11 */
#define MAX_DEPTH 64                /* recursion bound; the reference has none */
#define MAX_WALK (1u << 22)         /* tile-walk bound; the reference has none */

/* ------------------------------------------------------------------------ */
/* growable arrays                                                           */

typedef struct {
    uint32_t tile;       /* tile index inside the path's tile rect */
    uint16_t c[4];       /* from_x, from_y, to_x, to_y */
} fill_rec;

typedef struct {
    /* view box used for clipping (top is -inf, tiler.cpp:144) */
    float vb_left, vb_right, vb_bottom;
    /* tile rect */
    int32_t rx0, ry0, rx1, ry1, rw, rh;
    int32_t *col;        /* [rw] column sums, int32 (BuiltPathData::backdrops) */
    int8_t *bd;          /* [rw*rh] int8 tile backdrops (TileObjectPrimitive::backdrop) */
    uint32_t *fcount;    /* [rw*rh] fills per tile */
    fill_rec *fills;
    size_t nfill, capfill;
    uint64_t nleaf;
    int error;
} path_ctx;

static void push_fill(path_ctx *pc, uint32_t tile, uint16_t fx, uint16_t fy, uint16_t tx, uint16_t ty) {
    if (pc->nfill == pc->capfill) {
        size_t cap = pc->capfill ? pc->capfill * 2 : 256;
        fill_rec *n = (fill_rec *)realloc(pc->fills, cap * sizeof(fill_rec));
        if (!n) {
            pc->error = 1;
            return;
        }
        pc->fills = n;
        pc->capfill = cap;
    }
    fill_rec *f = &pc->fills[pc->nfill++];
    f->tile = tile;
    f->c[0] = fx;
    f->c[1] = fy;
    f->c[2] = tx;
    f->c[3] = ty;
}

/* ------------------------------------------------------------------------ */
/* ObjectBuilder::add_fill / adjust_alpha_tile_backdrop                      */
/* (pathfinder/core/d3d9/object_builder.cpp:19-64, 96-114)                    */

static float sse_max(float a, float b) { return a > b ? a : b; } /* _mm_max_ps */
static float sse_min(float a, float b) { return a < b ? a : b; } /* _mm_min_ps */

static void add_fill(path_ctx *pc, float x0, float y0, float x1, float y1, int32_t tx, int32_t ty) {
    /* RectI::contains_point(Vec2I): left <= x <= right-1, top <= y <= bottom-1 */
    if (!(pc->rx0 <= tx && tx <= pc->rx1 - 1 && pc->ry0 <= ty && ty <= pc->ry1 - 1)) return;
    const float ox = (float)tx * (float)TILE, oy = (float)ty * (float)TILE;
    float v[4] = {(x0 - ox) * 256.0f, (y0 - oy) * 256.0f, (x1 - ox) * 256.0f, (y1 - oy) * 256.0f};
    uint16_t q[4];
    for (int k = 0; k < 4; k++) {
        float c = sse_min(sse_max(v[k], 0.0f), (float)(TILE * 256 - 1));
        c = rintf(c); /* _mm_round_ps(_MM_FROUND_TO_NEAREST_INT): ties to even */
        q[k] = (uint16_t)c;
    }
    if (q[0] == q[2]) return; /* vertical after quantisation: culled */
    const uint32_t local = (uint32_t)((ty - pc->ry0) * pc->rw + (tx - pc->rx0));
    pc->fcount[local]++;
    push_fill(pc, local, q[0], q[1], q[2], q[3]);
}

static void adjust_backdrop(path_ctx *pc, int32_t tx, int32_t ty, int8_t delta) {
    const int32_t ox = tx - pc->rx0, oy = ty - pc->ry0;
    if (ox < 0 || ox >= pc->rw || oy >= pc->rh) return;
    if (oy < 0) {
        pc->col[ox] += delta;
        return;
    }
    int8_t *b = &pc->bd[oy * pc->rw + ox];
    *b = (int8_t)(*b + delta); /* int8 wraps */
}

/* ------------------------------------------------------------------------ */
/* clip_line_segment_to_rect (pathfinder/core/d3d9/tiler.cpp:46-125)          */

enum { OC_LEFT = 1, OC_RIGHT = 2, OC_TOP = 4, OC_BOTTOM = 8 };

static int outcode(const path_ctx *pc, float x, float y) {
    int o = 0;
    if (x < pc->vb_left) o |= OC_LEFT;
    else if (x > pc->vb_right) o |= OC_RIGHT;
    /* the clip box top is -inf: nothing is ever above it */
    if (y > pc->vb_bottom) o |= OC_BOTTOM;
    return o;
}

static float lerp_clamped(float a, float b, float t) { /* common/math/basic.h:50-53 */
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return a + (b - a) * t;
}

static int clip_line(const path_ctx *pc, float *x0, float *y0, float *x1, float *y1) {
    int of = outcode(pc, *x0, *y0), ot = outcode(pc, *x1, *y1);
    for (int iter = 0; iter < 64; iter++) {
        if (of == 0 && ot == 0) return 1;
        if ((of & ot) != 0) return 0;
        const int clip_from = of > ot;
        const int oc = clip_from ? of : ot;
        float px = clip_from ? *x0 : *x1, py = clip_from ? *y0 : *y1;
        if (oc & OC_LEFT) {
            px = pc->vb_left;
            py = lerp_clamped(*y0, *y1, (pc->vb_left - *x0) / (*x1 - *x0));
        } else if (oc & OC_RIGHT) {
            px = pc->vb_right;
            py = lerp_clamped(*y0, *y1, (pc->vb_right - *x0) / (*x1 - *x0));
        } else if (oc & OC_BOTTOM) {
            px = lerp_clamped(*x0, *x1, (pc->vb_bottom - *y0) / (*y1 - *y0));
            py = pc->vb_bottom;
        }
        if (clip_from) {
            *x0 = px;
            *y0 = py;
            of = outcode(pc, px, py);
        } else {
            *x1 = px;
            *y1 = py;
            ot = outcode(pc, px, py);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* process_line_segment (pathfinder/core/d3d9/tiler.cpp:131-279)              */

enum { STEP_NONE = 0, STEP_X = 1, STEP_Y = 2 };

static void process_line(path_ctx *pc, float x0, float y0, float x1, float y1) {
    pc->nleaf++;
    if (!isfinite(x0) || !isfinite(y0) || !isfinite(x1) || !isfinite(y1)) return;
    if (!clip_line(pc, &x0, &y0, &x1, &y1)) return;

    const float inv = 1.0f / (float)TILE;
    const int32_t fx = (int32_t)floorf(x0 * inv), fy = (int32_t)floorf(y0 * inv);
    const int32_t ex = (int32_t)floorf(x1 * inv), ey = (int32_t)floorf(y1 * inv);
    const float vx = x1 - x0, vy = y1 - y0;
    const int32_t sx = vx < 0.0f ? -1 : 1, sy = vy < 0.0f ? -1 : 1;
    const float cx = ((float)fx + (vx >= 0.0f ? 1.0f : 0.0f)) * (float)TILE;
    const float cy = ((float)fy + (vy >= 0.0f ? 1.0f : 0.0f)) * (float)TILE;
    float tmx = (cx - x0) / vx, tmy = (cy - y0) / vy;
    const float tdx = fabsf((float)TILE / vx), tdy = fabsf((float)TILE / vy);

    float curx = x0, cury = y0;
    int32_t tcx = fx, tcy = fy;
    int last = STEP_NONE;
    for (uint32_t it = 0;; it++) {
        if (it >= MAX_WALK) {
            pc->error = 2;
            return;
        }
        int next;
        if (tmx < tmy) next = STEP_X;
        else if (tmx > tmy) next = STEP_Y;
        else next = sx > 0 ? STEP_X : STEP_Y;
        float nt = next == STEP_X ? tmx : tmy;
        nt = (1.0f < nt) ? 1.0f : nt; /* std::min(next_t, 1.0f) */
        if (tcx == ex && tcy == ey) next = STEP_NONE;
        const float npx = x0 + vx * nt, npy = y0 + vy * nt; /* LineSegmentF::sample */

        add_fill(pc, curx, cury, npx, npy, tcx, tcy);
        if (sy < 0 && next == STEP_Y) {
            add_fill(pc, npx, npy, (float)tcx * (float)TILE, (float)tcy * (float)TILE, tcx, tcy);
        } else if (sy > 0 && last == STEP_Y) {
            add_fill(pc, (float)tcx * (float)TILE, (float)tcy * (float)TILE, curx, cury, tcx, tcy);
        }
        if (sx < 0 && last == STEP_X) adjust_backdrop(pc, tcx, tcy, 1);
        else if (sx > 0 && next == STEP_X) adjust_backdrop(pc, tcx, tcy, -1);

        if (next == STEP_X) {
            tmx += tdx;
            tcx += sx;
        } else if (next == STEP_Y) {
            tmy += tdy;
            tcy += sy;
        } else {
            break;
        }
        curx = npx;
        cury = npy;
        last = next;
    }
}

/* ------------------------------------------------------------------------ */
/* Recursive flattening (tiler.cpp:284-315; segment.cpp:12-126)               */

static int flat_cubic(const float b[4], const float c[4]) {
    /* uv = 3*ctrl - base - base - base.zwxy */
    float uv[4];
    const float bz[4] = {b[2], b[3], b[0], b[1]};
    for (int k = 0; k < 4; k++) {
        float t = 3.0f * c[k];
        t = t - b[k];
        t = t - b[k];
        t = t - bz[k];
        uv[k] = t * t;
    }
    const float m0 = uv[0] > uv[2] ? uv[0] : uv[2];
    const float m1 = uv[1] > uv[3] ? uv[1] : uv[3];
    return m0 + m1 <= FLATTENING_TOLERANCE;
}

static int flat_quad(const float b[4], const float c[2]) {
    const float mx = (b[0] + b[2]) * 0.5f, my = (b[1] + b[3]) * 0.5f;
    const float dx = c[0] - mx, dy = c[1] - my;
    const float dx2 = dx * dx, dy2 = dy * dy;
    return dx2 + dy2 <= FLATTENING_TOLERANCE * 0.25f;
}

static float half_lerp(float a, float b) { return a + 0.5f * (b - a); }

static void flatten_cubic(path_ctx *pc, const float b[4], const float c[4], int depth) {
    if (flat_cubic(b, c) || depth >= MAX_DEPTH) {
        if (depth >= MAX_DEPTH) pc->error = 3;
        process_line(pc, b[0], b[1], b[2], b[3]);
        return;
    }
    /* split_cubic at t = 0.5, lane by lane as in segment.cpp:62-95 */
    float p01[2], p12[2], p23[2], p012[2], p123[2], p0123[2];
    for (int k = 0; k < 2; k++) {
        p01[k] = b[k] + 0.5f * (c[k] - b[k]);
        p12[k] = c[k] + 0.5f * (c[2 + k] - c[k]);
        p23[k] = c[2 + k] + 0.5f * (b[2 + k] - c[2 + k]);
        p012[k] = p01[k] + 0.5f * (p12[k] - p01[k]);
        p123[k] = p12[k] + 0.5f * (p23[k] - p12[k]);
        p0123[k] = p012[k] + 0.5f * (p123[k] - p012[k]);
    }
    const float b0[4] = {b[0], b[1], p0123[0], p0123[1]}, c0[4] = {p01[0], p01[1], p012[0], p012[1]};
    const float b1[4] = {p0123[0], p0123[1], b[2], b[3]}, c1[4] = {p123[0], p123[1], p23[0], p23[1]};
    flatten_cubic(pc, b0, c0, depth + 1);
    flatten_cubic(pc, b1, c1, depth + 1);
}

static void flatten_quad(path_ctx *pc, const float b[4], const float c[2], int depth) {
    if (flat_quad(b, c) || depth >= MAX_DEPTH) {
        if (depth >= MAX_DEPTH) pc->error = 3;
        process_line(pc, b[0], b[1], b[2], b[3]);
        return;
    }
    /* split_quadratic at t = 0.5 (segment.cpp:102-126) */
    float a[2], bb[2], m[2];
    for (int k = 0; k < 2; k++) {
        a[k] = b[k] + (c[k] - b[k]) * 0.5f;
        bb[k] = c[k] + (b[2 + k] - c[k]) * 0.5f;
        m[k] = a[k] + (bb[k] - a[k]) * 0.5f;
    }
    const float b0[4] = {b[0], b[1], m[0], m[1]};
    const float b1[4] = {m[0], m[1], b[2], b[3]};
    flatten_quad(pc, b0, a, depth + 1);
    flatten_quad(pc, b1, bb, depth + 1);
}

/* ------------------------------------------------------------------------ */
/* SegmentsIter::get_next(force_closed = true) (pathfinder/core/data/contour.cpp:110-175) */

static void tile_contour(path_ctx *pc, const float *pts, const uint8_t *fl, uint32_t n) {
    if (n == 0) return;
    uint32_t head = 0;
    for (;;) {
        if (head >= n || fl[head] != PF_POINT_ON_CURVE) return;
        const float *p = pts + 2 * (size_t)head;
        if (head + 1 < n) {
            if (fl[head + 1] == PF_POINT_ON_CURVE) {
                process_line(pc, p[0], p[1], p[2], p[3]);
                head += 1;
            } else if (head + 2 < n) {
                if (fl[head + 1] == PF_POINT_CONTROL_0 && fl[head + 2] == PF_POINT_ON_CURVE) {
                    const float b[4] = {p[0], p[1], p[4], p[5]}, c[2] = {p[2], p[3]};
                    flatten_quad(pc, b, c, 0);
                    head += 2;
                } else if (head + 3 < n) {
                    if (fl[head + 1] == PF_POINT_CONTROL_0 && fl[head + 2] == PF_POINT_CONTROL_1 &&
                        fl[head + 3] == PF_POINT_ON_CURVE) {
                        const float b[4] = {p[0], p[1], p[6], p[7]}, c[4] = {p[2], p[3], p[4], p[5]};
                        flatten_cubic(pc, b, c, 0);
                        head += 3;
                    } else {
                        return;
                    }
                } else {
                    return;
                }
            } else {
                return;
            }
        } else {
            /* end of the contour: implicit closing line unless first ~= last (1e-4) */
            if (n > 1) {
                const float dx = pts[0] - pts[2 * (size_t)(n - 1)];
                const float dy = pts[1] - pts[2 * (size_t)(n - 1) + 1];
                const float dx2 = dx * dx, dy2 = dy * dy;
                if (!(sqrtf(dx2 + dy2) <= FLOAT_EPSILON)) {
                    process_line(pc, pts[2 * (size_t)(n - 1)], pts[2 * (size_t)(n - 1) + 1], pts[0], pts[1]);
                }
            }
            return;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Tiler::Tiler + generate_tiles + prepare_tiles (tiler.cpp:317-439)          */

static void path_rect(const pf_scene_view *s, uint32_t p, const float vb[4], int32_t r[4]) {
    /* Outline::bounds = union of the contours' point bounds */
    float l = 1.0f, t = 1.0f, rr = 0.0f, b = 0.0f;
    int valid = 0;
    for (uint32_t c = s->path_start[p]; c < s->path_start[p + 1]; c++) {
        for (uint32_t i = s->contour_start[c]; i < s->contour_start[c + 1]; i++) {
            const float x = s->points[2 * (size_t)i], y = s->points[2 * (size_t)i + 1];
            if (!valid) {
                l = rr = x;
                t = b = y;
                valid = 1;
            } else {
                l = x < l ? x : l;   /* Vec2::min -> std::min */
                t = y < t ? y : t;
                rr = rr < x ? x : rr; /* Vec2::max -> std::max */
                b = b < y ? y : b;
            }
        }
    }
    /* RectF::intersection with the view box vb = (left, top, right, bottom)
     * (common/math/rect.h:160-172): an invalid {1, 1, 0, 0} when they do not meet */
    float il, it, ir, ib;
    if (l > vb[2] || rr < vb[0] || t > vb[3] || b < vb[1]) {
        il = 1.0f;
        it = 1.0f;
        ir = 0.0f;
        ib = 0.0f;
    } else {
        il = l < vb[0] ? vb[0] : l;
        it = t < vb[1] ? vb[1] : t;
        ir = vb[2] < rr ? vb[2] : rr;
        ib = vb[3] < b ? vb[3] : b;
    }
    const float inv = 1.0f / (float)TILE;
    r[0] = (int32_t)floorf(il * inv);
    r[1] = (int32_t)floorf(it * inv);
    r[2] = (int32_t)ceilf(ir * inv);
    r[3] = (int32_t)ceilf(ib * inv);
}

static float view_box_right(float width) {
    /* Scene::set_view_box: right = round_up(ceil(right), 16) (pathfinder/core/scene.cpp:175) */
    int32_t w = (int32_t)ceilf(width);
    int32_t rem = (w < 0 ? -w : w) % TILE;
    if (rem != 0) w = w < 0 ? w + rem : w + TILE - rem;
    return (float)w;
}

/* The scene's view box as Scene::set_view_box stores it (scene.cpp:169-176): the given rect, or
 * (0, 0, width, height), with its right edge rounded up to a multiple of 16. */
static void scene_view_box(const pf_scene_view *s, float vb[4]) {
    vb[0] = s->view_box ? s->view_box[0] : 0.0f;
    vb[1] = s->view_box ? s->view_box[1] : 0.0f;
    vb[2] = view_box_right(s->view_box ? s->view_box[2] : s->width);
    vb[3] = s->view_box ? s->view_box[3] : s->height;
}

static int tile_path(const pf_scene_view *s, uint32_t p, path_ctx *pc) {
    memset(pc, 0, sizeof(*pc));
    float vb[4];
    scene_view_box(s, vb);
    pc->vb_left = vb[0];
    pc->vb_right = vb[2];
    pc->vb_bottom = vb[3];
    int32_t r[4];
    path_rect(s, p, vb, r);
    pc->rx0 = r[0];
    pc->ry0 = r[1];
    pc->rx1 = r[2];
    pc->ry1 = r[3];
    pc->rw = r[2] - r[0];
    pc->rh = r[3] - r[1];
    if (pc->rw < 0) pc->rw = 0;
    if (pc->rh < 0) pc->rh = 0;
    const size_t nt = (size_t)pc->rw * (size_t)pc->rh;
    pc->col = (int32_t *)calloc(pc->rw ? pc->rw : 1, sizeof(int32_t));
    pc->bd = (int8_t *)calloc(nt ? nt : 1, 1);
    pc->fcount = (uint32_t *)calloc(nt ? nt : 1, sizeof(uint32_t));
    if (!pc->col || !pc->bd || !pc->fcount) return 1;

    for (uint32_t c = s->path_start[p]; c < s->path_start[p + 1]; c++) {
        const uint32_t a = s->contour_start[c], e = s->contour_start[c + 1];
        tile_contour(pc, s->points + 2 * (size_t)a, s->point_flags + a, e - a);
    }
    /* prepare_tiles: running int32 column sums, tile backdrop = int8(sum above) */
    for (size_t i = 0; i < nt; i++) {
        const size_t column = i % (size_t)pc->rw;
        const int8_t delta = pc->bd[i];
        pc->bd[i] = (int8_t)pc->col[column];
        pc->col[column] += delta;
    }
    return pc->error ? 1 : 0;
}

/* ------------------------------------------------------------------------ */
/* threads over paths                                                        */

typedef struct {
    const pf_scene_view *s;
    path_ctx *pcs;
    uint32_t first, step;
    int status;
} tile_job;

static void *tile_worker(void *arg) {
    tile_job *j = (tile_job *)arg;
    for (uint32_t p = j->first; p < j->s->n_paths; p += j->step) {
        if (tile_path(j->s, p, &j->pcs[p])) j->status = 1;
    }
    return NULL;
}

static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static int validate(const pf_scene_view *s) {
    if (!s || s->n_paths == 0) return s ? 0 : 1;
    if (!s->path_start || !s->contour_start || !s->fill_rule || !s->color) return 1;
    if (s->path_start[0] != 0 || s->path_start[s->n_paths] != s->n_contours) return 1;
    if (s->contour_start[0] != 0 || s->contour_start[s->n_contours] != s->n_points) return 1;
    if (s->n_points && (!s->points || !s->point_flags)) return 1;
    for (uint32_t p = 0; p < s->n_paths; p++)
        if (s->path_start[p] > s->path_start[p + 1]) return 1;
    for (uint32_t c = 0; c < s->n_contours; c++)
        if (s->contour_start[c] > s->contour_start[c + 1]) return 1;
    if (!(s->width > 0.0f) || !(s->height > 0.0f)) return 1;
    for (uint32_t p = 0; s->path_paint && p < s->n_paths; p++) {
        const pf_paint *pp = &s->path_paint[p];
        if (pp->type > PF_PAINT_RADIAL || pp->wrap > PF_WRAP_REPEAT) return 1;
        if (pp->type != PF_PAINT_SOLID && ((uint64_t)pp->stop_first + pp->stop_count > s->n_stops ||
                                           (pp->stop_count && !s->stops)))
            return 1;
    }
    if (s->path_clip || s->path_is_clip) {
        /* clip paths follow the draw paths, are not clipped, and draw paths name clip paths */
        if (!s->path_clip || !s->path_is_clip) return 1;
        int seen_clip = 0;
        for (uint32_t p = 0; p < s->n_paths; p++) {
            const uint32_t c = s->path_clip[p];
            if (s->path_is_clip[p]) {
                seen_clip = 1;
                if (c != PF_NO_CLIP) return 1;
            } else {
                if (seen_clip) return 1;
                if (c != PF_NO_CLIP && (c >= s->n_paths || !s->path_is_clip[c])) return 1;
            }
        }
    }
    return 0;
}

static int is_clip_path(const pf_scene_view *s, uint32_t p) { return s->path_is_clip && s->path_is_clip[p]; }

int pfo_tile_scene_mt(const pf_scene_view *s, int z_rule, int threads, pfo_result *out) {
    if (!out) return 1;
    memset(out, 0, sizeof(*out));
    if (validate(s)) return 1;
    const uint32_t n = s->n_paths;
    path_ctx *pcs = (path_ctx *)calloc(n ? n : 1, sizeof(path_ctx));
    if (!pcs) return 1;
    if (threads < 1) threads = 1;
    if ((uint32_t)threads > n) threads = n ? (int)n : 1;
    tile_job *jobs = (tile_job *)calloc((size_t)threads, sizeof(tile_job));
    pthread_t *th = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    int status = 0;
    for (int t = 0; t < threads; t++) {
        jobs[t].s = s;
        jobs[t].pcs = pcs;
        jobs[t].first = (uint32_t)t;
        jobs[t].step = (uint32_t)threads;
        if (threads == 1) tile_worker(&jobs[t]);
        else pthread_create(&th[t], NULL, tile_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; t++) {
        if (threads > 1) pthread_join(th[t], NULL);
        status |= jobs[t].status;
    }
    free(jobs);
    free(th);

    /* assemble canonical arrays */
    out->n_paths = n;
    out->path_rect = (int32_t *)malloc(sizeof(int32_t) * 4 * (n ? n : 1));
    out->path_tile_first = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    out->path_column_first = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    out->path_microlines = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    out->path_fills = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    uint64_t nfill = 0;
    for (uint32_t p = 0; p < n; p++) {
        const path_ctx *pc = &pcs[p];
        out->path_rect[4 * p + 0] = pc->rx0;
        out->path_rect[4 * p + 1] = pc->ry0;
        out->path_rect[4 * p + 2] = pc->rx1;
        out->path_rect[4 * p + 3] = pc->ry1;
        out->path_tile_first[p + 1] = out->path_tile_first[p] + (uint64_t)pc->rw * (uint64_t)pc->rh;
        out->path_column_first[p + 1] = out->path_column_first[p] + (uint64_t)pc->rw;
        out->path_microlines[p] = (uint32_t)pc->nleaf;
        out->path_fills[p] = (uint32_t)pc->nfill;
        out->n_microlines += pc->nleaf;
        nfill += pc->nfill;
    }
    out->n_tiles = out->path_tile_first[n];
    out->n_columns = out->path_column_first[n];
    out->n_fills = nfill;
    out->tile_alpha = (uint8_t *)malloc(out->n_tiles ? out->n_tiles : 1);
    out->tile_backdrop = (int8_t *)malloc(out->n_tiles ? out->n_tiles : 1);
    out->tile_fill_count = (uint32_t *)malloc(sizeof(uint32_t) * (out->n_tiles ? out->n_tiles : 1));
    out->column_backdrop = (int32_t *)malloc(sizeof(int32_t) * (out->n_columns ? out->n_columns : 1));
    out->fills = (uint16_t *)malloc(sizeof(uint16_t) * 4 * (nfill ? nfill : 1));
    uint64_t *keys = NULL;
    size_t keycap = 0;
    uint64_t fo = 0;
    for (uint32_t p = 0; p < n; p++) {
        path_ctx *pc = &pcs[p];
        const uint64_t tb = out->path_tile_first[p];
        const size_t nt = (size_t)pc->rw * (size_t)pc->rh;
        for (size_t i = 0; i < nt; i++) {
            out->tile_alpha[tb + i] = pc->fcount[i] ? 1 : 0;
            out->tile_backdrop[tb + i] = pc->bd[i];
            out->tile_fill_count[tb + i] = pc->fcount[i];
        }
        memcpy(out->column_backdrop + out->path_column_first[p], pc->col, sizeof(int32_t) * (size_t)pc->rw);
        /* group the path's fills by tile (counting sort), then sort inside each tile */
        if (pc->nfill) {
            if (keycap < pc->nfill) {
                free(keys);
                keycap = pc->nfill;
                keys = (uint64_t *)malloc(sizeof(uint64_t) * keycap);
            }
            uint64_t *start = (uint64_t *)malloc(sizeof(uint64_t) * (nt + 1));
            start[0] = 0;
            for (size_t i = 0; i < nt; i++) start[i + 1] = start[i] + pc->fcount[i];
            uint64_t *cur = (uint64_t *)malloc(sizeof(uint64_t) * (nt ? nt : 1));
            memcpy(cur, start, sizeof(uint64_t) * nt);
            for (size_t k = 0; k < pc->nfill; k++) {
                const fill_rec *f = &pc->fills[k];
                keys[cur[f->tile]++] = ((uint64_t)f->c[0] << 48) | ((uint64_t)f->c[1] << 32) |
                                       ((uint64_t)f->c[2] << 16) | (uint64_t)f->c[3];
            }
            for (size_t i = 0; i < nt; i++) {
                const uint64_t a = start[i], e = start[i + 1];
                if (e - a > 1) qsort(keys + a, e - a, sizeof(uint64_t), cmp_u64);
            }
            for (size_t k = 0; k < pc->nfill; k++) {
                uint16_t *d = out->fills + 4 * (fo + k);
                d[0] = (uint16_t)(keys[k] >> 48);
                d[1] = (uint16_t)(keys[k] >> 32);
                d[2] = (uint16_t)(keys[k] >> 16);
                d[3] = (uint16_t)keys[k];
            }
            fo += pc->nfill;
            free(start);
            free(cur);
        }
    }
    free(keys);

    /* clipped draw tiles: Tiler::prepare_tiles (tiler.cpp:386-431) against the clip path's
     * tile at the same coordinates, which is not clipped itself */
    {
        const uint64_t nt = out->n_tiles ? out->n_tiles : 1;
        out->tile_mask = (uint8_t *)calloc(nt, 1);
        out->tile_clip = (uint64_t *)malloc(sizeof(uint64_t) * nt);
        out->tile_dest_backdrop = (int8_t *)calloc(nt, 1);
        for (uint64_t t = 0; t < out->n_tiles; t++) out->tile_clip[t] = UINT64_MAX;
        for (uint32_t p = 0; s->path_clip && p < n; p++) {
            const uint32_t c = s->path_clip[p];
            if (c == PF_NO_CLIP) continue;
            const path_ctx *pc = &pcs[p], *cc = &pcs[c];
            const uint64_t tb = out->path_tile_first[p], cb = out->path_tile_first[c];
            for (int32_t y = 0; y < pc->rh; y++)
                for (int32_t x = 0; x < pc->rw; x++) {
                    const uint64_t g = tb + (uint64_t)y * pc->rw + x;
                    const int32_t tx = pc->rx0 + x, ty = pc->ry0 + y;
                    const uint8_t da = out->tile_alpha[g];
                    const int8_t dbd = out->tile_backdrop[g];
                    if (tx < cc->rx0 || tx >= cc->rx1 || ty < cc->ry0 || ty >= cc->ry1) {
                        out->tile_alpha[g] = 0;  /* outside the clip's rect: culled */
                        out->tile_backdrop[g] = 0;
                        continue;
                    }
                    const uint64_t gc = cb + (uint64_t)(ty - cc->ry0) * cc->rw + (uint64_t)(tx - cc->rx0);
                    const uint8_t ca = out->tile_alpha[gc];
                    const int8_t cbd = out->tile_backdrop[gc];
                    if (ca && da) {
                        out->tile_mask[g] = 2;  /* both masks, combined */
                        out->tile_clip[g] = gc;
                        out->tile_dest_backdrop[g] = dbd;
                        out->tile_backdrop[g] = 0;
                    } else if (ca && !da && dbd != 0) {
                        out->tile_mask[g] = 1;  /* a solid tile takes the clip's mask */
                        out->tile_clip[g] = gc;
                        out->tile_alpha[g] = 1;
                        out->tile_backdrop[g] = cbd;
                    } else if (!ca && cbd == 0) {
                        out->tile_alpha[g] = 0;  /* blank clip tile: culled */
                        out->tile_backdrop[g] = 0;
                    }
                }
        }
    }

    /* z-buffer and composite lists (scene_builder.cpp:18-95; propagate.comp:190-205; sort.comp);
     * clip paths are not drawn */
    /* the framebuffer tile grid: d3d9's z-buffer covers the view box's tile rect
     * (round_rect_out_to_tile_bounds(view_box), scene_builder.cpp:50-54); the d3d11 tile pass
     * covers the destination image from tile (0, 0) (renderer.cpp:371, 443), and a tile outside
     * it is never composited */
    float vb[4];
    scene_view_box(s, vb);
    int32_t fx0 = 0, fy0 = 0;
    uint32_t fbw = (uint32_t)ceilf(view_box_right(s->width) / (float)TILE);
    uint32_t fbh = (uint32_t)ceilf(s->height / (float)TILE);
    if (z_rule == PFO_Z_D3D9) {
        const float inv = 1.0f / (float)TILE;
        fx0 = (int32_t)floorf(vb[0] * inv);
        fy0 = (int32_t)floorf(vb[1] * inv);
        fbw = (uint32_t)((int32_t)ceilf(vb[2] * inv) - fx0);
        fbh = (uint32_t)((int32_t)ceilf(vb[3] * inv) - fy0);
    }
    const size_t nfb = (size_t)fbw * fbh;
    out->fb_tiles_x = fbw;
    out->fb_tiles_y = fbh;
    out->z = (int32_t *)malloc(sizeof(int32_t) * (nfb ? nfb : 1));
    for (size_t i = 0; i < nfb; i++) out->z[i] = -1;
    for (uint32_t p = 0; p < n; p++) {
        const int occludes = pfo_paint_is_opaque(s, p);  /* PaintMetadata::is_opaque */
        if (!occludes || is_clip_path(s, p)) continue;
        const path_ctx *pc = &pcs[p];
        const uint64_t tb = out->path_tile_first[p];
        for (int32_t y = 0; y < pc->rh; y++)
            for (int32_t x = 0; x < pc->rw; x++) {
                const uint64_t g = tb + (uint64_t)y * pc->rw + x;
                const int8_t b = out->tile_backdrop[g];
                if (out->tile_alpha[g] || b == 0) continue;
                if (z_rule == PFO_Z_D3D11 && s->fill_rule[p] == PF_FILL_EVEN_ODD && (abs((int)b) % 2) == 0) continue;
                const int32_t tx = pc->rx0 + x - fx0, ty = pc->ry0 + y - fy0;
                if (tx < 0 || ty < 0 || tx >= (int32_t)fbw || ty >= (int32_t)fbh) continue;
                const size_t fb = (size_t)ty * fbw + (size_t)tx;
                if ((int32_t)p > out->z[fb]) out->z[fb] = (int32_t)p;
            }
    }
    out->fb_list_first = (uint64_t *)calloc(nfb + 1, sizeof(uint64_t));
    for (int pass = 0; pass < 2; pass++) {
        uint64_t *cur = NULL;
        if (pass == 1) {
            for (size_t i = 0; i < nfb; i++) out->fb_list_first[i + 1] += out->fb_list_first[i];
            out->n_list = out->fb_list_first[nfb];
            out->fb_list = (uint32_t *)malloc(sizeof(uint32_t) * (out->n_list ? out->n_list : 1));
            cur = (uint64_t *)malloc(sizeof(uint64_t) * (nfb ? nfb : 1));
            memcpy(cur, out->fb_list_first, sizeof(uint64_t) * nfb);
        }
        for (uint32_t p = 0; p < n; p++) {
            if (is_clip_path(s, p)) continue;
            const path_ctx *pc = &pcs[p];
            const uint64_t tb = out->path_tile_first[p];
            for (int32_t y = 0; y < pc->rh; y++)
                for (int32_t x = 0; x < pc->rw; x++) {
                    const uint64_t g = tb + (uint64_t)y * pc->rw + x;
                    if (!out->tile_alpha[g] && out->tile_backdrop[g] == 0) continue;
                    const int32_t tx = pc->rx0 + x - fx0, ty = pc->ry0 + y - fy0;
                    if (tx < 0 || ty < 0 || tx >= (int32_t)fbw || ty >= (int32_t)fbh) continue;
                    const size_t fb = (size_t)ty * fbw + (size_t)tx;
                    if ((int32_t)p < out->z[fb]) continue;
                    if (pass == 0) out->fb_list_first[fb + 1]++;
                    else out->fb_list[cur[fb]++] = (uint32_t)g;
                }
        }
        free(cur);
    }

    for (uint32_t p = 0; p < n; p++) {
        free(pcs[p].col);
        free(pcs[p].bd);
        free(pcs[p].fcount);
        free(pcs[p].fills);
    }
    free(pcs);
    return status ? 5 : 0;
}

int pfo_tile_scene(const pf_scene_view *s, int z_rule, pfo_result *out) {
    return pfo_tile_scene_mt(s, z_rule, 1, out);
}

void pfo_free(pfo_result *r) {
    if (!r) return;
    free(r->path_rect);
    free(r->path_tile_first);
    free(r->path_column_first);
    free(r->tile_alpha);
    free(r->tile_backdrop);
    free(r->tile_fill_count);
    free(r->fills);
    free(r->column_backdrop);
    free(r->z);
    free(r->fb_list_first);
    free(r->fb_list);
    free(r->path_microlines);
    free(r->path_fills);
    free(r->tile_mask);
    free(r->tile_clip);
    free(r->tile_dest_backdrop);
    memset(r, 0, sizeof(*r));
}

/* ------------------------------------------------------------------------ */
/* FP64 analytic-area coverage and src-over composite                         */
/*                                                                          */
/* Coverage of a pixel of an alpha tile = tile backdrop + sum over the tile's */
/* fills of the signed area, inside the pixel, between the fill and the tile  */
/* bottom (the quantity fill.comp:51-100 / fill.frag:25-44 sample from their  */
/* area LUT), followed by the fill rule of fill.comp:133-140.  Composite:     */
/* calculateColor + src-over of tile.comp:611-675, 841, with solid even-odd   */
/* tiles of even backdrop skipped (tile.comp:791-799).                        */

static double cover_u(double u) { return u <= 0.0 ? 0.0 : (u < 1.0 ? 0.5 * u * u : u - 0.5); }

/* signed area contributed by fill (x0,y0)->(x1,y1) (tile-local px) to pixel (i, j) */
static double fill_area(double x0, double y0, double x1, double y1, int i, int j) {
    if (x0 == x1) return 0.0;
    const double s = x0 > x1 ? 1.0 : -1.0;
    double xl = x0, yl = y0, xr = x1, yr = y1;
    if (x0 > x1) {
        xl = x1;
        yl = y1;
        xr = x0;
        yr = y0;
    }
    const double a = xl > (double)i ? xl : (double)i;
    const double b = xr < (double)(i + 1) ? xr : (double)(i + 1);
    if (!(b > a)) return 0.0;
    const double slope = (yr - yl) / (xr - xl);
    const double ya = yl + slope * (a - xl), yb = yl + slope * (b - xl);
    const double ua = (double)(j + 1) - ya, ub = (double)(j + 1) - yb;
    double integral;
    if (fabs(ub - ua) < 1e-12) {
        double u = 0.5 * (ua + ub);
        u = u < 0.0 ? 0.0 : (u > 1.0 ? 1.0 : u);
        integral = u * (b - a);
    } else {
        integral = (b - a) * (cover_u(ub) - cover_u(ua)) / (ub - ua);
    }
    return s * integral;
}

static double apply_rule(double c, int even_odd) {
    if (!even_odd) {
        c = fabs(c);
        return c > 1.0 ? 1.0 : c;
    }
    double m = c - 2.0 * floor(c / 2.0); /* GLSL mod */
    double v = 1.0 - fabs(1.0 - m);
    return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
}

/* backdrop + signed areas of the fills of tile g, before the fill rule, into raw[256] */
static void tile_raw(const pfo_result *r, const uint64_t *fill_first, uint64_t g, int8_t bd, double raw[256]) {
    for (int k = 0; k < 256; k++) raw[k] = (double)bd;
    for (uint64_t f = fill_first[g]; f < fill_first[g + 1]; f++) {
        const uint16_t *q = r->fills + 4 * f;
        const double x0 = q[0] / 256.0, y0 = q[1] / 256.0, x1 = q[2] / 256.0, y1 = q[3] / 256.0;
        const int i0 = (int)floor(x0 < x1 ? x0 : x1), i1 = (int)ceil(x0 < x1 ? x1 : x0);
        for (int i = i0; i < i1 && i < 16; i++) {
            if (i < 0) continue;
            for (int jj = 0; jj < 16; jj++) raw[jj * 16 + i] += fill_area(x0, y0, x1, y1, i, jj);
        }
    }
}

/* coverage of a visible alpha tile g after the fill rule, into cov[256]: its own mask, the
 * clip tile's mask (d3d9 tile.frag sampleMask with the draw path's rule), or both combined as
 * tile_clip_combine.frag does (min of |mask + backdrop|, then the draw path's rule) */
static void tile_coverage(const pfo_result *r, const uint64_t *fill_first, uint64_t g, int eo, double cov[256]) {
    const uint8_t mode = r->tile_mask ? r->tile_mask[g] : 0;
    if (mode == 0) {
        tile_raw(r, fill_first, g, r->tile_backdrop[g], cov);
    } else if (mode == 1) {
        tile_raw(r, fill_first, r->tile_clip[g], r->tile_backdrop[g], cov);
    } else {
        double clip[256];
        tile_raw(r, fill_first, g, r->tile_dest_backdrop[g], cov);
        const uint64_t gc = r->tile_clip[g];
        tile_raw(r, fill_first, gc, r->tile_backdrop[gc], clip);
        for (int k = 0; k < 256; k++) {
            const double a = fabs(cov[k]), b = fabs(clip[k]);
            cov[k] = a < b ? a : b;
        }
    }
    for (int k = 0; k < 256; k++) cov[k] = apply_rule(cov[k], eo);
}

typedef struct {
    const pf_scene_view *s;
    const pfo_result *r;
    const uint64_t *fill_first; /* [n_tiles + 1] */
    const uint32_t *tile_path;  /* [n_tiles] */
    uint8_t *rgba;
    float *cov_out;
    uint32_t w, h;
    size_t first, step;
    const uint32_t *ramps;      /* [n_paths][256] gradient ramps (gradient paths only) */
    const float *meta;          /* [n_paths][12] their half-float metadata */
} render_job;

static void *render_worker(void *arg) {
    render_job *j = (render_job *)arg;
    const pfo_result *r = j->r;
    const size_t nfb = (size_t)r->fb_tiles_x * r->fb_tiles_y;
    const uint32_t clear = j->s->clear_color;
    const double cr = (clear & 0xffu) / 255.0, cg = ((clear >> 8) & 0xffu) / 255.0,
                 cb = ((clear >> 16) & 0xffu) / 255.0, ca = ((clear >> 24) & 0xffu) / 255.0;
    double dest[256][4];
    double cov[256];
    for (size_t fb = j->first; fb < nfb; fb += j->step) {
        const uint32_t fx = (uint32_t)(fb % r->fb_tiles_x), fy = (uint32_t)(fb / r->fb_tiles_x);
        for (int k = 0; k < 256; k++) {
            const uint32_t px = fx * 16 + (uint32_t)(k & 15), py = fy * 16 + (uint32_t)(k >> 4);
            if (j->s->load_action == PF_LOAD_LOAD && px < j->w && py < j->h) {
                /* LOAD_ACTION_LOAD (tile.comp:744-757): start from the pixel already there */
                const uint8_t *d = j->rgba + ((size_t)py * j->w + px) * 4;
                for (int ch = 0; ch < 4; ch++) dest[k][ch] = d[ch] / 255.0;
                continue;
            }
            dest[k][0] = cr;
            dest[k][1] = cg;
            dest[k][2] = cb;
            dest[k][3] = ca;
        }
        for (uint64_t e = r->fb_list_first[fb]; e < r->fb_list_first[fb + 1]; e++) {
            const uint32_t g = r->fb_list[e];
            const uint32_t p = j->tile_path[g];
            const int eo = j->s->fill_rule[p] == PF_FILL_EVEN_ODD;
            const int8_t bd = r->tile_backdrop[g];
            if (r->tile_alpha[g]) {
                tile_coverage(r, j->fill_first, g, eo, cov);
            } else {
                if (eo && (abs((int)bd) % 2) == 0) continue;
                for (int k = 0; k < 256; k++) cov[k] = 1.0;
            }
            const uint32_t c = j->s->color[p];
            double pr = (c & 0xffu) / 255.0, pg = ((c >> 8) & 0xffu) / 255.0, pb = ((c >> 16) & 0xffu) / 255.0,
                   pa = ((c >> 24) & 0xffu) / 255.0;
            const pf_paint *pp = j->s->path_paint ? &j->s->path_paint[p] : NULL;
            const int grad = pp && pp->type != PF_PAINT_SOLID;
            for (int k = 0; k < 256; k++) {
                if (grad) {  /* tile.comp: the ramp's colour (SrcIn over the white base colour) */
                    double g[4];
                    pfo_paint_color(pp, j->meta + 12 * (size_t)p, j->ramps + 256 * (size_t)p,
                                    fx * 16.0 + (k & 15) + 0.5, fy * 16.0 + (k >> 4) + 0.5, g);
                    pr = g[0];
                    pg = g[1];
                    pb = g[2];
                    pa = g[3];
                }
                const double a = pa * cov[k];
                dest[k][0] = dest[k][0] * (1.0 - a) + pr * a;
                dest[k][1] = dest[k][1] * (1.0 - a) + pg * a;
                dest[k][2] = dest[k][2] * (1.0 - a) + pb * a;
                dest[k][3] = dest[k][3] * (1.0 - a) + a;
            }
        }
        for (int yy = 0; yy < 16; yy++) {
            const uint32_t py = fy * 16 + (uint32_t)yy;
            if (py >= j->h) break;
            for (int xx = 0; xx < 16; xx++) {
                const uint32_t px = fx * 16 + (uint32_t)xx;
                if (px >= j->w) break;
                uint8_t *o = j->rgba + ((size_t)py * j->w + px) * 4;
                for (int ch = 0; ch < 4; ch++) {
                    double v = dest[yy * 16 + xx][ch];
                    v = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
                    o[ch] = (uint8_t)nearbyint(v * 255.0);
                }
            }
        }
    }
    return NULL;
}

static void *coverage_worker(void *arg) {
    render_job *j = (render_job *)arg;
    const pfo_result *r = j->r;
    double cov[256];
    for (uint64_t g = j->first; g < r->n_tiles; g += j->step) {
        if (!r->tile_alpha[g]) continue;
        const uint32_t p = j->tile_path[g];
        tile_coverage(r, j->fill_first, g, j->s->fill_rule[p] == PF_FILL_EVEN_ODD, cov);
        for (int k = 0; k < 256; k++) j->cov_out[(size_t)g * 256 + k] = (float)cov[k];
    }
    return NULL;
}

int pfo_render(const pf_scene_view *s, const pfo_result *r, uint8_t *rgba, float *coverage_f, int threads) {
    if (!s || !r || !rgba) return 1;
    const uint64_t nt = r->n_tiles;
    uint64_t *fill_first = (uint64_t *)malloc(sizeof(uint64_t) * (nt + 1));
    uint32_t *tile_path = (uint32_t *)malloc(sizeof(uint32_t) * (nt ? nt : 1));
    if (!fill_first || !tile_path) return 1;
    fill_first[0] = 0;
    for (uint64_t t = 0; t < nt; t++) fill_first[t + 1] = fill_first[t] + r->tile_fill_count[t];
    for (uint32_t p = 0; p < r->n_paths; p++)
        for (uint64_t t = r->path_tile_first[p]; t < r->path_tile_first[p + 1]; t++) tile_path[t] = p;
    uint32_t *ramps = NULL;
    float *meta = NULL;
    if (s->path_paint) {
        ramps = (uint32_t *)calloc((size_t)r->n_paths * 256, sizeof(uint32_t));
        meta = (float *)calloc((size_t)r->n_paths * 12, sizeof(float));
        if (!ramps || !meta) return 1;
        for (uint32_t p = 0; p < r->n_paths; p++) {
            const pf_paint *pp = &s->path_paint[p];
            if (pp->type == PF_PAINT_SOLID) continue;
            pfo_gradient_ramp(s->stops + pp->stop_first, pp->stop_count, ramps + 256 * (size_t)p);
            pfo_paint_meta(pp, meta + 12 * (size_t)p);
        }
    }
    if (threads < 1) threads = 1;
    render_job *jobs = (render_job *)calloc((size_t)threads, sizeof(render_job));
    pthread_t *th = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; t++) {
        render_job *j = &jobs[t];
        j->s = s;
        j->r = r;
        j->fill_first = fill_first;
        j->tile_path = tile_path;
        j->rgba = rgba;
        j->cov_out = coverage_f;
        j->ramps = ramps;
        j->meta = meta;
        j->w = (uint32_t)ceilf(s->width);
        j->h = (uint32_t)ceilf(s->height);
        j->first = (size_t)t;
        j->step = (size_t)threads;
        if (threads == 1) render_worker(j);
        else pthread_create(&th[t], NULL, render_worker, j);
    }
    if (threads > 1)
        for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    if (coverage_f) {
        for (int t = 0; t < threads; t++) {
            if (threads == 1) coverage_worker(&jobs[t]);
            else pthread_create(&th[t], NULL, coverage_worker, &jobs[t]);
        }
        if (threads > 1)
            for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    }
    free(jobs);
    free(th);
    free(fill_first);
    free(tile_path);
    free(ramps);
    free(meta);
    return 0;
}
