/*
 * pf_stroke.c - CPU restatement of the reference's stroke-to-fill conversion and line
 * dashing (Canvas::stroke_path, pathfinder/core/canvas.cpp:270-300).
 *
 * TEST INFRASTRUCTURE ONLY (part of libpforacle.so): the checker for the GPU stroker, never on
 * the product path.  Pinned against the reference's own OutlineStrokeToFill / OutlineDash,
 * compiled from its sources (ref_harness.cpp, pfref_stroke_scene), bit for bit.
 *
 * Every float operation follows the reference's order (single precision, no contraction:
 * this file is compiled with -ffp-contract=off), so the output points are identical.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pf_oracle.h"

#define FLOAT_EPSILON 0.0001f       /* pathfinder/common/math/basic.h:11 */
#define GEOMETRIC_EPSILON 0.001f    /* pathfinder/common/math/basic.h:14 */
#define STROKE_TOL 0.1f             /* pathfinder/core/stroke.cpp:15 */
#define SAMPLE_COUNT 8u             /* pathfinder/core/stroke.cpp:21 */

enum { K_NONE, K_LINE, K_QUAD, K_CUBIC }; /* SegmentKind, core/data/line_segment.h:22-27 */
enum { F_ON = 0, F_C0 = 1, F_C1 = 2 };    /* PointFlag, core/data/data.h:42-52 */

typedef struct { float x, y; } v2;
typedef struct { v2 f, t; } lseg;                 /* LineSegmentF */
typedef struct { lseg base, ctrl; int kind; } seg;  /* Segment */
typedef struct { float v[4]; } mat2;              /* Mat2, column major (common/math/mat2.h) */
typedef struct { mat2 m; v2 t; } xform;           /* Transform2 (common/math/transform2.h) */

/* --- Vec2F (common/math/vec2.h) --------------------------------------------------------- */
static v2 V(float x, float y) { v2 r = {x, y}; return r; }
static v2 vadd(v2 a, v2 b) { return V(a.x + b.x, a.y + b.y); }
static v2 vsub(v2 a, v2 b) { return V(a.x - b.x, a.y - b.y); }
static v2 vmul(v2 a, v2 b) { return V(a.x * b.x, a.y * b.y); }
static v2 vscale(v2 a, float s) { return V(a.x * s, a.y * s); }
static v2 vadds(v2 a, float s) { return V(a.x + s, a.y + s); }
static v2 vneg(v2 a) { return V(-a.x, -a.y); }
static v2 vyx(v2 a) { return V(a.y, a.x); }
static float vsqlen(v2 a) { return a.x * a.x + a.y * a.y; }
static float vlen(v2 a) { return sqrtf(vsqlen(a)); }
static v2 vnormalize(v2 a) { const float l = vlen(a); return V(a.x / l, a.y / l); }
static int vapprox_eq(v2 a, v2 b, float eps) { return vlen(vsub(a, b)) <= eps; }
static int veq(v2 a, v2 b) { return a.x == b.x && a.y == b.y; }
static float fmax_std(float a, float b) { return a < b ? b : a; } /* std::max */
/* lerp(Vec2, Vec2, t) = a + t * (b - a)  (common/math/vec2.h:178-180) */
static v2 vlerp(v2 a, v2 b, float t) { return V(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y)); }

/* --- Mat2 / Transform2 / UnitVector ----------------------------------------------------- */
static mat2 M(float a, float b, float c, float d) { mat2 m = {{a, b, c, d}}; return m; }
static mat2 mmul(mat2 a, mat2 b) {
    return M(a.v[0] * b.v[0] + a.v[2] * b.v[1], a.v[1] * b.v[0] + a.v[3] * b.v[1],
             a.v[0] * b.v[2] + a.v[2] * b.v[3], a.v[1] * b.v[2] + a.v[3] * b.v[3]);
}
static v2 mvec(mat2 a, v2 p) { return V(a.v[0] * p.x + a.v[2] * p.y, a.v[1] * p.x + a.v[3] * p.y); }
static float mdet(mat2 a) { return a.v[0] * a.v[3] - a.v[1] * a.v[2]; }
static mat2 minverse(mat2 a) { /* adjugate() * (1 / det()) */
    const mat2 adj = M(a.v[3] * 1.0f, a.v[1] * -1.0f, a.v[2] * -1.0f, a.v[0] * 1.0f);
    const float s = 1.0f / mdet(a);
    return M(adj.v[0] * s, adj.v[1] * s, adj.v[2] * s, adj.v[3] * s);
}
static xform X(mat2 m, v2 t) { xform r = {m, t}; return r; }
static v2 xapply(xform a, v2 p) { return vadd(mvec(a.m, p), a.t); }
static xform xmul(xform a, xform b) { return X(mmul(a.m, b.m), xapply(a, b.t)); }
static xform xscale(v2 s) { return X(M(s.x, 0.0f, 0.0f, s.y), V(0.0f, 0.0f)); }
static xform xidentity(void) { return xscale(V(1.0f, 1.0f)); }
/* Transform2::translate: from_translation(v) * this (common/math/transform2.cpp:16-18) */
static xform xtranslate(xform a, v2 t) { return xmul(X(M(1.0f, 0.0f, 0.0f, 1.0f), t), a); }
static xform xrotation(v2 u) { return X(M(1.0f * u.x, 1.0f * u.y, -1.0f * u.y, 1.0f * u.x), V(0.0f, 0.0f)); }
/* UnitVector (common/math/unit_vector.cpp:9-20) */
static v2 urotate_by(v2 a, v2 o) { return V(a.x * o.x - a.y * o.y, a.y * o.x + a.x * o.y); }
static v2 urev_rotate_by(v2 a, v2 o) { return V(a.x * o.x + a.y * o.y, a.y * o.x - a.x * o.y); }
static v2 uhalve_angle(v2 a) {
    const v2 h = vmul(V(0.5f, 0.5f), vadd(V(1.0f, 1.0f), V(a.x, -a.x)));
    return V(sqrtf(fmax_std(h.x, 0.0f)), sqrtf(fmax_std(h.y, 0.0f)));
}

/* --- LineSegmentF (core/data/line_segment.cpp) ------------------------------------------ */
static lseg L(v2 f, v2 t) { lseg r = {f, t}; return r; }
static v2 lvec(lseg l) { return vsub(l.t, l.f); }
static float lsqlen(lseg l) { return vsqlen(lvec(l)); }
static v2 lsample(lseg l, float t) { return vadd(l.f, vscale(lvec(l), t)); }
static int lfinite(lseg l) { return isfinite(l.f.x) && isfinite(l.f.y) && isfinite(l.t.x) && isfinite(l.t.y); }
/* :37-48 */
static void lsplit(lseg l, float t, lseg *a, lseg *b) {
    const v2 d = vsub(l.t, l.f);
    const v2 mid = vadd(l.f, vscale(d, t));
    *a = L(l.f, mid);
    *b = L(mid, l.t);
}
/* :78-87 */
static int lintersection_t(lseg a, lseg o, float *out) {
    const v2 p0p1 = lvec(a), ov = lvec(o);
    const mat2 m = M(ov.x, ov.y, -p0p1.x, -p0p1.y);
    if (fabsf(mdet(m)) < FLOAT_EPSILON) return 0;
    *out = mvec(minverse(m), vsub(a.f, o.f)).y;
    return 1;
}
/* :89-95 */
static lseg loffset(lseg l, float distance) {
    const v2 v = lvec(l);
    if (v.x == 0 && v.y == 0) return l;
    const v2 d = vmul(vnormalize(vyx(v)), V(-distance, distance));
    return L(vadd(l.f, d), vadd(l.t, d));
}

/* --- Segment (core/data/segment.cpp) ----------------------------------------------------- */
static seg S(lseg b, lseg c, int k) { seg s = {b, c, k}; return s; }
static seg sline(lseg b) { return S(b, L(V(0, 0), V(0, 0)), K_LINE); }
static seg squad(lseg b, v2 c) { return S(b, L(c, c), K_QUAD); }
static seg scubic(lseg b, lseg c) { return S(b, c, K_CUBIC); }
/* :42-100 (the F32x4 lanes written out) */
static void split_cubic(const seg *s, float t, seg *a, seg *b) {
    if (t <= 0.0f) {
        const v2 f = s->base.f;
        *a = S(L(f, f), L(f, f), K_CUBIC);
        *b = S(s->base, s->ctrl, K_CUBIC);
    } else if (t >= 1.0f) {
        const v2 to = s->base.t;
        *a = S(s->base, s->ctrl, K_CUBIC);
        *b = S(L(to, to), L(to, to), K_CUBIC);
    } else {
        const v2 p0 = s->base.f, p3 = s->base.t, p1 = s->ctrl.f, p2 = s->ctrl.t;
        const v2 p01 = vadd(p0, vscale(vsub(p1, p0), t));
        const v2 p12 = vadd(p1, vscale(vsub(p2, p1), t));
        const v2 p23 = vadd(p2, vscale(vsub(p3, p2), t));
        const v2 p012 = vadd(p01, vscale(vsub(p12, p01), t));
        const v2 p123 = vadd(p12, vscale(vsub(p23, p12), t));
        const v2 p0123 = vadd(p012, vscale(vsub(p123, p012), t));
        *a = S(L(p0, p0123), L(p01, p012), K_CUBIC);
        *b = S(L(p0123, p3), L(p123, p23), K_CUBIC);
    }
}
/* :102-126 */
static void split_quad(const seg *s, float t, seg *a, seg *b) {
    const v2 p0 = s->base.f, p1 = s->ctrl.f, p2 = s->base.t;
    const v2 qa = vadd(p0, vscale(vsub(p1, p0), t));
    const v2 qb = vadd(p1, vscale(vsub(p2, p1), t));
    const v2 qc = vadd(qa, vscale(vsub(qb, qa), t));
    *a = S(L(p0, qc), L(qa, qa), K_QUAD);
    *b = S(L(qc, p2), L(qb, qb), K_QUAD);
}
/* :128-139 */
static void ssplit(const seg *s, float t, seg *a, seg *b) {
    if (s->kind == K_LINE) {
        lseg la, lb;
        lsplit(s->base, t, &la, &lb);
        *a = S(la, a->ctrl, K_LINE);
        *b = S(lb, b->ctrl, K_LINE);
    } else if (s->kind == K_QUAD) {
        split_quad(s, t, a, b);
    } else {
        split_cubic(s, t, a, b);
    }
}
/* :160-165 */
static v2 ssample(const seg *s, float t) {
    seg a = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, K_NONE}, b = a;
    ssplit(s, t, &a, &b);
    return a.base.t;
}
/* :153-158 */
static seg stransform(const seg *s, xform x) {
    return S(L(xapply(x, s->base.f), xapply(x, s->base.t)), L(xapply(x, s->ctrl.f), xapply(x, s->ctrl.t)), s->kind);
}
/* :189-200 */
static int svalid(const seg *s) {
    if (s->kind == K_LINE) return lfinite(s->base);
    if (s->kind == K_QUAD || s->kind == K_CUBIC) return lfinite(s->base) && lfinite(s->ctrl);
    return 0;
}
/* :141-151 */
static seg sto_cubic(const seg *s) {
    if (s->kind == K_CUBIC) return *s;
    const v2 p1_2 = vadd(s->ctrl.f, s->ctrl.f);
    const v2 c0 = vadd(s->base.f, p1_2), c1 = vadd(p1_2, s->base.t);
    return S(s->base, L(V(c0.x / 3.0f, c0.y / 3.0f), V(c1.x / 3.0f, c1.y / 3.0f)), K_CUBIC);
}
/* :168-187 */
static float sarc_length(const seg *s) {
    if (s->kind == K_LINE) return vlen(lvec(s->base));
    if (s->kind == K_QUAD || s->kind == K_CUBIC) {
        const seg c = sto_cubic(s);
        const float chord = vlen(lvec(c.base));
        const float cont_net = vlen(vsub(c.base.f, c.ctrl.f)) + vlen(lvec(c.ctrl)) + vlen(vsub(c.base.t, c.ctrl.t));
        return (cont_net + chord) * 0.5f;
    }
    return 0;
}
/* :202-211 */
static seg quarter_circle_arc(void) {
    const v2 p0 = V(sqrtf(2.0f) * 0.5f, sqrtf(2.0f) * 0.5f);
    const v2 p1 = V(-sqrtf(2.0f) / 6.0f + 4.0f / 3.0f, 7.0f * sqrtf(2.0f) / 6.0f - 4.0f / 3.0f);
    const v2 flip = V(1.0f, -1.0f);
    return S(L(vmul(p0, flip), p0), L(vmul(p1, flip), p1), K_CUBIC);
}
/* :213-240 (the threshold compares in double, as the reference's 1.0 - GEOMETRIC_EPSILON does) */
static seg arc_from_cos(float c) {
    if ((double)c >= 1.0 - (double)GEOMETRIC_EPSILON) return sline(L(V(1.0f, 0.0f), V(1.0f, 0.0f)));
    const v2 h = vmul(vadds(V(c, -c), 1.0f), V(0.5f, 0.5f));
    const v2 r = V(sqrtf(h.x), sqrtf(h.y));
    const v2 p3 = vmul(r, V(1.0f, -1.0f)), p0 = vmul(r, V(1.0f, 1.0f));
    const float p1x = 4.0f - p0.x;
    const float p1y = (1.0f - p0.x) * (3.0f - p0.x) / p0.y;
    const v2 p2 = vscale(V(p1x, -p1y), 1.0f / 3.0f), p1 = vscale(V(p1x, p1y), 1.0f / 3.0f);
    return scubic(L(p3, p0), L(p2, p1));
}

/* --- Contour output (core/data/contour.cpp) --------------------------------------------- */
typedef struct {
    v2 *p;
    uint8_t *f;
    size_t n, cap;
    int fail;
} cbuf;
static void cpush_point(cbuf *c, v2 p, uint8_t f) {
    if (c->n == c->cap) {
        const size_t cap = c->cap ? c->cap * 2 : 64;
        v2 *np = (v2 *)realloc(c->p, cap * sizeof(v2));
        uint8_t *nf = (uint8_t *)realloc(c->f, cap);
        if (!np || !nf) {
            if (np) c->p = np;
            if (nf) c->f = nf;
            c->fail = 1;
            return;
        }
        c->p = np;
        c->f = nf;
        c->cap = cap;
    }
    c->p[c->n] = p;
    c->f[c->n] = f;
    c->n++;
}
static v2 clast(const cbuf *c, int k) { return c->p[c->n - k]; } /* position_of_last, :7-9 */
/* :11-41 (the from point is pushed whatever the flags say) */
static void cpush_segment(cbuf *c, const seg *s) {
    if (s->kind == K_NONE || !svalid(s)) return;
    cpush_point(c, s->base.f, F_ON);
    if (s->kind != K_LINE) {
        cpush_point(c, s->ctrl.f, F_C0);
        if (s->kind != K_QUAD) cpush_point(c, s->ctrl.t, F_C1);
    }
    cpush_point(c, s->base.t, F_ON);
}
/* stroke.cpp:264-271 */
static int cmight_need_join(const cbuf *c, int join) {
    return c->n >= 2 && (join == PF_JOIN_MITER || join == PF_JOIN_ROUND);
}
/* stroke.cpp:326-368 (always clockwise here) */
static void cpush_arc(cbuf *c, xform x, lseg chord) {
    const xform dir = xidentity();
    v2 vec = chord.f;
    const v2 end = chord.t;
    for (int i = 0; i < 4; i++) {
        v2 sweep = urev_rotate_by(end, vec);
        const int last = sweep.x >= -FLOAT_EPSILON && sweep.y >= -FLOAT_EPSILON;
        seg s;
        if (!last) {
            sweep = V(0.0f, 1.0f);
            s = quarter_circle_arc();
        } else {
            s = arc_from_cos(sweep.x);
        }
        const v2 half = uhalve_angle(sweep);
        const xform rot = xrotation(urotate_by(half, vec));
        s = stransform(&s, xmul(xmul(x, dir), rot));
        cpush_segment(c, &s);
        if (last) break;
        vec = urotate_by(vec, sweep);
    }
}
/* stroke.cpp:273-324 */
static void cadd_join(cbuf *c, float distance, int join, v2 jp, lseg next, float miter_limit) {
    const lseg prev = L(clast(c, 2), clast(c, 1));
    if (lsqlen(prev) < FLOAT_EPSILON || lsqlen(next) < FLOAT_EPSILON) return;
    if (join == PF_JOIN_MITER) {
        float t;
        if (lintersection_t(prev, next, &t)) {
            if (t < -FLOAT_EPSILON) return;
            const v2 me = lsample(prev, t);
            const float threshold = miter_limit * distance;
            if (vsqlen(vsub(me, jp)) > threshold * threshold) return;
            cpush_point(c, me, F_ON);
        }
    } else if (join == PF_JOIN_ROUND) {
        if (vsqlen(vsub(prev.t, jp)) == 0 || vsqlen(vsub(next.t, jp)) == 0) return;
        const float scale = fabsf(distance);
        const xform x = xtranslate(xscale(V(scale, scale)), jp);
        const v2 cf = vnormalize(vsub(prev.t, jp)), ct = vnormalize(vsub(next.t, jp));
        cpush_arc(c, x, L(cf, ct));
    }
}

/* --- Segment offsetting (core/stroke.cpp) ----------------------------------------------- */
/* :370-442 */
static seg offset_once(const seg *s, float d) {
    if (s->kind == K_LINE) return sline(loffset(s->base, d));
    if (s->kind == K_QUAD) {
        const lseg s0 = loffset(L(s->base.f, s->ctrl.f), d), s1 = loffset(L(s->ctrl.f, s->base.t), d);
        float t;
        const v2 c = lintersection_t(s0, s1, &t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return squad(L(s0.f, s1.t), c);
    }
    if (veq(s->base.f, s->ctrl.f)) {
        const lseg s0 = loffset(L(s->base.f, s->ctrl.t), d), s1 = loffset(L(s->ctrl.t, s->base.t), d);
        float t;
        const v2 c = lintersection_t(s0, s1, &t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return scubic(L(s0.f, s1.t), L(s0.f, c));
    }
    if (veq(s->ctrl.t, s->base.t)) {
        const lseg s0 = loffset(L(s->base.f, s->ctrl.f), d), s1 = loffset(L(s->ctrl.f, s->base.t), d);
        float t;
        const v2 c = lintersection_t(s0, s1, &t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return scubic(L(s0.f, s1.t), L(c, s1.t));
    }
    const lseg s0 = loffset(L(s->base.f, s->ctrl.f), d), s1 = loffset(L(s->ctrl.f, s->ctrl.t), d),
               s2 = loffset(L(s->ctrl.t, s->base.t), d);
    v2 c0, c1;
    float t0, t1;
    /* both intersections are evaluated only while the first holds (&& short circuit) */
    if (lintersection_t(s0, s1, &t0) && lintersection_t(s1, s2, &t1)) {
        c0 = lsample(s0, t0);
        c1 = lsample(s1, t1);
    } else {
        c0 = vlerp(s0.t, s1.f, 0.5f);
        c1 = vlerp(s1.t, s2.f, 0.5f);
    }
    return scubic(L(s0.f, s2.t), L(c0, c1));
}
/* :455-477 */
static int within_tolerance(const seg *s, const seg *o, float d) {
    float lo = fabsf(d) - STROKE_TOL, hi = fabsf(d) + STROKE_TOL;
    lo = lo <= 0 ? 0.0f : lo * lo;
    hi = hi <= 0 ? 0.0f : hi * hi;
    for (uint32_t k = 0; k < SAMPLE_COUNT + 1; k++) {
        const float t = (float)k / (float)SAMPLE_COUNT;
        const float sq = vsqlen(vsub(ssample(s, t), ssample(o, t)));
        if (sq < lo || sq > hi) return 0;
    }
    return 1;
}
/* :479-500 */
static void add_to_contour(const seg *s, cbuf *c, float d, int join, v2 jp, float miter) {
    if (cmight_need_join(c, join)) {
        const v2 p3 = s->base.f;
        const v2 p4 = s->kind == K_LINE ? s->base.t : s->ctrl.f;
        cadd_join(c, d, join, jp, L(p4, p3), miter);
    }
    cpush_segment(c, s);
}
/* :502-540 */
static void soffset(const seg *s, float d, int join, float miter, cbuf *c, uint32_t depth) {
    if (!svalid(s)) return;
    const v2 jp = s->base.f;
    if (lsqlen(s->base) < STROKE_TOL * STROKE_TOL || depth >= 16) {
        add_to_contour(s, c, d, join, jp, miter);
        return;
    }
    if (s->kind == K_LINE) {
        const seg cand = offset_once(s, d);
        add_to_contour(&cand, c, d, join, jp, miter);
        return;
    }
    const seg cand = offset_once(s, d);
    if (within_tolerance(s, &cand, d)) {
        add_to_contour(&cand, c, d, join, jp, miter);
        return;
    }
    seg a, b;
    ssplit(s, 0.5f, &a, &b);
    soffset(&a, d, join, miter, c, depth + 1);
    soffset(&b, d, join, miter, c, depth + 1);
}

/* --- Input contours --------------------------------------------------------------------- */
typedef struct {
    const v2 *p;
    const uint8_t *f;
    size_t n;
    int closed;
} cin;
typedef struct {
    const cin *c;
    size_t head;
    int has_next;
} siter;
/* SegmentsIter::get_next, core/data/contour.cpp:110-173 (force_closed false) */
static seg siter_next(siter *it) {
    seg s = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, K_NONE};
    const cin *c = it->c;
    const size_t n = c->n, h = it->head;
    if (h >= n || c->f[h] != F_ON) return s;
    s.base.f = c->p[h];
    if (h + 1 < n) {
        if (c->f[h + 1] == F_ON) {
            s.base.t = c->p[h + 1];
            s.kind = K_LINE;
            it->head += 1;
        } else if (h + 2 < n) {
            if (c->f[h + 1] == F_C0 && c->f[h + 2] == F_ON) {
                s.ctrl.f = c->p[h + 1];
                s.base.t = c->p[h + 2];
                s.kind = K_QUAD;
                it->head += 2;
            } else if (h + 3 < n) {
                if (c->f[h + 1] == F_C0 && c->f[h + 2] == F_C1 && c->f[h + 3] == F_ON) {
                    s.ctrl.f = c->p[h + 1];
                    s.ctrl.t = c->p[h + 2];
                    s.base.t = c->p[h + 3];
                    s.kind = K_CUBIC;
                    it->head += 3;
                }
            }
        }
    } else {
        if (c->closed && n > 1 && !vapprox_eq(c->p[0], c->p[n - 1], FLOAT_EPSILON)) {
            s.base.f = c->p[n - 1];
            s.base.t = c->p[0];
            s.kind = K_LINE;
        }
        it->has_next = 0;
    }
    return s;
}

/* ContourStrokeToFill::offset_forward, stroke.cpp:27-49 */
static void offset_forward(const cin *in, float radius, int join, float miter, cbuf *out) {
    siter it = {in, 0, 1};
    int idx = -1;
    while (it.has_next) {
        const seg s = siter_next(&it);
        idx++;
        if (s.kind == K_NONE) break;
        soffset(&s, -radius, idx == 0 ? PF_JOIN_BEVEL : join, miter, out, 0);
    }
}
/* ContourStrokeToFill::offset_backward, stroke.cpp:51-122 */
static void offset_backward(const cin *in, float radius, int join, float miter, cbuf *out) {
    const int n = (int)in->n;
    int tail = n - 1, idx = -1;
    if (in->closed && n > 1 && !vapprox_eq(in->p[0], in->p[n - 1], FLOAT_EPSILON)) {
        const seg closing = sline(L(in->p[0], in->p[n - 1]));
        idx++;
        soffset(&closing, -radius, idx == 0 ? PF_JOIN_BEVEL : join, miter, out, 0);
    }
    while (tail >= 0) {
        if (in->f[tail] != F_ON) break;
        seg s = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, K_NONE};
        if (tail >= 3 && in->f[tail - 1] == F_C1 && in->f[tail - 2] == F_C0 && in->f[tail - 3] == F_ON) {
            s = scubic(L(in->p[tail], in->p[tail - 3]), L(in->p[tail - 1], in->p[tail - 2]));
            tail -= 3;
        } else if (tail >= 2 && in->f[tail - 1] == F_C0 && in->f[tail - 2] == F_ON) {
            s = squad(L(in->p[tail], in->p[tail - 2]), in->p[tail - 1]);
            tail -= 2;
        } else if (tail >= 1 && in->f[tail - 1] == F_ON) {
            s = sline(L(in->p[tail], in->p[tail - 1]));
            tail -= 1;
        } else {
            break;
        }
        idx++;
        soffset(&s, -radius, idx == 0 ? PF_JOIN_BEVEL : join, miter, out, 0);
    }
}
/* OutlineStrokeToFill::add_cap, stroke.cpp:206-258 */
static void add_cap(cbuf *c, const pf_stroke *st) {
    if (st->line_cap == PF_CAP_BUTT || c->n < 2) return;
    const float width = st->line_width;
    const v2 p1 = clast(c, 1);
    v2 p0;
    size_t i = c->n - 2;
    for (;;) {
        p0 = c->p[i];
        if (vsqlen(vsub(p1, p0)) > FLOAT_EPSILON) break;
        if (i == 0) return;
        i -= 1;
    }
    const v2 g = vnormalize(vsub(p1, p0));
    if (st->line_cap == PF_CAP_SQUARE) {
        const v2 off = vscale(g, width * 0.5f);
        const v2 p2 = vadd(p1, off);
        const v2 p3 = vadd(p2, vmul(vyx(g), V(-width, width)));
        const v2 p4 = vsub(p3, off);
        cpush_point(c, p2, F_ON);
        cpush_point(c, p3, F_ON);
        cpush_point(c, p4, F_ON);
    } else if (st->line_cap == PF_CAP_ROUND) {
        const float scale = width * 0.5f;
        const v2 off = vmul(vyx(g), V(-1.0f, 1.0f));
        const v2 tr = vadd(p1, vscale(off, width * 0.5f));
        const xform x = xtranslate(xscale(V(scale, scale)), tr);
        cpush_arc(c, x, L(vneg(off), off));
    }
}
/* OutlineStrokeToFill::push_stroked_contour's join, stroke.cpp:186-204 */
static void close_join(cbuf *c, const cin *in, const pf_stroke *st) {
    if (cmight_need_join(c, st->line_join)) {
        const lseg fin = L(c->p[1], c->p[0]);
        cadd_join(c, st->line_width * 0.5f, st->line_join, in->p[0], fin, st->miter_limit);
    }
}

/* --- Output ------------------------------------------------------------------------------ */
typedef struct {
    v2 *p;
    uint8_t *f;
    uint32_t *cs;  /* contour starts (+1) */
    size_t np, cap_p, nc, cap_c;
    int fail;
} obuf;
static void oreserve(obuf *o, size_t np) {
    if (o->np + np > o->cap_p) {
        size_t cap = o->cap_p ? o->cap_p : 256;
        while (cap < o->np + np) cap *= 2;
        v2 *p = (v2 *)realloc(o->p, cap * sizeof(v2));
        uint8_t *f = (uint8_t *)realloc(o->f, cap);
        if (!p || !f) {
            if (p) o->p = p;
            if (f) o->f = f;
            o->fail = 1;
            return;
        }
        o->p = p;
        o->f = f;
        o->cap_p = cap;
    }
    if (o->nc + 2 > o->cap_c) {
        const size_t cap = o->cap_c ? o->cap_c * 2 : 64;
        uint32_t *cs = (uint32_t *)realloc(o->cs, cap * sizeof(uint32_t));
        if (!cs) {
            o->fail = 1;
            return;
        }
        o->cs = cs;
        o->cap_c = cap;
    }
}
static void oemit(obuf *o, const v2 *p, const uint8_t *f, size_t n) {
    oreserve(o, n);
    if (o->fail) return;
    if (n) {
        memcpy(o->p + o->np, p, n * sizeof(v2));
        memcpy(o->f + o->np, f, n);
    }
    o->np += n;
    o->nc++;
    o->cs[o->nc] = (uint32_t)o->np;
}

/* One stroked contour (OutlineStrokeToFill::offset, stroke.cpp:124-167). */
static void stroke_contour(const cin *in, const pf_stroke *st, obuf *o, cbuf *c) {
    const float radius = st->line_width * 0.5f;
    c->n = 0;
    offset_forward(in, radius, st->line_join, st->miter_limit, c);
    if (in->closed) {
        close_join(c, in, st);
        oemit(o, c->p, c->f, c->n);
        c->n = 0;
    } else {
        add_cap(c, st);
    }
    offset_backward(in, radius, st->line_join, st->miter_limit, c);
    if (!in->closed) add_cap(c, st);
    else close_join(c, in, st);
    oemit(o, c->p, c->f, c->n);
}

/* Dashing (core/dash.cpp): the dashed contours of one path's outline, in order. */
typedef struct {
    cbuf cur;         /* DashState::output */
    const float *dashes;
    uint32_t count, idx;
    float left;       /* DashState::distance_left */
} dstate;
#define DASH_STEP_LIMIT (1u << 22)
/* DashState::DashState, dash.cpp:9-29.  Returns 1 when the phase runs past the pattern (the
 * reference would then read past its dash array). */
static int dstate_init(dstate *d, const float *dashes, uint32_t count, float offset) {
    float total = 0;
    for (uint32_t i = 0; i < count; i++) total += dashes[i];
    offset = fmodf(offset, total);
    d->dashes = dashes;
    d->count = count;
    d->idx = 0;
    while (d->idx < count) {
        const float dash = dashes[d->idx];
        if (offset < dash) break;
        offset -= dash;
        d->idx += 1;
    }
    d->left = offset;
    d->cur.n = 0;
    return d->idx >= count;
}
/* Outline::push_contour (core/data/path.cpp:24-38): empty contours are dropped */
static void dash_push(obuf *o, const cbuf *c) {
    if (c->n) oemit(o, c->p, c->f, c->n);
}
/* ContourDash::dash, dash.cpp:68-124; returns 0, or 1 past DASH_STEP_LIMIT steps */
static int dash_contour(const cin *in, dstate *d, obuf *o, uint32_t *steps) {
    siter it = {in, 0, 1};
    seg queued = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, K_NONE};
    int none = 1;
    for (;;) {
        if (none) {
            if (it.has_next) {
                queued = siter_next(&it);
                if (queued.kind == K_NONE) break;
                none = 0;
            } else {
                break;
            }
        }
        if (++*steps > DASH_STEP_LIMIT) return 1;
        seg cur = queued;
        float distance = d->left;
        const float t = distance / sarc_length(&cur);
        if (t < 1.0f) {
            seg a = cur, b = cur;
            ssplit(&cur, t, &a, &b);
            cur = a;
            queued = b;
            none = 0;
        } else {
            distance = sarc_length(&cur);
            none = 1;
        }
        if (d->idx % 2 == 0) cpush_segment(&d->cur, &cur);
        d->left -= distance;
        if (d->left < FLOAT_EPSILON) {
            if (d->idx % 2 == 0) {
                dash_push(o, &d->cur);
                d->cur.n = 0;
            }
            d->idx += 1;
            if (d->idx == d->count) d->idx = 0;
            d->left = d->dashes[d->idx];
        }
    }
    return 0;
}

static int path_is_stroked(const pf_scene_view *s, uint32_t p) {
    return s->path_stroke && s->path_stroke[p].line_width > 0.0f;
}

int pfo_stroke_check(const pf_scene_view *s) {
    if (!s->path_stroke) return 0;
    for (uint32_t p = 0; p < s->n_paths; p++) {
        const pf_stroke *st = &s->path_stroke[p];
        if (!(st->line_width >= 0.0f) || !isfinite(st->line_width) || !isfinite(st->miter_limit) ||
            st->line_cap > PF_CAP_ROUND || st->line_join > PF_JOIN_ROUND)
            return 1;
        if (st->line_width > 0.0f && st->dash_count) {
            if ((uint64_t)st->dash_first + st->dash_count > s->n_dashes || !s->dashes) return 1;
            float total = 0;
            for (uint32_t i = 0; i < st->dash_count; i++) {
                const float d = s->dashes[st->dash_first + i];
                if (!(d >= 0.0f) || !isfinite(d)) return 1;
                total += d;
            }
            if (!(total > 0.0f) || !isfinite(total) || !isfinite(st->dash_offset)) return 1;
        }
    }
    return 0;
}

int pfo_stroke_scene(const pf_scene_view *s, pfo_outline *out) {
    memset(out, 0, sizeof(*out));
    if (pfo_stroke_check(s)) return 1;
    obuf o = {0};
    cbuf c = {0};
    obuf dashed = {0};
    int status = 0;
    uint32_t *pstart = (uint32_t *)malloc(sizeof(uint32_t) * (s->n_paths + 1));
    uint8_t *rule = (uint8_t *)malloc(s->n_paths ? s->n_paths : 1);
    if (!pstart || !rule) {
        free(pstart);
        free(rule);
        return 3;
    }
    oreserve(&o, 0);
    if (o.fail) status = 3;
    if (o.cs) o.cs[0] = 0;
    pstart[0] = 0;
    const v2 *pts = (const v2 *)s->points;
    for (uint32_t p = 0; p < s->n_paths && !status; p++) {
        const uint32_t k0 = s->path_start[p], k1 = s->path_start[p + 1];
        rule[p] = s->fill_rule[p];
        if (!path_is_stroked(s, p)) {
            for (uint32_t k = k0; k < k1; k++) {
                const uint32_t a = s->contour_start[k], e = s->contour_start[k + 1];
                oemit(&o, pts + a, s->point_flags + a, e - a);
            }
        } else {
            const pf_stroke *st = &s->path_stroke[p];
            rule[p] = PF_FILL_NONZERO;  /* Canvas::stroke_path fills strokes nonzero */
            if (st->dash_count) {
                /* OutlineDash over the path's contours (one state for the whole outline), then the
                 * stroke of every dashed contour (open: Contour() starts open) */
                dstate d;
                memset(&d, 0, sizeof(d));
                if (dstate_init(&d, s->dashes + st->dash_first, st->dash_count, st->dash_offset)) status = 1;
                dashed.np = dashed.nc = 0;
                oreserve(&dashed, 0);
                if (dashed.cs) dashed.cs[0] = 0;
                uint32_t steps = 0;
                for (uint32_t k = k0; k < k1 && !status; k++) {
                    const uint32_t a = s->contour_start[k], e = s->contour_start[k + 1];
                    const cin in = {pts + a, s->point_flags + a, e - a,
                                    s->contour_closed ? s->contour_closed[k] != 0 : 0};
                    if (dash_contour(&in, &d, &dashed, &steps)) status = 5;
                }
                if (!status && d.idx % 2 == 0) dash_push(&dashed, &d.cur);
                free(d.cur.p);
                free(d.cur.f);
                if (dashed.fail) status = 3;
                for (size_t k = 0; k < dashed.nc && !status; k++) {
                    const cin in = {dashed.p + dashed.cs[k], dashed.f + dashed.cs[k],
                                    dashed.cs[k + 1] - dashed.cs[k], 0};
                    stroke_contour(&in, st, &o, &c);
                }
            } else {
                for (uint32_t k = k0; k < k1; k++) {
                    const uint32_t a = s->contour_start[k], e = s->contour_start[k + 1];
                    if (a == e) continue;  /* an outline has no empty contours (Outline::push_contour) */
                    const cin in = {pts + a, s->point_flags + a, e - a,
                                    s->contour_closed ? s->contour_closed[k] != 0 : 0};
                    stroke_contour(&in, st, &o, &c);
                }
            }
        }
        if (o.fail || c.fail) status = 3;
        if (o.nc >= UINT32_MAX || o.np >= ((size_t)1 << 31)) status = 4;
        pstart[p + 1] = (uint32_t)o.nc;
    }
    free(c.p);
    free(c.f);
    free(dashed.p);
    free(dashed.f);
    free(dashed.cs);
    if (status) {
        free(o.p);
        free(o.f);
        free(o.cs);
        free(pstart);
        free(rule);
        return status;
    }
    out->n_points = (uint32_t)o.np;
    out->n_contours = (uint32_t)o.nc;
    out->n_paths = s->n_paths;
    out->points = (float *)o.p;
    out->point_flags = o.f;
    out->contour_start = o.cs;
    out->path_start = pstart;
    out->fill_rule = rule;
    if (!out->points) out->points = (float *)calloc(2, sizeof(float));
    if (!out->point_flags) out->point_flags = (uint8_t *)calloc(1, 1);
    return 0;
}

void pfo_outline_free(pfo_outline *o) {
    if (!o) return;
    free(o->points);
    free(o->point_flags);
    free(o->contour_start);
    free(o->path_start);
    free(o->fill_rule);
    memset(o, 0, sizeof(*o));
}
