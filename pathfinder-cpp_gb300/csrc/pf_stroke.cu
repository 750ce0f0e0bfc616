// pf_stroke.cu - stroke-to-fill conversion and line dashing on the GPU, run when a scene with
// stroked paths is uploaded (Canvas::stroke_path, pathfinder/core/canvas.cpp:270-300: dash the
// outline with OutlineDash, convert it with OutlineStrokeToFill, fill the result nonzero).
//
// Layout of the work:
//   k_dash<count/write>        one thread per dashed path walks its contours in order (the dash
//                              state runs on across contours, core/dash.cpp:51-55), writing
//                              the dashed contours into a side buffer;
//   k_stroke_jobs<count/fill>  one job per output contour: a copied contour (filled paths), an
//                              open stroked contour (forward offset, cap, backward offset, cap)
//                              or one of the two contours of a closed stroked contour (forward
//                              or backward offset plus the closing join);
//   k_stroke<count/write>      one thread per job runs it: the segment offset recursion is an
//                              explicit depth-first stack, joins and caps read the contour's
//                              last points from a small ring, so the count pass and the write
//                              pass take the same steps;
//   k_outline_starts           the scene-local contour and path offsets of the new outline.
//
// Every float operation is the reference's, in its order, with explicit round-to-nearest
// intrinsics (no contraction into FMA), so the stroke outline matches the reference's bit for
// bit: Segment::offset and its helpers (core/stroke.cpp:370-540), LineSegmentF
// (core/data/line_segment.cpp), Segment (core/data/segment.cpp), Mat2 / Transform2 /
// UnitVector (common/math).
#include "pf_internal.h"

namespace pfc {
namespace {

constexpr float kFloatEps = 0.0001f;   // FLOAT_EPSILON, common/math/basic.h:11
constexpr float kGeomEps = 0.001f;     // GEOMETRIC_EPSILON, common/math/basic.h:14
constexpr float kStrokeTol = 0.1f;     // STROKE_TOL, core/stroke.cpp:15
constexpr uint32_t kSamples = 8;       // SAMPLE_COUNT, core/stroke.cpp:21
constexpr int kRing = 64;              // points a job can look back (caps search backwards)
constexpr int kStack = 18;             // offset recursion: depth 16 (stroke.cpp:521)
constexpr uint32_t kDashStepLimit = 1u << 22;

enum : int { kNone = 0, kLine = 1, kQuad = 2, kCubic = 3 };
enum : uint8_t { kOn = 0, kC0 = 1, kC1 = 2 };

// first index i in [0, n) with a[i] > v (a non-decreasing), n if none
__device__ __forceinline__ uint32_t upper_bound(const uint32_t *a, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

struct V2 {
    float x, y;
};
struct LSeg {
    V2 f, t;
};
struct Seg {
    LSeg b, c;
    int kind;
};
struct Mat {
    float v[4];
};
struct Xf {
    Mat m;
    V2 t;
};

__device__ __forceinline__ V2 mk(float x, float y) { return V2{x, y}; }
__device__ __forceinline__ V2 vadd(V2 a, V2 b) { return mk(fa(a.x, b.x), fa(a.y, b.y)); }
__device__ __forceinline__ V2 vsub(V2 a, V2 b) { return mk(fs(a.x, b.x), fs(a.y, b.y)); }
__device__ __forceinline__ V2 vmul(V2 a, V2 b) { return mk(fm(a.x, b.x), fm(a.y, b.y)); }
__device__ __forceinline__ V2 vscale(V2 a, float s) { return mk(fm(a.x, s), fm(a.y, s)); }
__device__ __forceinline__ float vsqlen(V2 a) { return fa(fm(a.x, a.x), fm(a.y, a.y)); }
__device__ __forceinline__ float vlen(V2 a) { return fsqrt(vsqlen(a)); }
__device__ __forceinline__ V2 vnorm(V2 a) {
    const float l = vlen(a);
    return mk(fd(a.x, l), fd(a.y, l));
}
__device__ __forceinline__ bool veq(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
__device__ __forceinline__ float max_std(float a, float b) { return a < b ? b : a; }  // std::max
__device__ __forceinline__ V2 vlerp(V2 a, V2 b, float t) {  // common/math/vec2.h:178-180
    return mk(fa(a.x, fm(t, fs(b.x, a.x))), fa(a.y, fm(t, fs(b.y, a.y))));
}

// Mat2 (common/math/mat2.h), Transform2 (common/math/transform2.*), UnitVector
// (common/math/unit_vector.cpp)
__device__ __forceinline__ Mat mat(float a, float b, float c, float d) { return Mat{{a, b, c, d}}; }
__device__ __forceinline__ Mat mmul(const Mat &a, const Mat &b) {
    return mat(fa(fm(a.v[0], b.v[0]), fm(a.v[2], b.v[1])), fa(fm(a.v[1], b.v[0]), fm(a.v[3], b.v[1])),
               fa(fm(a.v[0], b.v[2]), fm(a.v[2], b.v[3])), fa(fm(a.v[1], b.v[2]), fm(a.v[3], b.v[3])));
}
__device__ __forceinline__ V2 mvec(const Mat &a, V2 p) {
    return mk(fa(fm(a.v[0], p.x), fm(a.v[2], p.y)), fa(fm(a.v[1], p.x), fm(a.v[3], p.y)));
}
__device__ __forceinline__ float mdet(const Mat &a) { return fs(fm(a.v[0], a.v[3]), fm(a.v[1], a.v[2])); }
__device__ __forceinline__ V2 xapply(const Xf &a, V2 p) { return vadd(mvec(a.m, p), a.t); }
__device__ __forceinline__ Xf xmul(const Xf &a, const Xf &b) { return Xf{mmul(a.m, b.m), xapply(a, b.t)}; }
__device__ __forceinline__ Xf xscale(V2 s) { return Xf{mat(s.x, 0.0f, 0.0f, s.y), mk(0.0f, 0.0f)}; }
__device__ __forceinline__ Xf xtranslate(const Xf &a, V2 t) {  // from_translation(t) * a
    return xmul(Xf{mat(1.0f, 0.0f, 0.0f, 1.0f), t}, a);
}
__device__ __forceinline__ Xf xrotation(V2 u) {
    return Xf{mat(fm(1.0f, u.x), fm(1.0f, u.y), fm(-1.0f, u.y), fm(1.0f, u.x)), mk(0.0f, 0.0f)};
}
__device__ __forceinline__ V2 urot(V2 a, V2 o) { return mk(fs(fm(a.x, o.x), fm(a.y, o.y)), fa(fm(a.y, o.x), fm(a.x, o.y))); }
__device__ __forceinline__ V2 urevrot(V2 a, V2 o) {
    return mk(fa(fm(a.x, o.x), fm(a.y, o.y)), fs(fm(a.y, o.x), fm(a.x, o.y)));
}
__device__ __forceinline__ V2 uhalve(V2 a) {
    const V2 h = vmul(mk(0.5f, 0.5f), vadd(mk(1.0f, 1.0f), mk(a.x, -a.x)));
    return mk(fsqrt(max_std(h.x, 0.0f)), fsqrt(max_std(h.y, 0.0f)));
}

// LineSegmentF (core/data/line_segment.cpp)
__device__ __forceinline__ LSeg ls(V2 f, V2 t) { return LSeg{f, t}; }
__device__ __forceinline__ V2 lvec(const LSeg &l) { return vsub(l.t, l.f); }
__device__ __forceinline__ float lsqlen(const LSeg &l) { return vsqlen(lvec(l)); }
__device__ __forceinline__ V2 lsample(const LSeg &l, float t) { return vadd(l.f, vscale(lvec(l), t)); }
__device__ __forceinline__ bool lfinite(const LSeg &l) {
    return isfinite(l.f.x) && isfinite(l.f.y) && isfinite(l.t.x) && isfinite(l.t.y);
}
// :78-87
__device__ __forceinline__ bool lintersect(const LSeg &a, const LSeg &o, float &out) {
    const V2 p0p1 = lvec(a), ov = lvec(o);
    const Mat m = mat(ov.x, ov.y, -p0p1.x, -p0p1.y);
    const float det = mdet(m);
    if (fabsf(det) < kFloatEps) return false;
    const float s = fd(1.0f, det);
    const Mat adj = mat(fm(m.v[3], 1.0f), fm(m.v[1], -1.0f), fm(m.v[2], -1.0f), fm(m.v[0], 1.0f));
    const Mat inv = mat(fm(adj.v[0], s), fm(adj.v[1], s), fm(adj.v[2], s), fm(adj.v[3], s));
    out = mvec(inv, vsub(a.f, o.f)).y;
    return true;
}
// :89-95
__device__ __forceinline__ LSeg loffset(const LSeg &l, float d) {
    const V2 v = lvec(l);
    if (v.x == 0.0f && v.y == 0.0f) return l;
    const V2 o = vmul(vnorm(mk(v.y, v.x)), mk(-d, d));
    return ls(vadd(l.f, o), vadd(l.t, o));
}

// Segment (core/data/segment.cpp)
__device__ __forceinline__ Seg sline(LSeg b) { return Seg{b, ls(mk(0, 0), mk(0, 0)), kLine}; }
__device__ __forceinline__ Seg squad(LSeg b, V2 c) { return Seg{b, ls(c, c), kQuad}; }
__device__ __forceinline__ Seg scubic(LSeg b, LSeg c) { return Seg{b, c, kCubic}; }
__device__ __forceinline__ V2 lerp_t(V2 a, V2 b, float t) { return vadd(a, vscale(vsub(b, a), t)); }
// split :42-139
__device__ void ssplit(const Seg &s, float t, Seg &a, Seg &b) {
    if (s.kind == kLine) {
        const V2 mid = vadd(s.b.f, vscale(vsub(s.b.t, s.b.f), t));
        a = Seg{ls(s.b.f, mid), s.c, kLine};
        b = Seg{ls(mid, s.b.t), s.c, kLine};
    } else if (s.kind == kQuad) {
        const V2 p0 = s.b.f, p1 = s.c.f, p2 = s.b.t;
        const V2 qa = lerp_t(p0, p1, t), qb = lerp_t(p1, p2, t), qc = lerp_t(qa, qb, t);
        a = Seg{ls(p0, qc), ls(qa, qa), kQuad};
        b = Seg{ls(qc, p2), ls(qb, qb), kQuad};
    } else if (t <= 0.0f) {
        const V2 f = s.b.f;
        a = Seg{ls(f, f), ls(f, f), kCubic};
        b = Seg{s.b, s.c, kCubic};
    } else if (t >= 1.0f) {
        const V2 to = s.b.t;
        a = Seg{s.b, s.c, kCubic};
        b = Seg{ls(to, to), ls(to, to), kCubic};
    } else {
        const V2 p0 = s.b.f, p3 = s.b.t, p1 = s.c.f, p2 = s.c.t;
        const V2 p01 = lerp_t(p0, p1, t), p12 = lerp_t(p1, p2, t), p23 = lerp_t(p2, p3, t);
        const V2 p012 = lerp_t(p01, p12, t), p123 = lerp_t(p12, p23, t);
        const V2 p0123 = lerp_t(p012, p123, t);
        a = Seg{ls(p0, p0123), ls(p01, p012), kCubic};
        b = Seg{ls(p0123, p3), ls(p123, p23), kCubic};
    }
}
__device__ __forceinline__ V2 ssample(const Seg &s, float t) {  // :160-165
    Seg a, b;
    ssplit(s, t, a, b);
    return a.b.t;
}
__device__ __forceinline__ Seg sxform(const Seg &s, const Xf &x) {  // :153-158
    return Seg{ls(xapply(x, s.b.f), xapply(x, s.b.t)), ls(xapply(x, s.c.f), xapply(x, s.c.t)), s.kind};
}
__device__ __forceinline__ bool svalid(const Seg &s) {  // :189-200
    if (s.kind == kLine) return lfinite(s.b);
    if (s.kind == kQuad || s.kind == kCubic) return lfinite(s.b) && lfinite(s.c);
    return false;
}
__device__ float sarc_length(const Seg &s) {  // :141-187 (quadratics through to_cubic)
    if (s.kind == kLine) return vlen(lvec(s.b));
    if (s.kind != kQuad && s.kind != kCubic) return 0.0f;
    LSeg c = s.c;
    if (s.kind == kQuad) {
        const V2 p1_2 = vadd(s.c.f, s.c.f);
        const V2 c0 = vadd(s.b.f, p1_2), c1 = vadd(p1_2, s.b.t);
        c = ls(mk(fd(c0.x, 3.0f), fd(c0.y, 3.0f)), mk(fd(c1.x, 3.0f), fd(c1.y, 3.0f)));
    }
    const float chord = vlen(lvec(s.b));
    const float net = fa(fa(vlen(vsub(s.b.f, c.f)), vlen(lvec(c))), vlen(vsub(s.b.t, c.t)));
    return fm(fa(net, chord), 0.5f);
}
__device__ __forceinline__ Seg quarter_arc() {  // :202-211
    const float r2 = fsqrt(2.0f);
    const V2 p0 = mk(fm(r2, 0.5f), fm(r2, 0.5f));
    const float third4 = fd(4.0f, 3.0f);
    const V2 p1 = mk(fa(fd(-r2, 6.0f), third4), fs(fd(fm(7.0f, r2), 6.0f), third4));
    const V2 flip = mk(1.0f, -1.0f);
    return Seg{ls(vmul(p0, flip), p0), ls(vmul(p1, flip), p1), kCubic};
}
__device__ __forceinline__ Seg arc_from_cos(float c) {  // :213-240 (the threshold in double)
    if ((double)c >= 1.0 - (double)kGeomEps) return sline(ls(mk(1.0f, 0.0f), mk(1.0f, 0.0f)));
    const V2 h = vmul(mk(fa(c, 1.0f), fa(-c, 1.0f)), mk(0.5f, 0.5f));
    const V2 r = mk(fsqrt(h.x), fsqrt(h.y));
    const V2 p3 = vmul(r, mk(1.0f, -1.0f)), p0 = vmul(r, mk(1.0f, 1.0f));
    const float p1x = fs(4.0f, p0.x);
    const float p1y = fd(fm(fs(1.0f, p0.x), fs(3.0f, p0.x)), p0.y);
    const float third = fd(1.0f, 3.0f);
    return scubic(ls(p3, p0), ls(vscale(mk(p1x, -p1y), third), vscale(mk(p1x, p1y), third)));
}

// One output contour: counts its points; with a destination also stores them.  Joins read
// the last two points, the closing join the first two, caps search back through the ring.
struct Sink {
    float2 *pts;
    uint8_t *fl;
    uint32_t n;
    bool lost;  // a cap searched further back than the ring holds
    V2 first[2];
    V2 ring[kRing];
    __device__ void push(V2 p, uint8_t f) {
        if (pts) {
            pts[n] = make_float2(p.x, p.y);
            fl[n] = f;
        }
        if (n < 2) first[n] = p;
        ring[n % kRing] = p;
        n++;
    }
    __device__ V2 last(uint32_t k) const { return ring[(n - k) % kRing]; }
};

__device__ void push_seg(Sink &o, const Seg &s) {  // core/data/contour.cpp:11-41
    if (s.kind == kNone || !svalid(s)) return;
    o.push(s.b.f, kOn);
    if (s.kind != kLine) {
        o.push(s.c.f, kC0);
        if (s.kind != kQuad) o.push(s.c.t, kC1);
    }
    o.push(s.b.t, kOn);
}
__device__ __forceinline__ bool might_join(const Sink &o, int join) {  // stroke.cpp:264-271
    return o.n >= 2 && (join == PF_JOIN_MITER || join == PF_JOIN_ROUND);
}
__device__ void push_arc(Sink &o, const Xf &x, LSeg chord) {  // stroke.cpp:326-368, clockwise
    const Xf dir = xscale(mk(1.0f, 1.0f));
    V2 vec = chord.f;
    const V2 end = chord.t;
    for (int i = 0; i < 4; i++) {
        V2 sweep = urevrot(end, vec);
        const bool last = sweep.x >= -kFloatEps && sweep.y >= -kFloatEps;
        Seg s;
        if (!last) {
            sweep = mk(0.0f, 1.0f);
            s = quarter_arc();
        } else {
            s = arc_from_cos(sweep.x);
        }
        const Xf rot = xrotation(urot(uhalve(sweep), vec));
        s = sxform(s, xmul(xmul(x, dir), rot));
        push_seg(o, s);
        if (last) break;
        vec = urot(vec, sweep);
    }
}
__device__ void add_join(Sink &o, float d, int join, V2 jp, const LSeg &next, float miter) {  // :273-324
    const LSeg prev = ls(o.last(2), o.last(1));
    if (lsqlen(prev) < kFloatEps || lsqlen(next) < kFloatEps) return;
    if (join == PF_JOIN_MITER) {
        float t;
        if (lintersect(prev, next, t)) {
            if (t < -kFloatEps) return;
            const V2 me = lsample(prev, t);
            const float th = fm(miter, d);
            if (vsqlen(vsub(me, jp)) > fm(th, th)) return;
            o.push(me, kOn);
        }
    } else if (join == PF_JOIN_ROUND) {
        if (vsqlen(vsub(prev.t, jp)) == 0.0f || vsqlen(vsub(next.t, jp)) == 0.0f) return;
        const float sc = fabsf(d);
        const Xf x = xtranslate(xscale(mk(sc, sc)), jp);
        push_arc(o, x, ls(vnorm(vsub(prev.t, jp)), vnorm(vsub(next.t, jp))));
    }
}

// Segment::offset_once, stroke.cpp:370-442
__device__ Seg offset_once(const Seg &s, float d) {
    if (s.kind == kLine) return sline(loffset(s.b, d));
    if (s.kind == kQuad) {
        const LSeg s0 = loffset(ls(s.b.f, s.c.f), d), s1 = loffset(ls(s.c.f, s.b.t), d);
        float t;
        const V2 c = lintersect(s0, s1, t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return squad(ls(s0.f, s1.t), c);
    }
    if (veq(s.b.f, s.c.f)) {
        const LSeg s0 = loffset(ls(s.b.f, s.c.t), d), s1 = loffset(ls(s.c.t, s.b.t), d);
        float t;
        const V2 c = lintersect(s0, s1, t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return scubic(ls(s0.f, s1.t), ls(s0.f, c));
    }
    if (veq(s.c.t, s.b.t)) {
        const LSeg s0 = loffset(ls(s.b.f, s.c.f), d), s1 = loffset(ls(s.c.f, s.b.t), d);
        float t;
        const V2 c = lintersect(s0, s1, t) ? lsample(s0, t) : vlerp(s0.t, s1.f, 0.5f);
        return scubic(ls(s0.f, s1.t), ls(c, s1.t));
    }
    const LSeg s0 = loffset(ls(s.b.f, s.c.f), d), s1 = loffset(ls(s.c.f, s.c.t), d), s2 = loffset(ls(s.c.t, s.b.t), d);
    float t0, t1;
    V2 c0, c1;
    if (lintersect(s0, s1, t0) && lintersect(s1, s2, t1)) {
        c0 = lsample(s0, t0);
        c1 = lsample(s1, t1);
    } else {
        c0 = vlerp(s0.t, s1.f, 0.5f);
        c1 = vlerp(s1.t, s2.f, 0.5f);
    }
    return scubic(ls(s0.f, s2.t), ls(c0, c1));
}
// Segment::error_is_within_tolerance, stroke.cpp:455-477
__device__ bool within_tol(const Seg &s, const Seg &o, float d) {
    float lo = fs(fabsf(d), kStrokeTol), hi = fa(fabsf(d), kStrokeTol);
    lo = lo <= 0.0f ? 0.0f : fm(lo, lo);
    hi = hi <= 0.0f ? 0.0f : fm(hi, hi);
    for (uint32_t k = 0; k < kSamples + 1; k++) {
        const float t = fd((float)k, (float)kSamples);
        const float sq = vsqlen(vsub(ssample(s, t), ssample(o, t)));
        if (sq < lo || sq > hi) return false;
    }
    return true;
}
// Segment::add_to_contour, stroke.cpp:479-500
__device__ void add_to_contour(Sink &o, const Seg &s, float d, int join, V2 jp, float miter) {
    if (might_join(o, join)) {
        const V2 p3 = s.b.f, p4 = s.kind == kLine ? s.b.t : s.c.f;
        add_join(o, d, join, jp, ls(p4, p3), miter);
    }
    push_seg(o, s);
}
// Segment::offset, stroke.cpp:502-540, depth first through an explicit stack
__device__ void seg_offset(Sink &o, const Seg &root, float d, int join, float miter) {
    Seg stack[kStack];
    uint8_t depth[kStack];
    int sp = 0;
    stack[0] = root;
    depth[0] = 0;
    sp = 1;
    const float tol2 = fm(kStrokeTol, kStrokeTol);
    while (sp > 0) {
        sp--;
        const Seg s = stack[sp];
        const uint32_t dep = depth[sp];
        if (!svalid(s)) continue;
        const V2 jp = s.b.f;
        if (lsqlen(s.b) < tol2 || dep >= 16) {
            add_to_contour(o, s, d, join, jp, miter);
            continue;
        }
        const Seg cand = offset_once(s, d);
        if (s.kind == kLine || within_tol(s, cand, d)) {
            add_to_contour(o, cand, d, join, jp, miter);
            continue;
        }
        Seg a, b;
        ssplit(s, 0.5f, a, b);
        stack[sp] = b;
        depth[sp] = (uint8_t)(dep + 1);
        stack[sp + 1] = a;
        depth[sp + 1] = (uint8_t)(dep + 1);
        sp += 2;
    }
}

struct Contour {
    const float2 *p;
    const uint8_t *f;
    uint32_t n;
    bool closed;
    __device__ V2 at(uint32_t i) const {
        const float2 q = p[i];
        return mk(q.x, q.y);
    }
};

// SegmentsIter::get_next, core/data/contour.cpp:110-173 (force_closed false)
struct SegIter {
    const Contour *c;
    uint32_t head;
    bool has_next;
    __device__ Seg next() {
        Seg s{ls(mk(0, 0), mk(0, 0)), ls(mk(0, 0), mk(0, 0)), kNone};
        const uint32_t n = c->n, h = head;
        if (h >= n || c->f[h] != kOn) return s;
        s.b.f = c->at(h);
        if (h + 1 < n) {
            if (c->f[h + 1] == kOn) {
                s.b.t = c->at(h + 1);
                s.kind = kLine;
                head += 1;
            } else if (h + 2 < n) {
                if (c->f[h + 1] == kC0 && c->f[h + 2] == kOn) {
                    s.c.f = c->at(h + 1);
                    s.b.t = c->at(h + 2);
                    s.kind = kQuad;
                    head += 2;
                } else if (h + 3 < n) {
                    if (c->f[h + 1] == kC0 && c->f[h + 2] == kC1 && c->f[h + 3] == kOn) {
                        s.c.f = c->at(h + 1);
                        s.c.t = c->at(h + 2);
                        s.b.t = c->at(h + 3);
                        s.kind = kCubic;
                        head += 3;
                    }
                }
            }
        } else {
            const V2 a = c->at(0), z = c->at(n - 1);
            if (c->closed && n > 1 && !(vlen(vsub(a, z)) <= kFloatEps)) {
                s.b = ls(z, a);
                s.kind = kLine;
            }
            has_next = false;
        }
        return s;
    }
};

// ContourStrokeToFill::offset_forward / offset_backward, stroke.cpp:27-122
__device__ void offset_forward(Sink &o, const Contour &c, float r, int join, float miter) {
    SegIter it{&c, 0, true};
    int idx = -1;
    while (it.has_next) {
        const Seg s = it.next();
        idx++;
        if (s.kind == kNone) break;
        seg_offset(o, s, -r, idx == 0 ? (int)PF_JOIN_BEVEL : join, miter);
    }
}
__device__ void offset_backward(Sink &o, const Contour &c, float r, int join, float miter) {
    const int n = (int)c.n;
    int tail = n - 1, idx = -1;
    if (c.closed && n > 1 && !(vlen(vsub(c.at(0), c.at(n - 1))) <= kFloatEps)) {
        idx++;
        seg_offset(o, sline(ls(c.at(0), c.at(n - 1))), -r, idx == 0 ? (int)PF_JOIN_BEVEL : join, miter);
    }
    while (tail >= 0) {
        if (c.f[tail] != kOn) break;
        Seg s;
        if (tail >= 3 && c.f[tail - 1] == kC1 && c.f[tail - 2] == kC0 && c.f[tail - 3] == kOn) {
            s = scubic(ls(c.at(tail), c.at(tail - 3)), ls(c.at(tail - 1), c.at(tail - 2)));
            tail -= 3;
        } else if (tail >= 2 && c.f[tail - 1] == kC0 && c.f[tail - 2] == kOn) {
            s = squad(ls(c.at(tail), c.at(tail - 2)), c.at(tail - 1));
            tail -= 2;
        } else if (tail >= 1 && c.f[tail - 1] == kOn) {
            s = sline(ls(c.at(tail), c.at(tail - 1)));
            tail -= 1;
        } else {
            break;
        }
        idx++;
        seg_offset(o, s, -r, idx == 0 ? (int)PF_JOIN_BEVEL : join, miter);
    }
}
// OutlineStrokeToFill::add_cap, stroke.cpp:206-258
__device__ void add_cap(Sink &o, const pf_stroke &st) {
    if (st.line_cap == PF_CAP_BUTT || o.n < 2) return;
    const float w = st.line_width;
    const V2 p1 = o.last(1);
    V2 p0;
    uint32_t i = o.n - 2;
    for (;;) {
        if (o.n - i > (uint32_t)kRing) {
            o.lost = true;
            return;
        }
        p0 = o.ring[i % kRing];
        if (vsqlen(vsub(p1, p0)) > kFloatEps) break;
        if (i == 0) return;
        i -= 1;
    }
    const V2 g = vnorm(vsub(p1, p0));
    if (st.line_cap == PF_CAP_SQUARE) {
        const V2 off = vscale(g, fm(w, 0.5f));
        const V2 p2 = vadd(p1, off);
        const V2 p3 = vadd(p2, vmul(mk(g.y, g.x), mk(-w, w)));
        const V2 p4 = vsub(p3, off);
        o.push(p2, kOn);
        o.push(p3, kOn);
        o.push(p4, kOn);
    } else {
        const float sc = fm(w, 0.5f);
        const V2 off = vmul(mk(g.y, g.x), mk(-1.0f, 1.0f));
        const V2 tr = vadd(p1, vscale(off, fm(w, 0.5f)));
        push_arc(o, xtranslate(xscale(mk(sc, sc)), tr), ls(mk(-off.x, -off.y), off));
    }
}
// OutlineStrokeToFill::push_stroked_contour's join, stroke.cpp:186-204
__device__ void close_join(Sink &o, const Contour &c, const pf_stroke &st) {
    if (might_join(o, st.line_join))
        add_join(o, fm(st.line_width, 0.5f), st.line_join, c.at(0), ls(o.first[1], o.first[0]), st.miter_limit);
}

// Job kinds (one output contour each).
enum : uint32_t { kJobCopy = 0, kJobOpen = 1, kJobClosedFwd = 2, kJobClosedBwd = 3 };

__device__ __forceinline__ const pf_stroke &path_stroke(const StrokeIn &in, uint32_t p) { return in.stroke[p]; }
__device__ __forceinline__ bool stroked(const StrokeIn &in, uint32_t p) { return in.stroke[p].line_width > 0.0f; }

// Global contour k of the uploaded outline: its points.
__device__ __forceinline__ Contour raw_contour(const StrokeIn &in, uint32_t k) {
    const uint32_t s = upper_bound(in.scene_contour_first, in.n_scenes + 1, k) - 1;
    const SceneDev &S = in.scenes[s];
    const uint32_t local = k - S.contour_first;
    const uint32_t a = in.cstart[S.cstart_base + local], e = in.cstart[S.cstart_base + local + 1];
    Contour c;
    c.p = in.points + S.point_first + a;
    c.f = in.flags + S.point_first + a;
    c.n = e - a;
    c.closed = in.closed && in.closed[k] != 0;
    return c;
}
__device__ __forceinline__ uint2 path_contours(const StrokeIn &in, uint32_t p) {
    const uint32_t s = upper_bound(in.scene_path_first, in.n_scenes + 1, p) - 1;
    const SceneDev &S = in.scenes[s];
    const uint32_t local = p - S.path_first;
    return make_uint2(S.contour_first + in.pstart[S.pstart_base + local],
                      S.contour_first + in.pstart[S.pstart_base + local + 1]);
}

// --- Dashing (core/dash.cpp) -------------------------------------------------------------
// One thread per path.  count: dash_pts[p], dash_cnt[p] (contours); write: the contours at
// dash_pts[p] / dash_cnt[p] (scanned), their ends in dash_end.
template <bool kWrite>
__global__ void k_dash(StrokeIn in, uint32_t *status) {
    // the dashed paths, largest first (dash_order); every other path's counts are zeroed
    // before the count pass
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= in.n_dashed) return;
    const uint32_t p = in.dash_order[t];
    const pf_stroke &st = path_stroke(in, p);
    if (!stroked(in, p) || st.dash_count == 0) return;
    // DashState::DashState, dash.cpp:9-29
    const float *dashes = in.dashes + st.dash_first;
    const uint32_t count = st.dash_count;
    float total = 0.0f;
    for (uint32_t i = 0; i < count; i++) total = fa(total, dashes[i]);
    float offset = fmodf(st.dash_offset, total);
    uint32_t idx = 0;
    while (idx < count) {
        const float dash = dashes[idx];
        if (offset < dash) break;
        offset = fs(offset, dash);
        idx += 1;
    }
    if (idx >= count) {  // the phase ran past the pattern
        atomicOr(&status[kStErr], kErrStroke);
        return;
    }
    float left = offset;
    uint32_t pts = kWrite ? in.dash_pts[p] : 0u, cnt = kWrite ? in.dash_cnt[p] : 0u;
    Sink cur;
    cur.pts = kWrite ? in.dash_points + pts : nullptr;
    cur.fl = kWrite ? in.dash_flags + pts : nullptr;
    cur.n = 0;
    cur.lost = false;
    uint32_t steps = 0;
    auto flush = [&]() {  // Outline::push_contour: empty contours are dropped
        if (cur.n == 0) return;
        pts += cur.n;
        if (kWrite) in.dash_end[cnt] = pts;
        cnt++;
        cur.n = 0;
        if (kWrite) {
            cur.pts = in.dash_points + pts;
            cur.fl = in.dash_flags + pts;
        }
    };
    const uint2 kr = path_contours(in, p);
    for (uint32_t k = kr.x; k < kr.y; k++) {
        const Contour c = raw_contour(in, k);
        // ContourDash::dash, dash.cpp:68-124
        SegIter it{&c, 0, true};
        Seg queued{};
        bool none = true;
        for (;;) {
            if (none) {
                if (!it.has_next) break;
                queued = it.next();
                if (queued.kind == kNone) break;
                none = false;
            }
            if (++steps > kDashStepLimit) {
                atomicOr(&status[kStErr], kErrStroke);
                return;
            }
            Seg segc = queued;
            float distance = left;
            const float t = fd(distance, sarc_length(segc));
            if (t < 1.0f) {
                Seg a = segc, b = segc;
                ssplit(segc, t, a, b);
                segc = a;
                queued = b;
                none = false;
            } else {
                distance = sarc_length(segc);
                none = true;
            }
            if (idx % 2 == 0) push_seg(cur, segc);
            left = fs(left, distance);
            if (left < kFloatEps) {
                if (idx % 2 == 0) flush();
                idx += 1;
                if (idx == count) idx = 0;
                left = dashes[idx];
            }
        }
    }
    if (idx % 2 == 0) flush();  // OutlineDash::into_outline, dash.cpp:57-63
    if (!kWrite) {
        in.dash_pts[p] = pts;
        in.dash_cnt[p] = cnt;
        // 64-bit total beside the 32-bit scan, so that an overflowing batch is caught
        atomicAdd(reinterpret_cast<unsigned long long *>(status + kStFill64), (unsigned long long)pts);
    }
}

// --- Jobs --------------------------------------------------------------------------------
// count: job_first[p] = output contours of path p.  fill: the jobs (x: first point, y: points,
// z: kind | closed << 2 | from the dash buffer << 3, w: path).
template <bool kFill>
__global__ void k_stroke_jobs(StrokeIn in) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= in.n_paths) return;
    uint32_t j = kFill ? in.job_first[p] : 0u;
    if (stroked(in, p) && path_stroke(in, p).dash_count) {
        // the dashed contours, all open (dash_cnt is scanned by now: the path's contours are
        // [dash_cnt[p], dash_cnt[p + 1]))
        const uint32_t c0 = in.dash_cnt[p], n = in.dash_cnt[p + 1] - c0;
        if (kFill) {
            for (uint32_t k = 0; k < n; k++) {
                const uint32_t a = c0 + k == 0 ? 0u : in.dash_end[c0 + k - 1], e = in.dash_end[c0 + k];
                in.jobs[j++] = make_uint4(a, e - a, kJobOpen | 8u, p);
            }
        } else {
            in.job_first[p] = n;
        }
        return;
    }
    const uint2 kr = path_contours(in, p);
    const bool st = stroked(in, p);
    uint32_t n = 0;
    for (uint32_t k = kr.x; k < kr.y; k++) {
        const uint32_t s = upper_bound(in.scene_contour_first, in.n_scenes + 1, k) - 1;
        const SceneDev &S = in.scenes[s];
        const uint32_t local = k - S.contour_first;
        const uint32_t a = in.cstart[S.cstart_base + local], e = in.cstart[S.cstart_base + local + 1];
        const uint32_t first = S.point_first + a, np = e - a;
        if (!st) {
            if (kFill) in.jobs[j++] = make_uint4(first, np, kJobCopy, p);
            n++;
        } else if (np) {  // an outline has no empty contours (Outline::push_contour)
            const bool closed = in.closed && in.closed[k];
            if (closed) {
                if (kFill) {
                    in.jobs[j++] = make_uint4(first, np, kJobClosedFwd | 4u, p);
                    in.jobs[j++] = make_uint4(first, np, kJobClosedBwd | 4u, p);
                }
                n += 2;
            } else {
                if (kFill) in.jobs[j++] = make_uint4(first, np, kJobOpen, p);
                n++;
            }
        }
    }
    if (!kFill) in.job_first[p] = n;
}

// One output contour.  count: job_pts[j]; write: its points at job_pts[j] (scanned).
template <bool kWrite>
__global__ void __launch_bounds__(128) k_stroke(StrokeIn in, uint32_t *status) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= in.n_jobs) return;
    const uint4 job = in.jobs[j];
    const uint32_t kind = job.z & 3u;
    // stroked contours go through the segment-parallel kernels unless marked degenerate
    if (kind != kJobCopy && !(in.job_flags[j] & 1u)) return;
    Contour c;
    const bool from_dash = (job.z & 8u) != 0;
    c.p = (from_dash ? in.dash_points : in.points) + job.x;
    c.f = (from_dash ? in.dash_flags : in.flags) + job.x;
    c.n = job.y;
    c.closed = (job.z & 4u) != 0;
    const uint32_t base = kWrite ? in.job_pts[j] : 0u;
    if (kind == kJobCopy) {
        if (kWrite)
            for (uint32_t i = 0; i < c.n; i++) {
                in.out_points[base + i] = c.p[i];
                in.out_flags[base + i] = c.f[i];
            }
        else
            in.job_pts[j] = c.n;
        return;
    }
    const pf_stroke st = in.stroke[job.w];
    const float r = fm(st.line_width, 0.5f);
    Sink o;
    o.pts = kWrite ? in.out_points + base : nullptr;
    o.fl = kWrite ? in.out_flags + base : nullptr;
    o.n = 0;
    o.lost = false;
    // OutlineStrokeToFill::offset, stroke.cpp:124-167
    if (kind == kJobOpen) {
        offset_forward(o, c, r, st.line_join, st.miter_limit);
        add_cap(o, st);
        offset_backward(o, c, r, st.line_join, st.miter_limit);
        add_cap(o, st);
    } else if (kind == kJobClosedFwd) {
        offset_forward(o, c, r, st.line_join, st.miter_limit);
        close_join(o, c, st);
    } else {
        offset_backward(o, c, r, st.line_join, st.miter_limit);
        close_join(o, c, st);
    }
    if (o.lost) atomicOr(&status[kStErr], kErrStroke);
    if (!kWrite) in.job_pts[j] = o.n;
}


// --- Segment-parallel stroking --------------------------------------------------------------
// The sequential algorithm pushes, per input segment in order, the leaves of its offset
// recursion, each preceded by the join with the contour's last two points.  When every leaf
// is a valid segment (it then pushes at least two points), those two points are the previous
// leaf's last two, so every leaf's join and points depend on that leaf and its predecessor
// only; caps and the closing join depend on the first and last leaves.  Contours for which
// this does not hold (an invalid leaf, a cap that searches back past the last leaf, one
// direction empty) are marked and redone by the sequential k_stroke.

// Unit record: float4 baseline, float4 control, float4 (kind, job, dir << 31 | index, -).
__device__ __forceinline__ void put_seg(float4 *dst, const Seg &s, uint32_t w0, uint32_t w1, uint32_t w2) {
    dst[0] = make_float4(s.b.f.x, s.b.f.y, s.b.t.x, s.b.t.y);
    dst[1] = make_float4(s.c.f.x, s.c.f.y, s.c.t.x, s.c.t.y);
    dst[2] = make_float4(__uint_as_float((uint32_t)s.kind), __uint_as_float(w0), __uint_as_float(w1),
                         __uint_as_float(w2));
}
__device__ __forceinline__ Seg get_seg(const float4 *src, uint4 &meta) {
    const float4 b = src[0], c = src[1], m = src[2];
    meta = make_uint4(__float_as_uint(m.x), __float_as_uint(m.y), __float_as_uint(m.z), __float_as_uint(m.w));
    return Seg{ls(mk(b.x, b.y), mk(b.z, b.w)), ls(mk(c.x, c.y), mk(c.z, c.w)), (int)meta.x};
}

__device__ __forceinline__ Contour job_contour(const StrokeIn &in, const uint4 &job) {
    Contour c;
    const bool from_dash = (job.z & 8u) != 0;
    c.p = (from_dash ? in.dash_points : in.points) + job.x;
    c.f = (from_dash ? in.dash_flags : in.flags) + job.x;
    c.n = job.y;
    c.closed = (job.z & 4u) != 0;
    return c;
}

// count: job_units[j], job_nfwd[j]; write: the units (forward: SegmentsIter order; backward:
// the closing line first, then the segments reversed, stroke.cpp:51-122).
template <bool kWrite>
__global__ void k_units(StrokeIn in) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= in.n_jobs) return;
    const uint4 job = in.jobs[j];
    const uint32_t kind = job.z & 3u;
    uint32_t u = kWrite ? in.job_units[j] : 0u;
    const uint32_t u0 = u;
    if (kind == kJobCopy) {
        if (!kWrite) in.job_units[j] = in.job_nfwd[j] = 0;
        return;
    }
    const Contour c = job_contour(in, job);
    if (kind == kJobOpen || kind == kJobClosedFwd) {
        SegIter it{&c, 0, true};
        uint32_t idx = 0;
        while (it.has_next) {
            const Seg s = it.next();
            if (s.kind == kNone) break;
            if (kWrite) put_seg(in.units + 3 * (size_t)u, s, j, idx, 0);
            u++;
            idx++;
        }
    }
    const uint32_t nfwd = u - u0;
    if (kind == kJobOpen || kind == kJobClosedBwd) {
        const int n = (int)c.n;
        int tail = n - 1;
        uint32_t idx = 0;
        if (c.closed && n > 1 && !(vlen(vsub(c.at(0), c.at(n - 1))) <= kFloatEps)) {
            if (kWrite) put_seg(in.units + 3 * (size_t)u, sline(ls(c.at(0), c.at(n - 1))), j, 1u << 31 | idx, 0);
            u++;
            idx++;
        }
        while (tail >= 0) {
            if (c.f[tail] != kOn) break;
            Seg s;
            if (tail >= 3 && c.f[tail - 1] == kC1 && c.f[tail - 2] == kC0 && c.f[tail - 3] == kOn) {
                s = scubic(ls(c.at(tail), c.at(tail - 3)), ls(c.at(tail - 1), c.at(tail - 2)));
                tail -= 3;
            } else if (tail >= 2 && c.f[tail - 1] == kC0 && c.f[tail - 2] == kOn) {
                s = squad(ls(c.at(tail), c.at(tail - 2)), c.at(tail - 1));
                tail -= 2;
            } else if (tail >= 1 && c.f[tail - 1] == kOn) {
                s = sline(ls(c.at(tail), c.at(tail - 1)));
                tail -= 1;
            } else {
                break;
            }
            if (kWrite) put_seg(in.units + 3 * (size_t)u, s, j, 1u << 31 | idx, 0);
            u++;
            idx++;
        }
    }
    if (!kWrite) {
        in.job_units[j] = u - u0;
        in.job_nfwd[j] = nfwd;
    }
}

// count: unit_leaves[u]; write: the leaves of the unit's offset recursion (Segment::offset,
// stroke.cpp:502-540), each the segment it pushes, its join point and (job, meta): meta =
// kind | direction << 2 | (unit index > 0) << 3.  An invalid leaf marks the job.
template <bool kWrite>
__global__ void __launch_bounds__(128) k_unit_leaves(StrokeIn in) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= in.n_units) return;
    const uint32_t u = in.unit_order ? in.unit_order[t] : t;
    uint4 um;
    const Seg root = get_seg(in.units + 3 * (size_t)u, um);
    const uint32_t job = um.y, dir = um.z >> 31, idx = um.z & 0x7fffffffu;
    const float d = -fm(in.stroke[in.jobs[job].w].line_width, 0.5f);
    uint32_t leaf = kWrite ? in.unit_leaves[u] : 0u;
    const uint32_t l0 = leaf;
    Seg stack[kStack];
    uint8_t depth[kStack];
    stack[0] = root;
    depth[0] = 0;
    int sp = 1;
    const float tol2 = fm(kStrokeTol, kStrokeTol);
    bool bad = false;
    auto emit = [&](const Seg &s, V2 jp) {
        bad |= !svalid(s);
        if (kWrite) {
            float4 *r = in.leaves + 3 * (size_t)leaf;
            r[0] = make_float4(s.b.f.x, s.b.f.y, s.b.t.x, s.b.t.y);
            r[1] = make_float4(s.c.f.x, s.c.f.y, s.c.t.x, s.c.t.y);
            r[2] = make_float4(jp.y, __uint_as_float(job),
                               __uint_as_float((uint32_t)s.kind | dir << 2 | (idx > 0 ? 8u : 0u)), jp.x);
        }
        leaf++;
    };
    while (sp > 0) {
        sp--;
        const Seg s = stack[sp];
        const uint32_t dep = depth[sp];
        if (!svalid(s)) continue;
        const V2 jp = s.b.f;
        if (lsqlen(s.b) < tol2 || dep >= 16) {
            emit(s, jp);
            continue;
        }
        const Seg cand = offset_once(s, d);
        if (s.kind == kLine || within_tol(s, cand, d)) {
            emit(cand, jp);
            continue;
        }
        Seg a, b;
        ssplit(s, 0.5f, a, b);
        stack[sp] = b;
        depth[sp] = (uint8_t)(dep + 1);
        stack[sp + 1] = a;
        depth[sp + 1] = (uint8_t)(dep + 1);
        sp += 2;
    }
    if (!kWrite) in.unit_leaves[u] = leaf - l0;
    // an invalid leaf, or a unit without leaves (a later leaf's predecessor would not be its
    // own direction's), leaves the contour to the sequential kernel
    if (!kWrite && (bad || leaf == l0)) atomicOr(&in.job_flags[job], 1u);
}

// A leaf record: float4 baseline, float4 control, float4 (join point y, job, meta, join point x);
// the pushed segment's kind rides in the meta word.
__device__ __forceinline__ Seg get_leaf(const StrokeIn &in, uint32_t l, V2 &jp, uint32_t &job, uint32_t &meta) {
    const float4 *r = in.leaves + 3 * (size_t)l;
    const float4 b = r[0], c = r[1], m = r[2];
    job = __float_as_uint(m.y);
    meta = __float_as_uint(m.z);
    jp = mk(m.w, m.x);
    return Seg{ls(mk(b.x, b.y), mk(b.z, b.w)), ls(mk(c.x, c.y), mk(c.z, c.w)), (int)(meta & 3u)};
}
// The points a segment pushes (contour.cpp:11-41), in order.
__device__ __forceinline__ uint32_t seg_points(const Seg &s, V2 *p) {
    uint32_t n = 0;
    p[n++] = s.b.f;
    if (s.kind != kLine) {
        p[n++] = s.c.f;
        if (s.kind != kQuad) p[n++] = s.c.t;
    }
    p[n++] = s.b.t;
    return n;
}

__device__ __forceinline__ uint32_t first_leaf_of_job(const StrokeIn &in, uint32_t j) {
    return in.unit_leaves[in.job_units[j]];
}
// Output position of a job's leaf: the job's start, the leaves before it, and (open
// contours, backward leaves) the first cap.
__device__ __forceinline__ uint32_t leaf_pos(const StrokeIn &in, uint32_t l, uint32_t job, uint32_t meta) {
    const uint32_t l0 = first_leaf_of_job(in, job);
    const bool open = (in.jobs[job].z & 3u) == kJobOpen;
    return in.job_pts[job] + (in.leaf_pts[l] - in.leaf_pts[l0]) + (open && (meta & 4u) ? in.job_cap1[job] : 0u);
}

// count: leaf_pts[l] = the join before the leaf plus its points; write: those points.
template <bool kWrite>
__global__ void __launch_bounds__(128) k_leaf_pts(StrokeIn in) {
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= in.n_leaves) return;
    V2 jp;
    uint32_t job, meta;
    const Seg s = get_leaf(in, l, jp, job, meta);
    if (in.job_flags[job] & 1u) {
        if (!kWrite) in.leaf_pts[l] = 0;
        return;
    }
    const pf_stroke st = in.stroke[in.jobs[job].w];
    const float d = -fm(st.line_width, 0.5f);
    const bool joins = (meta & 8u) && st.line_join != PF_JOIN_BEVEL;
    Sink o;
    o.n = 2;
    o.lost = false;
    o.pts = nullptr;
    o.fl = nullptr;
    if (joins) {  // the contour's last two points: the previous leaf's
        V2 pj, pp[4];
        uint32_t pjob, pmeta;
        const Seg prev = get_leaf(in, l - 1, pj, pjob, pmeta);
        const uint32_t k = seg_points(prev, pp);
        o.ring[0] = pp[k - 2];
        o.ring[1] = pp[k - 1];
    }
    if (kWrite) {
        const uint32_t pos = leaf_pos(in, l, job, meta);
        o.pts = in.out_points + pos - 2;
        o.fl = in.out_flags + pos - 2;
    }
    if (joins) add_to_contour(o, s, d, st.line_join, jp, st.miter_limit);
    else push_seg(o, s);
    if (!kWrite) in.leaf_pts[l] = o.n - 2;
}

// A cap after leaf l (OutlineStrokeToFill::add_cap, stroke.cpp:206-258) with the search for
// the tangent's start kept inside the leaf's points.  first: the leaf starts the contour (a
// search that reaches its first point ends without a cap); otherwise leaving the leaf marks
// the job.  Returns false when the job must be redone sequentially.
__device__ bool leaf_cap(const StrokeIn &in, uint32_t l, const pf_stroke &st, bool first, float2 *pts, uint8_t *fl,
                         uint32_t &count) {
    V2 jp, p[4];
    uint32_t job, meta;
    const Seg s = get_leaf(in, l, jp, job, meta);
    const uint32_t k = seg_points(s, p);
    count = 0;
    if (st.line_cap == PF_CAP_BUTT) return true;
    const V2 p1 = p[k - 1];
    int i = (int)k - 2;
    for (;;) {
        if (vsqlen(vsub(p1, p[i])) > kFloatEps) break;
        if (i == 0) {
            if (first) return true;
            return false;
        }
        i--;
    }
    Sink o;
    o.n = 2;
    o.lost = false;
    o.pts = pts ? pts - 2 : nullptr;
    o.fl = fl ? fl - 2 : nullptr;
    const V2 g = vnorm(vsub(p1, p[i]));
    const float w = st.line_width;
    if (st.line_cap == PF_CAP_SQUARE) {
        const V2 off = vscale(g, fm(w, 0.5f));
        const V2 p2 = vadd(p1, off);
        const V2 p3 = vadd(p2, vmul(mk(g.y, g.x), mk(-w, w)));
        o.push(p2, kOn);
        o.push(p3, kOn);
        o.push(vsub(p3, off), kOn);
    } else {
        const float sc = fm(w, 0.5f);
        const V2 off = vmul(mk(g.y, g.x), mk(-1.0f, 1.0f));
        const V2 tr = vadd(p1, vscale(off, fm(w, 0.5f)));
        push_arc(o, xtranslate(xscale(mk(sc, sc)), tr), ls(mk(-off.x, -off.y), off));
    }
    count = o.n - 2;
    return true;
}

// count: job_cap1[j], job_end[j] (and the marks for degenerate contours); write: the caps /
// the closing join (push_stroked_contour, stroke.cpp:186-204).
template <bool kWrite>
__global__ void k_job_ends(StrokeIn in) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= in.n_jobs) return;
    const uint4 job = in.jobs[j];
    const uint32_t kind = job.z & 3u;
    if (kind == kJobCopy || (in.job_flags[j] & 1u)) {
        if (!kWrite) in.job_cap1[j] = in.job_end[j] = 0;
        return;
    }
    const uint32_t u0 = in.job_units[j], u1 = in.job_units[j + 1];
    const uint32_t l0 = in.unit_leaves[u0], l1 = in.unit_leaves[u1];
    if (l0 == l1) {  // nothing pushed: no cap, no join
        if (!kWrite) in.job_cap1[j] = in.job_end[j] = 0;
        return;
    }
    const pf_stroke st = in.stroke[job.w];
    const uint32_t base = kWrite ? in.job_pts[j] + (in.leaf_pts[l1] - in.leaf_pts[l0]) : 0u;
    if (kind == kJobOpen) {
        const uint32_t lb = in.unit_leaves[u0 + in.job_nfwd[j]];
        if (lb == l0 || lb == l1) {  // one direction pushed nothing
            if (!kWrite) atomicOr(&in.job_flags[j], 1u);
            return;
        }
        uint32_t c1 = 0, c2 = 0;
        const uint32_t pos1 = kWrite ? in.job_pts[j] + (in.leaf_pts[lb] - in.leaf_pts[l0]) : 0u;
        bool ok = leaf_cap(in, lb - 1, st, lb - 1 == l0, kWrite ? in.out_points + pos1 : nullptr,
                           kWrite ? in.out_flags + pos1 : nullptr, c1);
        const uint32_t cap1 = kWrite ? in.job_cap1[j] : c1;
        ok = ok && leaf_cap(in, l1 - 1, st, false, kWrite ? in.out_points + base + cap1 : nullptr,
                            kWrite ? in.out_flags + base + cap1 : nullptr, c2);
        if (!kWrite) {
            if (!ok) atomicOr(&in.job_flags[j], 1u);
            in.job_cap1[j] = c1;
            in.job_end[j] = c2;
        }
        return;
    }
    // closed: the join from the last leaf back to the contour's first two points
    V2 jp, a[4], z[4];
    uint32_t jb, meta;
    const uint32_t ka = seg_points(get_leaf(in, l0, jp, jb, meta), a);
    const uint32_t kz = seg_points(get_leaf(in, l1 - 1, jp, jb, meta), z);
    Sink o;
    o.n = 2;
    o.lost = false;
    o.ring[0] = z[kz - 2];
    o.ring[1] = z[kz - 1];
    o.first[0] = a[0];
    o.first[1] = a[1];
    (void)ka;
    o.pts = kWrite ? in.out_points + base - 2 : nullptr;
    o.fl = kWrite ? in.out_flags + base - 2 : nullptr;
    const Contour c = job_contour(in, job);
    close_join(o, c, st);
    if (!kWrite) {
        in.job_cap1[j] = 0;
        in.job_end[j] = o.n - 2;
    }
}

// job_pts[j] for the segment-parallel jobs (the sequential kernel has set the others), and
// the 64-bit total of all jobs beside the 32-bit scan.
__global__ void k_job_totals(StrokeIn in, uint32_t *status) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long n = 0;
    if (j < in.n_jobs) {
        const uint4 job = in.jobs[j];
        if ((job.z & 3u) == kJobCopy || (in.job_flags[j] & 1u)) {
            n = in.job_pts[j];
        } else {
            const uint32_t l0 = in.unit_leaves[in.job_units[j]], l1 = in.unit_leaves[in.job_units[j + 1]];
            const uint32_t c = (in.leaf_pts[l1] - in.leaf_pts[l0]) + in.job_cap1[j] + in.job_end[j];
            in.job_pts[j] = c;
            n = c;
        }
    }
    // one atomic per warp (one hot address for millions of jobs otherwise)
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n)
        atomicAdd(reinterpret_cast<unsigned long long *>(status + kStFill64 + 2), n);
}

// --- Work ordering ---------------------------------------------------------------------------
// A warp's lanes run their items in step, so a warp takes as long as its longest item.  Items
// are bucketed by an estimate of their work, largest first: units by kind and the flatness of
// their control polygon (lines split never; curves split more the more they bend), dashed paths
// by their point count.  A fixed grid counts the buckets per block in shared memory, a single
// block turns the counts into each block's first slot, and the grid places the items.
constexpr int kOrderBuckets = 16;
constexpr int kOrderBlocks = 608;  // 4 per SM of 152

__device__ __forceinline__ int unit_bucket(const StrokeIn &in, uint32_t u) {
    uint4 m;
    const Seg s = get_seg(in.units + 3 * (size_t)u, m);
    if (s.kind == kLine) return 0;
    const V2 p0 = s.b.f, p3 = s.b.t, c0 = s.c.f;
    const V2 c1 = s.kind == kQuad ? s.c.f : s.c.t;
    const float ux = 3.0f * c0.x - 2.0f * p0.x - p3.x, uy = 3.0f * c0.y - 2.0f * p0.y - p3.y;
    const float vx = 3.0f * c1.x - 2.0f * p3.x - p0.x, vy = 3.0f * c1.y - 2.0f * p3.y - p0.y;
    const float f = fmaxf(ux * ux, vx * vx) + fmaxf(uy * uy, vy * vy);
    if (!(f > 1.0f)) return 1;
    const int d = 1 + (int)ceilf(__log2f(f) * 0.25f);
    return d < kOrderBuckets - 1 ? d : kOrderBuckets - 1;
}

__device__ __forceinline__ int dash_bucket(const StrokeIn &in, uint32_t p) {
    if (!stroked(in, p) || path_stroke(in, p).dash_count == 0) return -1;
    const uint2 kr = path_contours(in, p);
    uint32_t pts = 0;
    for (uint32_t k = kr.x; k < kr.y; k++) pts += raw_contour(in, k).n;
    const int d = pts ? 32 - __clz(pts) : 0;
    return d < kOrderBuckets - 1 ? d : kOrderBuckets - 1;
}

// kWhat 0: units, 1: dashed paths.  ctl[kOrderBuckets * block + bucket].
template <int kWhat, bool kScatter>
__global__ void __launch_bounds__(256) k_order(StrokeIn in, uint32_t *ctl, uint32_t *order) {
    __shared__ uint32_t s_cnt[kOrderBuckets];
    const uint32_t n = kWhat == 0 ? in.n_units : in.n_paths;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < kOrderBuckets) s_cnt[threadIdx.x] = kScatter ? ctl[kOrderBuckets * blockIdx.x + threadIdx.x] : 0u;
    __syncthreads();
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const int bk = i < n ? (kWhat == 0 ? unit_bucket(in, i) : dash_bucket(in, i)) : -1;
        const unsigned group = __match_any_sync(0xffffffffu, bk);
        const int leader = __ffs(group) - 1;
        uint32_t slot = 0;
        if (bk >= 0 && lane == leader) slot = atomicAdd(&s_cnt[bk], (uint32_t)__popc(group));
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (kScatter && bk >= 0) order[slot + __popc(group & ((1u << lane) - 1u))] = i;
    }
    __syncthreads();
    if (!kScatter && threadIdx.x < kOrderBuckets) ctl[kOrderBuckets * blockIdx.x + threadIdx.x] = s_cnt[threadIdx.x];
}

// Each block's first slot per bucket, largest bucket first; ctl[kOrderBuckets * kOrderBlocks]
// receives the number of items placed.
__global__ void k_order_starts(uint32_t *ctl) {
    __shared__ uint32_t total[kOrderBuckets];
    const int bk = threadIdx.x;
    if (bk < kOrderBuckets) {
        uint32_t t = 0;
        for (int blk = 0; blk < kOrderBlocks; blk++) t += ctl[kOrderBuckets * blk + bk];
        total[bk] = t;
    }
    __syncthreads();
    if (bk < kOrderBuckets) {
        uint32_t run = 0;
        for (int d = kOrderBuckets - 1; d > bk; d--) run += total[d];
        for (int blk = 0; blk < kOrderBlocks; blk++) {
            const uint32_t c = ctl[kOrderBuckets * blk + bk];
            ctl[kOrderBuckets * blk + bk] = run;
            run += c;
        }
        if (bk == 0) ctl[kOrderBuckets * kOrderBlocks] = run;
    }
}

// The new outline's per-scene offset arrays (the layout the upload uses: scene s's contour
// offsets at cstart_base = its first contour + s, path offsets at pstart_base).
__global__ void k_outline_starts(StrokeIn in, const SceneDev *out_scenes, uint32_t *cstart, uint32_t *pstart) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < in.n_jobs) {
        const uint32_t p = in.jobs[i].w;
        const uint32_t s = upper_bound(in.scene_path_first, in.n_scenes + 1, p) - 1;
        const SceneDev &S = out_scenes[s];
        cstart[S.cstart_base + (i - S.contour_first)] = in.job_pts[i] - S.point_first;
    }
    if (i < in.n_paths) {
        const uint32_t s = upper_bound(in.scene_path_first, in.n_scenes + 1, i) - 1;
        const SceneDev &S = out_scenes[s];
        pstart[S.pstart_base + (i - S.path_first)] = in.job_first[i] - S.contour_first;
    }
    if (i < in.n_scenes) {
        const SceneDev &S = out_scenes[i];
        cstart[S.cstart_base + (S.contour_end - S.contour_first)] = S.point_end - S.point_first;
        pstart[S.pstart_base + (S.path_end - S.path_first)] = S.contour_end - S.contour_first;
    }
}

// Per scene: its first output contour and point (scene boundaries of the scanned arrays).
__global__ void k_scene_bounds(StrokeIn in, uint32_t *out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > in.n_scenes) return;
    const uint32_t p = in.scene_path_first[s];
    const uint32_t k = p < in.n_paths ? in.job_first[p] : in.n_jobs;
    out[2 * s] = k;
    out[2 * s + 1] = k < in.n_jobs ? in.job_pts[k] : in.n_out_points;
}

}  // namespace

static uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

cudaError_t launch_dash(const StrokeIn &in, bool write, uint32_t *status, cudaStream_t st) {
    if (!in.n_dashed) return cudaSuccess;
    if (write) k_dash<true><<<blocks(in.n_dashed, 64), 64, 0, st>>>(in, status);
    else k_dash<false><<<blocks(in.n_dashed, 64), 64, 0, st>>>(in, status);
    count_launches(1);
    return cudaGetLastError();
}

size_t stroke_order_ctl_bytes() { return (size_t(kOrderBuckets) * kOrderBlocks + 1) * 4; }

// what: 0 units (order: [n_units]), 1 dashed paths (order: [n_paths]; the count lands in
// ctl[kOrderBuckets * kOrderBlocks])
cudaError_t launch_stroke_order(const StrokeIn &in, int what, uint32_t *ctl, uint32_t *order, cudaStream_t st) {
    if (what == 0) {
        if (!in.n_units) return cudaSuccess;
        k_order<0, false><<<kOrderBlocks, 256, 0, st>>>(in, ctl, order);
        k_order_starts<<<1, 32, 0, st>>>(ctl);
        k_order<0, true><<<kOrderBlocks, 256, 0, st>>>(in, ctl, order);
    } else {
        if (!in.n_paths) return cudaSuccess;
        k_order<1, false><<<kOrderBlocks, 256, 0, st>>>(in, ctl, order);
        k_order_starts<<<1, 32, 0, st>>>(ctl);
        k_order<1, true><<<kOrderBlocks, 256, 0, st>>>(in, ctl, order);
    }
    count_launches(3);
    return cudaGetLastError();
}

cudaError_t launch_stroke_jobs(const StrokeIn &in, bool fill, cudaStream_t st) {
    if (!in.n_paths) return cudaSuccess;
    if (fill) k_stroke_jobs<true><<<blocks(in.n_paths, 128), 128, 0, st>>>(in);
    else k_stroke_jobs<false><<<blocks(in.n_paths, 128), 128, 0, st>>>(in);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_stroke(const StrokeIn &in, bool write, uint32_t *status, cudaStream_t st) {
    if (!in.n_jobs) return cudaSuccess;
    if (write) k_stroke<true><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in, status);
    else k_stroke<false><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in, status);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_units(const StrokeIn &in, bool write, cudaStream_t st) {
    if (!in.n_jobs) return cudaSuccess;
    if (write) k_units<true><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in);
    else k_units<false><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_unit_leaves(const StrokeIn &in, bool write, cudaStream_t st) {
    if (!in.n_units) return cudaSuccess;
    if (write) k_unit_leaves<true><<<blocks(in.n_units, 128), 128, 0, st>>>(in);
    else k_unit_leaves<false><<<blocks(in.n_units, 128), 128, 0, st>>>(in);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_job_ends(const StrokeIn &in, bool write, cudaStream_t st) {
    if (!in.n_jobs) return cudaSuccess;
    if (write) k_job_ends<true><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in);
    else k_job_ends<false><<<blocks(in.n_jobs, 128), 128, 0, st>>>(in);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_leaf_pts(const StrokeIn &in, bool write, cudaStream_t st) {
    if (!in.n_leaves) return cudaSuccess;
    if (write) k_leaf_pts<true><<<blocks(in.n_leaves, 128), 128, 0, st>>>(in);
    else k_leaf_pts<false><<<blocks(in.n_leaves, 128), 128, 0, st>>>(in);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_job_totals(const StrokeIn &in, uint32_t *status, cudaStream_t st) {
    if (!in.n_jobs) return cudaSuccess;
    k_job_totals<<<blocks(in.n_jobs, 256), 256, 0, st>>>(in, status);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_outline_starts(const StrokeIn &in, const SceneDev *out_scenes, uint32_t *cstart, uint32_t *pstart,
                                  cudaStream_t st) {
    const uint32_t n = max(max(in.n_jobs, in.n_paths), in.n_scenes);
    if (!n) return cudaSuccess;
    k_outline_starts<<<blocks(n, 256), 256, 0, st>>>(in, out_scenes, cstart, pstart);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_scene_bounds(const StrokeIn &in, uint32_t *out, cudaStream_t st) {
    k_scene_bounds<<<blocks(in.n_scenes + 1, 128), 128, 0, st>>>(in, out);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace pfc
