// pf_svg.cu - SVG ingestion (host code): SVG text straight to the C-ABI scene format.
//
// The reference loads SVG with nanosvg (third_party/nanosvg.h: nsvgParse(text, "px", dpi)) and
// replays the result through its canvas (SvgScene::SvgScene, pathfinder/core/svg.cpp:135-205):
// per shape a Path2d of cubic segments, a fill (Canvas::fill_path) and a stroke
// (Canvas::stroke_path: dash, stroke-to-fill).  Here one pass writes the scene arrays directly:
// the fill as a path, the stroke as a path with a pf_stroke (the GPU strokes it at upload).
//
// Two kinds of code are in this file.
//
// * Written for this library: the tag reader (read_tag / parse_document), the element and
//   attribute dispatch tables (kElements, kAttrRules), style declarations (apply_style), units,
//   colours, url() and dash lists, and the scene assembly (SceneOut, convert_paint,
//   emit_contours, pf_svg_parse).  They accept exactly the documents nanosvg accepts and read them
//   the same way (that is what makes the scene equal to the reference's), but they are not
//   nanosvg's code.
// * ALTERED FROM NANOSVG (the notice below applies to these parts): the arithmetic whose
//   operation order fixes the output bits - the number reader (parse_atof, parse_number,
//   next_path_item), the 2x3 transforms and transform lists (xf_*, transform_args,
//   parse_transform), curve bounds (eval_bezier, curve_bounds, local_bounds), path data and
//   shapes (parse_path, arc_to, parse_rect / circle / ellipse / line / poly, Parser::move_to /
//   line_to / cubic_to / add_path), gradients (parse_gradient, parse_stop, create_gradient) and
//   the view-box scaling (scale_to_viewbox).  They are restated in this library's own types and
//   names from nanosvg.h (nsvg__atof, nsvg__parseNumber, nsvg__xform*, nsvg__parseTransform,
//   nsvg__pathArcTo, nsvg__parsePath, nsvg__parseRect..Poly, nsvg__createGradient,
//   nsvg__scaleToViewbox), and altered: zeros where nanosvg reads memory it never wrote (a
//   transform item without its arguments, the inverse of a singular transform), no parser-state
//   allocation, C++ containers for its linked lists.
//
// Float arithmetic follows nanosvg operation by operation (this file is compiled without FMA
// contraction), so the scene's points are the reference's bit for bit.
//
// nanosvg's notice, which travels with the altered parts:
//
//   Copyright (c) 2013-14 Mikko Mononen memon@inside.org
//
//   This software is provided 'as-is', without any express or implied
//   warranty.  In no event will the authors be held liable for any damages
//   arising from the use of this software.
//
//   Permission is granted to anyone to use this software for any purpose,
//   including commercial applications, and to alter it and redistribute it
//   freely, subject to the following restrictions:
//
//   1. The origin of this software must not be misrepresented; you must not
//   claim that you wrote the original software. If you use this software
//   in a product, an acknowledgment in the product documentation would be
//   appreciated but is not required.
//   2. Altered source versions must be plainly marked as such, and must not be
//   misrepresented as being the original software.
//   3. This notice may not be removed or altered from any source distribution.
//
//   The SVG parser is based on Anti-Grain Geometry 2.4 SVG example
//   Copyright (C) 2002-2004 Maxim Shemanarev (McSeem) (http://www.antigrain.com/)
//
//   Arc calculation code based on canvg (https://code.google.com/p/canvg/)
//
//   Bounding box calculation based on http://blog.hackers-cafe.net/2009/06/how-to-calculate-bezier-curves-bounding.html
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pfcuda.h"

namespace {

constexpr float kPi = 3.14159265358979323846264338327f;  // NSVG_PI
constexpr float kKappa90 = 0.5522847493f;                // NSVG_KAPPA90
constexpr int kMaxAttr = 128;
constexpr int kMaxDashes = 8;

enum Units { kUser, kPx, kPt, kPc, kMm, kCm, kIn, kPercent, kEm, kEx };
enum Paint { kNone = 0, kColor = 1, kLinear = 2, kRadial = 3 };
enum Align { kAlignMin, kAlignMid, kAlignMax, kAlignNone = 0, kAlignMeet = 1, kAlignSlice = 2 };

inline bool is_space(char c) { return std::strchr(" \t\n\v\f\r", c) != nullptr; }  // '\0' counts
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
inline float minf(float a, float b) { return a < b ? a : b; }
inline float maxf(float a, float b) { return a > b ? a : b; }
inline uint32_t rgb(uint32_t r, uint32_t g, uint32_t b) { return r | g << 8 | b << 16; }

struct Coord {
    float value;
    int units;
};

// --- numbers ---------------------------------------------------------------------------------
double parse_atof(const char *s) {
    const char *cur = s;
    char *end = nullptr;
    double res = 0.0, sign = 1.0;
    bool has_int = false, has_frac = false;
    if (*cur == '+') cur++;
    else if (*cur == '-') {
        sign = -1;
        cur++;
    }
    if (is_digit(*cur)) {
        const long long ip = std::strtoll(cur, &end, 10);
        if (cur != end) {
            res = (double)ip;
            has_int = true;
            cur = end;
        }
    }
    if (*cur == '.') {
        cur++;
        if (is_digit(*cur)) {
            const long long fp = std::strtoll(cur, &end, 10);
            if (cur != end) {
                res += (double)fp / std::pow(10.0, (double)(end - cur));
                has_frac = true;
                cur = end;
            }
        }
    }
    if (!has_int && !has_frac) return 0.0;
    if (*cur == 'e' || *cur == 'E') {
        cur++;
        const long ep = std::strtol(cur, &end, 10);
        if (cur != end) res *= std::pow(10.0, (double)ep);
    }
    return res * sign;
}

const char *parse_number(const char *s, char *it, int size) {
    const int last = size - 1;
    int i = 0;
    if (*s == '-' || *s == '+') {
        if (i < last) it[i++] = *s;
        s++;
    }
    while (*s && is_digit(*s)) {
        if (i < last) it[i++] = *s;
        s++;
    }
    if (*s == '.') {
        if (i < last) it[i++] = *s;
        s++;
        while (*s && is_digit(*s)) {
            if (i < last) it[i++] = *s;
            s++;
        }
    }
    if ((*s == 'e' || *s == 'E') && (s[1] != 'm' && s[1] != 'x')) {
        if (i < last) it[i++] = *s;
        s++;
        if (*s == '-' || *s == '+') {
            if (i < last) it[i++] = *s;
            s++;
        }
        while (*s && is_digit(*s)) {
            if (i < last) it[i++] = *s;
            s++;
        }
    }
    it[i] = '\0';
    return s;
}

const char *next_path_item(const char *s, char *it) {
    it[0] = '\0';
    while (*s && (is_space(*s) || *s == ',')) s++;
    if (!*s) return s;
    if (*s == '-' || *s == '+' || *s == '.' || is_digit(*s)) {
        s = parse_number(s, it, 64);
    } else {
        it[0] = *s++;
        it[1] = '\0';
    }
    return s;
}

// --- transforms (a, b, c, d, e, f: x' = a x + c y + e) -----------------------------------------
void xf_identity(float *t) {
    t[0] = 1.0f, t[1] = 0.0f, t[2] = 0.0f, t[3] = 1.0f, t[4] = 0.0f, t[5] = 0.0f;
}
void xf_translation(float *t, float tx, float ty) {
    t[0] = 1.0f, t[1] = 0.0f, t[2] = 0.0f, t[3] = 1.0f, t[4] = tx, t[5] = ty;
}
void xf_scale(float *t, float sx, float sy) {
    t[0] = sx, t[1] = 0.0f, t[2] = 0.0f, t[3] = sy, t[4] = 0.0f, t[5] = 0.0f;
}
void xf_multiply(float *t, const float *s) {  // t = t * s
    const float t0 = t[0] * s[0] + t[1] * s[2];
    const float t2 = t[2] * s[0] + t[3] * s[2];
    const float t4 = t[4] * s[0] + t[5] * s[2] + s[4];
    t[1] = t[0] * s[1] + t[1] * s[3];
    t[3] = t[2] * s[1] + t[3] * s[3];
    t[5] = t[4] * s[1] + t[5] * s[3] + s[5];
    t[0] = t0;
    t[2] = t2;
    t[4] = t4;
}
void xf_premultiply(float *t, const float *s) {  // t = s * t
    float s2[6];
    std::memcpy(s2, s, sizeof s2);
    xf_multiply(s2, t);
    std::memcpy(t, s2, sizeof s2);
}
void xf_point(float *dx, float *dy, float x, float y, const float *t) {
    *dx = x * t[0] + y * t[2] + t[4];
    *dy = x * t[1] + y * t[3] + t[5];
}
void xf_vec(float *dx, float *dy, float x, float y, const float *t) {
    *dx = x * t[0] + y * t[2];
    *dy = x * t[1] + y * t[3];
}
void xf_inverse(float *inv, float *t) {
    const double det = (double)t[0] * t[3] - (double)t[2] * t[1];
    if (det > -1e-6 && det < 1e-6) {
        xf_identity(t);
        return;
    }
    const double invdet = 1.0 / det;
    inv[0] = (float)(t[3] * invdet);
    inv[2] = (float)(-t[2] * invdet);
    inv[4] = (float)(((double)t[2] * t[5] - (double)t[3] * t[4]) * invdet);
    inv[1] = (float)(-t[1] * invdet);
    inv[3] = (float)(t[0] * invdet);
    inv[5] = (float)(((double)t[1] * t[4] - (double)t[0] * t[5]) * invdet);
}

// --- curve bounds (the image's bounds when the document gives no size) --------------------------
double eval_bezier(double t, double p0, double p1, double p2, double p3) {
    const double it = 1.0 - t;
    return it * it * it * p0 + 3.0 * it * it * t * p1 + 3.0 * it * t * t * p2 + t * t * t * p3;
}
bool pt_in_bounds(const float *pt, const float *b) {
    return pt[0] >= b[0] && pt[0] <= b[2] && pt[1] >= b[1] && pt[1] <= b[3];
}
void curve_bounds(float *bounds, const float *curve) {
    const float *v0 = &curve[0], *v1 = &curve[2], *v2 = &curve[4], *v3 = &curve[6];
    bounds[0] = minf(v0[0], v3[0]);
    bounds[1] = minf(v0[1], v3[1]);
    bounds[2] = maxf(v0[0], v3[0]);
    bounds[3] = maxf(v0[1], v3[1]);
    if (pt_in_bounds(v1, bounds) && pt_in_bounds(v2, bounds)) return;
    const double eps = 1e-12;
    for (int i = 0; i < 2; i++) {
        const double a = -3.0 * v0[i] + 9.0 * v1[i] - 9.0 * v2[i] + 3.0 * v3[i];
        const double b = 6.0 * v0[i] - 12.0 * v1[i] + 6.0 * v2[i];
        const double c = 3.0 * v1[i] - 3.0 * v0[i];
        double roots[2];
        int count = 0;
        if (std::fabs(a) < eps) {
            if (std::fabs(b) > eps) {
                const double t = -c / b;
                if (t > eps && t < 1.0 - eps) roots[count++] = t;
            }
        } else {
            const double b2ac = b * b - 4.0 * c * a;
            if (b2ac > eps) {
                double t = (-b + std::sqrt(b2ac)) / (2.0 * a);
                if (t > eps && t < 1.0 - eps) roots[count++] = t;
                t = (-b - std::sqrt(b2ac)) / (2.0 * a);
                if (t > eps && t < 1.0 - eps) roots[count++] = t;
            }
        }
        for (int j = 0; j < count; j++) {
            const double v = eval_bezier(roots[j], v0[i], v1[i], v2[i], v3[i]);
            bounds[0 + i] = minf(bounds[0 + i], (float)v);
            bounds[2 + i] = maxf(bounds[2 + i], (float)v);
        }
    }
}

// --- document model ------------------------------------------------------------------------------
struct GradStop {
    uint32_t color;
    float offset;
};

struct GradData {
    std::string id, ref;
    int type = kLinear;
    // nanosvg keeps the linear and radial coordinates in one union, so x1/cx, y1/cy, x2/r and
    // y2/fx share a slot (an attribute of the other kind lands in it); fy has its own
    Coord u[5] = {{0.0f, kUser}, {0.0f, kUser}, {0.0f, kUser}, {0.0f, kUser}, {0.0f, kUser}};
    int spread = 0;  // pad, reflect, repeat
    bool object_space = true;
    float xform[6];
    std::vector<GradStop> stops;
};

struct Grad {  // a gradient paint as SvgScene reads it
    int type;
    float x1, y1, x2, y2, cx, cy, fx, fy, r;
    float xform2[6], xform3[6];  // the gradient's transform, the shape's transform
    int spread;
    std::vector<GradStop> stops;
};

struct PaintDesc {
    int type = kNone;
    uint32_t color = 0;
    Grad grad{};
};

struct SubPath {
    std::vector<float> pts;
    bool closed = false;
    float bounds[4];
};

struct Shape {
    PaintDesc fill, stroke;
    float stroke_width, dash_offset, dashes[kMaxDashes];
    int dash_count;
    char join, cap, fill_rule;
    float miter;
    float bounds[4];
    std::vector<SubPath> paths;  // most recent first, as nanosvg lists them
};

struct Attr {
    char id[64];
    float xform[6];
    uint32_t fill_color, stroke_color;
    float opacity, fill_opacity, stroke_opacity;
    char fill_grad[64], stroke_grad[64];
    float stroke_width, dash_offset, dashes[kMaxDashes];
    int dash_count;
    char join, cap;
    float miter;
    char fill_rule;
    float font_size;
    uint32_t stop_color;
    float stop_opacity, stop_offset;
    char has_fill, has_stroke, visible;
};

struct Parser {
    Attr attr[kMaxAttr];
    int head = 0;
    std::vector<float> pts;
    std::vector<SubPath> plist;  // paths of the shape being built, most recent first
    std::vector<Shape> shapes;
    std::vector<GradData> grads;  // most recent first
    float width = 0, height = 0;
    float view_minx = 0, view_miny = 0, view_width = 0, view_height = 0;
    int align_x = kAlignMin, align_y = kAlignMin, align_type = kAlignNone;
    float dpi = 96.0f;
    bool defs_flag = false;

    Parser() {
        std::memset(attr, 0, sizeof attr);
        Attr &a = attr[0];
        xf_identity(a.xform);
        a.fill_color = rgb(0, 0, 0);
        a.stroke_color = rgb(0, 0, 0);
        a.opacity = a.fill_opacity = a.stroke_opacity = a.stop_opacity = 1;
        a.stroke_width = 1;
        a.join = 0;  // miter
        a.cap = 0;   // butt
        a.miter = 4;
        a.fill_rule = 0;  // nonzero
        a.has_fill = 1;
        a.visible = 1;
    }
    Attr &cur() { return attr[head]; }
    void push() {
        if (head < kMaxAttr - 1) {
            head++;
            std::memcpy(&attr[head], &attr[head - 1], sizeof(Attr));
        }
    }
    void pop() {
        if (head > 0) head--;
    }
    float actual_length() const {
        const float w = view_width, h = view_height;
        return std::sqrt(w * w + h * h) / std::sqrt(2.0f);
    }
    float to_pixels(Coord c, float orig, float length) {
        const Attr &a = cur();
        switch (c.units) {
            case kUser: return c.value;
            case kPx: return c.value;
            case kPt: return c.value / 72.0f * dpi;
            case kPc: return c.value / 6.0f * dpi;
            case kMm: return c.value / 25.4f * dpi;
            case kCm: return c.value / 2.54f * dpi;
            case kIn: return c.value * dpi;
            case kEm: return c.value * a.font_size;
            case kEx: return c.value * a.font_size * 0.52f;
            case kPercent: return orig + c.value / 100.0f * length;
            default: return c.value;
        }
    }
    // path building (points: 1 + 3n, lines as cubics at thirds)
    void add_point(float x, float y) {
        pts.push_back(x);
        pts.push_back(y);
    }
    size_t npts() const { return pts.size() / 2; }
    void move_to(float x, float y) {
        if (npts() > 0) {
            pts[pts.size() - 2] = x;
            pts[pts.size() - 1] = y;
        } else {
            add_point(x, y);
        }
    }
    void line_to(float x, float y) {
        if (npts() > 0) {
            const float px = pts[pts.size() - 2], py = pts[pts.size() - 1];
            const float dx = x - px, dy = y - py;
            add_point(px + dx / 3.0f, py + dy / 3.0f);
            add_point(x - dx / 3.0f, y - dy / 3.0f);
            add_point(x, y);
        }
    }
    void cubic_to(float c1x, float c1y, float c2x, float c2y, float x, float y) {
        if (npts() > 0) {
            add_point(c1x, c1y);
            add_point(c2x, c2y);
            add_point(x, y);
        }
    }
    void add_path(bool closed);
    void add_shape();
};

void Parser::add_path(bool closed) {
    if (npts() < 4) return;
    if (closed) line_to(pts[0], pts[1]);
    if ((npts() % 3) != 1) return;
    SubPath sp;
    sp.closed = closed;
    sp.pts.resize(pts.size());
    const Attr &a = cur();
    for (size_t i = 0; i < npts(); i++) xf_point(&sp.pts[2 * i], &sp.pts[2 * i + 1], pts[2 * i], pts[2 * i + 1], a.xform);
    for (size_t i = 0; i + 1 < npts(); i += 3) {
        float b[4];
        curve_bounds(b, &sp.pts[2 * i]);
        if (i == 0) {
            std::memcpy(sp.bounds, b, sizeof b);
        } else {
            sp.bounds[0] = minf(sp.bounds[0], b[0]);
            sp.bounds[1] = minf(sp.bounds[1], b[1]);
            sp.bounds[2] = maxf(sp.bounds[2], b[2]);
            sp.bounds[3] = maxf(sp.bounds[3], b[3]);
        }
    }
    plist.insert(plist.begin(), std::move(sp));
}

float average_scale(const float *t) {
    const float sx = std::sqrt(t[0] * t[0] + t[2] * t[2]);
    const float sy = std::sqrt(t[1] * t[1] + t[3] * t[3]);
    return (sx + sy) * 0.5f;
}

void local_bounds(float *bounds, const Shape &shape, const float *xform) {
    bool first = true;
    for (const SubPath &path : shape.paths) {
        float curve[8];
        xf_point(&curve[0], &curve[1], path.pts[0], path.pts[1], xform);
        const size_t n = path.pts.size() / 2;
        for (size_t i = 0; i + 1 < n; i += 3) {
            xf_point(&curve[2], &curve[3], path.pts[(i + 1) * 2], path.pts[(i + 1) * 2 + 1], xform);
            xf_point(&curve[4], &curve[5], path.pts[(i + 2) * 2], path.pts[(i + 2) * 2 + 1], xform);
            xf_point(&curve[6], &curve[7], path.pts[(i + 3) * 2], path.pts[(i + 3) * 2 + 1], xform);
            float cb[4];
            curve_bounds(cb, curve);
            if (first) {
                std::memcpy(bounds, cb, sizeof cb);
                first = false;
            } else {
                bounds[0] = minf(bounds[0], cb[0]);
                bounds[1] = minf(bounds[1], cb[1]);
                bounds[2] = maxf(bounds[2], cb[2]);
                bounds[3] = maxf(bounds[3], cb[3]);
            }
            curve[0] = curve[6];
            curve[1] = curve[7];
        }
    }
}

const GradData *find_grad(const Parser &p, const std::string &id) {
    if (id.empty()) return nullptr;
    for (const GradData &g : p.grads)
        if (g.id == id) return &g;
    return nullptr;
}

// nsvg__createGradient: false when the id is unknown or no gradient in its chain has stops
bool create_gradient(Parser &p, const char *id, const float *lb, PaintDesc &out) {
    const GradData *data = find_grad(p, id);
    if (!data) return false;
    const std::vector<GradStop> *stops = nullptr;
    const GradData *ref = data;
    int iter = 0;
    while (ref) {
        if (!ref->stops.empty()) {
            stops = &ref->stops;
            break;
        }
        const GradData *next = find_grad(p, ref->ref);
        if (next == ref) break;
        ref = next;
        if (++iter > 32) break;
    }
    if (!stops) return false;
    float ox, oy, sw, sh;
    if (data->object_space) {
        ox = lb[0];
        oy = lb[1];
        sw = lb[2] - lb[0];
        sh = lb[3] - lb[1];
    } else {
        ox = p.view_minx;
        oy = p.view_miny;
        sw = p.view_width;
        sh = p.view_height;
    }
    const float sl = std::sqrt(sw * sw + sh * sh) / std::sqrt(2.0f);
    Grad g{};
    g.type = data->type;
    if (data->type == kLinear) {
        g.x1 = p.to_pixels(data->u[0], ox, sw);
        g.y1 = p.to_pixels(data->u[1], oy, sh);
        g.x2 = p.to_pixels(data->u[2], ox, sw);
        g.y2 = p.to_pixels(data->u[3], oy, sh);
    } else {
        g.cx = p.to_pixels(data->u[0], ox, sw);
        g.cy = p.to_pixels(data->u[1], oy, sh);
        g.fx = p.to_pixels(data->u[3], ox, sw);
        g.fy = p.to_pixels(data->u[4], oy, sh);
        g.r = p.to_pixels(data->u[2], 0, sl);
    }
    std::memcpy(g.xform2, data->xform, sizeof g.xform2);
    std::memcpy(g.xform3, p.cur().xform, sizeof g.xform3);
    g.spread = data->spread;
    g.stops = *stops;
    out.type = data->type;
    out.grad = std::move(g);
    return true;
}

void Parser::add_shape() {
    if (plist.empty()) return;
    const Attr &a = cur();
    Shape s;
    const float scale = average_scale(a.xform);
    s.stroke_width = a.stroke_width * scale;
    s.dash_offset = a.dash_offset * scale;
    s.dash_count = a.dash_count;
    for (int i = 0; i < a.dash_count; i++) s.dashes[i] = a.dashes[i] * scale;
    s.join = a.join;
    s.cap = a.cap;
    s.miter = a.miter;
    s.fill_rule = a.fill_rule;
    s.paths = std::move(plist);
    plist.clear();
    std::memcpy(s.bounds, s.paths[0].bounds, sizeof s.bounds);
    for (size_t i = 1; i < s.paths.size(); i++) {
        s.bounds[0] = minf(s.bounds[0], s.paths[i].bounds[0]);
        s.bounds[1] = minf(s.bounds[1], s.paths[i].bounds[1]);
        s.bounds[2] = maxf(s.bounds[2], s.paths[i].bounds[2]);
        s.bounds[3] = maxf(s.bounds[3], s.paths[i].bounds[3]);
    }
    auto paint = [&](char has, uint32_t color, float opacity, const char *grad, PaintDesc &out) {
        if (has == 0) {
            out.type = kNone;
        } else if (has == 1) {
            out.type = kColor;
            out.color = color | (uint32_t)(opacity * 255) << 24;
        } else if (has == 2) {
            // a singular transform leaves nanosvg's inverse unwritten (it resets the transform
            // instead); here that inverse is zero, so the shape's local bounds are zero
            float inv[6] = {0, 0, 0, 0, 0, 0}, lb[4] = {0, 0, 0, 0};
            float xf[6];
            std::memcpy(xf, a.xform, sizeof xf);
            xf_inverse(inv, xf);
            local_bounds(lb, s, inv);
            if (!create_gradient(*this, grad, lb, out)) out.type = kNone;
        }
    };
    paint(a.has_fill, a.fill_color, a.fill_opacity, a.fill_grad, s.fill);
    paint(a.has_stroke, a.stroke_color, a.stroke_opacity, a.stroke_grad, s.stroke);
    shapes.push_back(std::move(s));
}

// --- attributes ----------------------------------------------------------------------------------
// A length's unit is named by the first characters after its number: the two-letter CSS units and
// '%' (anything else is a user unit).
int parse_units(const char *u) {
    static const struct {
        char c0, c1;
        int unit;
    } kUnits[] = {{'p', 'x', kPx}, {'p', 't', kPt}, {'p', 'c', kPc}, {'m', 'm', kMm}, {'c', 'm', kCm},
                  {'i', 'n', kIn}, {'e', 'm', kEm}, {'e', 'x', kEx}};
    if (u[0] == '%') return kPercent;
    if (u[0] == '\0') return kUser;
    for (const auto &k : kUnits)
        if (u[0] == k.c0 && u[1] == k.c1) return k.unit;
    return kUser;
}
Coord parse_coord_raw(const char *s) {
    char buf[64];
    Coord c{0, kUser};
    c.units = parse_units(parse_number(s, buf, 64));
    c.value = (float)parse_atof(buf);
    return c;
}
float parse_coord(Parser &p, const char *s, float orig, float length) {
    return p.to_pixels(parse_coord_raw(s), orig, length);
}
bool is_coordinate(const char *s) {
    if (*s == '-' || *s == '+') s++;
    return is_digit(*s) || *s == '.';
}

// Colours: "#rrggbb" / "#rgb" (read with the C library's %x conversions, white space and all),
// "rgb(r, g, b)" with integers (%u) or with percentages, and the colour keywords the reference's
// build of nanosvg knows (its short table: other names, and anything malformed, read as gray).
constexpr uint32_t kGray = 128u | 128u << 8 | 128u << 16;

uint32_t hex_color(const char *s) {
    unsigned c[3] = {0, 0, 0};
    if (std::sscanf(s, "#%2x%2x%2x", &c[0], &c[1], &c[2]) == 3) return rgb(c[0], c[1], c[2]);
    if (std::sscanf(s, "#%1x%1x%1x", &c[0], &c[1], &c[2]) == 3) return rgb(17 * c[0], 17 * c[1], 17 * c[2]);
    return kGray;
}

// One "<number>%" component of rgb(...), then white space and the expected delimiter; false when
// the text does not have that form.
bool percent_component(const char *&s, char delim, float &out) {
    while (*s && is_space(*s)) s++;
    if (*s == '+') s++;
    if (!*s) return false;
    out = (float)parse_atof(s);
    while (is_digit(*s)) s++;
    if (*s == '.') {
        if (!is_digit(*++s)) return false;
        while (is_digit(*s)) s++;
    }
    if (*s++ != '%') return false;
    while (*s && is_space(*s)) s++;  // (nanosvg's loop here also steps over the string's end)
    return *s++ == delim;
}

uint32_t function_color(const char *s) {
    unsigned v[3];
    if (std::sscanf(s, "rgb(%u, %u, %u)", &v[0], &v[1], &v[2]) != 3) {
        const char *q = s + 4;
        float f[3];
        if (!percent_component(q, ',', f[0]) || !percent_component(q, ',', f[1]) || !percent_component(q, ')', f[2]))
            return kGray;
        for (int k = 0; k < 3; k++) v[k] = (unsigned)std::round(f[k] * 2.55f);
    }
    return rgb(v[0] > 255 ? 255 : v[0], v[1] > 255 ? 255 : v[1], v[2] > 255 ? 255 : v[2]);
}

uint32_t keyword_color(const char *s) {
    static const std::pair<const char *, uint32_t> kWords[] = {  // sorted by name
        {"black", 0x000000u}, {"blue", 0xff0000u},    {"cyan", 0xffff00u},  {"gray", 0x808080u},
        {"green", 0x008000u}, {"grey", 0x808080u},    {"magenta", 0xff00ffu}, {"red", 0x0000ffu},
        {"white", 0xffffffu}, {"yellow", 0x00ffffu}};
    const auto *end = kWords + sizeof kWords / sizeof kWords[0];
    const auto *it = std::lower_bound(kWords, end, s, [](const std::pair<const char *, uint32_t> &w, const char *k) {
        return std::strcmp(w.first, k) < 0;
    });
    return it != end && std::strcmp(it->first, s) == 0 ? it->second : kGray;
}

uint32_t parse_color(const char *s) {
    while (*s == ' ') ++s;
    if (*s == '#') return hex_color(s);
    if (std::strncmp(s, "rgb(", 4) == 0) return function_color(s);
    return keyword_color(s);
}
float parse_opacity(const char *s) {
    float v = (float)parse_atof(s);
    if (v < 0.0f) v = 0.0f;
    if (v > 1.0f) v = 1.0f;
    return v;
}

int transform_args(const char *str, float *args, int max_na, int *na) {
    char it[64];
    *na = 0;
    const char *ptr = str;
    while (*ptr && *ptr != '(') ++ptr;
    if (*ptr == 0) return 1;
    const char *end = ptr;
    while (*end && *end != ')') ++end;
    if (*end == 0) return 1;
    while (ptr < end) {
        if (*ptr == '-' || *ptr == '+' || *ptr == '.' || is_digit(*ptr)) {
            if (*na >= max_na) return 0;
            ptr = parse_number(ptr, it, 64);
            args[(*na)++] = (float)parse_atof(it);
        } else {
            ++ptr;
        }
    }
    return (int)(end - str);
}

void parse_transform(float *xform, const char *str) {
    xf_identity(xform);
    // t carries over between items: a matrix() without six numbers applies the previous item
    // again (identity before the first), as nanosvg's reused array does
    float t[6];
    xf_identity(t);
    while (*str) {
        float args[6] = {0, 0, 0, 0, 0, 0};
        int na = 0, len;
        if (std::strncmp(str, "matrix", 6) == 0) {
            len = transform_args(str, args, 6, &na);
            if (na == 6) std::memcpy(t, args, sizeof t);
        } else if (std::strncmp(str, "translate", 9) == 0) {
            len = transform_args(str, args, 2, &na);
            if (na == 1) args[1] = 0.0f;
            xf_translation(t, args[0], args[1]);
        } else if (std::strncmp(str, "scale", 5) == 0) {
            len = transform_args(str, args, 2, &na);
            if (na == 1) args[1] = args[0];
            xf_scale(t, args[0], args[1]);
        } else if (std::strncmp(str, "rotate", 6) == 0) {
            len = transform_args(str, args, 3, &na);
            if (na == 1) args[1] = args[2] = 0.0f;
            float m[6], s[6];
            xf_identity(m);
            if (na > 1) {
                xf_translation(s, -args[1], -args[2]);
                xf_multiply(m, s);
            }
            const float a = args[0] / 180.0f * kPi;
            const float cs = std::cos(a), sn = std::sin(a);
            s[0] = cs, s[1] = sn, s[2] = -sn, s[3] = cs, s[4] = 0.0f, s[5] = 0.0f;
            xf_multiply(m, s);
            if (na > 1) {
                xf_translation(s, args[1], args[2]);
                xf_multiply(m, s);
            }
            std::memcpy(t, m, sizeof t);
        } else if (std::strncmp(str, "skewX", 5) == 0) {
            len = transform_args(str, args, 1, &na);
            xf_identity(t);
            t[2] = std::tan(args[0] / 180.0f * kPi);
        } else if (std::strncmp(str, "skewY", 5) == 0) {
            len = transform_args(str, args, 1, &na);
            xf_identity(t);
            t[1] = std::tan(args[0] / 180.0f * kPi);
        } else {
            ++str;
            continue;
        }
        if (len != 0) {
            str += len;
        } else {
            ++str;
            continue;
        }
        xf_premultiply(xform, t);
    }
}

// "url(#name)" (the '#' optional): the name, up to 63 characters or the ')'.
void url_target(char *id, const char *value) {
    const char *q = value + 4;
    if (*q == '#') q++;
    size_t n = 0;
    while (n < 63 && q[n] && q[n] != ')') n++;
    std::memcpy(id, q, n);
    id[n] = '\0';
}

// stroke-dasharray: "none" (anything starting with 'n'), or lengths split by white space and
// commas, at most kMaxDashes kept (absolute values); a pattern whose sum is not above 1e-6 is
// no pattern.  Each length is read from at most 63 of its characters.
int dash_pattern(Parser &p, const char *str, float *dashes) {
    if (str[0] == 'n') return 0;
    int count = 0;
    const char *q = str;
    for (;;) {
        while (*q && (is_space(*q) || *q == ',')) q++;
        const char *b = q;
        while (*q && !is_space(*q) && *q != ',') q++;
        if (q == b) break;
        char item[64];
        const size_t n = std::min<size_t>(size_t(q - b), 63);
        std::memcpy(item, b, n);
        item[n] = '\0';
        if (count < kMaxDashes) dashes[count++] = std::fabs(parse_coord(p, item, 0.0f, p.actual_length()));
    }
    float sum = 0.0f;
    for (int i = 0; i < count; i++) sum += dashes[i];
    return sum <= 1e-6f ? 0 : count;
}

// Presentation attributes and style properties (the ones the reference's nanosvg build reads),
// applied to the current attribute state: one handler per name, found by binary search.
void apply_style(Parser &p, const char *text);

// "none", "url(#id)" (a gradient, kind 2) or a colour (kind 1)
void paint_attr(const char *v, char &kind, uint32_t &color, char *grad) {
    if (std::strcmp(v, "none") == 0) {
        kind = 0;
    } else if (std::strncmp(v, "url(", 4) == 0) {
        kind = 2;
        url_target(grad, v);
    } else {
        kind = 1;
        color = parse_color(v);
    }
}

using AttrFn = void (*)(Parser &, Attr &, const char *);
struct AttrRule {
    const char *name;
    AttrFn apply;
};

const AttrRule kAttrRules[] = {  // sorted by name (strcmp)
    {"display", [](Parser &, Attr &a, const char *v) { if (std::strcmp(v, "none") == 0) a.visible = 0; }},
    {"fill", [](Parser &, Attr &a, const char *v) { paint_attr(v, a.has_fill, a.fill_color, a.fill_grad); }},
    {"fill-opacity", [](Parser &, Attr &a, const char *v) { a.fill_opacity = parse_opacity(v); }},
    {"fill-rule", [](Parser &, Attr &a, const char *v) { a.fill_rule = std::strcmp(v, "evenodd") == 0; }},
    {"font-size", [](Parser &p, Attr &a, const char *v) { a.font_size = parse_coord(p, v, 0.0f, p.actual_length()); }},
    {"id", [](Parser &, Attr &a, const char *v) {
         std::strncpy(a.id, v, 63);
         a.id[63] = '\0';
     }},
    {"offset", [](Parser &p, Attr &a, const char *v) { a.stop_offset = parse_coord(p, v, 0.0f, 1.0f); }},
    {"opacity", [](Parser &, Attr &a, const char *v) { a.opacity = parse_opacity(v); }},
    {"stop-color", [](Parser &, Attr &a, const char *v) { a.stop_color = parse_color(v); }},
    {"stop-opacity", [](Parser &, Attr &a, const char *v) { a.stop_opacity = parse_opacity(v); }},
    {"stroke", [](Parser &, Attr &a, const char *v) { paint_attr(v, a.has_stroke, a.stroke_color, a.stroke_grad); }},
    {"stroke-dasharray", [](Parser &p, Attr &a, const char *v) { a.dash_count = dash_pattern(p, v, a.dashes); }},
    {"stroke-dashoffset",
     [](Parser &p, Attr &a, const char *v) { a.dash_offset = parse_coord(p, v, 0.0f, p.actual_length()); }},
    {"stroke-linecap", [](Parser &, Attr &a, const char *v) {
         a.cap = std::strcmp(v, "round") == 0 ? 1 : std::strcmp(v, "square") == 0 ? 2 : 0;
     }},
    {"stroke-linejoin", [](Parser &, Attr &a, const char *v) {
         a.join = std::strcmp(v, "round") == 0 ? 1 : std::strcmp(v, "bevel") == 0 ? 2 : 0;
     }},
    {"stroke-miterlimit", [](Parser &, Attr &a, const char *v) {
         const float m = (float)parse_atof(v);
         a.miter = m < 0.0f ? 0.0f : m;
     }},
    {"stroke-opacity", [](Parser &, Attr &a, const char *v) { a.stroke_opacity = parse_opacity(v); }},
    {"stroke-width",
     [](Parser &p, Attr &a, const char *v) { a.stroke_width = parse_coord(p, v, 0.0f, p.actual_length()); }},
    {"style", [](Parser &p, Attr &, const char *v) { apply_style(p, v); }},
    {"transform", [](Parser &, Attr &a, const char *v) {
         float xf[6];
         parse_transform(xf, v);
         xf_premultiply(a.xform, xf);
     }},
};

// Applies a known attribute to the current state; false for a name no rule has.
bool parse_attr(Parser &p, const char *name, const char *value) {
    const AttrRule *end = kAttrRules + sizeof kAttrRules / sizeof kAttrRules[0];
    const AttrRule *r = std::lower_bound(kAttrRules, end, name,
                                         [](const AttrRule &a, const char *n) { return std::strcmp(a.name, n) < 0; });
    if (r == end || std::strcmp(r->name, name) != 0) return false;
    r->apply(p, p.cur(), value);
    return true;
}

// A style attribute: declarations split at ';'; in each, the name is what precedes the first
// ':' and the value what follows it, each trimmed of white space (and of the ':' and ';'
// separators next to it), at most 511 characters each.  Empty declarations are skipped.  A
// declaration without ':' is its own name with an empty value, unless a ';' follows it at once:
// nanosvg then reads the ';' into the name, which names no attribute.
void apply_style(Parser &p, const char *text) {
    const char *q = text;
    while (*q) {
        while (*q && is_space(*q)) q++;
        const char *b = q;
        while (*q && *q != ';') q++;
        const char *e = q;
        if (*q) q++;
        while (e > b && (is_space(e[-1]) || e[-1] == ';')) e--;
        if (e == b) continue;
        const char *colon = b;
        while (colon < e && *colon != ':') colon++;
        if (colon == e && *e == ';') continue;
        const char *ne = colon;
        while (ne > b && (is_space(ne[-1]) || ne[-1] == ':')) ne--;
        const char *vb = colon;
        while (vb < e && (is_space(*vb) || *vb == ':')) vb++;
        char name[512], value[512];
        const size_t nn = std::min<size_t>(size_t(ne - b), 511), nv = std::min<size_t>(size_t(e - vb), 511);
        std::memcpy(name, b, nn);
        name[nn] = '\0';
        std::memcpy(value, vb, nv);
        value[nv] = '\0';
        parse_attr(p, name, value);
    }
}

void parse_attribs(Parser &p, const char **attr) {
    for (int i = 0; attr[i]; i += 2) parse_attr(p, attr[i], attr[i + 1]);
}

// --- path data -----------------------------------------------------------------------------------
int args_per(char cmd) {
    switch (cmd) {
        case 'v': case 'V': case 'h': case 'H': return 1;
        case 'm': case 'M': case 'l': case 'L': case 't': case 'T': return 2;
        case 'q': case 'Q': case 's': case 'S': return 4;
        case 'c': case 'C': return 6;
        case 'a': case 'A': return 7;
        case 'z': case 'Z': return 0;
    }
    return -1;
}

inline float sqr(float x) { return x * x; }
inline float vmag(float x, float y) { return std::sqrt(x * x + y * y); }
float vecrat(float ux, float uy, float vx, float vy) { return (ux * vx + uy * vy) / (vmag(ux, uy) * vmag(vx, vy)); }
float vecang(float ux, float uy, float vx, float vy) {
    float r = vecrat(ux, uy, vx, vy);
    if (r < -1.0f) r = -1.0f;
    if (r > 1.0f) r = 1.0f;
    return ((ux * vy < uy * vx) ? -1.0f : 1.0f) * std::acos(r);
}

// nsvg__pathArcTo (canvg's arc conversion)
void arc_to(Parser &p, float *cpx, float *cpy, const float *args, bool rel) {
    float rx = std::fabs(args[0]), ry = std::fabs(args[1]);
    const float rotx = args[2] / 180.0f * kPi;
    const int fa = std::fabs(args[3]) > 1e-6 ? 1 : 0, fs = std::fabs(args[4]) > 1e-6 ? 1 : 0;
    const float x1 = *cpx, y1 = *cpy;
    float x2, y2;
    if (rel) {
        x2 = *cpx + args[5];
        y2 = *cpy + args[6];
    } else {
        x2 = args[5];
        y2 = args[6];
    }
    float dx = x1 - x2, dy = y1 - y2;
    float d = std::sqrt(dx * dx + dy * dy);
    if (d < 1e-6f || rx < 1e-6f || ry < 1e-6f) {
        p.line_to(x2, y2);
        *cpx = x2;
        *cpy = y2;
        return;
    }
    const float sinrx = std::sin(rotx), cosrx = std::cos(rotx);
    const float x1p = cosrx * dx / 2.0f + sinrx * dy / 2.0f;
    const float y1p = -sinrx * dx / 2.0f + cosrx * dy / 2.0f;
    d = sqr(x1p) / sqr(rx) + sqr(y1p) / sqr(ry);
    if (d > 1) {
        d = std::sqrt(d);
        rx *= d;
        ry *= d;
    }
    float s = 0.0f;
    float sa = sqr(rx) * sqr(ry) - sqr(rx) * sqr(y1p) - sqr(ry) * sqr(x1p);
    const float sb = sqr(rx) * sqr(y1p) + sqr(ry) * sqr(x1p);
    if (sa < 0.0f) sa = 0.0f;
    if (sb > 0.0f) s = std::sqrt(sa / sb);
    if (fa == fs) s = -s;
    const float cxp = s * rx * y1p / ry;
    const float cyp = s * -ry * x1p / rx;
    const float cx = (x1 + x2) / 2.0f + cosrx * cxp - sinrx * cyp;
    const float cy = (y1 + y2) / 2.0f + sinrx * cxp + cosrx * cyp;
    const float ux = (x1p - cxp) / rx, uy = (y1p - cyp) / ry;
    const float vx = (-x1p - cxp) / rx, vy = (-y1p - cyp) / ry;
    const float a1 = vecang(1.0f, 0.0f, ux, uy);
    float da = vecang(ux, uy, vx, vy);
    if (fs == 0 && da > 0) da -= 2 * kPi;
    else if (fs == 1 && da < 0) da += 2 * kPi;
    float t[6] = {cosrx, sinrx, -sinrx, cosrx, cx, cy};
    const int ndivs = (int)(std::fabs(da) / (kPi * 0.5f) + 1.0f);
    float hda = (da / (float)ndivs) / 2.0f;
    if ((hda < 1e-3f) && (hda > -1e-3f)) hda *= 0.5f;
    else hda = (1.0f - std::cos(hda)) / std::sin(hda);
    float kappa = std::fabs(4.0f / 3.0f * hda);
    if (da < 0.0f) kappa = -kappa;
    float px = 0, py = 0, ptanx = 0, ptany = 0;
    for (int i = 0; i <= ndivs; i++) {
        const float a = a1 + da * ((float)i / (float)ndivs);
        dx = std::cos(a);
        dy = std::sin(a);
        float x, y, tanx, tany;
        xf_point(&x, &y, dx * rx, dy * ry, t);
        xf_vec(&tanx, &tany, -dy * rx * kappa, dx * ry * kappa, t);
        if (i > 0) p.cubic_to(px + ptanx, py + ptany, x - tanx, y - tany, x, y);
        px = x;
        py = y;
        ptanx = tanx;
        ptany = tany;
    }
    *cpx = x2;
    *cpy = y2;
}

void parse_path(Parser &p, const char **attr) {
    const char *s = nullptr;
    for (int i = 0; attr[i]; i += 2) {
        if (std::strcmp(attr[i], "d") == 0) {
            s = attr[i + 1];
        } else {
            const char *tmp[4] = {attr[i], attr[i + 1], nullptr, nullptr};
            parse_attribs(p, tmp);
        }
    }
    if (s) {
        char item[64], cmd = '\0';
        float args[10];
        int nargs = 0, rargs = 0;
        bool init = false, closed = false;
        float cpx = 0, cpy = 0, cpx2 = 0, cpy2 = 0;
        p.pts.clear();
        while (*s) {
            s = next_path_item(s, item);
            if (!*item) break;
            if (cmd != '\0' && is_coordinate(item)) {
                if (nargs < 10) args[nargs++] = (float)parse_atof(item);
                if (nargs >= rargs) {
                    const bool rel = cmd >= 'a';
                    switch (cmd) {
                        case 'm': case 'M':
                            if (rel) cpx += args[0], cpy += args[1];
                            else cpx = args[0], cpy = args[1];
                            p.move_to(cpx, cpy);
                            cmd = rel ? 'l' : 'L';
                            rargs = args_per(cmd);
                            cpx2 = cpx;
                            cpy2 = cpy;
                            init = true;
                            break;
                        case 'l': case 'L':
                            if (rel) cpx += args[0], cpy += args[1];
                            else cpx = args[0], cpy = args[1];
                            p.line_to(cpx, cpy);
                            cpx2 = cpx;
                            cpy2 = cpy;
                            break;
                        case 'h': case 'H':
                            if (rel) cpx += args[0];
                            else cpx = args[0];
                            p.line_to(cpx, cpy);
                            cpx2 = cpx;
                            cpy2 = cpy;
                            break;
                        case 'v': case 'V':
                            if (rel) cpy += args[0];
                            else cpy = args[0];
                            p.line_to(cpx, cpy);
                            cpx2 = cpx;
                            cpy2 = cpy;
                            break;
                        case 'c': case 'C': {
                            float c1x, c1y, c2x, c2y, x2, y2;
                            if (rel) {
                                c1x = cpx + args[0], c1y = cpy + args[1], c2x = cpx + args[2], c2y = cpy + args[3];
                                x2 = cpx + args[4], y2 = cpy + args[5];
                            } else {
                                c1x = args[0], c1y = args[1], c2x = args[2], c2y = args[3], x2 = args[4], y2 = args[5];
                            }
                            p.cubic_to(c1x, c1y, c2x, c2y, x2, y2);
                            cpx2 = c2x, cpy2 = c2y, cpx = x2, cpy = y2;
                        } break;
                        case 's': case 'S': {
                            const float x1 = cpx, y1 = cpy;
                            float c2x, c2y, x2, y2;
                            if (rel) c2x = cpx + args[0], c2y = cpy + args[1], x2 = cpx + args[2], y2 = cpy + args[3];
                            else c2x = args[0], c2y = args[1], x2 = args[2], y2 = args[3];
                            const float c1x = 2 * x1 - cpx2, c1y = 2 * y1 - cpy2;
                            p.cubic_to(c1x, c1y, c2x, c2y, x2, y2);
                            cpx2 = c2x, cpy2 = c2y, cpx = x2, cpy = y2;
                        } break;
                        case 'q': case 'Q': {
                            const float x1 = cpx, y1 = cpy;
                            float cx, cy, x2, y2;
                            if (rel) cx = cpx + args[0], cy = cpy + args[1], x2 = cpx + args[2], y2 = cpy + args[3];
                            else cx = args[0], cy = args[1], x2 = args[2], y2 = args[3];
                            const float c1x = x1 + 2.0f / 3.0f * (cx - x1), c1y = y1 + 2.0f / 3.0f * (cy - y1);
                            const float c2x = x2 + 2.0f / 3.0f * (cx - x2), c2y = y2 + 2.0f / 3.0f * (cy - y2);
                            p.cubic_to(c1x, c1y, c2x, c2y, x2, y2);
                            cpx2 = cx, cpy2 = cy, cpx = x2, cpy = y2;
                        } break;
                        case 't': case 'T': {
                            const float x1 = cpx, y1 = cpy;
                            float x2, y2;
                            if (rel) x2 = cpx + args[0], y2 = cpy + args[1];
                            else x2 = args[0], y2 = args[1];
                            const float cx = 2 * x1 - cpx2, cy = 2 * y1 - cpy2;
                            const float c1x = x1 + 2.0f / 3.0f * (cx - x1), c1y = y1 + 2.0f / 3.0f * (cy - y1);
                            const float c2x = x2 + 2.0f / 3.0f * (cx - x2), c2y = y2 + 2.0f / 3.0f * (cy - y2);
                            p.cubic_to(c1x, c1y, c2x, c2y, x2, y2);
                            cpx2 = cx, cpy2 = cy, cpx = x2, cpy = y2;
                        } break;
                        case 'a': case 'A':
                            arc_to(p, &cpx, &cpy, args, rel);
                            cpx2 = cpx;
                            cpy2 = cpy;
                            break;
                        default:
                            if (nargs >= 2) {
                                cpx = args[nargs - 2];
                                cpy = args[nargs - 1];
                                cpx2 = cpx;
                                cpy2 = cpy;
                            }
                            break;
                    }
                    nargs = 0;
                }
            } else {
                cmd = item[0];
                if (cmd == 'M' || cmd == 'm') {
                    if (p.npts() > 0) p.add_path(closed);
                    p.pts.clear();
                    closed = false;
                    nargs = 0;
                } else if (!init) {
                    cmd = '\0';
                }
                if (cmd == 'Z' || cmd == 'z') {
                    closed = true;
                    if (p.npts() > 0) {
                        cpx = p.pts[0];
                        cpy = p.pts[1];
                        cpx2 = cpx;
                        cpy2 = cpy;
                        p.add_path(closed);
                    }
                    p.pts.clear();
                    p.move_to(cpx, cpy);
                    closed = false;
                    nargs = 0;
                }
                rargs = args_per(cmd);
                if (rargs == -1) {
                    cmd = '\0';
                    rargs = 0;
                }
            }
        }
        if (p.npts()) p.add_path(closed);
    }
    p.add_shape();
}

void parse_rect(Parser &p, const char **attr) {
    float x = 0.0f, y = 0.0f, w = 0.0f, h = 0.0f, rx = -1.0f, ry = -1.0f;
    for (int i = 0; attr[i]; i += 2) {
        if (!parse_attr(p, attr[i], attr[i + 1])) {
            if (std::strcmp(attr[i], "x") == 0) x = parse_coord(p, attr[i + 1], p.view_minx, p.view_width);
            if (std::strcmp(attr[i], "y") == 0) y = parse_coord(p, attr[i + 1], p.view_miny, p.view_height);
            if (std::strcmp(attr[i], "width") == 0) w = parse_coord(p, attr[i + 1], 0.0f, p.view_width);
            if (std::strcmp(attr[i], "height") == 0) h = parse_coord(p, attr[i + 1], 0.0f, p.view_height);
            if (std::strcmp(attr[i], "rx") == 0) rx = std::fabs(parse_coord(p, attr[i + 1], 0.0f, p.view_width));
            if (std::strcmp(attr[i], "ry") == 0) ry = std::fabs(parse_coord(p, attr[i + 1], 0.0f, p.view_height));
        }
    }
    if (rx < 0.0f && ry > 0.0f) rx = ry;
    if (ry < 0.0f && rx > 0.0f) ry = rx;
    if (rx < 0.0f) rx = 0.0f;
    if (ry < 0.0f) ry = 0.0f;
    if (rx > w / 2.0f) rx = w / 2.0f;
    if (ry > h / 2.0f) ry = h / 2.0f;
    if (w != 0.0f && h != 0.0f) {
        p.pts.clear();
        if (rx < 0.00001f || ry < 0.0001f) {
            p.move_to(x, y);
            p.line_to(x + w, y);
            p.line_to(x + w, y + h);
            p.line_to(x, y + h);
        } else {
            const float k = 1 - kKappa90;
            p.move_to(x + rx, y);
            p.line_to(x + w - rx, y);
            p.cubic_to(x + w - rx * k, y, x + w, y + ry * k, x + w, y + ry);
            p.line_to(x + w, y + h - ry);
            p.cubic_to(x + w, y + h - ry * k, x + w - rx * k, y + h, x + w - rx, y + h);
            p.line_to(x + rx, y + h);
            p.cubic_to(x + rx * k, y + h, x, y + h - ry * k, x, y + h - ry);
            p.line_to(x, y + ry);
            p.cubic_to(x, y + ry * k, x + rx * k, y, x + rx, y);
        }
        p.add_path(true);
        p.add_shape();
    }
}

void ellipse_path(Parser &p, float cx, float cy, float rx, float ry) {
    p.pts.clear();
    p.move_to(cx + rx, cy);
    p.cubic_to(cx + rx, cy + ry * kKappa90, cx + rx * kKappa90, cy + ry, cx, cy + ry);
    p.cubic_to(cx - rx * kKappa90, cy + ry, cx - rx, cy + ry * kKappa90, cx - rx, cy);
    p.cubic_to(cx - rx, cy - ry * kKappa90, cx - rx * kKappa90, cy - ry, cx, cy - ry);
    p.cubic_to(cx + rx * kKappa90, cy - ry, cx + rx, cy - ry * kKappa90, cx + rx, cy);
    p.add_path(true);
    p.add_shape();
}

void parse_circle(Parser &p, const char **attr) {
    float cx = 0.0f, cy = 0.0f, r = 0.0f;
    for (int i = 0; attr[i]; i += 2) {
        if (!parse_attr(p, attr[i], attr[i + 1])) {
            if (std::strcmp(attr[i], "cx") == 0) cx = parse_coord(p, attr[i + 1], p.view_minx, p.view_width);
            if (std::strcmp(attr[i], "cy") == 0) cy = parse_coord(p, attr[i + 1], p.view_miny, p.view_height);
            if (std::strcmp(attr[i], "r") == 0) r = std::fabs(parse_coord(p, attr[i + 1], 0.0f, p.actual_length()));
        }
    }
    if (r > 0.0f) ellipse_path(p, cx, cy, r, r);
}

void parse_ellipse(Parser &p, const char **attr) {
    float cx = 0.0f, cy = 0.0f, rx = 0.0f, ry = 0.0f;
    for (int i = 0; attr[i]; i += 2) {
        if (!parse_attr(p, attr[i], attr[i + 1])) {
            if (std::strcmp(attr[i], "cx") == 0) cx = parse_coord(p, attr[i + 1], p.view_minx, p.view_width);
            if (std::strcmp(attr[i], "cy") == 0) cy = parse_coord(p, attr[i + 1], p.view_miny, p.view_height);
            if (std::strcmp(attr[i], "rx") == 0) rx = std::fabs(parse_coord(p, attr[i + 1], 0.0f, p.view_width));
            if (std::strcmp(attr[i], "ry") == 0) ry = std::fabs(parse_coord(p, attr[i + 1], 0.0f, p.view_height));
        }
    }
    if (rx > 0.0f && ry > 0.0f) ellipse_path(p, cx, cy, rx, ry);
}

void parse_line(Parser &p, const char **attr) {
    float x1 = 0.0f, y1 = 0.0f, x2 = 0.0f, y2 = 0.0f;
    for (int i = 0; attr[i]; i += 2) {
        if (!parse_attr(p, attr[i], attr[i + 1])) {
            if (std::strcmp(attr[i], "x1") == 0) x1 = parse_coord(p, attr[i + 1], p.view_minx, p.view_width);
            if (std::strcmp(attr[i], "y1") == 0) y1 = parse_coord(p, attr[i + 1], p.view_miny, p.view_height);
            if (std::strcmp(attr[i], "x2") == 0) x2 = parse_coord(p, attr[i + 1], p.view_minx, p.view_width);
            if (std::strcmp(attr[i], "y2") == 0) y2 = parse_coord(p, attr[i + 1], p.view_miny, p.view_height);
        }
    }
    p.pts.clear();
    p.move_to(x1, y1);
    p.line_to(x2, y2);
    p.add_path(false);
    p.add_shape();
}

void parse_poly(Parser &p, const char **attr, bool close) {
    char item[64];
    int npts = 0;
    p.pts.clear();
    for (int i = 0; attr[i]; i += 2) {
        if (!parse_attr(p, attr[i], attr[i + 1])) {
            if (std::strcmp(attr[i], "points") == 0) {
                const char *s = attr[i + 1];
                float args[2];
                int nargs = 0;
                while (*s) {
                    s = next_path_item(s, item);
                    args[nargs++] = (float)parse_atof(item);
                    if (nargs >= 2) {
                        if (npts == 0) p.move_to(args[0], args[1]);
                        else p.line_to(args[0], args[1]);
                        nargs = 0;
                        npts++;
                    }
                }
            }
        }
    }
    p.add_path(close);
    p.add_shape();
}

// The <svg> element: presentation attributes, then its size, view box and alignment.
// Four numbers separated by white space, commas or '%'.  False when the text ends before the
// fourth: nanosvg then stops reading the element's attributes.
bool svg_view_box(Parser &p, const char *s) {
    float *dst[4] = {&p.view_minx, &p.view_miny, &p.view_width, &p.view_height};
    char buf[64];
    for (int k = 0; k < 4; k++) {
        if (k) {
            while (*s && (is_space(*s) || *s == '%' || *s == ',')) s++;
            if (!*s) return false;
        }
        s = parse_number(s, buf, 64);
        *dst[k] = (float)parse_atof(buf);
    }
    return true;
}

void svg_align(Parser &p, const char *v) {
    // "none", or an x and a y alignment keyword and "meet" / "slice" anywhere in the value
    if (std::strstr(v, "none")) {
        p.align_type = kAlignNone;
        return;
    }
    static const struct {
        const char *word;
        int *(*field)(Parser &);
        int value;
    } kWords[] = {{"xMin", [](Parser &q) { return &q.align_x; }, kAlignMin},
                  {"xMid", [](Parser &q) { return &q.align_x; }, kAlignMid},
                  {"xMax", [](Parser &q) { return &q.align_x; }, kAlignMax},
                  {"yMin", [](Parser &q) { return &q.align_y; }, kAlignMin},
                  {"yMid", [](Parser &q) { return &q.align_y; }, kAlignMid},
                  {"yMax", [](Parser &q) { return &q.align_y; }, kAlignMax}};
    bool x_done = false, y_done = false;
    for (const auto &w : kWords) {
        bool &done = w.word[0] == 'x' ? x_done : y_done;
        if (!done && std::strstr(v, w.word)) {
            *w.field(p) = w.value;
            done = true;
        }
    }
    p.align_type = std::strstr(v, "slice") ? kAlignSlice : kAlignMeet;
}

void parse_svg(Parser &p, const char **attr) {
    for (int i = 0; attr[i]; i += 2) {
        const char *n = attr[i], *v = attr[i + 1];
        if (parse_attr(p, n, v)) continue;
        if (std::strcmp(n, "width") == 0) p.width = parse_coord(p, v, 0.0f, 0.0f);
        else if (std::strcmp(n, "height") == 0) p.height = parse_coord(p, v, 0.0f, 0.0f);
        else if (std::strcmp(n, "viewBox") == 0 && !svg_view_box(p, v)) return;
        else if (std::strcmp(n, "preserveAspectRatio") == 0) svg_align(p, v);
    }
}

void parse_gradient(Parser &p, const char **attr, int type) {
    GradData g;
    g.type = type;
    if (type == kLinear) {  // x1 0%, y1 0%, x2 100%, y2 0%
        g.u[0] = {0.0f, kPercent}, g.u[1] = {0.0f, kPercent}, g.u[2] = {100.0f, kPercent}, g.u[3] = {0.0f, kPercent};
    } else {  // cx, cy, r 50%
        g.u[0] = {50.0f, kPercent}, g.u[1] = {50.0f, kPercent}, g.u[2] = {50.0f, kPercent};
    }
    xf_identity(g.xform);
    for (int i = 0; attr[i]; i += 2) {
        if (std::strcmp(attr[i], "id") == 0) {
            g.id = std::string(attr[i + 1]).substr(0, 63);
        } else if (!parse_attr(p, attr[i], attr[i + 1])) {
            const char *n = attr[i], *v = attr[i + 1];
            if (std::strcmp(n, "gradientUnits") == 0) g.object_space = std::strcmp(v, "objectBoundingBox") == 0;
            else if (std::strcmp(n, "gradientTransform") == 0) parse_transform(g.xform, v);
            else if (std::strcmp(n, "cx") == 0) g.u[0] = parse_coord_raw(v);
            else if (std::strcmp(n, "cy") == 0) g.u[1] = parse_coord_raw(v);
            else if (std::strcmp(n, "r") == 0) g.u[2] = parse_coord_raw(v);
            else if (std::strcmp(n, "fx") == 0) g.u[3] = parse_coord_raw(v);
            else if (std::strcmp(n, "fy") == 0) g.u[4] = parse_coord_raw(v);
            else if (std::strcmp(n, "x1") == 0) g.u[0] = parse_coord_raw(v);
            else if (std::strcmp(n, "y1") == 0) g.u[1] = parse_coord_raw(v);
            else if (std::strcmp(n, "x2") == 0) g.u[2] = parse_coord_raw(v);
            else if (std::strcmp(n, "y2") == 0) g.u[3] = parse_coord_raw(v);
            else if (std::strcmp(n, "spreadMethod") == 0) {
                if (std::strcmp(v, "pad") == 0) g.spread = 0;
                else if (std::strcmp(v, "reflect") == 0) g.spread = 1;
                else if (std::strcmp(v, "repeat") == 0) g.spread = 2;
            } else if (std::strcmp(n, "xlink:href") == 0) {
                g.ref = std::string(v + 1).substr(0, 62);
            }
        }
    }
    p.grads.insert(p.grads.begin(), std::move(g));
}

void parse_stop(Parser &p, const char **attr) {
    Attr &a = p.cur();
    a.stop_offset = 0;
    a.stop_color = 0;
    a.stop_opacity = 1.0f;
    for (int i = 0; attr[i]; i += 2) parse_attr(p, attr[i], attr[i + 1]);
    if (p.grads.empty()) return;
    std::vector<GradStop> &stops = p.grads.front().stops;
    size_t idx = stops.size();
    for (size_t i = 0; i < stops.size(); i++)
        if (a.stop_offset < stops[i].offset) {
            idx = i;
            break;
        }
    stops.insert(stops.begin() + idx, GradStop{a.stop_color | (uint32_t)(a.stop_opacity * 255) << 24, a.stop_offset});
}

// --- elements ----------------------------------------------------------------------------------
// What each element does when it opens and closes.  Inside <defs> only gradients and their stops
// open.  A shape element reads its attributes into a state of its own (pushed, then popped);
// <g> pushes a state that its closing tag pops.
void parse_shape(Parser &p, const char **attr, void (*read)(Parser &, const char **)) {
    p.push();
    read(p, attr);
    p.pop();
}

struct ElementRule {
    const char *name;
    bool in_defs;                                   // also read inside <defs>
    void (*open)(Parser &, const char **);
    void (*close)(Parser &);                        // null: nothing to do
};

const ElementRule kElements[] = {  // sorted by name (strcmp)
    {"circle", false, [](Parser &p, const char **a) { parse_shape(p, a, parse_circle); }, nullptr},
    {"defs", false, [](Parser &p, const char **) { p.defs_flag = true; }, [](Parser &p) { p.defs_flag = false; }},
    {"ellipse", false, [](Parser &p, const char **a) { parse_shape(p, a, parse_ellipse); }, nullptr},
    {"g", false, [](Parser &p, const char **a) {
         p.push();
         parse_attribs(p, a);
     }, [](Parser &p) { p.pop(); }},
    {"line", false, [](Parser &p, const char **a) { parse_shape(p, a, parse_line); }, nullptr},
    {"linearGradient", true, [](Parser &p, const char **a) { parse_gradient(p, a, kLinear); }, nullptr},
    {"path", false, [](Parser &p, const char **a) { parse_shape(p, a, parse_path); }, nullptr},
    {"polygon", false, [](Parser &p, const char **a) {
         parse_shape(p, a, [](Parser &q, const char **b) { parse_poly(q, b, true); });
     }, nullptr},
    {"polyline", false, [](Parser &p, const char **a) {
         parse_shape(p, a, [](Parser &q, const char **b) { parse_poly(q, b, false); });
     }, nullptr},
    {"radialGradient", true, [](Parser &p, const char **a) { parse_gradient(p, a, kRadial); }, nullptr},
    {"rect", false, [](Parser &p, const char **a) { parse_shape(p, a, parse_rect); }, nullptr},
    {"stop", true, [](Parser &p, const char **a) { parse_stop(p, a); }, nullptr},
    {"svg", false, [](Parser &p, const char **a) { parse_svg(p, a); }, nullptr},
};

const ElementRule *element_rule(const char *name) {
    const ElementRule *end = kElements + sizeof kElements / sizeof kElements[0];
    const ElementRule *r = std::lower_bound(kElements, end, name,
                                            [](const ElementRule &e, const char *n) { return std::strcmp(e.name, n) < 0; });
    return r != end && std::strcmp(r->name, name) == 0 ? r : nullptr;
}

// --- XML -----------------------------------------------------------------------------------------
// The document is cut into tags the way the reference's parser (nanosvg) cuts it, so that every
// document gives the reference's scene, quirks included: text outside tags is skipped; a tag runs
// from a '<' to the next '>' (quotes do not hide a '>'), and one left open at the end is dropped;
// "<?...>", "<!...>" and empty tags are skipped; after an optional '/' (a closing tag) the name runs
// to the first white space; in an opening tag, attributes follow until a '/' (which also closes
// it): a name ends at white space or '=', and its value is the next quoted string (single or
// double quotes) - so an unquoted value takes the next attribute's.  At most 127 attributes.
constexpr int kMaxTagAttrs = 127;

struct Tag {
    std::string name;
    bool opens = false, closes = false;
    std::vector<std::string> kv;     // name, value, name, value, ...
    std::vector<const char *> argv;  // the same as C strings, then two null pointers
};

// Reads the tag whose text (between '<' and '>') is [b, e); false for one that is skipped.
bool read_tag(const char *b, const char *e, Tag &t) {
    t.name.clear();
    t.kv.clear();
    t.opens = t.closes = false;
    const char *q = b;
    while (q < e && is_space(*q)) q++;
    if (q < e && *q == '/') {
        t.closes = true;
        q++;
    } else {
        t.opens = true;
    }
    if (q == e || *q == '?' || *q == '!') return false;
    const char *nb = q;
    while (q < e && !is_space(*q)) q++;
    t.name.assign(nb, q);
    if (q < e) q++;  // the white space after the name
    while (!t.closes && q < e && (int)t.kv.size() < 2 * kMaxTagAttrs) {
        while (q < e && is_space(*q)) q++;
        if (q == e) break;
        if (*q == '/') {
            t.closes = true;
            break;
        }
        const char *ab = q;
        while (q < e && !is_space(*q) && *q != '=') q++;
        const char *ae = q;
        if (q < e) q++;  // the '=' or white space after the name
        while (q < e && *q != '"' && *q != '\'') q++;
        if (q == e) break;
        const char quote = *q++;
        const char *vb = q;
        while (q < e && *q != quote) q++;
        t.kv.emplace_back(ab, ae);
        t.kv.emplace_back(vb, q);
        if (q < e) q++;  // the closing quote
    }
    t.argv.clear();
    for (const std::string &x : t.kv) t.argv.push_back(x.c_str());
    t.argv.push_back(nullptr);
    t.argv.push_back(nullptr);
    return true;
}

void parse_document(Parser &p, const char *text, size_t n) {
    Tag t;
    const char *q = text, *end = text + n;
    while (q < end) {
        const char *lt = static_cast<const char *>(std::memchr(q, '<', size_t(end - q)));
        if (!lt) break;
        const char *gt = static_cast<const char *>(std::memchr(lt + 1, '>', size_t(end - lt - 1)));
        if (!gt) break;
        q = gt + 1;
        if (!read_tag(lt + 1, gt, t)) continue;
        const ElementRule *r = element_rule(t.name.c_str());
        if (!r) continue;
        if (t.opens && (r->in_defs || !p.defs_flag)) r->open(p, t.argv.data());
        if (t.closes && r->close) r->close(p);  // closing tags act inside <defs> too
    }
}

float view_align(float content, float container, int type) {
    if (type == kAlignMin) return 0;
    if (type == kAlignMax) return container - content;
    return (container - content) * 0.5f;
}

// nsvg__scaleToViewbox with units "px"
void scale_to_viewbox(Parser &p) {
    float bounds[4] = {0, 0, 0, 0};
    if (!p.shapes.empty()) {
        std::memcpy(bounds, p.shapes[0].bounds, sizeof bounds);
        for (size_t i = 1; i < p.shapes.size(); i++) {
            bounds[0] = minf(bounds[0], p.shapes[i].bounds[0]);
            bounds[1] = minf(bounds[1], p.shapes[i].bounds[1]);
            bounds[2] = maxf(bounds[2], p.shapes[i].bounds[2]);
            bounds[3] = maxf(bounds[3], p.shapes[i].bounds[3]);
        }
    }
    if (p.view_width == 0) {
        if (p.width > 0) {
            p.view_width = p.width;
        } else {
            p.view_minx = bounds[0];
            p.view_width = bounds[2] - bounds[0];
        }
    }
    if (p.view_height == 0) {
        if (p.height > 0) {
            p.view_height = p.height;
        } else {
            p.view_miny = bounds[1];
            p.view_height = bounds[3] - bounds[1];
        }
    }
    if (p.width == 0) p.width = p.view_width;
    if (p.height == 0) p.height = p.view_height;
    float tx = -p.view_minx, ty = -p.view_miny;
    float sx = p.view_width > 0 ? p.width / p.view_width : 0;
    float sy = p.view_height > 0 ? p.height / p.view_height : 0;
    const float us = 1.0f / p.to_pixels(Coord{1.0f, kPx}, 0.0f, 1.0f);
    if (p.align_type == kAlignMeet) {
        sx = sy = minf(sx, sy);
        tx += view_align(p.view_width * sx, p.width, p.align_x) / sx;
        ty += view_align(p.view_height * sy, p.height, p.align_y) / sy;
    } else if (p.align_type == kAlignSlice) {
        sx = sy = maxf(sx, sy);
        tx += view_align(p.view_width * sx, p.width, p.align_x) / sx;
        ty += view_align(p.view_height * sy, p.height, p.align_y) / sy;
    }
    sx *= us;
    sy *= us;
    const float avgs = (sx + sy) / 2.0f;
    for (Shape &shape : p.shapes) {
        for (SubPath &path : shape.paths)
            for (size_t i = 0; i < path.pts.size(); i += 2) {
                path.pts[i] = (path.pts[i] + tx) * sx;
                path.pts[i + 1] = (path.pts[i + 1] + ty) * sy;
            }
        shape.stroke_width *= avgs;
        shape.dash_offset *= avgs;
        for (int i = 0; i < shape.dash_count; i++) shape.dashes[i] *= avgs;
    }
}

// --- scene assembly (SvgScene, Path2d, Canvas) ----------------------------------------------------
constexpr float kPathMinDist = 0.05f;  // PATH_MIN_DIST, core/path2d.cpp:9

struct SceneOut {
    std::vector<float> points;
    std::vector<uint8_t> flags, closed, fill_rule;
    std::vector<uint32_t> cstart{0}, pstart{0}, color;
    std::vector<pf_stroke> stroke;
    std::vector<float> dashes;
    std::vector<pf_paint> paint;
    std::vector<pf_color_stop> stops;
    float width = 0, height = 0;
    pf_scene_view view{};
};

// Transform2 (common/math/transform2.*): {matrix m11 m21 m12 m22, vector}, A * B and A * p
void t2_mul(const float *a, const float *b, float *out) {
    const float m0 = a[0] * b[0] + a[2] * b[1], m1 = a[1] * b[0] + a[3] * b[1];
    const float m2 = a[0] * b[2] + a[2] * b[3], m3 = a[1] * b[2] + a[3] * b[3];
    const float vx = (a[0] * b[4] + a[2] * b[5]) + a[4], vy = (a[1] * b[4] + a[3] * b[5]) + a[5];
    out[0] = m0, out[1] = m1, out[2] = m2, out[3] = m3, out[4] = vx, out[5] = vy;
}
void t2_apply(const float *t, float x, float y, float *ox, float *oy) {
    *ox = (t[0] * x + t[2] * y) + t[4];
    *oy = (t[1] * x + t[3] * y) + t[5];
}

// convert_nsvg_paint (core/svg.cpp:63-133): colour, or a gradient; base colour visible?
bool convert_paint(const PaintDesc &pd, SceneOut &o, uint32_t &color, pf_paint &paint) {
    std::memset(&paint, 0, sizeof paint);
    paint.transform[0] = paint.transform[3] = 1.0f;
    if (pd.type == kColor) {
        color = pd.color;
        return (color >> 24) != 0;  // Canvas::push_path draws only a visible base colour
    }
    if (pd.type != kLinear && pd.type != kRadial) return false;
    const Grad &g = pd.grad;
    float pg[6];
    t2_mul(g.xform3, g.xform2, pg);  // path_xform * gradient_xform
    paint.type = pd.type == kLinear ? PF_PAINT_LINEAR : PF_PAINT_RADIAL;
    if (pd.type == kLinear) {
        t2_apply(pg, g.x1, g.y1, &paint.line[0], &paint.line[1]);
        t2_apply(pg, g.x2, g.y2, &paint.line[2], &paint.line[3]);
    } else {
        paint.line[0] = g.cx, paint.line[1] = g.cy, paint.line[2] = g.fx, paint.line[3] = g.fy;
        paint.radii[0] = 0.0f;
        paint.radii[1] = g.r;
        std::memcpy(paint.transform, pg, sizeof pg);
    }
    paint.wrap = g.spread == 2 ? PF_WRAP_REPEAT : PF_WRAP_CLAMP;  // reflect is not supported (clamps)
    // Paint::is_visible: a gradient is visible when one of its stops is
    bool visible = false;
    for (const GradStop &s : g.stops) visible |= (s.color >> 24) != 0;
    if (!visible) return false;
    paint.stop_first = (uint32_t)o.stops.size();
    paint.stop_count = (uint32_t)g.stops.size();
    for (const GradStop &s : g.stops) o.stops.push_back(pf_color_stop{s.offset, s.color});
    color = 0xffffffffu;  // from_gradient's white base colour
    return true;
}

// Path2d of a shape's subpaths (move_to, cubic_to with its line fallback, close_path): the
// contours go to o, with their closed flags.
void emit_contours(const Shape &s, SceneOut &o) {
    for (const SubPath &sp : s.paths) {
        const size_t n = sp.pts.size() / 2;
        o.points.push_back(sp.pts[0]);
        o.points.push_back(sp.pts[1]);
        o.flags.push_back(PF_POINT_ON_CURVE);
        auto approx = [](float ax, float ay, float bx, float by, float eps) {
            const float dx = ax - bx, dy = ay - by;
            return std::sqrt(dx * dx + dy * dy) <= eps;
        };
        for (size_t i = 0; i + 3 < n; i += 3) {
            const float *q = &sp.pts[i * 2];
            const float c0x = q[2], c0y = q[3], c1x = q[4], c1y = q[5], x = q[6], y = q[7];
            if (approx(c0x, c0y, c1x, c1y, kPathMinDist) && approx(c1x, c1y, x, y, kPathMinDist)) {
                // Path2d::line_to: dropped within 0.05 of the last point
                const float lx = o.points[o.points.size() - 2], ly = o.points[o.points.size() - 1];
                const float dx = x - lx, dy = y - ly;
                if (dx * dx + dy * dy < kPathMinDist * kPathMinDist) continue;
                o.points.push_back(x);
                o.points.push_back(y);
                o.flags.push_back(PF_POINT_ON_CURVE);
            } else {
                o.points.insert(o.points.end(), {c0x, c0y, c1x, c1y, x, y});
                o.flags.insert(o.flags.end(), {PF_POINT_CONTROL_0, PF_POINT_CONTROL_1, PF_POINT_ON_CURVE});
            }
        }
        o.cstart.push_back((uint32_t)o.flags.size());
        o.closed.push_back(sp.closed ? 1 : 0);
    }
}

}  // namespace

struct pf_svg {
    SceneOut out;
};

extern "C" {

int pf_svg_parse(const char *text, size_t length, float dpi, pf_svg **out) {
    if (!text || !out) return PF_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    Parser *p = new (std::nothrow) Parser();
    pf_svg *svg = new (std::nothrow) pf_svg();
    if (!p || !svg) {
        delete p;
        delete svg;
        return PF_ERR_OUT_OF_MEMORY;
    }
    p->dpi = dpi;
    parse_document(*p, text, strnlen(text, length));  // the text ends at its first NUL, as C text does
    scale_to_viewbox(*p);
    SceneOut &o = svg->out;
    o.width = p->width;
    o.height = p->height;
    // SvgScene: per shape a fill (if its paint is visible) and then a stroke (if its paint is
    // visible and its width positive), both over the same Path2d
    for (const Shape &s : p->shapes) {
        uint32_t color;
        pf_paint paint;
        if (convert_paint(s.fill, o, color, paint)) {
            emit_contours(s, o);
            o.pstart.push_back((uint32_t)(o.cstart.size() - 1));
            o.color.push_back(color);
            o.fill_rule.push_back(s.fill_rule ? PF_FILL_EVEN_ODD : PF_FILL_NONZERO);
            o.paint.push_back(paint);
            pf_stroke none{};
            o.stroke.push_back(none);
        }
        if (s.stroke_width > 0.0f && convert_paint(s.stroke, o, color, paint)) {
            emit_contours(s, o);
            o.pstart.push_back((uint32_t)(o.cstart.size() - 1));
            o.color.push_back(color);
            o.fill_rule.push_back(PF_FILL_NONZERO);
            o.paint.push_back(paint);
            pf_stroke st{};
            st.line_width = s.stroke_width;
            st.miter_limit = s.miter;
            // nanosvg caps butt/round/square and joins miter/round/bevel to LineCap / LineJoin
            // (convert_nsvg_line_cap / _join, core/svg.cpp:22-61)
            st.line_cap = s.cap == 1 ? PF_CAP_ROUND : s.cap == 2 ? PF_CAP_SQUARE : PF_CAP_BUTT;
            st.line_join = s.join == 1 ? PF_JOIN_ROUND : s.join == 2 ? PF_JOIN_BEVEL : PF_JOIN_MITER;
            if (s.dash_count) {  // Canvas::stroke_path dashes with phase 0
                st.dash_first = (uint32_t)o.dashes.size();
                st.dash_count = (uint32_t)s.dash_count;
                st.dash_offset = 0.0f;
                o.dashes.insert(o.dashes.end(), s.dashes, s.dashes + s.dash_count);
            }
            o.stroke.push_back(st);
        }
    }
    delete p;
    // the counts are the real ones; an empty array still gets a valid pointer
    const uint32_t n_dashes = (uint32_t)o.dashes.size(), n_stops = (uint32_t)o.stops.size();
    if (o.dashes.empty()) o.dashes.push_back(0.0f);
    if (o.stops.empty()) o.stops.push_back(pf_color_stop{0.0f, 0u});
    pf_scene_view &v = o.view;
    v = pf_scene_view{};
    v.points = o.points.data();
    v.point_flags = o.flags.data();
    v.contour_start = o.cstart.data();
    v.path_start = o.pstart.data();
    v.fill_rule = o.fill_rule.data();
    v.color = o.color.data();
    v.n_points = (uint32_t)o.flags.size();
    v.n_contours = (uint32_t)(o.cstart.size() - 1);
    v.n_paths = (uint32_t)o.color.size();
    v.width = o.width;
    v.height = o.height;
    v.clear_color = 0;
    v.path_stroke = o.stroke.data();
    v.contour_closed = o.closed.data();
    v.dashes = o.dashes.data();
    v.n_dashes = n_dashes;
    v.path_paint = o.paint.data();
    v.stops = o.stops.data();
    v.n_stops = n_stops;
    *out = svg;
    return PF_OK;
}

int pf_svg_scene(const pf_svg *svg, pf_scene_view *out) {
    if (!svg || !out) return PF_ERR_INVALID_ARGUMENT;
    *out = svg->out.view;
    return PF_OK;
}

void pf_svg_free(pf_svg *svg) { delete svg; }

}  // extern "C"
