/*
 * pf_paint.c - CPU restatement of the reference's gradient paints for the pixel oracle.
 *
 * TEST INFRASTRUCTURE ONLY (part of libpforacle.so): the checker for the GPU composite's
 * gradients, never on the product path.
 *
 *   - colour ramps: Gradient::add / Gradient::sample / GradientTileBuilder::allocate
 *     (pathfinder/core/paint/gradient.cpp:5-110), single precision, bit-exact (pinned against the
 *     reference's own Gradient through ref_harness.cpp);
 *   - texture metadata: the gradient texture transform (Palette, core/paint/palette.cpp:420-435)
 *     and the radial filter parameters (palette.cpp:36-39, core/paint/paint.cpp:45-65), stored as
 *     half floats with umHalf's truncating conversion (core/renderer.cpp:167-250), bit-exact;
 *   - per pixel: tile.comp's colour-texture coordinate (computeTileVaryings, tile.comp:694-724),
 *     filterRadialGradient (tile.comp:319-347) and a linearly filtered texture fetch, in double
 *     precision (the shader's own arithmetic is GPU float; tolerance-checked).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pf_oracle.h"

#define RAMP 256  /* GRADIENT_TILE_LENGTH, core/paint/gradient.h */

/* umHalf's float -> half -> float round trip (third_party/umHalf.inl): the exponent is
 * rebiased, the mantissa truncated; below 2^-24 zero, below 2^-14 a subnormal (truncated),
 * above 2^15 infinity. */
float pfo_half_trunc(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    const uint32_t sign = b & 0x80000000u;
    const int32_t e = (int32_t)((b >> 23) & 0xffu);
    const uint32_t frac = b & 0x7fffffu;
    uint32_t hexp, hfrac;
    if (e == 0) {
        hexp = 0;
        hfrac = 0;
    } else if (e == 255) {
        hexp = 31;
        hfrac = frac ? 1u : 0u;
    } else {
        const int32_t adj = e - 127;
        if (adj < -24) {
            hexp = 0;
            hfrac = 0;
        } else if (adj < -14) {
            const int32_t ne = -14 - adj;
            hexp = 0;
            hfrac = (1024u >> ne) + (frac >> (13 + ne));
        } else if (adj > 15) {
            hexp = 31;
            hfrac = 0;
        } else {
            hexp = (uint32_t)(adj + 15);
            hfrac = frac >> 13;
        }
    }
    /* back to float */
    float out;
    if (hexp == 0) {
        out = hfrac ? ((float)hfrac / 1024.0f) * (1.0f / 16384.0f) : 0.0f;
        if (sign) out = -out;
        return out;
    }
    uint32_t ob;
    if (hexp == 31) ob = sign | 0x7f800000u | (hfrac ? 1u : 0u);
    else ob = sign | ((hexp - 15 + 127) << 23) | (hfrac << 13);
    memcpy(&out, &ob, 4);
    return out;
}

typedef struct {
    float offset;
    uint8_t c[4];
} stop_t;

/* Gradient::add: a stop goes before the first stop whose offset is not smaller */
static uint32_t sorted_stops(const pf_color_stop *in, uint32_t n, stop_t *out) {
    uint32_t m = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t at = 0;
        while (at < m && out[at].offset < in[i].offset) at++;
        memmove(out + at + 1, out + at, (m - at) * sizeof(stop_t));
        out[at].offset = in[i].offset;
        for (int k = 0; k < 4; k++) out[at].c[k] = (uint8_t)(in[i].color >> (8 * k));
        m++;
    }
    return m;
}

/* Gradient::sample (gradient.cpp:16-45) with ColorF::lerp and ColorU(ColorF) (common/color.cpp) */
static void sample(const stop_t *st, uint32_t n, float t, uint8_t out[4]) {
    if (n == 0) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    const uint32_t last = n - 1;
    uint32_t it = 0;
    while (it < n && (st[it].offset < t || st[it].offset == 0)) it++;
    const uint32_t upper = it < last ? it : last;
    const uint32_t lower = upper > 0 ? upper - 1 : upper;
    const float denom = st[upper].offset - st[lower].offset;
    if (denom == 0) {
        memcpy(out, st[lower].c, 4);
        return;
    }
    float ratio = (t - st[lower].offset) / denom;
    ratio = ratio < 1.0f ? ratio : 1.0f;
    ratio = ratio < 0.0f ? 0.0f : (ratio > 1.0f ? 1.0f : ratio);  /* ColorF::lerp clamps */
    const float factor = 1.f / 255.f;
    for (int k = 0; k < 4; k++) {
        const float a = (float)st[lower].c[k] * factor, b = (float)st[upper].c[k] * factor;
        const float v = a + (b - a) * ratio;
        out[k] = (uint8_t)(v * 255.f);
    }
}

/* GradientTileBuilder::allocate's row: texel x holds sample((x + 0.5) / 256) */
void pfo_gradient_ramp(const pf_color_stop *stops, uint32_t n, uint32_t *ramp) {
    stop_t st[64];
    stop_t *buf = n <= 64 ? st : (stop_t *)malloc(sizeof(stop_t) * n);
    const uint32_t m = sorted_stops(stops, n, buf);
    for (int x = 0; x < RAMP; x++) {
        uint8_t c[4];
        sample(buf, m, ((float)x + 0.5f) / (float)RAMP, c);
        ramp[x] = (uint32_t)c[0] | (uint32_t)c[1] << 8 | (uint32_t)c[2] << 16 | (uint32_t)c[3] << 24;
    }
    if (buf != st) free(buf);
}

int pfo_paint_is_opaque(const pf_scene_view *s, uint32_t p) {
    if (!s->path_paint || s->path_paint[p].type == PF_PAINT_SOLID) return ((s->color[p] >> 24) & 0xffu) == 0xffu;
    const pf_paint *pp = &s->path_paint[p];
    if (pp->stop_count == 0) return 0;  /* Gradient::is_opaque */
    for (uint32_t i = 0; i < pp->stop_count; i++)
        if ((s->stops[pp->stop_first + i].color >> 24) != 0xffu) return 0;
    return 1;
}

/*
 * The metadata of a gradient path, as the shader reads it (half floats):
 * linear: colour transform (m0.x, 0, m0.y, 0 | m13.x + m13.y, v0) with m0 = dp / |dp|^2 and
 * m13 = m0 * -from (palette.cpp:420-431); radial: the inverse of the gradient's transform
 * (palette.cpp:433-434), p0 = (from, to - from), p1 = (r0, r1, uv origin) (palette.cpp:36-39).
 * The ramp's row is texel-centred, so v picks it exactly; u is all that matters here.
 */
void pfo_paint_meta(const pf_paint *pp, float meta[12]) {
    memset(meta, 0, 12 * sizeof(float));
    if (pp->type == PF_PAINT_LINEAR) {
        const float fx = pp->line[0], fy = pp->line[1];
        const float dx = pp->line[2] - fx, dy = pp->line[3] - fy;
        const float sq = dx * dx + dy * dy;
        const float m0x = dx / sq, m0y = dy / sq;
        const float m13x = m0x * -fx, m13y = m0y * -fy;
        meta[0] = pfo_half_trunc(m0x);
        meta[2] = pfo_half_trunc(m0y);
        meta[4] = pfo_half_trunc(m13x + m13y);
    } else if (pp->type == PF_PAINT_RADIAL) {
        /* Transform2::inverse (common/math/transform2.cpp:32-36): adjugate / det, then
         * -(inverse matrix * vector) */
        const float *t = pp->transform;
        const float det = t[0] * t[3] - t[1] * t[2];
        const float s = 1.0f / det;
        const float a = (t[3] * 1.0f) * s, b = (t[1] * -1.0f) * s, c = (t[2] * -1.0f) * s, d = (t[0] * 1.0f) * s;
        const float vx = -(a * t[4] + c * t[5]), vy = -(b * t[4] + d * t[5]);
        meta[0] = pfo_half_trunc(a);
        meta[1] = pfo_half_trunc(b);
        meta[2] = pfo_half_trunc(c);
        meta[3] = pfo_half_trunc(d);
        meta[4] = pfo_half_trunc(vx);
        meta[5] = pfo_half_trunc(vy);
        meta[6] = pfo_half_trunc(pp->line[0]);
        meta[7] = pfo_half_trunc(pp->line[1]);
        meta[8] = pfo_half_trunc(pp->line[2] - pp->line[0]);
        meta[9] = pfo_half_trunc(pp->line[3] - pp->line[1]);
        meta[10] = pfo_half_trunc(pp->radii[0]);
        meta[11] = pfo_half_trunc(pp->radii[1]);
    }
}

/* a linearly filtered fetch of the ramp at u (texel centres at (i + 0.5) / 256) */
static void fetch(const uint32_t *ramp, int repeat, double u, double out[4]) {
    if (!isfinite(u)) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    if (repeat) u -= floor(u);
    const double s = u * RAMP - 0.5;
    const double f0 = floor(s), f = s - f0;
    long i0 = (long)f0, i1 = i0 + 1;
    if (repeat) {
        i0 = ((i0 % RAMP) + RAMP) % RAMP;
        i1 = ((i1 % RAMP) + RAMP) % RAMP;
    } else {
        i0 = i0 < 0 ? 0 : (i0 > RAMP - 1 ? RAMP - 1 : i0);
        i1 = i1 < 0 ? 0 : (i1 > RAMP - 1 ? RAMP - 1 : i1);
    }
    for (int k = 0; k < 4; k++) {
        const double a = (double)((ramp[i0] >> (8 * k)) & 0xffu) / 255.0;
        const double b = (double)((ramp[i1] >> (8 * k)) & 0xffu) / 255.0;
        out[k] = a + (b - a) * f;
    }
}

/* The colour (straight alpha) a gradient path gives the pixel centred at (x, y). */
void pfo_paint_color(const pf_paint *pp, const float meta[12], const uint32_t *ramp, double x, double y,
                     double out[4]) {
    const int repeat = pp->wrap == PF_WRAP_REPEAT;
    if (pp->type == PF_PAINT_LINEAR) {
        fetch(ramp, repeat, (double)meta[0] * x + (double)meta[2] * y + (double)meta[4], out);
        return;
    }
    /* filterRadialGradient (tile.comp:319-347) */
    const double cx = (double)meta[0] * x + (double)meta[2] * y + (double)meta[4];
    const double cy = (double)meta[1] * x + (double)meta[3] * y + (double)meta[5];
    const double dpx = cx - meta[6], dpy = cy - meta[7], dcx = meta[8], dcy = meta[9];
    const double r0 = meta[10], dr = (double)meta[11] - r0;
    const double a = dcx * dcx + dcy * dcy - dr * dr;
    const double b = dpx * dcx + dpy * dcy + r0 * dr;
    const double c = dpx * dpx + dpy * dpy - r0 * r0;
    const double disc = b * b - a * c;
    if (disc == 0.0 || !(disc > 0.0)) {  /* zero: the shader's transparent; negative: no real t */
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    const double sq = sqrt(disc);
    double t0 = (sq + b) / a, t1 = (-sq + b) / a;
    if (t0 > t1) {
        const double tmp = t0;
        t0 = t1;
        t1 = tmp;
    }
    fetch(ramp, repeat, t0 >= 0.0 ? t0 : t1, out);
}
