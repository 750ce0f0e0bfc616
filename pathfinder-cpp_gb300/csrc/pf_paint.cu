// pf_paint.cu - gradient paints: each gradient's 256-texel colour ramp and the metadata the
// reference's tile shader reads for it, built once per upload (one block per gradient).
//
// Ramp: GradientTileBuilder::allocate (pathfinder/core/paint/gradient.cpp:61-110) fills a
// texture row with Gradient::sample((x + 0.5) / 256), which finds the stops around t, lerps
// their colours as floats (ColorF::lerp, common/color.cpp:61-71) and truncates to 8 bits
// (ColorU(ColorF), common/color.cpp:15-21).  Stops arrive sorted the way Gradient::add inserts
// them.  Metadata: the texture transform (core/paint/palette.cpp:420-435) and radial filter
// parameters (palette.cpp:36-39, core/paint/paint.cpp:45-65) as half floats with umHalf's
// truncating conversion (core/renderer.cpp:167-250).  Single precision throughout, with
// explicit round-to-nearest intrinsics so the values are the reference's bit for bit.
#include "pf_internal.h"

namespace pfc {
namespace {

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// umHalf: float -> half (exponent rebiased, mantissa truncated) -> float
__device__ float half_trunc(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t sign = b & 0x80000000u, frac = b & 0x7fffffu;
    const int32_t e = (int32_t)((b >> 23) & 0xffu);
    uint32_t hexp = 0, hfrac = 0;
    if (e == 255) {
        hexp = 31;
        hfrac = frac ? 1u : 0u;
    } else if (e != 0) {
        const int32_t adj = e - 127;
        if (adj < -24) {
        } else if (adj < -14) {
            const int32_t ne = -14 - adj;
            hfrac = (1024u >> ne) + (frac >> (13 + ne));
        } else if (adj > 15) {
            hexp = 31;
        } else {
            hexp = (uint32_t)(adj + 15);
            hfrac = frac >> 13;
        }
    }
    if (hexp == 0) {
        const float m = hfrac ? fm(fd((float)hfrac, 1024.0f), fd(1.0f, 16384.0f)) : 0.0f;
        return sign ? -m : m;
    }
    if (hexp == 31) return __uint_as_float(sign | 0x7f800000u | (hfrac ? 1u : 0u));
    return __uint_as_float(sign | ((hexp - 15 + 127) << 23) | (hfrac << 13));
}

__device__ __forceinline__ uint32_t upper_bound(const uint32_t *a, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void k_gradient_flags(const pf_paint *paints, uint32_t n, uint32_t *flags) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) flags[p] = paints[p].type != PF_PAINT_SOLID ? 1u : 0u;
}

__global__ void k_gradient_index(const pf_paint *paints, uint32_t n, const uint32_t *scanned, uint32_t *path_grad,
                                 uint32_t *grad_path) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const bool g = paints[p].type != PF_PAINT_SOLID;
    path_grad[p] = g ? scanned[p] : kNone;
    if (g) grad_path[scanned[p]] = p;
}

__global__ void __launch_bounds__(256) k_gradients(const pf_paint *paints, const uint32_t *grad_path,
                                                   const uint32_t *scene_path_first, uint32_t n_scenes,
                                                   const uint32_t *stop_base, const pf_color_stop *stops, uint32_t n,
                                                   float4 *meta, uint32_t *ramps) {
    __shared__ pf_color_stop st[kMaxGradientStops];
    const uint32_t g = blockIdx.x;
    if (g >= n) return;
    const uint32_t path = grad_path[g];
    const pf_paint pp = paints[path];
    const uint32_t scene = upper_bound(scene_path_first, n_scenes + 1, path) - 1;
    const pf_color_stop *src = stops + stop_base[scene] + pp.stop_first;
    const uint32_t cnt = min(pp.stop_count, kMaxGradientStops);
    if (threadIdx.x == 0) {
        // Gradient::add: each stop goes before the first stop whose offset is not smaller
        for (uint32_t i = 0; i < cnt; i++) {
            const pf_color_stop s = src[i];
            uint32_t at = 0;
            while (at < i && st[at].offset < s.offset) at++;
            for (uint32_t k = i; k > at; k--) st[k] = st[k - 1];
            st[at] = s;
        }
    }
    __syncthreads();
    // Gradient::sample((x + 0.5) / 256)
    const uint32_t x = threadIdx.x;
    float t = fd(fa((float)x, 0.5f), 256.0f);
    uint32_t out = 0;
    if (cnt) {
        t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
        uint32_t it = 0;
        while (it < cnt && (st[it].offset < t || st[it].offset == 0.0f)) it++;
        const uint32_t upper = min(it, cnt - 1), lower = upper > 0 ? upper - 1 : upper;
        const float denom = fs(st[upper].offset, st[lower].offset);
        if (denom == 0.0f) {
            out = st[lower].color;
        } else {
            float ratio = fd(fs(t, st[lower].offset), denom);
            ratio = ratio < 1.0f ? ratio : 1.0f;
            ratio = ratio < 0.0f ? 0.0f : (ratio > 1.0f ? 1.0f : ratio);
            const float factor = fd(1.0f, 255.0f);
            for (int k = 0; k < 4; k++) {
                const float a = fm((float)((st[lower].color >> (8 * k)) & 0xffu), factor);
                const float c = fm((float)((st[upper].color >> (8 * k)) & 0xffu), factor);
                const float v = fa(a, fm(fs(c, a), ratio));
                out |= (uint32_t)(uint8_t)fm(v, 255.0f) << (8 * k);
            }
        }
    }
    ramps[(size_t)g * 256 + x] = out;
    if (x != 0) return;
    float m[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (pp.type == PF_PAINT_LINEAR) {
        const float fx = pp.line[0], fy = pp.line[1];
        const float dx = fs(pp.line[2], fx), dy = fs(pp.line[3], fy);
        const float sq = fa(fm(dx, dx), fm(dy, dy));
        const float m0x = fd(dx, sq), m0y = fd(dy, sq);
        m[0] = half_trunc(m0x);
        m[2] = half_trunc(m0y);
        m[4] = half_trunc(fa(fm(m0x, -fx), fm(m0y, -fy)));
    } else if (pp.type == PF_PAINT_RADIAL) {
        const float *tr = pp.transform;
        const float det = fs(fm(tr[0], tr[3]), fm(tr[1], tr[2]));
        const float s = fd(1.0f, det);
        const float a = fm(fm(tr[3], 1.0f), s), b = fm(fm(tr[1], -1.0f), s), c = fm(fm(tr[2], -1.0f), s),
                    d = fm(fm(tr[0], 1.0f), s);
        m[0] = half_trunc(a);
        m[1] = half_trunc(b);
        m[2] = half_trunc(c);
        m[3] = half_trunc(d);
        m[4] = half_trunc(-fa(fm(a, tr[4]), fm(c, tr[5])));
        m[5] = half_trunc(-fa(fm(b, tr[4]), fm(d, tr[5])));
        m[6] = half_trunc(pp.line[0]);
        m[7] = half_trunc(pp.line[1]);
        m[8] = half_trunc(fs(pp.line[2], pp.line[0]));
        m[9] = half_trunc(fs(pp.line[3], pp.line[1]));
        m[10] = half_trunc(pp.radii[0]);
        m[11] = half_trunc(pp.radii[1]);
    }
    bool opaque = cnt > 0;  // Gradient::is_opaque (the base colour is opaque white)
    for (uint32_t i = 0; i < cnt; i++) opaque &= (st[i].color >> 24) == 0xffu;
    float4 *r = meta + 4 * (size_t)g;
    r[0] = make_float4(m[0], m[1], m[2], m[3]);
    r[1] = make_float4(m[4], m[5], m[6], m[7]);
    r[2] = make_float4(m[8], m[9], m[10], m[11]);
    r[3] = make_float4(__uint_as_float(pp.type), __uint_as_float(pp.wrap), __uint_as_float(opaque ? 1u : 0u), 0.0f);
}

}  // namespace

cudaError_t launch_gradient_index(const pf_paint *paints, uint32_t n_paths, uint32_t *flags, uint32_t *path_grad,
                                  uint32_t *grad_path, void *scan_temp, uint32_t *status, cudaStream_t st) {
    if (!n_paths) return cudaSuccess;
    const uint32_t blocks = (n_paths + 255) / 256;
    k_gradient_flags<<<blocks, 256, 0, st>>>(paints, n_paths, flags);
    cudaError_t e = scan_exclusive_u32(flags, flags, n_paths, flags + n_paths, scan_temp, st, status + kStErr);
    if (e != cudaSuccess) return e;
    k_gradient_index<<<blocks, 256, 0, st>>>(paints, n_paths, flags, path_grad, grad_path);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t launch_gradients(const pf_paint *paints, const uint32_t *grad_path, const uint32_t *scene_path_first,
                             uint32_t n_scenes, const uint32_t *stop_base, const pf_color_stop *stops, uint32_t n,
                             float4 *meta, uint32_t *ramps, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_gradients<<<n, 256, 0, st>>>(paints, grad_path, scene_path_first, n_scenes, stop_base, stops, n, meta, ramps);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace pfc
