// pf_sizer.cu - the learned per-path sizer: features, a 12 -> 64 -> 64 -> 2 MLP
// (bf16 weights, fp32 accumulation), and its training kernels (forward, backward, Adam).
//
// The reference sizes its microline and fill buffers by running dice/bin, reading the
// count back and re-running on overflow (pathfinder/core/d3d11/renderer.cpp:540-577,
// 707-724, 834-845).  The sizer predicts, per path, log1p(leaf lines) and log1p(fills)
// from cheap geometric features, so a frame can lay out per-path leaf regions and fill
// capacity before flattening, in one pass; the exact count-then-allocate frame remains
// the fallback when a prediction overflows.
#include <math.h>

#include "pf_internal.h"

namespace pfc {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t global_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ float leg_len(float2 a, float2 b) {
    const float dx = b.x - a.x, dy = b.y - a.y;
    return sqrtf(dx * dx + dy * dy);
}

// absolute turning angle between legs a->b and b->c
__device__ __forceinline__ float turn(float2 a, float2 b, float2 c) {
    const float ux = b.x - a.x, uy = b.y - a.y, vx = c.x - b.x, vy = c.y - b.y;
    const float cr = ux * vy - uy * vx, dt = ux * vx + uy * vy;
    if (cr == 0.0f && dt == 0.0f) return 0.0f;
    return fabsf(atan2f(cr, dt));
}

// Per contour: its point-flag counts, control-polygon length and summed turning angle
// (closed around the contour).  Paths sum them over their contours, so a path of thousands of
// contours (a dashed stroke's outline) costs its warp one strided pass over those sums.  A
// thread takes its contour alone up to kBigContour points; longer contours are taken by the
// whole warp afterwards, one at a time, so no thread walks thousands of points.
constexpr uint32_t kBigContour = 64;

__device__ __forceinline__ void point_terms(const Batch &b, uint32_t a, uint32_t n, uint32_t i, float &n_on,
                                            float &n_c0, float &n_c1, float &length, float &turning) {
    const uint8_t f = b.flags[a + i];
    n_on += f == 0;
    n_c0 += f == 1;
    n_c1 += f == 2;
    if (n > 1) {
        const float2 q0 = b.points[a + (i == 0 ? n - 1 : i - 1)], q1 = b.points[a + i],
                     q2 = b.points[a + (i + 1 == n ? 0 : i + 1)];
        length += leg_len(q1, q2);
        turning += turn(q0, q1, q2);
    }
}

__global__ void k_contour_features(Batch b, float4 *cf) {
    const uint32_t c = global_tid();
    const int lane = threadIdx.x & 31;
    const bool in = c < b.n_contours;
    uint32_t a = 0, n = 0;
    if (in) {
        a = b.contour_point_first[c];
        n = b.contour_point_first[c + 1] - a;
    }
    const bool big = in && n > kBigContour;
    if (in && !big) {
        float n_on = 0, n_c0 = 0, n_c1 = 0, length = 0, turning = 0;
        for (uint32_t i = 0; i < n; i++) point_terms(b, a, n, i, n_on, n_c0, n_c1, length, turning);
        cf[2 * (size_t)c] = make_float4(n_on, n_c0, n_c1, length);
        cf[2 * (size_t)c + 1] = make_float4(turning, 0.0f, 0.0f, 0.0f);
    }
    unsigned pending = __ballot_sync(0xffffffffu, big);
    while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t ba = __shfl_sync(0xffffffffu, a, src), bn = __shfl_sync(0xffffffffu, n, src);
        float n_on = 0, n_c0 = 0, n_c1 = 0, length = 0, turning = 0;
        for (uint32_t i = lane; i < bn; i += 32) point_terms(b, ba, bn, i, n_on, n_c0, n_c1, length, turning);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            n_on += __shfl_xor_sync(0xffffffffu, n_on, d);
            n_c0 += __shfl_xor_sync(0xffffffffu, n_c0, d);
            n_c1 += __shfl_xor_sync(0xffffffffu, n_c1, d);
            length += __shfl_xor_sync(0xffffffffu, length, d);
            turning += __shfl_xor_sync(0xffffffffu, turning, d);
        }
        if (lane == src) {
            cf[2 * (size_t)c] = make_float4(n_on, n_c0, n_c1, length);
            cf[2 * (size_t)c + 1] = make_float4(turning, 0.0f, 0.0f, 0.0f);
        }
    }
}

// One warp per path: features from its contours' sums and its bounds / tile rect (after
// k_path_setup); they need no segment records, so they are ready before the first host
// synchronisation of a frame:
//   0 segments   1 lines   2 quadratics   3 cubics   4 contours   5 box width   6 box height
//   7 box area   8 control-polygon length   9 summed turning angle   10 tiles in the rect
//   11 even-odd flag
// (log1p of every count / length; the reference's outlines are already in canvas space, so
// the transform-scale feature is replaced by the tile count of the clipped rect).
__global__ void k_features(Batch b, const uint2 *path_contours, const float4 *cf, float *feat) {
    const uint32_t p = global_tid() >> 5;
    const int lane = threadIdx.x & 31;
    if (p >= b.n_paths) return;
    const uint2 cr = path_contours[p];
    float n_on = 0, n_c0 = 0, n_c1 = 0, length = 0, turning = 0;
    for (uint32_t c = cr.x + lane; c < cr.y; c += 32) {
        const float4 u = cf[2 * (size_t)c], v = cf[2 * (size_t)c + 1];
        n_on += u.x;
        n_c0 += u.y;
        n_c1 += u.z;
        length += u.w;
        turning += v.x;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        n_on += __shfl_xor_sync(0xffffffffu, n_on, d);
        n_c0 += __shfl_xor_sync(0xffffffffu, n_c0, d);
        n_c1 += __shfl_xor_sync(0xffffffffu, n_c1, d);
        length += __shfl_xor_sync(0xffffffffu, length, d);
        turning += __shfl_xor_sync(0xffffffffu, turning, d);
    }
    if (lane != 0) return;
    const float4 bb = b.path_bounds[p];
    const float w = fmaxf(bb.z - bb.x, 0.0f), h = fmaxf(bb.w - bb.y, 0.0f);
    const PathDev P = b.paths[p];
    const float tiles = (float)max(P.rx1 - P.rx0, 0) * (float)max(P.ry1 - P.ry0, 0);
    const float n_cubic = n_c1, n_quad = fmaxf(n_c0 - n_c1, 0.0f), n_line = fmaxf(n_on - n_c0, 0.0f);
    float *f = feat + (size_t)p * kSizerIn;
    f[0] = log1pf(n_on);
    f[1] = log1pf(n_line);
    f[2] = log1pf(n_quad);
    f[3] = log1pf(n_cubic);
    f[4] = log1pf((float)(cr.y - cr.x));
    f[5] = log1pf(w);
    f[6] = log1pf(h);
    f[7] = log1pf(w * h);
    f[8] = log1pf(length);
    f[9] = log1pf(turning);
    f[10] = log1pf(tiles);
    f[11] = (P.flags & 1u) ? 1.0f : 0.0f;
}

// Per-path leaf budget (and fill estimate) from the sizer's prediction:
// budget = ceil(expm1(prediction) * mul + add), and at least the path's segment count: every
// segment yields at least one leaf, and a segment's first leaf goes to the slot of its own
// index in the path's region (k_flatten_pool), so the region's write cursor starts past them.
__global__ void k_budgets(Batch b, const float *pred, float mul, float add, uint32_t *leaf_budget,
                          uint32_t *fill_budget, uint32_t *leaf_cursor) {
    const uint32_t p = global_tid();
    if (p >= b.n_paths) return;
    const float l = fmaxf(expm1f(fminf(pred[2 * p + 0], 30.0f)), 0.0f);
    const float f = fmaxf(expm1f(fminf(pred[2 * p + 1], 30.0f)), 0.0f);
    const uint2 cr = b.path_contours[p];
    const uint32_t n_segs = b.contour_segs[cr.y] - b.contour_segs[cr.x];
    leaf_budget[p] = max((uint32_t)fminf(ceilf(l * mul + add), 1.0e9f), n_segs);
    fill_budget[p] = (uint32_t)fminf(ceilf(f * mul + add), 1.0e9f);
    leaf_cursor[p] = n_segs;
}

// Exact per-path counts of the last exact frame (training labels): leaf lines and fills.
__global__ void k_path_counts(Batch b, const uint2 *path_contours, uint32_t *leaves, uint32_t *fills) {
    const uint32_t p = global_tid();
    if (p >= b.n_paths) return;
    const uint2 cr = path_contours[p];
    const uint32_t s0 = b.contour_segs[cr.x], s1 = b.contour_segs[cr.y];
    leaves[p] = b.seg_leaves[s1] - b.seg_leaves[s0];
    const uint32_t t0 = b.path_tiles[p], t1 = b.path_tiles[p + 1];
    fills[p] = t1 > t0 ? b.tile_fills[t1 - 1] - b.path_fill[p] : 0u;
}

// ---------------------------------------------------------------------------
// MLP.  Parameter block layout (floats): W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2].

constexpr int kH = kSizerHidden, kI = kSizerIn, kO = kSizerOut;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kI, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kH * kH,
              kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kO * kH, kParams = kOffB3 + kO;
static_assert(kParams == kSizerParams, "parameter count");

// Weights are stored and used in bf16; accumulation is fp32.
__device__ __forceinline__ void load_params_smem(const __nv_bfloat16 *w, float *s) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) s[i] = __bfloat162float(w[i]);
    __syncthreads();
}

__device__ __forceinline__ void mlp_forward(const float *s, const float x[kI], float h1[kH], float h2[kH],
                                            float y[kO]) {
#pragma unroll 4
    for (int i = 0; i < kH; i++) {
        float a = s[kOffB1 + i];
#pragma unroll
        for (int k = 0; k < kI; k++) a += s[kOffW1 + i * kI + k] * x[k];
        h1[i] = fmaxf(a, 0.0f);
    }
#pragma unroll 2
    for (int i = 0; i < kH; i++) {
        float a = s[kOffB2 + i];
#pragma unroll 8
        for (int k = 0; k < kH; k++) a += s[kOffW2 + i * kH + k] * h1[k];
        h2[i] = fmaxf(a, 0.0f);
    }
#pragma unroll
    for (int o = 0; o < kO; o++) {
        float a = s[kOffB3 + o];
#pragma unroll 8
        for (int k = 0; k < kH; k++) a += s[kOffW3 + o * kH + k] * h2[k];
        y[o] = a;
    }
}

__global__ void __launch_bounds__(128) k_mlp_predict(const __nv_bfloat16 *w, const float *feat, uint32_t n,
                                                     float *out) {
    __shared__ float s[kParams];
    load_params_smem(w, s);
    const uint32_t i = global_tid();
    if (i >= n) return;
    float x[kI], h1[kH], h2[kH], y[kO];
#pragma unroll
    for (int k = 0; k < kI; k++) x[k] = feat[(size_t)i * kI + k];
    mlp_forward(s, x, h1, h2, y);
#pragma unroll
    for (int o = 0; o < kO; o++) out[(size_t)i * kO + o] = y[o];
}

// Training step, part 1: forward + backward of a mini-batch, weight gradients summed over
// the block's samples (a reduction over the batch dimension, no per-sample atomics) and
// added to the global gradient.  Loss: mean over samples and outputs of (y - t)^2.
constexpr int kTrainSamples = 64;  // samples per block

__global__ void __launch_bounds__(kTrainSamples) k_mlp_grad(const __nv_bfloat16 *w, const float *feat,
                                                            const float *target, const uint32_t *index,
                                                            uint32_t n, float inv_count, float *grad,
                                                            float *loss) {
    __shared__ float s[kParams];
    __shared__ float sx[kTrainSamples][kI];
    __shared__ float sh1[kTrainSamples][kH + 1];
    __shared__ float sh2[kTrainSamples][kH + 1];
    __shared__ float sd2[kTrainSamples][kH + 1];  // dL/d(pre-activation 2)
    __shared__ float sd1[kTrainSamples][kH + 1];  // dL/d(pre-activation 1)
    __shared__ float sdy[kTrainSamples][kO];
    load_params_smem(w, s);
    const int t = threadIdx.x;
    const uint32_t j = blockIdx.x * kTrainSamples + t;
    const bool valid = j < n;
    float x[kI], h1[kH], h2[kH], y[kO];
    float l = 0.0f;
    if (valid) {
        const uint32_t src = index ? index[j] : j;
#pragma unroll
        for (int k = 0; k < kI; k++) x[k] = feat[(size_t)src * kI + k];
        mlp_forward(s, x, h1, h2, y);
#pragma unroll
        for (int o = 0; o < kO; o++) {
            const float e = y[o] - target[(size_t)src * kO + o];
            l += e * e;
            sdy[t][o] = 2.0f * e * inv_count;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kI; k++) x[k] = 0.0f;
#pragma unroll
        for (int k = 0; k < kH; k++) h1[k] = h2[k] = 0.0f;
#pragma unroll
        for (int o = 0; o < kO; o++) sdy[t][o] = 0.0f;
    }
#pragma unroll
    for (int k = 0; k < kI; k++) sx[t][k] = x[k];
    for (int k = 0; k < kH; k++) {
        sh1[t][k] = h1[k];
        sh2[t][k] = h2[k];
    }
    // backprop through layer 3 and the ReLU of layer 2
    for (int k = 0; k < kH; k++) {
        float d = 0.0f;
#pragma unroll
        for (int o = 0; o < kO; o++) d += s[kOffW3 + o * kH + k] * sdy[t][o];
        sd2[t][k] = h2[k] > 0.0f ? d : 0.0f;
    }
    // backprop through layer 2 and the ReLU of layer 1
    for (int k = 0; k < kH; k++) {
        float d = 0.0f;
        for (int i = 0; i < kH; i++) d += s[kOffW2 + i * kH + k] * sd2[t][i];
        sd1[t][k] = h1[k] > 0.0f ? d : 0.0f;
    }
    __syncthreads();
    // weight gradients: every thread owns a strided set of parameters and sums over samples
    for (int q = t; q < kParams; q += kTrainSamples) {
        float g = 0.0f;
        if (q < kOffB1) {
            const int i = q / kI, k = q % kI;
            for (int m = 0; m < kTrainSamples; m++) g += sd1[m][i] * sx[m][k];
        } else if (q < kOffW2) {
            const int i = q - kOffB1;
            for (int m = 0; m < kTrainSamples; m++) g += sd1[m][i];
        } else if (q < kOffB2) {
            const int i = (q - kOffW2) / kH, k = (q - kOffW2) % kH;
            for (int m = 0; m < kTrainSamples; m++) g += sd2[m][i] * sh1[m][k];
        } else if (q < kOffW3) {
            const int i = q - kOffB2;
            for (int m = 0; m < kTrainSamples; m++) g += sd2[m][i];
        } else if (q < kOffB3) {
            const int o = (q - kOffW3) / kH, k = (q - kOffW3) % kH;
            for (int m = 0; m < kTrainSamples; m++) g += sdy[m][o] * sh2[m][k];
        } else {
            const int o = q - kOffB3;
            for (int m = 0; m < kTrainSamples; m++) g += sdy[m][o];
        }
        atomicAdd(&grad[q], g);
    }
    // loss (sum of squared errors; the caller divides)
    for (int d = 16; d > 0; d >>= 1) l += __shfl_xor_sync(0xffffffffu, l, d);
    if ((t & 31) == 0) atomicAdd(loss, l);
}

// Training step, part 2: Adam on fp32 master weights, bf16 copy for the next forward.
__global__ void k_adam(float *master, __nv_bfloat16 *w, float *grad, float *m, float *v, float lr, float beta1,
                       float beta2, float eps, float bc1, float bc2) {
    const int q = global_tid();
    if (q >= kParams) return;
    const float g = grad[q];
    const float mq = beta1 * m[q] + (1.0f - beta1) * g;
    const float vq = beta2 * v[q] + (1.0f - beta2) * g * g;
    m[q] = mq;
    v[q] = vq;
    const float upd = lr * (mq / bc1) / (sqrtf(vq / bc2) + eps);
    const float nw = master[q] - upd;
    master[q] = nw;
    w[q] = __float2bfloat16_rn(nw);
    grad[q] = 0.0f;
}

}  // namespace

cudaError_t launch_features(const Batch &b, const uint2 *path_contours, float4 *contour_scratch, float *feat,
                            cudaStream_t st) {
    if (b.n_paths) {
        if (b.n_contours) {
            k_contour_features<<<(b.n_contours + kThreads - 1) / kThreads, kThreads, 0, st>>>(b, contour_scratch);
            count_launches(1);
        }
        k_features<<<(unsigned)((uint64_t(b.n_paths) * 32 + kThreads - 1) / kThreads), kThreads, 0, st>>>(
            b, path_contours, contour_scratch, feat);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_budgets(const Batch &b, const float *pred, float mul, float add, uint32_t *leaf_budget,
                           uint32_t *fill_budget, uint32_t *leaf_cursor, cudaStream_t st) {
    if (b.n_paths) {
        k_budgets<<<(b.n_paths + kThreads - 1) / kThreads, kThreads, 0, st>>>(b, pred, mul, add, leaf_budget,
                                                                             fill_budget, leaf_cursor);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_path_counts(const Batch &b, const uint2 *path_contours, uint32_t *leaves, uint32_t *fills,
                               cudaStream_t st) {
    if (b.n_paths) {
        k_path_counts<<<(b.n_paths + kThreads - 1) / kThreads, kThreads, 0, st>>>(b, path_contours, leaves, fills);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict(const __nv_bfloat16 *w, const float *feat, uint32_t n, float *out, cudaStream_t st) {
    if (n) {
        k_mlp_predict<<<(n + 127) / 128, 128, 0, st>>>(w, feat, n, out);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const __nv_bfloat16 *w, const float *feat, const float *target, const uint32_t *index,
                            uint32_t n, float *grad, float *loss, cudaStream_t st) {
    if (n) {
        k_mlp_grad<<<(n + kTrainSamples - 1) / kTrainSamples, kTrainSamples, 0, st>>>(
            w, feat, target, index, n, 1.0f / (float)(n * kO), grad, loss);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_adam(float *master, __nv_bfloat16 *w, float *grad, float *m, float *v, float lr, int step,
                        cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    k_adam<<<(kParams + 255) / 256, 256, 0, st>>>(master, w, grad, m, v, lr, b1, b2, 1e-8f, bc1, bc2);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace pfc
