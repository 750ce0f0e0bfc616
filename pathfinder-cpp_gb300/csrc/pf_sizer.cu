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

// One warp per path: features from the path's segments (after k_contour_segments<write>)
// and its bounds / tile rect (after k_path_setup).
__global__ void k_features(Batch b, const uint2 *path_contours, const float4 *bounds, float *feat) {
    const uint32_t p = global_tid() >> 5;
    const int lane = threadIdx.x & 31;
    if (p >= b.n_paths) return;
    const uint2 cr = path_contours[p];
    const uint32_t s0 = b.contour_segs[cr.x], s1 = b.contour_segs[cr.y];
    float n_line = 0, n_quad = 0, n_cubic = 0, length = 0, turning = 0;
    for (uint32_t i = s0 + lane; i < s1; i += 32) {
        const SegDev sg = b.segs[i];
        const float2 p0 = b.points[sg.a];
        if (sg.kind == kSegLine || sg.kind == kSegClose) {
            n_line += 1;
            length += leg_len(p0, b.points[sg.kind == kSegClose ? sg.b : sg.a + 1]);
        } else if (sg.kind == kSegQuad) {
            n_quad += 1;
            const float2 c = b.points[sg.a + 1], p2 = b.points[sg.a + 2];
            length += leg_len(p0, c) + leg_len(c, p2);
            turning += turn(p0, c, p2);
        } else {
            n_cubic += 1;
            const float2 c0 = b.points[sg.a + 1], c1 = b.points[sg.a + 2], p3 = b.points[sg.a + 3];
            length += leg_len(p0, c0) + leg_len(c0, c1) + leg_len(c1, p3);
            turning += turn(p0, c0, c1) + turn(c0, c1, p3);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        n_line += __shfl_xor_sync(0xffffffffu, n_line, d);
        n_quad += __shfl_xor_sync(0xffffffffu, n_quad, d);
        n_cubic += __shfl_xor_sync(0xffffffffu, n_cubic, d);
        length += __shfl_xor_sync(0xffffffffu, length, d);
        turning += __shfl_xor_sync(0xffffffffu, turning, d);
    }
    if (lane != 0) return;
    const float4 bb = bounds[p];
    const float w = fmaxf(bb.z - bb.x, 0.0f), h = fmaxf(bb.w - bb.y, 0.0f);
    const PathDev P = b.paths[p];
    const float tiles = (float)max(P.rx1 - P.rx0, 0) * (float)max(P.ry1 - P.ry0, 0);
    float *f = feat + (size_t)p * kSizerIn;
    f[0] = log1pf(n_line + n_quad + n_cubic);
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

cudaError_t launch_features(const Batch &b, const uint2 *path_contours, const float4 *bounds, float *feat,
                            cudaStream_t st) {
    if (b.n_paths) {
        k_features<<<(unsigned)((uint64_t(b.n_paths) * 32 + kThreads - 1) / kThreads), kThreads, 0, st>>>(
            b, path_contours, bounds, feat);
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
