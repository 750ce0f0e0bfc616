// pf_kernels.cu - the stages of the GPU-driven fill pipeline for sm_103a.
//
// Stage map (reference -> here):
//   SegmentsD3D11::add_path / SegmentsIter   -> k_contour_segments (count + emit)
//   BuiltPath / round_rect_out_to_tile_bounds -> k_path_setup
//   dice.comp (here: the d3d9 recursive bisection, tiler.cpp:284-315)  -> k_flatten<count|write>
//   bin.comp (here: the d3d9 tile walk + add_fill, tiler.cpp:131-279,
//             object_builder.cpp:19-114),
//   bound.comp (tile records), propagate.comp / Tiler::prepare_tiles
//                                              -> k_bin_fused (one CTA per path: counts, backdrops,
//                                                 offsets, fills grouped by tile; no linked lists);
//                                                 k_bin_large* for rects too big for a CTA
//   sort.comp (z-culled per-framebuffer-tile lists)
//                                              -> k_rows (per framebuffer row: the spanning paths in
//                                                 path order) + the front-to-back walk of k_composite,
//                                                 which stops at the first occluder; k_list_dump
//                                                 writes the lists out for the canonical read-back
//   fill.comp + tile.comp                      -> k_composite (coverage never leaves the SM)
//   (learned frame) per-path budgets            -> pf_sizer.cu: k_features, k_mlp_predict, k_budgets;
//                                                 here k_flatten_pool and the spill-pool lists
//
// Integer outputs follow the reference's d3d9 CPU tiler bit for bit, so every float
// operation on that path is written with __f*_rn intrinsics (no FMA contraction), in the
// same order as the reference's SSE lanes (pathfinder/common/f32x4.h).
#include <algorithm>
#include <atomic>

#include "pf_internal.h"

namespace pfc {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

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

__device__ __forceinline__ uint32_t global_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

inline unsigned grid_for(uint64_t n, int threads = kThreads) {
    return static_cast<unsigned>((n + threads - 1) / threads);
}

// ---------------------------------------------------------------------------
// Normalisation: scene-local offsets -> global offsets.

__global__ void k_normalize_contours(Batch b) {
    const uint32_t c = global_tid();
    if (c >= b.n_contours) return;
    const uint32_t cg = b.contour_base + c;
    const uint32_t s = upper_bound(b.scene_contour_first, b.n_scenes_all + 1, cg) - 1;
    const SceneDev &S = b.scenes[s];
    const uint32_t local = cg - S.contour_first;
    b.contour_point_first[c] = S.point_first + b.contour_start_cat[S.cstart_base + local];
    if (c == b.n_contours - 1)
        b.contour_point_first[b.n_contours] = S.point_first + b.contour_start_cat[S.cstart_base + local + 1];
}

__global__ void k_normalize_paths(Batch b, uint2 *path_contours) {
    const uint32_t p = global_tid();
    if (p >= b.n_paths) return;
    const uint32_t pg = b.path_base + p;
    const uint32_t s = upper_bound(b.scene_path_first, b.n_scenes_all + 1, pg) - 1;
    const SceneDev &S = b.scenes[s];
    const uint32_t local = pg - S.path_first;
    const uint32_t c0 = S.contour_first + b.path_start_cat[S.pstart_base + local] - b.contour_base;
    const uint32_t c1 = S.contour_first + b.path_start_cat[S.pstart_base + local + 1] - b.contour_base;
    path_contours[p] = make_uint2(c0, c1);
    for (uint32_t c = c0; c < c1; c++) b.contour_path[c] = p;
    PathDev P{};
    P.scene = s;
    // occludes: an opaque paint (PaintMetadata::is_opaque): an opaque colour, or a gradient
    // whose stops are all opaque
    bool opaque = (b.color[pg] >> 24) == 0xffu;
    if (b.path_grad && b.path_grad[pg] != kNone) opaque = __float_as_uint(b.grad_meta[4 * b.path_grad[pg] + 3].z) != 0;
    P.flags = (b.fill_rule[pg] ? 1u : 0u) | (opaque ? 2u : 0u);
    if (b.path_clip_cat) {
        // clip paths are tiled like the others but never drawn; a clipped path's clip is in its
        // scene, addressed here within the frame
        if (b.path_is_clip_cat[pg]) P.flags |= kPathIsClip;
        const uint32_t lc = b.path_clip_cat[pg];
        b.path_clip_rel[p] = lc == kNone ? kNone : S.path_first - b.path_base + lc;
    }
    b.paths[p] = P;
}

// ---------------------------------------------------------------------------
// Per-path bounds and tile rect (one warp per path).
// Outline::bounds (pathfinder/core/data/path.cpp), RectF::intersection and
// round_rect_out_to_tile_bounds (pathfinder/core/data/data.h:131-133), Tiler::Tiler
// (pathfinder/core/d3d9/tiler.cpp:317-335).

__global__ void k_path_setup(Batch b, const uint2 *path_contours) {
    const uint32_t p = global_tid() >> 5;
    const int lane = threadIdx.x & 31;
    if (p >= b.n_paths) return;
    const uint2 cr = path_contours[p];
    const uint32_t a = b.contour_point_first[cr.x], e = b.contour_point_first[cr.y];
    float l = INFINITY, t = INFINITY, r = -INFINITY, bt = -INFINITY;
    bool bad = false;
    for (uint32_t i = a + lane; i < e; i += 32) {
        const float2 q = b.points[i];
        bad |= !(isfinite(q.x) && isfinite(q.y));
        l = fminf(l, q.x);
        t = fminf(t, q.y);
        r = fmaxf(r, q.x);
        bt = fmaxf(bt, q.y);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        l = fminf(l, __shfl_xor_sync(0xffffffffu, l, d));
        t = fminf(t, __shfl_xor_sync(0xffffffffu, t, d));
        r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, d));
        bt = fmaxf(bt, __shfl_xor_sync(0xffffffffu, bt, d));
    }
    bad = __any_sync(0xffffffffu, bad);
    if (lane != 0) return;
    if (bad) atomicOr(&b.status[kStErr], kErrNonFinite);
    PathDev P = b.paths[p];
    const SceneDev &S = b.scenes[P.scene];
    float il, it, ir, ib;
    if (e == a) {  // no points: the default (invalid) RectF {1, 1, 0, 0}
        l = 1.0f;
        t = 1.0f;
        r = 0.0f;
        bt = 0.0f;
    }
    // RectF::intersection with the view box (common/math/rect.h:160-172)
    if (l > S.vb_right || r < S.vb_left || t > S.vb_bottom || bt < S.vb_top) {
        il = 1.0f;
        it = 1.0f;
        ir = 0.0f;
        ib = 0.0f;
    } else {
        il = l < S.vb_left ? S.vb_left : l;
        it = t < S.vb_top ? S.vb_top : t;
        ir = S.vb_right < r ? S.vb_right : r;
        ib = S.vb_bottom < bt ? S.vb_bottom : bt;
    }
    b.path_bounds[p] = make_float4(l, t, r, bt);
    const float inv = 1.0f / kTile;
    P.rx0 = (int32_t)floorf(fmul(il, inv));
    P.ry0 = (int32_t)floorf(fmul(it, inv));
    P.rx1 = (int32_t)ceilf(fmul(ir, inv));
    P.ry1 = (int32_t)ceilf(fmul(ib, inv));
    const int32_t w = max(P.rx1 - P.rx0, 0), h = max(P.ry1 - P.ry0, 0);
    b.paths[p] = P;
    b.path_tiles[p] = (uint32_t)(w * h);
    b.path_cols[p] = (uint32_t)w;
}

__global__ void k_path_offsets(Batch b) {
    const uint32_t p = global_tid();
    if (p >= b.n_paths) return;
    b.paths[p].tile_first = b.path_tiles[p];
    b.paths[p].col_first = b.path_cols[p];
}

// ---------------------------------------------------------------------------
// Segments of a contour, as SegmentsIter::get_next(force_closed = true) yields them
// (pathfinder/core/data/contour.cpp:110-175): stop at the first malformed point pattern;
// at the end, an implicit closing line unless first ~= last within 1e-4.

template <bool kWrite>
__global__ void k_contour_segments(Batch b) {
    const uint32_t c = global_tid();
    if (c >= b.n_contours) return;
    const uint32_t a = b.contour_point_first[c], n = b.contour_point_first[c + 1] - a;
    const uint8_t *fl = b.flags + a;
    uint32_t out = 0, path = 0;
    if (kWrite) {
        out = b.contour_segs[c];
        path = b.contour_path[c];
        if (out > b.seg_cap) return;
    }
    uint32_t count = 0, head = 0;
    auto emit = [&](uint32_t kind, uint32_t first, uint32_t second) {
        if (kWrite) {
            const uint32_t k = out + count;
            if (k < b.seg_cap) b.segs[k] = SegDev{first, second, kind, path};
            else atomicOr(&b.status[kStErr], kErrOverflowSeg);
        }
        count++;
    };
    if (n != 0) {
        for (;;) {
            if (head >= n || fl[head] != 0) break;
            if (head + 1 < n) {
                const uint8_t f1 = fl[head + 1];
                if (f1 == 0) {
                    emit(kSegLine, a + head, 0);
                    head += 1;
                } else if (head + 2 < n) {
                    const uint8_t f2 = fl[head + 2];
                    if (f1 == 1 && f2 == 0) {
                        emit(kSegQuad, a + head, 0);
                        head += 2;
                    } else if (head + 3 < n) {
                        if (f1 == 1 && f2 == 2 && fl[head + 3] == 0) {
                            emit(kSegCubic, a + head, 0);
                            head += 3;
                        } else {
                            break;
                        }
                    } else {
                        break;
                    }
                } else {
                    break;
                }
            } else {
                if (n > 1) {
                    const float2 f = b.points[a], l = b.points[a + n - 1];
                    const float dx = fsub(f.x, l.x), dy = fsub(f.y, l.y);
                    const float len = __fsqrt_rn(fadd(fmul(dx, dx), fmul(dy, dy)));
                    if (!(len <= 0.0001f)) emit(kSegClose, a + n - 1, a);
                }
                break;
            }
        }
    }
    if (!kWrite) b.contour_segs[c] = count;
}

// ---------------------------------------------------------------------------
// Flattening: the d3d9 recursive bisection (process_segment, tiler.cpp:284-315) run
// depth first with an explicit stack, so leaves come out in the reference's order.
// Segment::is_flat_cubic (segment.cpp:12-20), is_flat_quadratic (:22-36), split_cubic
// at t = 0.5 (:42-100) and split_quadratic (:102-126), with the same operation order.

__device__ __forceinline__ bool flat_cubic(const float bb[4], const float cc[4]) {
    const float bz[4] = {bb[2], bb[3], bb[0], bb[1]};
    float uv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float t = fmul(3.0f, cc[k]);
        t = fsub(t, bb[k]);
        t = fsub(t, bb[k]);
        t = fsub(t, bz[k]);
        uv[k] = fmul(t, t);
    }
    const float m0 = uv[0] > uv[2] ? uv[0] : uv[2];
    const float m1 = uv[1] > uv[3] ? uv[1] : uv[3];
    return fadd(m0, m1) <= 1.0f;
}

__device__ __forceinline__ bool flat_quad(const float bb[4], const float cc[2]) {
    const float mx = fmul(fadd(bb[0], bb[2]), 0.5f), my = fmul(fadd(bb[1], bb[3]), 0.5f);
    const float dx = fsub(cc[0], mx), dy = fsub(cc[1], my);
    return fadd(fmul(dx, dx), fmul(dy, dy)) <= 0.25f;
}

__device__ __forceinline__ float half_lerp(float a, float b) { return fadd(a, fmul(0.5f, fsub(b, a))); }

// The stack of pending second halves is kept small, as it lives in local memory: an entry
// holds a half's start point and control points only.  A half ends where the half pushed
// before it (the entry below) begins, or at the segment's end for the bottom entry, because
// each split pushes the second half of the current piece, whose end is the current piece's.
// Depths need no slot either: the path from the root has at most one pending half per depth,
// so a bit mask of pending depths gives the top entry's depth (its highest bit).

template <class Emit>
__device__ void flatten_cubic(float b0, float b1, float b2, float b3, float c0, float c1, float c2, float c3,
                              Emit &&emit, uint32_t *status, int depth0 = 0) {
    float4 sa[kMaxDepth];  // start x, y, first control x, y
    float2 sb[kMaxDepth];  // second control x, y
    uint32_t pending = 0;
    int sp = 0;
    float bb[4] = {b0, b1, b2, b3}, cc[4] = {c0, c1, c2, c3};
    int depth = depth0;
    for (;;) {
        if (depth >= kMaxDepth - 1 || flat_cubic(bb, cc)) {
            if (depth >= kMaxDepth - 1) atomicOr(status, kErrDepth);
            emit(bb[0], bb[1], bb[2], bb[3]);
            if (sp == 0) return;
            sp--;
            const float4 a = sa[sp];
            const float2 c = sb[sp];
            bb[0] = a.x;
            bb[1] = a.y;
            cc[0] = a.z;
            cc[1] = a.w;
            cc[2] = c.x;
            cc[3] = c.y;
            if (sp > 0) {
                const float4 below = sa[sp - 1];
                bb[2] = below.x;
                bb[3] = below.y;
            } else {
                bb[2] = b2;
                bb[3] = b3;
            }
            depth = 31 - __clz(pending);
            pending &= ~(1u << depth);
            continue;
        }
        float p01[2], p12[2], p23[2], p012[2], p123[2], p0123[2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            p01[k] = half_lerp(bb[k], cc[k]);
            p12[k] = half_lerp(cc[k], cc[2 + k]);
            p23[k] = half_lerp(cc[2 + k], bb[2 + k]);
            p012[k] = half_lerp(p01[k], p12[k]);
            p123[k] = half_lerp(p12[k], p23[k]);
            p0123[k] = half_lerp(p012[k], p123[k]);
        }
        // push the second half, continue with the first
        sa[sp] = make_float4(p0123[0], p0123[1], p123[0], p123[1]);
        sb[sp] = make_float2(p23[0], p23[1]);
        sp++;
        depth++;
        pending |= 1u << depth;
        bb[2] = p0123[0];
        bb[3] = p0123[1];
        cc[0] = p01[0];
        cc[1] = p01[1];
        cc[2] = p012[0];
        cc[3] = p012[1];
    }
}

template <class Emit>
__device__ void flatten_quad(float b0, float b1, float b2, float b3, float c0, float c1, Emit &&emit,
                             uint32_t *status, int depth0 = 0) {
    float4 sa[kMaxDepth];  // start x, y, control x, y
    uint32_t pending = 0;
    int sp = 0;
    float bb[4] = {b0, b1, b2, b3}, cc[2] = {c0, c1};
    int depth = depth0;
    for (;;) {
        if (depth >= kMaxDepth - 1 || flat_quad(bb, cc)) {
            if (depth >= kMaxDepth - 1) atomicOr(status, kErrDepth);
            emit(bb[0], bb[1], bb[2], bb[3]);
            if (sp == 0) return;
            sp--;
            const float4 a = sa[sp];
            bb[0] = a.x;
            bb[1] = a.y;
            cc[0] = a.z;
            cc[1] = a.w;
            if (sp > 0) {
                const float4 below = sa[sp - 1];
                bb[2] = below.x;
                bb[3] = below.y;
            } else {
                bb[2] = b2;
                bb[3] = b3;
            }
            depth = 31 - __clz(pending);
            pending &= ~(1u << depth);
            continue;
        }
        float a[2], q[2], m[2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            a[k] = fadd(bb[k], fmul(fsub(cc[k], bb[k]), 0.5f));
            q[k] = fadd(cc[k], fmul(fsub(bb[2 + k], cc[k]), 0.5f));
            m[k] = fadd(a[k], fmul(fsub(q[k], a[k]), 0.5f));
        }
        sa[sp] = make_float4(m[0], m[1], q[0], q[1]);
        sp++;
        depth++;
        pending |= 1u << depth;
        bb[2] = m[0];
        bb[3] = m[1];
        cc[0] = a[0];
        cc[1] = a[1];
    }
}

// Segment order for the flattening kernels.  A warp's lanes flatten 32 segments in step, so
// its time is its largest segment's.  Segments are bucketed by sixteenths of the depth a
// uniform bisection would need, ceil(4 log2 of the root's flatness value) - the value shrinks
// about 16-fold per level - and the kernels take them bucket by bucket, deepest first, so a
// warp's segments have like leaf counts, and the learned frame's leaf regions get runs of like
// lines, which the binning walk takes 32 at a time.  (512-scene frame, flattening + binning:
// whole levels 6.28 + 20.66 ms, quarters 5.92 + 20.44 ms, eighths 5.90 + 20.18 ms, sixteenths
// 5.98 + 20.02 ms.)  The order changes no output: every segment writes its own leaf range (exact
// frame) or reserves slots in its path's region (learned frame).
constexpr int kSegBuckets = 256;

__device__ __forceinline__ int seg_bucket(const Batch &b, const SegDev &sg) {
    if (sg.kind == kSegLine || sg.kind == kSegClose) return 0;
    const float2 p0 = b.points[sg.a], c0 = b.points[sg.a + 1], c1 = b.points[sg.a + 2];
    float m;
    if (sg.kind == kSegQuad) {
        const float dx = c0.x - 0.5f * (p0.x + c1.x), dy = c0.y - 0.5f * (p0.y + c1.y);
        m = 4.0f * (dx * dx + dy * dy);
    } else {
        const float2 p3 = b.points[sg.a + 3];
        const float ux = 3.0f * c0.x - 2.0f * p0.x - p3.x, uy = 3.0f * c0.y - 2.0f * p0.y - p3.y;
        const float vx = 3.0f * c1.x - 2.0f * p3.x - p0.x, vy = 3.0f * c1.y - 2.0f * p3.y - p0.y;
        m = fmaxf(ux * ux, vx * vx) + fmaxf(uy * uy, vy * vy);
    }
    if (!(m > 1.0f)) return 0;  // also NaN
    const int d = (int)ceilf(__log2f(m) * 4.0f);
    return d < kSegBuckets - 1 ? d : kSegBuckets - 1;
}

// A fixed grid of kSegBlocks blocks walks the segments grid-stride.  The count pass leaves
// each block's per-bucket counts in ctl[kSegBuckets * block + bucket]; the totals and starts
// kernels turn them into each block's first slot per bucket (buckets deepest first); the scatter
// pass walks the same segments and places them from those slots.  Counters live in shared
// memory: no global atomics (one hot global counter per bucket serialised millions of them).
constexpr int kSegBlocks = 1216;  // 8 blocks per SM of 152

template <bool kScatter>
__global__ void __launch_bounds__(kThreads) k_seg_buckets(Batch b, uint32_t *ctl) {
    __shared__ uint32_t s_cnt[kSegBuckets];
    const uint32_t n = b.status[kStSegs];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < kSegBuckets)
        s_cnt[threadIdx.x] = kScatter ? ctl[kSegBuckets * blockIdx.x + threadIdx.x] : 0u;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const int bk = i < n ? seg_bucket(b, b.segs[i]) : -1;
        const unsigned group = __match_any_sync(0xffffffffu, bk);
        const int leader = __ffs(group) - 1;
        uint32_t slot = 0;
        if (bk >= 0 && lane == leader) slot = atomicAdd(&s_cnt[bk], (uint32_t)__popc(group));
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (kScatter && bk >= 0) b.seg_order[slot + __popc(group & ((1u << lane) - 1u))] = i;
    }
    __syncthreads();
    if (!kScatter && threadIdx.x < kSegBuckets) ctl[kSegBuckets * blockIdx.x + threadIdx.x] = s_cnt[threadIdx.x];
}

// Each bucket's total over the blocks (one CTA per bucket), stored after the per-block counts.
__global__ void __launch_bounds__(kThreads) k_seg_bucket_totals(uint32_t *ctl) {
    __shared__ uint32_t red[kThreads / 32];
    const int bk = blockIdx.x, tid = threadIdx.x;
    uint32_t t = 0;
    for (int blk = tid; blk < kSegBlocks; blk += kThreads) t += ctl[kSegBuckets * blk + bk];
    t = __reduce_add_sync(0xffffffffu, t);
    if ((tid & 31) == 0) red[tid >> 5] = t;
    __syncthreads();
    if (tid == 0) {
        uint32_t sum = 0;
        for (int w = 0; w < kThreads / 32; w++) sum += red[w];
        ctl[kSegBuckets * kSegBlocks + bk] = sum;
    }
}

// Every block's first slot per bucket, buckets deepest first (one CTA per bucket): the deeper
// buckets' totals, then an exclusive scan of the bucket's per-block counts.
__global__ void __launch_bounds__(kThreads) k_seg_bucket_starts(uint32_t *ctl) {
    constexpr int kPer = (kSegBlocks + kThreads - 1) / kThreads;  // blocks per thread
    __shared__ uint32_t red[kThreads / 32];
    __shared__ uint32_t s_base;
    const int bk = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t *total = ctl + kSegBuckets * kSegBlocks;
    uint32_t deeper = 0;
    for (int k = bk + 1 + tid; k < kSegBuckets; k += kThreads) deeper += total[k];
    deeper = __reduce_add_sync(0xffffffffu, deeper);
    if (lane == 0) red[warp] = deeper;
    __syncthreads();
    if (tid == 0) {
        uint32_t sum = 0;
        for (int w = 0; w < kThreads / 32; w++) sum += red[w];
        s_base = sum;
    }
    uint32_t v[kPer];
    uint32_t own = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const int blk = tid * kPer + j;
        v[j] = blk < kSegBlocks ? ctl[kSegBuckets * blk + bk] : 0u;
        own += v[j];
    }
    uint32_t incl = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    __syncthreads();  // red is reused
    if (lane == 31) red[warp] = incl;
    __syncthreads();
    uint32_t before = s_base;
    for (int w = 0; w < warp; w++) before += red[w];
    uint32_t run = before + incl - own;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const int blk = tid * kPer + j;
        if (blk < kSegBlocks) ctl[kSegBuckets * blk + bk] = run;
        run += v[j];
    }
}

template <bool kWrite>
__global__ void __launch_bounds__(kThreads) k_flatten(Batch b, uint32_t n_segs) {
    const uint32_t t = global_tid();
    if (t >= n_segs || t >= b.status[kStSegs]) return;
    if (kWrite && b.status[kStLeaves] > b.leaf_cap) {
        if (t == 0) atomicOr(&b.status[kStErr], kErrOverflowLeaf);
        return;
    }
    const uint32_t i = b.seg_order ? b.seg_order[t] : t;
    const SegDev sg = b.segs[i];
    uint32_t out = kWrite ? b.seg_leaves[i] : 0u;
    uint32_t count = 0;
    auto emit = [&](float x0, float y0, float x1, float y1) {
        if (kWrite) b.leaves[out + count] = make_float4(x0, y0, x1, y1);
        count++;
    };
    const float2 p0 = b.points[sg.a];
    switch (sg.kind) {
        case kSegLine: {
            const float2 p1 = b.points[sg.a + 1];
            emit(p0.x, p0.y, p1.x, p1.y);
        } break;
        case kSegClose: {
            const float2 p1 = b.points[sg.b];
            emit(p0.x, p0.y, p1.x, p1.y);
        } break;
        case kSegQuad: {
            const float2 c = b.points[sg.a + 1], p2 = b.points[sg.a + 2];
            flatten_quad(p0.x, p0.y, p2.x, p2.y, c.x, c.y, emit, &b.status[kStErr]);
        } break;
        default: {
            const float2 c0 = b.points[sg.a + 1], c1 = b.points[sg.a + 2], p3 = b.points[sg.a + 3];
            flatten_cubic(p0.x, p0.y, p3.x, p3.y, c0.x, c0.y, c1.x, c1.y, emit, &b.status[kStErr]);
        } break;
    }
    if (!kWrite) b.seg_leaves[i] = count;
}

// ---------------------------------------------------------------------------
// Binning: the d3d9 tile walk of one leaf line (process_line_segment, tiler.cpp:131-279),
// with clip_line_segment_to_rect (:46-125, clip box top = -inf), ObjectBuilder::add_fill
// (object_builder.cpp:19-64: cull outside the tile rect, x256 local coordinates, clamp to
// [0, 4095], round half to even, cull vertical) and adjust_alpha_tile_backdrop (:96-114).

struct WalkCtx {
    int32_t rx0, ry0, rx1, ry1, rw, rh;
    float vb_left, vb_right, vb_bottom;  // the clip box: the view box with its top at -infinity
};

__device__ __forceinline__ int outcode(const WalkCtx &w, float x, float y) {
    int o = 0;
    if (x < w.vb_left) o |= 1;
    else if (x > w.vb_right) o |= 2;
    if (y > w.vb_bottom) o |= 8;
    return o;
}

__device__ __forceinline__ float lerp_clamped(float a, float b, float t) {
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return fadd(a, fmul(fsub(b, a), t));
}

__device__ __forceinline__ int clip_line(const WalkCtx &w, float &x0, float &y0, float &x1, float &y1,
                                         uint32_t *status) {
    int of = outcode(w, x0, y0), ot = outcode(w, x1, y1);
    for (int iter = 0; iter < 64; iter++) {
        if (of == 0 && ot == 0) return 1;
        if ((of & ot) != 0) return 0;
        const bool clip_from = of > ot;
        const int oc = clip_from ? of : ot;
        float px = clip_from ? x0 : x1, py = clip_from ? y0 : y1;
        if (oc & 1) {
            px = w.vb_left;
            py = lerp_clamped(y0, y1, fdiv(fsub(w.vb_left, x0), fsub(x1, x0)));
        } else if (oc & 2) {
            px = w.vb_right;
            py = lerp_clamped(y0, y1, fdiv(fsub(w.vb_right, x0), fsub(x1, x0)));
        } else if (oc & 8) {
            px = lerp_clamped(x0, x1, fdiv(fsub(w.vb_bottom, y0), fsub(y1, y0)));
            py = w.vb_bottom;
        }
        if (clip_from) {
            x0 = px;
            y0 = py;
            of = outcode(w, px, py);
        } else {
            x1 = px;
            y1 = py;
            ot = outcode(w, px, py);
        }
    }
    atomicOr(status, kErrClip);
    return 0;
}

// Quantise a piece of line in tile (tx, ty); returns false when add_fill culls it.
__device__ __forceinline__ bool quantise(const WalkCtx &w, float x0, float y0, float x1, float y1, int32_t tx,
                                         int32_t ty, uint2 &packed) {
    if (!(w.rx0 <= tx && tx <= w.rx1 - 1 && w.ry0 <= ty && ty <= w.ry1 - 1)) return false;
    const float ox = fmul((float)tx, 16.0f), oy = fmul((float)ty, 16.0f);
    float v[4] = {fmul(fsub(x0, ox), 256.0f), fmul(fsub(y0, oy), 256.0f), fmul(fsub(x1, ox), 256.0f),
                  fmul(fsub(y1, oy), 256.0f)};
    uint32_t q[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float c = v[k] > 0.0f ? v[k] : 0.0f;
        c = c < 4095.0f ? c : 4095.0f;
        q[k] = (uint32_t)rintf(c);
    }
    if (q[0] == q[2]) return false;
    packed = make_uint2(q[0] | (q[1] << 16), q[2] | (q[3] << 16));
    return true;
}

// Walk of one line, split into a set-up and steps.  A step has a decision - which tile
// boundary the line crosses next and at which parameter (crossing parameters accumulate, so
// decisions are sequential) - and an emission: the fill(s) and backdrop delta of the tile,
// which depend only on that step's decision and the one before.  on_fill(local_tile, packed)
// for every fill kept; on_delta(local_tile or -1 - column, delta) for every backdrop change
// that lands in the rect or above it.
struct WalkState {
    float x0, y0, vx, vy, tmx, tmy, tdx, tdy, curx, cury;
    int32_t tcx, tcy, ex, ey, sx, sy;
    int last;  // 0 none, 1 x, 2 y
    uint32_t it;
};

struct WalkStep {
    float curx, cury, nt;
    int32_t tcx, tcy;
    int last, next;
};

// False when nothing is left to step: a non-finite or clipped-away line, or a line inside one
// tile, whose single fill is emitted here.
template <class OnFill>
__device__ __forceinline__ bool walk_begin(const WalkCtx &w, float x0, float y0, float x1, float y1, WalkState &s,
                                           OnFill &&on_fill, uint32_t *status) {
    if (!(isfinite(x0) && isfinite(y0) && isfinite(x1) && isfinite(y1))) return false;
    if (!clip_line(w, x0, y0, x1, y1, status)) return false;
    const float inv = 1.0f / kTile;
    const int32_t fx = (int32_t)floorf(fmul(x0, inv)), fy = (int32_t)floorf(fmul(y0, inv));
    const int32_t ex = (int32_t)floorf(fmul(x1, inv)), ey = (int32_t)floorf(fmul(y1, inv));
    const float vx = fsub(x1, x0), vy = fsub(y1, y0);
    if (fx == ex && fy == ey) {
        // A line inside one tile: the walk would stop at its first step with t = 1 (the next
        // tile boundary in each direction lies beyond the end point, so both crossing
        // parameters are >= 1 or infinite), add the one fill from (x0, y0) to
        // (x0 + vx * 1, y0 + vy * 1), and neither an extra fill nor a backdrop delta.
        uint2 q;
        if (quantise(w, x0, y0, fadd(x0, vx), fadd(y0, vy), fx, fy, q))
            on_fill((fy - w.ry0) * w.rw + (fx - w.rx0), q);
        return false;
    }
    s.x0 = x0;
    s.y0 = y0;
    s.vx = vx;
    s.vy = vy;
    s.sx = vx < 0.0f ? -1 : 1;
    s.sy = vy < 0.0f ? -1 : 1;
    const float cx = fmul(fadd((float)fx, vx >= 0.0f ? 1.0f : 0.0f), 16.0f);
    const float cy = fmul(fadd((float)fy, vy >= 0.0f ? 1.0f : 0.0f), 16.0f);
    s.tmx = fdiv(fsub(cx, x0), vx);
    s.tmy = fdiv(fsub(cy, y0), vy);
    s.tdx = fabsf(fdiv(16.0f, vx));
    s.tdy = fabsf(fdiv(16.0f, vy));
    s.curx = x0;
    s.cury = y0;
    s.tcx = fx;
    s.tcy = fy;
    s.ex = ex;
    s.ey = ey;
    s.last = 0;
    s.it = 0;
    return true;
}

// The decision of the next step, which it records, and the walk state advanced past it;
// false once the line is done (or the step bound is hit).
__device__ __forceinline__ bool walk_decide(WalkState &s, WalkStep &r, uint32_t *status) {
    if (s.it >= kMaxWalk) {
        atomicOr(status, kErrWalk);
        r.next = -1;  // nothing to emit
        return false;
    }
    s.it++;
    int next;
    if (s.tmx < s.tmy) next = 1;
    else if (s.tmx > s.tmy) next = 2;
    else next = s.sx > 0 ? 1 : 2;
    float nt = next == 1 ? s.tmx : s.tmy;
    nt = (1.0f < nt) ? 1.0f : nt;
    if (s.tcx == s.ex && s.tcy == s.ey) next = 0;
    r.curx = s.curx;
    r.cury = s.cury;
    r.nt = nt;
    r.tcx = s.tcx;
    r.tcy = s.tcy;
    r.last = s.last;
    r.next = next;
    if (next == 1) {
        s.tmx = fadd(s.tmx, s.tdx);
        s.tcx += s.sx;
    } else if (next == 2) {
        s.tmy = fadd(s.tmy, s.tdy);
        s.tcy += s.sy;
    } else {
        return false;
    }
    s.curx = fadd(s.x0, fmul(s.vx, nt));
    s.cury = fadd(s.y0, fmul(s.vy, nt));
    s.last = next;
    return true;
}

// The fills and backdrop delta of one decided step.
template <class OnFill, class OnDelta>
__device__ __forceinline__ void walk_emit(const WalkCtx &w, const WalkState &s, const WalkStep &r, OnFill &&on_fill,
                                          OnDelta &&on_delta) {
    const float npx = fadd(s.x0, fmul(s.vx, r.nt)), npy = fadd(s.y0, fmul(s.vy, r.nt));
    const int32_t lx = r.tcx - w.rx0, ly = r.tcy - w.ry0;
    uint2 q;
    if (quantise(w, r.curx, r.cury, npx, npy, r.tcx, r.tcy, q)) on_fill(ly * w.rw + lx, q);
    if (s.sy < 0 && r.next == 2) {
        if (quantise(w, npx, npy, fmul((float)r.tcx, 16.0f), fmul((float)r.tcy, 16.0f), r.tcx, r.tcy, q))
            on_fill(ly * w.rw + lx, q);
    } else if (s.sy > 0 && r.last == 2) {
        if (quantise(w, fmul((float)r.tcx, 16.0f), fmul((float)r.tcy, 16.0f), r.curx, r.cury, r.tcx, r.tcy, q))
            on_fill(ly * w.rw + lx, q);
    }
    int delta = 0;
    if (s.sx < 0 && r.last == 1) delta = 1;
    else if (s.sx > 0 && r.next == 1) delta = -1;
    if (delta != 0 && lx >= 0 && lx < w.rw && ly < w.rh) {
        if (ly < 0) on_delta(-1 - lx, delta);
        else on_delta(ly * w.rw + lx, delta);
    }
}

// One lane walks one line.
template <class OnFill, class OnDelta>
__device__ void walk_line(const WalkCtx &w, float x0, float y0, float x1, float y1, OnFill &&on_fill,
                          OnDelta &&on_delta, uint32_t *status) {
    WalkState s;
    if (!walk_begin(w, x0, y0, x1, y1, s, on_fill, status)) return;
    for (;;) {
        WalkStep r;
        const bool more = walk_decide(s, r, status);
        if (r.next >= 0) walk_emit(w, s, r, on_fill, on_delta);
        if (!more) return;
    }
}

// The whole warp walks one (long) line: every lane runs the same sequence of decisions, lane
// j % 32 keeps step j, and the lanes emit their steps together, 32 steps per round.  The
// decisions are a few instructions each, the emissions (clip, quantise, fills) the bulk.
template <class OnFill, class OnDelta>
__device__ void walk_line_warp(const WalkCtx &w, float4 f, OnFill &&on_fill, OnDelta &&on_delta, uint32_t *status) {
    const int lane = threadIdx.x & 31;
    WalkState s;
    if (!walk_begin(w, f.x, f.y, f.z, f.w, s,
                    [&](int32_t local, uint2 q) {
                        if (lane == 0) on_fill(local, q);
                    },
                    status))
        return;
    bool more = true;
    while (more) {
        WalkStep mine;
        mine.next = -1;
#pragma unroll 1
        for (int j = 0; j < 32 && more; j++) {
            WalkStep r;
            more = walk_decide(s, r, status);
            if (j == lane) mine = r;
        }
        if (mine.next >= 0) walk_emit(w, s, mine, on_fill, on_delta);
        __syncwarp();
    }
}

// Flattening shared by the lanes of a warp, for both frames:
// * learned frame (kExact false): each path's leaf lines go to the path's region, laid out from
//   the sizer's budget; lines past the budget spill into the shared pool, and an exhausted pool
//   sets the overflow bit (the frame is then redone by the exact two-pass method);
// * exact frame's write pass (kExact true): each segment's lines go to its range of the leaf
//   buffer, counted by the count pass.
//
// The bisection is shared by the 32 lanes of a warp.  With one segment per lane (as the exact
// frame's k_flatten does) a warp runs the split branch and the emit branch of every step one after
// the other, with only the lanes on one side doing work in each (13 of 32 lanes active on the
// 512-scene batch, flattening 5.93 ms of the learned frame).  Here the lanes share the work of the
// warp's segments instead (flattening 4.54 ms):
//
// * a split round: each lane takes a pending (not flat) piece from the warp's pool in shared
//   memory, splits it at t = 0.5, and tests both halves: a flat half (or one at the depth bound)
//   joins the warp's leaf queue, the other goes back on the pool;
// * an emit round: each lane takes a queued leaf line and stores it.  Learned frame: the
//   segment's first leaf (its leftmost piece) at the segment's own slot in its path's region, the
//   others at slots reserved with one atomic per path among the round's lines (lanes grouped by
//   path) and stored one round later, so that the atomic's round trip overlaps the next split
//   round; lines past the budget go to the spill pool.  Exact frame: at the next slots of the
//   segment's range, from a counter in the warp's segment table (no global atomics).
//
// Every piece is split with the same operations as in the depth-first walk, so the leaf lines
// are the same lines bit for bit; only their order within a path's region differs, which no
// output depends on (fills are counted and placed per tile, coverage sums are integers).  The
// pool is a stack, so it stays near 32 pieces per level of the warp's deepest segments; a half
// that finds it full is flattened depth first by its lane alone (about 0.02% of the lines of the
// 512-scene batch, in a CPU model of this kernel).  Warps take their segments 32 at a time, in the bucketed order, from a
// frame-wide ticket, up to kPoolSets groups in flight: a group's slot in the segment table is
// reused once no pending piece or queued line refers to it.
constexpr int kPoolWarps = 2;     // warps per block
constexpr int kPoolCap = 224;     // pending pieces per warp
constexpr int kPoolLeafCap = 96;  // queued leaf lines per warp: < 32 before a round, + 2 per lane
constexpr int kPoolSets = 4;      // groups of 32 segments in flight per warp
// piece and line tags: bits 0-6 the segment's table entry (group * 32 + lane), bit 7 the
// segment's leftmost piece, bit 8 a cubic (else a quadratic), bits 9-13 the depth
constexpr uint32_t kTagEntry = 127u, kTagLeft = 1u << 7, kTagCubic = 1u << 8;
constexpr int kTagDepthShift = 9;

struct FlattenPool {
    float4 pend_ends[kPoolCap];   // x0, y0, x1, y1
    float4 pend_ctrl[kPoolCap];   // first control x, y, second control x, y (quadratic: first only)
    uint32_t pend_tag[kPoolCap];
    float4 leaf[kPoolLeafCap];    // x0, y0, x1, y1
    uint32_t leaf_tag[kPoolLeafCap];
    uint4 seg[kPoolSets * 32];    // learned frame: path, region, budget, own slot; exact frame:
                                  // the segment's first leaf slot and its lines stored so far
};

// Where a lane stores leaf lines by itself.
struct LeafSink {
    float4 *leaves;
    uint32_t *cursor, *status, *pool_path;
    uint32_t pool_first, pool_cap;
};

// A half that found the pool full: flattened depth first from its depth, its lines stored one
// slot at a time.  Returns the lines it produced.
__device__ __noinline__ uint32_t flatten_piece_alone(LeafSink out, uint4 sg, float4 ends, float4 ctrl, uint32_t tag) {
    bool left = (tag & kTagLeft) != 0;
    uint32_t produced = 0;
    auto emit = [&](float x0, float y0, float x1, float y1) {
        const float4 v = make_float4(x0, y0, x1, y1);
        produced++;
        if (left) {
            out.leaves[sg.w] = v;
            left = false;
            return;
        }
        const uint32_t slot = atomicAdd(&out.cursor[sg.x], 1u);
        if (slot < sg.z) {
            out.leaves[sg.y + slot] = v;
            return;
        }
        if (slot == sg.z) atomicAdd(&out.status[kStPathsOver], 1u);
        const uint32_t j = atomicAdd(&out.status[kStPoolUsed], 1u);
        if (j < out.pool_cap) {
            out.leaves[out.pool_first + j] = v;
            out.pool_path[j] = sg.x;
        } else {
            atomicOr(&out.status[kStErr], kErrOverflowLeaf);
        }
    };
    const int depth = (int)(tag >> kTagDepthShift) & 31;
    if (tag & kTagCubic)
        flatten_cubic(ends.x, ends.y, ends.z, ends.w, ctrl.x, ctrl.y, ctrl.z, ctrl.w, emit, &out.status[kStErr],
                      depth);
    else
        flatten_quad(ends.x, ends.y, ends.z, ends.w, ctrl.x, ctrl.y, emit, &out.status[kStErr], depth);
    return produced;
}

// The same for the exact frame: the segment's lines go to its range of the leaf buffer (from the
// count pass), the next slot taken from the segment's counter in the warp's table.
__device__ __noinline__ void flatten_piece_alone_exact(float4 *leaves, uint32_t leaf_cap, uint32_t *status,
                                                       uint32_t *stored, uint32_t first, float4 ends, float4 ctrl,
                                                       uint32_t tag) {
    auto emit = [&](float x0, float y0, float x1, float y1) {
        const uint32_t idx = first + atomicAdd(stored, 1u);
        if (idx < leaf_cap) leaves[idx] = make_float4(x0, y0, x1, y1);
        else atomicOr(&status[kStErr], kErrOverflowLeaf);
    };
    const int depth = (int)(tag >> kTagDepthShift) & 31;
    if (tag & kTagCubic)
        flatten_cubic(ends.x, ends.y, ends.z, ends.w, ctrl.x, ctrl.y, ctrl.z, ctrl.w, emit, &status[kStErr], depth);
    else
        flatten_quad(ends.x, ends.y, ends.z, ends.w, ctrl.x, ctrl.y, emit, &status[kStErr], depth);
}

__device__ __forceinline__ bool piece_flat(bool cubic, float4 e, float4 c) {
    const float bb[4] = {e.x, e.y, e.z, e.w}, cc[4] = {c.x, c.y, c.z, c.w};
    return cubic ? flat_cubic(bb, cc) : flat_quad(bb, cc);
}

template <bool kExact>
__global__ void __launch_bounds__(kPoolWarps * 32) k_flatten_pool(Batch b, uint32_t n_segs) {
    __shared__ FlattenPool pools[kPoolWarps];
    FlattenPool &W = pools[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    uint32_t *const err = &b.status[kStErr];
    if (kExact && b.status[kStLeaves] > b.leaf_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrOverflowLeaf);
        return;
    }
    n_segs = min(n_segs, b.status[kStSegs]);
    const uint32_t n_groups = (n_segs + 31u) / 32u;
    // a group of 32 segments: lane 0 takes the ticket, and the lanes read it when they need it,
    // so the atomic's round trip overlaps the work in between
    uint32_t ticket = lane == 0 ? atomicAdd(&b.status[kStFlatTicket], 1u) : 0u;
    auto current_group = [&]() { return __shfl_sync(~0u, ticket, 0); };
    int top = 0, nleaf = 0;  // pool and queue sizes (the same in every lane)
    uint32_t produced = 0;

    // An emit round reserves its lines' slots and stores them one round later: the reservation's
    // round trip overlaps the split rounds in between.  The lines waiting for their slots:
    bool held = false;                                   // this lane holds one
    float4 held_line = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t held_path = 0, held_region = 0, held_budget = 0;
    uint32_t held_first = 0;                             // the reservation's first slot (its leader lane)
    uint32_t held_count = 0, held_rank = 0;
    int held_leader = 0;
    auto store_held = [&]() {
        const unsigned held_mask = __ballot_sync(~0u, held);
        if (!held_mask) return;
        bool spill = false;
        if (held) {
            const uint32_t slot = __shfl_sync(held_mask, held_first, held_leader) + held_rank;
            if (lane == held_leader && held_first <= held_budget && held_first + held_count > held_budget)
                atomicAdd(&b.status[kStPathsOver], 1u);
            spill = slot >= held_budget;
            if (!spill) b.leaves[held_region + slot] = held_line;
        }
        const unsigned spill_mask = __ballot_sync(~0u, spill);
        if (spill_mask) {
            const int first = __ffs(spill_mask) - 1;
            uint32_t q = 0;
            if (lane == first) q = atomicAdd(&b.status[kStPoolUsed], (uint32_t)__popc(spill_mask));
            q = __shfl_sync(~0u, q, first);
            if (spill) {
                const uint32_t j = q + __popc(spill_mask & below);
                if (j < b.leaf_pool_cap) {
                    b.leaves[b.leaf_pool_first + j] = held_line;
                    b.pool_path[j] = held_path;
                } else {
                    atomicOr(err, kErrOverflowLeaf);
                }
            }
        }
        held = false;
    };

    // n (1..32) queued lines from the top of the queue, one per lane: a segment's leftmost line
    // goes to the segment's own slot, the others reserve slots (one atomic per path)
    auto emit_round = [&](int n) {
        if constexpr (kExact) {
            // exact frame: each segment's lines fill its counted range, slots taken from the
            // segment's counter by one lane per segment among the round's lines
            const bool act = lane < n;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            uint32_t entry = 0;
            if (act) {
                const int k = nleaf - 1 - lane;
                v = W.leaf[k];
                entry = W.leaf_tag[k] & kTagEntry;
            }
            nleaf -= n;
            const unsigned act_mask = __ballot_sync(~0u, act);
            if (act) {
                const unsigned same = __match_any_sync(act_mask, entry);
                const int leader = __ffs(same) - 1;
                uint32_t stored = 0;
                if (lane == leader) {
                    stored = W.seg[entry].y;
                    W.seg[entry].y = stored + __popc(same);
                }
                stored = __shfl_sync(act_mask, stored, leader);
                const uint32_t idx = W.seg[entry].x + stored + __popc(same & below);
                if (idx < b.leaf_cap) b.leaves[idx] = v;
                else atomicOr(err, kErrOverflowLeaf);
            }
            __syncwarp();
            return;
        }
        store_held();
        const bool act = lane < n;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint32_t tag = 0;
        uint4 sg = make_uint4(0u, 0u, 0u, 0u);
        if (act) {
            const int k = nleaf - 1 - lane;
            v = W.leaf[k];
            tag = W.leaf_tag[k];
            sg = W.seg[tag & kTagEntry];
        }
        nleaf -= n;
        produced += act ? 1u : 0u;
        const bool left = act && (tag & kTagLeft);
        if (left) b.leaves[sg.w] = v;
        held = act && !left;
        const unsigned held_mask = __ballot_sync(~0u, held);
        if (held) {
            const unsigned same = __match_any_sync(held_mask, sg.x);
            held_leader = __ffs(same) - 1;
            held_count = __popc(same);
            held_rank = __popc(same & below);
            if (lane == held_leader) held_first = atomicAdd(&b.path_leaf_cursor[sg.x], held_count);
            held_line = v;
            held_path = sg.x;
            held_region = sg.y;
            held_budget = sg.z;
        }
        __syncwarp();
    };
    auto drain = [&]() {
        while (nleaf >= 32) emit_round(32);
    };

    for (;;) {
        drain();
        if (top < 32 && current_group() < n_groups) {
            // a table group that no pending piece or queued line refers to
            uint32_t used = 0;
            for (int k = lane; k < top; k += 32) used |= 1u << ((W.pend_tag[k] & kTagEntry) >> 5);
            for (int k = lane; k < nleaf; k += 32) used |= 1u << ((W.leaf_tag[k] & kTagEntry) >> 5);
            used = __reduce_or_sync(~0u, used);
            if (used != (1u << kPoolSets) - 1u) {
                const uint32_t set = __ffs(~used) - 1;
                const uint32_t t = current_group() * 32u + (uint32_t)lane;
                const bool valid = t < n_segs;
                bool is_leaf = false, is_piece = false;
                float4 ends = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ctrl = ends;
                uint32_t tag = set * 32u + (uint32_t)lane | kTagLeft;
                if (valid) {
                    const uint32_t i = b.seg_order ? b.seg_order[t] : t;
                    const SegDev sg = b.segs[i];
                    if constexpr (kExact) {
                        W.seg[set * 32u + lane] = make_uint4(b.seg_leaves[i], 0u, 0u, 0u);
                    } else {
                        const uint32_t region = b.path_leaf_first[sg.path];
                        const uint32_t own = region + (i - b.contour_segs[b.path_contours[sg.path].x]);
                        W.seg[set * 32u + lane] = make_uint4(sg.path, region, b.path_leaf_budget[sg.path], own);
                    }
                    const float2 p0 = b.points[sg.a];
                    if (sg.kind == kSegLine || sg.kind == kSegClose) {
                        const float2 p1 = b.points[sg.kind == kSegLine ? sg.a + 1 : sg.b];
                        ends = make_float4(p0.x, p0.y, p1.x, p1.y);
                        is_leaf = true;
                    } else if (sg.kind == kSegQuad) {
                        const float2 c = b.points[sg.a + 1], p2 = b.points[sg.a + 2];
                        ends = make_float4(p0.x, p0.y, p2.x, p2.y);
                        ctrl = make_float4(c.x, c.y, 0.0f, 0.0f);
                    } else {
                        const float2 c0 = b.points[sg.a + 1], c1 = b.points[sg.a + 2], p3 = b.points[sg.a + 3];
                        ends = make_float4(p0.x, p0.y, p3.x, p3.y);
                        ctrl = make_float4(c0.x, c0.y, c1.x, c1.y);
                        tag |= kTagCubic;
                    }
                    if (!is_leaf) {
                        is_leaf = piece_flat(tag & kTagCubic, ends, ctrl);
                        is_piece = !is_leaf;
                    }
                }
                const unsigned leaf_mask = __ballot_sync(~0u, is_leaf), piece_mask = __ballot_sync(~0u, is_piece);
                // nleaf < 32 and top < 32 here: the group fits (checked all the same)
                if (is_leaf) {
                    const int k = nleaf + __popc(leaf_mask & below);
                    if (k < kPoolLeafCap) {
                        W.leaf[k] = ends;
                        W.leaf_tag[k] = tag;
                    } else {
                        atomicOr(err, kErrOverflowLeaf);
                    }
                }
                if (is_piece) {
                    const int k = top + __popc(piece_mask & below);
                    if (k < kPoolCap) {
                        W.pend_ends[k] = ends;
                        W.pend_ctrl[k] = ctrl;
                        W.pend_tag[k] = tag;
                    } else {
                        atomicOr(err, kErrOverflowLeaf);
                    }
                }
                nleaf = min(nleaf + __popc(leaf_mask), kPoolLeafCap);
                top = min(top + __popc(piece_mask), kPoolCap);
                __syncwarp();
                if (lane == 0) ticket = atomicAdd(&b.status[kStFlatTicket], 1u);
                drain();
            }
        }
        if (top == 0) {
            if (nleaf > 0) emit_round(nleaf);
            if (current_group() >= n_groups) break;
            continue;
        }

        // split round: up to 32 pieces from the top of the pool
        const int n = min(top, 32);
        const bool act = lane < n;
        float4 ends = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ctrl = ends;
        uint32_t tag = 0;
        if (act) {
            const int k = top - 1 - lane;
            ends = W.pend_ends[k];
            ctrl = W.pend_ctrl[k];
            tag = W.pend_tag[k];
        }
        top -= n;
        __syncwarp();
        const bool cubic = (tag & kTagCubic) != 0;
        float4 e0 = ends, c0 = ctrl, e1 = ends, c1 = ctrl;  // first and second halves
        if (cubic) {
            const float p01x = half_lerp(ends.x, ctrl.x), p01y = half_lerp(ends.y, ctrl.y);
            const float p12x = half_lerp(ctrl.x, ctrl.z), p12y = half_lerp(ctrl.y, ctrl.w);
            const float p23x = half_lerp(ctrl.z, ends.z), p23y = half_lerp(ctrl.w, ends.w);
            const float p012x = half_lerp(p01x, p12x), p012y = half_lerp(p01y, p12y);
            const float p123x = half_lerp(p12x, p23x), p123y = half_lerp(p12y, p23y);
            const float mx = half_lerp(p012x, p123x), my = half_lerp(p012y, p123y);
            e0 = make_float4(ends.x, ends.y, mx, my);
            c0 = make_float4(p01x, p01y, p012x, p012y);
            e1 = make_float4(mx, my, ends.z, ends.w);
            c1 = make_float4(p123x, p123y, p23x, p23y);
        } else {
            const float ax = fadd(ends.x, fmul(fsub(ctrl.x, ends.x), 0.5f));
            const float ay = fadd(ends.y, fmul(fsub(ctrl.y, ends.y), 0.5f));
            const float qx = fadd(ctrl.x, fmul(fsub(ends.z, ctrl.x), 0.5f));
            const float qy = fadd(ctrl.y, fmul(fsub(ends.w, ctrl.y), 0.5f));
            const float mx = fadd(ax, fmul(fsub(qx, ax), 0.5f)), my = fadd(ay, fmul(fsub(qy, ay), 0.5f));
            e0 = make_float4(ends.x, ends.y, mx, my);
            c0 = make_float4(ax, ay, 0.0f, 0.0f);
            e1 = make_float4(mx, my, ends.z, ends.w);
            c1 = make_float4(qx, qy, 0.0f, 0.0f);
        }
        const uint32_t depth = ((tag >> kTagDepthShift) & 31u) + 1u;
        const bool deep = depth >= (uint32_t)(kMaxDepth - 1);
        if (act && deep) atomicOr(err, kErrDepth);
        const uint32_t tag0 = (tag & ~(31u << kTagDepthShift)) | depth << kTagDepthShift;
        const uint32_t tag1 = tag0 & ~kTagLeft;
        const bool leaf0 = act && (deep || piece_flat(cubic, e0, c0));
        const bool leaf1 = act && (deep || piece_flat(cubic, e1, c1));
        const unsigned l0 = __ballot_sync(~0u, leaf0), l1 = __ballot_sync(~0u, leaf1);
        // nleaf < 32 before the round, so at most 31 + 64 lines are queued after it (the
        // bounds checks below never fail; a failure would send the frame to the exact redo)
        if (leaf0) {
            const int k = nleaf + __popc(l0 & below);
            if (k < kPoolLeafCap) {
                W.leaf[k] = e0;
                W.leaf_tag[k] = tag0;
            } else {
                atomicOr(err, kErrOverflowLeaf);
            }
        }
        if (leaf1) {
            const int k = nleaf + __popc(l0) + __popc(l1 & below);
            if (k < kPoolLeafCap) {
                W.leaf[k] = e1;
                W.leaf_tag[k] = tag1;
            } else {
                atomicOr(err, kErrOverflowLeaf);
            }
        }
        nleaf = min(nleaf + __popc(l0) + __popc(l1), kPoolLeafCap);
        // halves that are not flat go back on the pool, the second below the first
        const bool keep0 = act && !leaf0, keep1 = act && !leaf1;
        const unsigned m0 = __ballot_sync(~0u, keep0), m1 = __ballot_sync(~0u, keep1);
        const int k1 = top + __popc(m1 & below), k0 = top + __popc(m1) + __popc(m0 & below);
        if (keep1) {
            if (k1 < kPoolCap) {
                W.pend_ends[k1] = e1;
                W.pend_ctrl[k1] = c1;
                W.pend_tag[k1] = tag1;
            }
        }
        if (keep0) {
            if (k0 < kPoolCap) {
                W.pend_ends[k0] = e0;
                W.pend_ctrl[k0] = c0;
                W.pend_tag[k0] = tag0;
            }
        }
        top = min(top + __popc(m0) + __popc(m1), kPoolCap);
        if ((keep1 && k1 >= kPoolCap) || (keep0 && k0 >= kPoolCap)) {
            if constexpr (kExact) {
                if (keep1 && k1 >= kPoolCap) {
                    uint4 &sg = W.seg[tag1 & kTagEntry];
                    flatten_piece_alone_exact(b.leaves, b.leaf_cap, b.status, &sg.y, sg.x, e1, c1, tag1);
                }
                if (keep0 && k0 >= kPoolCap) {
                    uint4 &sg = W.seg[tag0 & kTagEntry];
                    flatten_piece_alone_exact(b.leaves, b.leaf_cap, b.status, &sg.y, sg.x, e0, c0, tag0);
                }
            } else {
                const LeafSink out{b.leaves, b.path_leaf_cursor, b.status, b.pool_path, b.leaf_pool_first,
                                   b.leaf_pool_cap};
                if (keep1 && k1 >= kPoolCap)
                    produced += flatten_piece_alone(out, W.seg[tag1 & kTagEntry], e1, c1, tag1);
                if (keep0 && k0 >= kPoolCap)
                    produced += flatten_piece_alone(out, W.seg[tag0 & kTagEntry], e0, c0, tag0);
            }
        }
        __syncwarp();
    }
    if constexpr (!kExact) {
        store_held();
        const uint32_t total = __reduce_add_sync(~0u, produced);
        if (lane == 0) atomicAdd(&b.status[kStLeafCount], total);
    }
}

// ---------------------------------------------------------------------------
// Binning by path (the d3d9 Tiler::process_line_segment walk and Tiler::prepare_tiles,
// tiler.cpp:131-279 / 369-439, which the reference's GPU frame runs as bin.comp and
// propagate.comp).  A path's tiles belong to it alone, so one CTA bins all of a path's leaf
// lines in shared memory: it counts fills and backdrop deltas per tile, propagates the
// backdrops down each column, scans the counts into fill offsets (reserving the path's block
// of fills with one atomic), and walks the lines again to write the fills grouped by tile.
// No tile needs clearing, there is no frame-wide scan over tiles and no global atomic per
// fill.  Paths too large for a CTA (class 3) take global passes: counts with atomics, a CTA
// per path for backdrops and offsets, then the writes with atomics.

// Size classes by shared-memory words: one per tile (fill count in bits 0-23, the int8 sum of
// backdrop deltas in bits 24-31, later the tile's write cursor) and one per column (deltas
// landing above the rect, summed as int32).
constexpr int kCtaClasses = 3;
__host__ __device__ constexpr uint32_t class_words(int c) { return c == 0 ? 1088u : c == 1 ? 4352u : 16896u; }
// Small CTAs for the small classes: a path's barriers then hold few warps, and more paths are in
// flight per SM (A/B on the 512-scene batch, binning: 21.56 ms with 256-thread CTAs, 6 per SM, for
// classes 0 and 1; 20.80 ms with 128-thread CTAs, 12 per SM; 20.72 ms with class 0 at 64 threads,
// 24 per SM).  Class 2 keeps 384 threads: its shared words allow 3 CTAs per SM (256 or 512 threads
// ran slower).
__host__ __device__ constexpr int class_threads(int c) { return c == 2 ? 384 : c == 1 ? 128 : 64; }
// CTAs per SM the register budget is set for (shared memory allows 3 of class 2, 12 of class 1):
// class 0 at 20 (48 registers) and class 1 at 8 (64 registers, no spills) beat 24 and 12 at 40
// registers with 148-208 B of spills (binning 20.00 -> 19.30 ms per 512-scene frame)
__host__ __device__ constexpr int class_min_ctas(int c) { return c == 2 ? 3 : c == 1 ? 8 : 20; }
// Fills a CTA stages during its count walk (8 bytes each, in its own slice of a global buffer
// that stays in L2): the fills are then placed without walking the lines again.  A path with
// more fills than this walks its lines twice.
__host__ __device__ constexpr uint32_t class_stage(int c) { return c == 0 ? 3072u : c == 1 ? 6144u : 12288u; }
// One line gives a tile at most two fills (the walk visits a tile once, with at most one
// extra fill for a vertical crossing), so with at most 2^22 lines per CTA-binned path the
// 24-bit counters cannot carry into the delta byte.
constexpr uint32_t kCtaMaxLeaves = 1u << 22;
// bin_ctl slots: paths per CTA class, work tickets per CTA class, tickets of the class-3
// zeroing and set-up passes, and at slot 12 a 64-bit word: class-3 paths << 40 | their lines.
enum : int { kCtlCount = 0, kCtlTicket = 4, kCtlTicketZero = 8, kCtlTicketPrep = 9, kCtl3 = 12 };
// and from slot 16 the CTA classes' paths counted by log2 of their leaf lines (3 x 32), then
// the write cursors of those buckets (3 x 32): each class's list runs from its largest paths to
// its smallest, so the last CTAs to start take the shortest paths
enum : int { kCtlBucket = 16, kCtlCursor = 16 + 3 * 32, kCtlWords = 16 + 6 * 32, kCtlCompTicket = kCtlWords };
static_assert((kCtlCompTicket + 1) * 4 <= 1024, "bin_ctl holds 1024 bytes");
constexpr uint64_t kLow40 = (1ull << 40) - 1;

__device__ __forceinline__ unsigned long long *ctl3_word(const Batch &b) {
    return reinterpret_cast<unsigned long long *>(b.bin_ctl + kCtl3);
}
__device__ __forceinline__ unsigned long long *fill_total(const Batch &b) {
    return reinterpret_cast<unsigned long long *>(b.status + kStFill64);
}

// -1: no columns (nothing can land); 0-2: CTA classes; 3: global passes
__device__ __forceinline__ int path_class(const PathDev &P, uint32_t leaves) {
    const int32_t rw = max(P.rx1 - P.rx0, 0), rh = max(P.ry1 - P.ry0, 0);
    if (rw == 0) return -1;
    if (leaves > kCtaMaxLeaves) return 3;
    const uint32_t words = (uint32_t)rw * (uint32_t)rh + (uint32_t)rw;
    return words <= class_words(0) ? 0 : words <= class_words(1) ? 1 : words <= class_words(2) ? 2 : 3;
}

// The leaf lines of one path: its region of the leaf buffer, then (learned frame) its lines
// in the spill pool, listed by k_pool_scatter.
struct PathLeaves {
    uint32_t first, nreg, pool0, n;
    __device__ __forceinline__ uint32_t index(const Batch &b, uint32_t k) const {
        return k < nreg ? first + k : b.leaf_pool_first + b.pool_idx[pool0 + (k - nreg)];
    }
};

__device__ __forceinline__ PathLeaves path_leaves(const Batch &b, uint32_t p) {
    const uint2 r = b.path_leaf_range[p];
    PathLeaves L{r.x, r.y - r.x, 0u, r.y - r.x};
    if (b.pool_cnt) {
        L.pool0 = b.pool_cnt[(int64_t)p - 1];
        L.n += b.pool_cnt[p] - L.pool0;
    }
    return L;
}

__device__ __forceinline__ WalkCtx walk_ctx(const Batch &b, const PathDev &P) {
    const SceneDev &S = b.scenes[P.scene];
    WalkCtx w;
    w.rx0 = P.rx0;
    w.ry0 = P.ry0;
    w.rx1 = P.rx1;
    w.ry1 = P.ry1;
    w.rw = max(P.rx1 - P.rx0, 0);
    w.rh = max(P.ry1 - P.ry0, 0);
    w.vb_left = S.vb_left;
    w.vb_right = S.vb_right;
    w.vb_bottom = S.vb_bottom;
    return w;
}

// Adds an int8 delta to the low byte of a 16-bit tile state (class-3 count pass; the high
// byte is still zero).  A compare-and-swap on the enclosing word: every failed round means
// another thread's update went in, and the loop is bounded all the same.
__device__ __forceinline__ void add_delta_u16(uint16_t *a, int d, uint32_t *status) {
    uint32_t *word = reinterpret_cast<uint32_t *>(reinterpret_cast<uintptr_t>(a) & ~uintptr_t(3));
    const int sh = (reinterpret_cast<uintptr_t>(a) & 2) ? 16 : 0;
    uint32_t old = *word;
    for (int it = 0; it < (1 << 20); it++) {
        const uint32_t byte = ((old >> sh) + (uint32_t)d) & 0xffu;
        const uint32_t want = (old & ~(0xffu << sh)) | (byte << sh);
        const uint32_t seen = atomicCAS(word, old, want);
        if (seen == old) return;
        old = seen;
    }
    atomicOr(status, kErrWalk);
}

// Leaf ranges of every path and the size classes.  Classes 0-2 are listed with one atomic per
// warp and class; class-3 paths take a 64-bit atomic that also hands out their offsets in the
// class-3 line numbering the global passes stride over.
// log2 of a path's leaf lines (its range and its spill-pool lines), after k_bin_classify
// stored the range
__device__ __forceinline__ int bin_bucket(const Batch &b, uint32_t p) {
    const uint2 range = b.path_leaf_range[p];
    uint32_t n = range.y - range.x;
    if (b.pool_cnt) n += b.pool_cnt[p] - b.pool_cnt[(int64_t)p - 1];
    return 31 - __clz(max(n, 1u));
}

__global__ void k_bin_classify(Batch b, bool learned) {
    const uint32_t p = global_tid();
    const int lane = threadIdx.x & 31;
    int cls = -1;
    if (p < b.n_paths) {
        const PathDev P = b.paths[p];
        uint2 range;
        if (learned) {
            const uint32_t f = b.path_leaf_first[p];
            range = make_uint2(f, f + min(b.path_leaf_cursor[p], b.path_leaf_budget[p]));
        } else {
            const uint2 pc = b.path_contours[p];
            range = make_uint2(b.seg_leaves[b.contour_segs[pc.x]], b.seg_leaves[b.contour_segs[pc.y]]);
        }
        b.path_leaf_range[p] = range;
        uint32_t n = range.y - range.x;
        if (b.pool_cnt) n += b.pool_cnt[p] - b.pool_cnt[(int64_t)p - 1];
        cls = path_class(P, n);
        b.path_cls[p] = (uint8_t)cls;
        if (cls < 0) b.path_fill[p] = 0;
        if (cls == 3) {
            const unsigned long long old = atomicAdd(ctl3_word(b), (1ull << 40) | (unsigned long long)n);
            const uint32_t item = (uint32_t)(old >> 40);
            b.bin_list[(size_t)3 * b.n_paths + item] = p;
            b.bin_list[(size_t)4 * b.n_paths + item] = (uint32_t)(old & kLow40);
        }
    }
#pragma unroll
    for (int c = 0; c < kCtaClasses; c++) {
        const uint32_t m = __ballot_sync(0xffffffffu, cls == c);
        if (m && lane == __ffs(m) - 1) atomicAdd(&b.bin_ctl[kCtlCount + c], (uint32_t)__popc(m));
    }
    // the bucket of a CTA-class path: log2 of its leaf lines
    const int key = cls >= 0 && cls < kCtaClasses ? cls * 32 + bin_bucket(b, p) : -1;
    const unsigned g = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(g) - 1) atomicAdd(&b.bin_ctl[kCtlBucket + key], (uint32_t)__popc(g));
}

// The buckets' cursors, largest lines first within each class.
__global__ void k_bin_bucket_starts(Batch b) {
    const int c = threadIdx.x;
    if (c >= kCtaClasses) return;
    uint32_t off = 0;
    for (int k = 31; k >= 0; k--) {
        b.bin_ctl[kCtlCursor + c * 32 + k] = off;
        off += b.bin_ctl[kCtlBucket + c * 32 + k];
    }
}

// Each CTA-class path into its class list at its bucket's cursor.
__global__ void k_bin_scatter(Batch b) {
    const uint32_t p = global_tid();
    const int lane = threadIdx.x & 31;
    int key = -1;
    if (p < b.n_paths) {
        const int cls = (int)(int8_t)b.path_cls[p];
        if (cls >= 0 && cls < kCtaClasses) key = cls * 32 + bin_bucket(b, p);
    }
    const unsigned g = __match_any_sync(0xffffffffu, key);
    if (key < 0) return;
    const int leader = __ffs(g) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&b.bin_ctl[kCtlCursor + key], (uint32_t)__popc(g));
    base = __shfl_sync(g, base, leader);
    b.bin_list[(size_t)(key >> 5) * b.n_paths + base + __popc(g & ((1u << lane) - 1u))] = p;
}

// Tiles a line's walk visits at most (its end points' tile distance, before clipping, plus one):
// lines above Batch::long_line (8 unless tuned) are walked by a whole warp.
__device__ __forceinline__ float line_span(const float4 &f) {
    return fabsf(floorf(f.z * 0.0625f) - floorf(f.x * 0.0625f)) + fabsf(floorf(f.w * 0.0625f) - floorf(f.y * 0.0625f)) +
           1.0f;
}

// A staged fill: the four 12-bit coordinates of the packed u16 fill and the tile (< 2^16).
__device__ __forceinline__ uint2 stage_pack(uint2 q, uint32_t local) {
    const uint32_t x0 = q.x & 0xfffu, y0 = q.x >> 16, x1 = q.y & 0xfffu, y1 = q.y >> 16;
    return make_uint2(x0 | y0 << 12 | (x1 & 0xffu) << 24, x1 >> 8 | y1 << 4 | local << 16);
}
__device__ __forceinline__ uint2 stage_fill(uint2 v) {
    const uint32_t x0 = v.x & 0xfffu, y0 = (v.x >> 12) & 0xfffu, x1 = v.x >> 24 | (v.y & 0xfu) << 8,
                   y1 = (v.y >> 4) & 0xfffu;
    return make_uint2(x0 | y0 << 16, x1 | y1 << 16);
}

template <int kCls>
__global__ void __launch_bounds__(class_threads(kCls), class_min_ctas(kCls)) k_bin_fused(Batch b) {
    constexpr int kThr = class_threads(kCls), kWarps = kThr / 32;
    constexpr uint32_t kStage = class_stage(kCls);
    static_assert(class_words(kCls) <= 65536u, "a staged fill holds its tile in 16 bits");
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t s_item, s_base, s_write, s_next, s_nstage;
    uint2 *const stage = b.stage ? b.stage + (size_t)blockIdx.x * kStage : nullptr;
    __shared__ int32_t s_seg[kThr];
    __shared__ uint32_t s_warp[kWarps];
    __shared__ unsigned long long s_wsum[kWarps];
    const uint32_t tid = threadIdx.x;
    const int lane = (int)(tid & 31), warp = (int)(tid >> 5);
    const uint32_t *list = b.bin_list + (size_t)kCls * b.n_paths;
    const uint32_t n_items = b.bin_ctl[kCtlCount + kCls];
    uint32_t *const err = &b.status[kStErr];
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&b.bin_ctl[kCtlTicket + kCls], 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) return;
        const uint32_t p = list[item];
        const PathDev P = b.paths[p];
        const WalkCtx w = walk_ctx(b, P);
        const uint32_t rw = (uint32_t)w.rw, rh = (uint32_t)w.rh, T = rw * rh, tb = P.tile_first, cb = P.col_first;
        uint32_t *cnt = sm;                                   // per tile: count | delta << 24, then cursor
        int32_t *above = reinterpret_cast<int32_t *>(sm + T);  // per column
        const PathLeaves L = path_leaves(b, p);
        for (uint32_t t = tid; t < T + rw; t += kThr) sm[t] = 0;
        if (tid == 0) {
            s_next = 0;
            s_nstage = 0;
        }
        __syncthreads();

        // 1. fill counts and backdrop deltas, the fills staged with their tiles.  Warps take
        //    the lines 32 at a time, so a warp that drew short lines takes more.
        //    A line of many tiles (a contour's closing line spans the canvas) would hold its
        //    warp, and at the barrier its CTA, for tens of steps: such lines are walked by the
        //    whole warp after its short lines.
        auto on_fill = [&](int32_t local, uint2 q) {
            atomicAdd(&cnt[local], 1u);
            const uint32_t slot = atomicAdd(&s_nstage, 1u);
            if (stage && slot < kStage) stage[slot] = stage_pack(q, (uint32_t)local);
        };
        auto on_delta = [&](int32_t where, int d) {
            if (where >= 0) atomicAdd(&cnt[where], (uint32_t)d << 24);
            else atomicAdd(&above[-1 - where], d);
        };
        for (;;) {
            uint32_t k0 = 0;
            if (lane == 0) k0 = atomicAdd(&s_next, 32u);
            k0 = __shfl_sync(0xffffffffu, k0, 0);
            if (k0 >= L.n) break;
            const uint32_t k = k0 + (uint32_t)lane;
            float4 f = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            bool along = false;
            if (k < L.n) {
                f = b.leaves[L.index(b, k)];
                along = line_span(f) > b.long_line;
                if (!along) walk_line(w, f.x, f.y, f.z, f.w, on_fill, on_delta, err);
            }
            for (unsigned m = __ballot_sync(0xffffffffu, along); m; m &= m - 1) {
                const int l = __ffs(m) - 1;
                const float4 g = make_float4(__shfl_sync(0xffffffffu, f.x, l), __shfl_sync(0xffffffffu, f.y, l),
                                             __shfl_sync(0xffffffffu, f.z, l), __shfl_sync(0xffffffffu, f.w, l));
                walk_line_warp(w, g, on_fill, on_delta, err);
            }
        }
        __syncthreads();

        // 2. the count of each warp's chunk of tiles; thread 0 reserves the path's block of
        //    fills with one atomic whose result it reads only after the column pass
        const uint32_t chunk = ((T + kWarps - 1) / kWarps + 127u) & ~127u;
        const uint32_t c0 = min(T, (uint32_t)warp * chunk), c1 = min(T, c0 + chunk);
        unsigned long long wsum = 0;  // 64-bit: a path's fills need not fit 32 bits (it then overflows)
        for (uint32_t t = c0 + lane; t < c1; t += 32) wsum += cnt[t] & 0xffffffu;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wsum += __shfl_down_sync(0xffffffffu, wsum, o);
        if (lane == 0) s_wsum[warp] = wsum;
        __syncthreads();
        unsigned long long base = 0, total = 0;
        if (tid == 0) {
            for (int k = 0; k < kWarps; k++) {
                const unsigned long long v = s_wsum[k];
                s_warp[k] = (uint32_t)total;
                total += v;
            }
            base = atomicAdd(fill_total(b), total);
        }

        // 3. backdrops down each column (tile backdrop = int8 of the running column sum before
        //    the tile's own delta); columns are cut into segments of rows so every thread has
        //    work: segment sums first, then each segment's walk from its starting sum.
        const uint32_t segs = rw >= (uint32_t)kThr ? 1u : (uint32_t)kThr / rw;
        const uint32_t seg_rows = (rh + segs - 1) / segs;
        if (segs > 1) {
            if (tid < rw * segs) {
                const uint32_t x = tid % rw, s = tid / rw;
                const uint32_t y0 = min(rh, s * seg_rows), y1 = min(rh, y0 + seg_rows);
                int32_t sum = 0;
                for (uint32_t y = y0; y < y1; y++) sum += (int8_t)(cnt[y * rw + x] >> 24);
                s_seg[tid] = sum;
            }
            __syncthreads();
        }
        for (uint32_t u = tid; u < rw * segs; u += kThr) {
            const uint32_t x = u % rw, s = u / rw;
            int32_t run = above[x];
            for (uint32_t k = 0; k < s; k++) run += s_seg[k * rw + x];
            const uint32_t y0 = min(rh, s * seg_rows), y1 = min(rh, y0 + seg_rows);
            for (uint32_t y = y0; y < y1; y++) {
                const uint32_t t = y * rw + x, c = cnt[t];
                b.tile_state[tb + t] = (uint16_t)((uint32_t)(uint8_t)(int8_t)run | ((c & 0xffffffu) ? 0x100u : 0u));
                run += (int8_t)(c >> 24);
            }
            if (s == segs - 1) b.col_final[cb + x] = run;
        }
        if (tid == 0) {
            const bool fits = base + total <= (unsigned long long)b.fill_cap;
            if (!fits) atomicOr(err, kErrOverflowFill);
            b.path_fill[p] = (uint32_t)base;
            s_base = (uint32_t)base;
            s_write = fits && total > 0;
        }
        __syncthreads();

        // 4. each warp scans its chunk into write cursors (shared) and end offsets (global): a
        //    lane takes four consecutive tiles (one 16-byte shared load; chunks start on
        //    multiples of 128 tiles), and one warp scan covers 128 tiles
        uint32_t carry = s_base + s_warp[warp];
        for (uint32_t t0 = c0; t0 < c1; t0 += 128) {
            const uint32_t t = t0 + 4 * (uint32_t)lane;
            uint32_t v[4];
            if (t + 4 <= c1) {
                const uint4 q = *reinterpret_cast<const uint4 *>(&cnt[t]);
                v[0] = q.x & 0xffffffu;
                v[1] = q.y & 0xffffffu;
                v[2] = q.z & 0xffffffu;
                v[3] = q.w & 0xffffffu;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) v[j] = t + j < c1 ? (cnt[t + j] & 0xffffffu) : 0u;
            }
            const uint32_t own = v[0] + v[1] + v[2] + v[3];
            uint32_t incl = own;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += n;
            }
            uint32_t e[5];
            e[0] = carry + incl - own;
#pragma unroll
            for (int j = 0; j < 4; j++) e[j + 1] = e[j] + v[j];
            if (t + 4 <= c1) {
                *reinterpret_cast<uint4 *>(&cnt[t]) = make_uint4(e[0], e[1], e[2], e[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (t + j < c1) cnt[t + j] = e[j];
            }
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (t + j < c1) b.tile_fills[tb + t + j] = e[j + 1];
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        __syncthreads();

        // 5. the fills, grouped by tile: from the stage (four loads in flight per thread), or by
        //    walking the lines again
        const uint32_t nstage = s_nstage;
        if (s_write && stage && nstage <= kStage) {
            for (uint32_t k = tid; k < nstage; k += 4 * kThr) {
                uint2 v[4];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (k + j * kThr < nstage) v[j] = stage[k + j * kThr];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (k + j * kThr < nstage) b.fills[atomicAdd(&cnt[v[j].y >> 16], 1u)] = stage_fill(v[j]);
            }
        } else if (s_write) {
            for (uint32_t k = tid; k < L.n; k += kThr) {
                const float4 f = b.leaves[L.index(b, k)];
                walk_line(
                    w, f.x, f.y, f.z, f.w,
                    [&](int32_t local, uint2 q) { b.fills[atomicAdd(&cnt[local], 1u)] = q; },
                    [&](int32_t, int) {}, err);
            }
        }
        __syncthreads();
    }
}

// Class 3: clear the counters, deltas and column sums of the paths' tiles.
__global__ void k_bin_zero_large(Batch b) {
    __shared__ uint32_t s_item;
    const uint32_t n3 = (uint32_t)(*ctl3_word(b) >> 40);
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&b.bin_ctl[kCtlTicketZero], 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();
        if (item >= n3) return;
        const PathDev P = b.paths[b.bin_list[(size_t)3 * b.n_paths + item]];
        const uint32_t rw = (uint32_t)(P.rx1 - P.rx0), T = rw * (uint32_t)max(P.ry1 - P.ry0, 0);
        for (uint32_t t = threadIdx.x; t < T; t += blockDim.x) {
            b.tile_fills[P.tile_first + t] = 0;
            b.tile_state[P.tile_first + t] = 0;
        }
        for (uint32_t x = threadIdx.x; x < rw; x += blockDim.x) b.col_above[P.col_first + x] = 0;
    }
}

// Class 3, per line (strided over the class-3 numbering of lines): count (global atomics on
// the tile counters, deltas into the low byte of the tile state) or write (the counters have
// become cursors).
template <bool kWrite>
__global__ void __launch_bounds__(kThreads) k_bin_large(Batch b) {
    const unsigned long long c3 = *ctl3_word(b);
    const uint32_t n3 = (uint32_t)(c3 >> 40), total = (uint32_t)(c3 & kLow40);
    if (n3 == 0) return;
    if (kWrite && (b.status[kStErr] & kErrOverflowFill)) return;
    const uint32_t *list = b.bin_list + (size_t)3 * b.n_paths, *first = b.bin_list + (size_t)4 * b.n_paths;
    for (uint32_t j = global_tid(); j < total; j += gridDim.x * blockDim.x) {
        const uint32_t item = upper_bound(first, n3, j) - 1;
        const uint32_t p = list[item];
        const PathDev P = b.paths[p];
        const PathLeaves L = path_leaves(b, p);
        const float4 f = b.leaves[L.index(b, j - first[item])];
        const WalkCtx w = walk_ctx(b, P);
        const uint32_t tb = P.tile_first, cb = P.col_first;
        if (kWrite) {
            walk_line(
                w, f.x, f.y, f.z, f.w,
                [&](int32_t local, uint2 q) { b.fills[atomicAdd(&b.tile_fills[tb + (uint32_t)local], 1u)] = q; },
                [&](int32_t, int) {}, &b.status[kStErr]);
        } else {
            walk_line(
                w, f.x, f.y, f.z, f.w, [&](int32_t local, uint2) { atomicAdd(&b.tile_fills[tb + (uint32_t)local], 1u); },
                [&](int32_t where, int d) {
                    if (where >= 0) add_delta_u16(&b.tile_state[tb + (uint32_t)where], d, &b.status[kStErr]);
                    else atomicAdd(&b.col_above[cb + (uint32_t)(-1 - where)], d);
                },
                &b.status[kStErr]);
        }
    }
}

// Class 3, one CTA per path: backdrops down each column, then the path's block of fills and
// the counts scanned into write cursors.
constexpr int kPrepThreads = 256;

__global__ void __launch_bounds__(kPrepThreads) k_bin_large_prep(Batch b) {
    constexpr int kWarps = kPrepThreads / 32;
    __shared__ uint32_t s_item, s_base;
    __shared__ unsigned long long s_red[kWarps];
    __shared__ uint32_t s_warp[kWarps];
    const uint32_t tid = threadIdx.x;
    const int lane = (int)(tid & 31), warp = (int)(tid >> 5);
    const uint32_t n3 = (uint32_t)(*ctl3_word(b) >> 40);
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&b.bin_ctl[kCtlTicketPrep], 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n3) return;
        const uint32_t p = b.bin_list[(size_t)3 * b.n_paths + item];
        const PathDev P = b.paths[p];
        const uint32_t rw = (uint32_t)max(P.rx1 - P.rx0, 0), rh = (uint32_t)max(P.ry1 - P.ry0, 0), T = rw * rh;
        const uint32_t tb = P.tile_first, cb = P.col_first;
        unsigned long long sum = 0;
        for (uint32_t x = tid; x < rw; x += kPrepThreads) {
            int32_t run = b.col_above[cb + x];
            uint32_t y = 0;
            // eight rows at a time: their counters and deltas are loaded before any of the
            // eight states is rewritten, so the loads overlap instead of following each store
            for (; y + 8 <= rh; y += 8) {
                uint32_t cnt[8];
                uint16_t state[8];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const uint32_t t = tb + (y + k) * rw + x;
                    cnt[k] = b.tile_fills[t];
                    state[k] = b.tile_state[t];
                }
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const uint32_t t = tb + (y + k) * rw + x;
                    b.tile_state[t] = (uint16_t)((uint32_t)(uint8_t)(int8_t)run | (cnt[k] ? 0x100u : 0u));
                    run += (int8_t)(state[k] & 0xffu);
                    sum += cnt[k];
                }
            }
            for (; y < rh; y++) {
                const uint32_t t = tb + y * rw + x, c = b.tile_fills[t];
                const int8_t delta = (int8_t)(b.tile_state[t] & 0xffu);
                b.tile_state[t] = (uint16_t)((uint32_t)(uint8_t)(int8_t)run | (c ? 0x100u : 0u));
                run += delta;
                sum += c;
            }
            b.col_final[cb + x] = run;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) s_red[warp] = sum;
        __syncthreads();
        if (tid == 0) {
            unsigned long long total = 0;
            for (int k = 0; k < kWarps; k++) total += s_red[k];
            const unsigned long long base = atomicAdd(fill_total(b), total);
            if (base + total > (unsigned long long)b.fill_cap) atomicOr(&b.status[kStErr], kErrOverflowFill);
            b.path_fill[p] = (uint32_t)base;
            s_base = (uint32_t)base;
        }
        __syncthreads();
        // exclusive scan of the counters into write cursors, four consecutive tiles a thread
        uint32_t carry = s_base;
        for (uint32_t t0 = 0; t0 < T; t0 += 4 * kPrepThreads) {
            const uint32_t t = t0 + 4 * tid;
            uint32_t v[4], own = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                v[k] = t + k < T ? b.tile_fills[tb + t + k] : 0u;
                own += v[k];
            }
            uint32_t incl = own;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += n;
            }
            if (lane == 31) s_warp[warp] = incl;
            __syncthreads();
            uint32_t before = 0, chunk_total = 0;
            for (int k = 0; k < kWarps; k++) {
                if (k < warp) before += s_warp[k];
                chunk_total += s_warp[k];
            }
            uint32_t cur = carry + before + incl - own;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (t + k < T) b.tile_fills[tb + t + k] = cur;
                cur += v[k];
            }
            carry += chunk_total;
            __syncthreads();
        }
    }
}

// Learned frame: list the spill pool's lines by path (count, scan, scatter), so each path's
// CTA finds its pooled lines.
__global__ void k_pool_count(Batch b) {
    const uint32_t n = min(b.status[kStPoolUsed], b.leaf_pool_cap);
    for (uint32_t j = global_tid(); j < n; j += gridDim.x * blockDim.x) atomicAdd(&b.pool_cnt[b.pool_path[j]], 1u);
}

__global__ void k_pool_scatter(Batch b) {
    const uint32_t n = min(b.status[kStPoolUsed], b.leaf_pool_cap);
    for (uint32_t j = global_tid(); j < n; j += gridDim.x * blockDim.x)
        b.pool_idx[atomicAdd(&b.pool_cnt[b.pool_path[j]], 1u)] = j;
}

// ---------------------------------------------------------------------------
// Per framebuffer-tile row of each scene: the scene's paths whose tile rect spans the row,
// in path order (one block per row; a block scan keeps the order, no sort is needed).

constexpr int kRowThreads = 256;
// Row-entry flag of a clipped path; mask sources of a clipped tile.
constexpr uint32_t kRowClipped = 16u;
enum : uint32_t { kMaskOwn = 0, kMaskClip = 1, kMaskBoth = 2 };

template <bool kWrite>
__global__ void __launch_bounds__(kRowThreads) k_rows(Batch b) {
    __shared__ uint32_t warp_counts[kRowThreads / 32];
    __shared__ uint32_t chunk_total;
    const uint32_t r = blockIdx.x;
    const uint32_t rg = b.row_base + r;
    const uint32_t s = upper_bound(b.scene_row_first, b.n_scenes_all + 1, rg) - 1;
    const SceneDev &S = b.scenes[s];
    const int32_t y = (int32_t)(rg - S.row_first);
    const uint32_t p0 = S.path_first - b.path_base, p1 = S.path_end - b.path_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t out = kWrite ? b.row_first[r] : 0u;
    uint32_t total = 0;
    for (uint32_t base = p0; base < p1; base += kRowThreads) {
        const uint32_t p = base + threadIdx.x;
        bool spans = false;
        int4 rect = make_int4(0, 0, 0, 0);
        int32_t cx0 = 0, cx1 = 0;  // the rect's columns inside the framebuffer
        if (p < p1) {
            rect = *reinterpret_cast<const int4 *>(&b.paths[p].rx0);
            cx0 = max(rect.x, 0);
            cx1 = min(rect.z, (int32_t)S.fbw);
            spans = rect.y <= y && y < rect.w && cx0 < cx1 && !(b.paths[p].flags & kPathIsClip);
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, spans);
        if (lane == 0) warp_counts[warp] = __popc(ballot);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int k = 0; k < kRowThreads / 32; k++) {
                const uint32_t c = warp_counts[k];
                warp_counts[k] = run;
                run += c;
            }
            chunk_total = run;
        }
        __syncthreads();
        if (kWrite && spans) {
            const uint32_t rank = warp_counts[warp] + __popc(ballot & ((1u << lane) - 1u));
            // tile index of column 0 of this row in the path's numbering (may underflow by rx0;
            // adding fx >= rx0 brings it back into range)
            const uint32_t row_tile = b.paths[p].tile_first + (uint32_t)(y - rect.y) * (uint32_t)(rect.z - rect.x) -
                                      (uint32_t)rect.x;
            // flags: bit 0 even-odd, bit 1 occludes, bit 2 the rect's first tile (its first
            // row, first column) is in this row of the framebuffer, bit 4 the path is clipped
            const bool clipped = b.path_clip_cat && b.path_clip_rel[p] != kNone;
            const bool first = y == rect.y && rect.x >= 0;
            if (out + rank < b.row_cap)
                b.row_paths[out + rank] = make_uint4(p, (uint32_t)cx0 | ((uint32_t)cx1 << 16), row_tile,
                                                     b.paths[p].flags | (first ? 4u : 0u) |
                                                         (clipped ? kRowClipped : 0u));
        }
        out += chunk_total;
        total += chunk_total;
        __syncthreads();
    }
    if (!kWrite && threadIdx.x == 0) b.row_first[r] = total;
}

// ---------------------------------------------------------------------------
// Coverage of one alpha tile, accumulated by a warp into shared memory.
//
// A fill contributes, to the pixel (i, j) of its tile, the signed area inside the pixel
// between the fill and the tile bottom (the quantity fill.comp:51-100 looks up in its area
// LUT).  Along a pixel column that area steps from 0 (rows above the line) to the fill's
// x-extent (rows below it), so the fill is stored as per-row differences: every piece of
// the fill inside one cell (i, r) with x-width w and mean in-row depth m adds w(1-m) to
// row r and w*m to row r+1; a prefix sum down the column restores the area.  Values are
// int32 fixed point (kCovShift fraction bits), so the result does not depend on fill order.

__device__ __forceinline__ int cov_index(int row, int col) { return row * 16 + col + ((row >> 3) << 4); }
constexpr int kCovCells = 16 * 16 + 16;

__device__ __forceinline__ void cov_add(int *D, int row, int col, float v) {
    if (row < 16) atomicAdd(&D[cov_index(row, col)], __float2int_rn(v * (float)(1 << kCovShift)));
}

// Per-fill set-up shared by the (fill, column) work items of one alpha tile.
struct FillPrep {
    float xl, yl, xr, yr, dydx, s;
    int i0;
    int first;  // first work item of this fill
};

// The piece of fill `fp` inside pixel column i: per-row differences into D.
__device__ __forceinline__ void raster_column(const FillPrep &fp, int i, int *D) {
    const float xa = fmaxf(fp.xl, (float)i), xb = fminf(fp.xr, (float)(i + 1));
    const float w = xb - xa;
    if (!(w > 0.0f)) return;
    const float ya = xa == fp.xl ? fp.yl : fp.yl + fp.dydx * (xa - fp.xl);
    const float yb = xb == fp.xr ? fp.yr : fp.yl + fp.dydx * (xb - fp.xl);
    const float ylo = fminf(ya, yb), yhi = fmaxf(ya, yb);
    const int r0 = (int)floorf(ylo);
    const float sw = fp.s * w;
    if (yhi <= (float)(r0 + 1)) {
        const float m = 0.5f * (ylo + yhi) - (float)r0;
        cov_add(D, r0, i, sw * (1.0f - m));
        cov_add(D, r0 + 1, i, sw * m);
    } else {
        const int r1 = min((int)ceilf(yhi) - 1, 15);
        const float inv_h = 1.0f / (yhi - ylo);
        for (int r = r0; r <= r1; r++) {
            const float lo = fmaxf(ylo, (float)r), hi = fminf(yhi, (float)(r + 1));
            const float hgt = hi - lo;
            if (!(hgt > 0.0f)) continue;
            const float wr = sw * hgt * inv_h;
            const float m = 0.5f * (lo + hi) - (float)r;
            cov_add(D, r, i, wr * (1.0f - m));
            cov_add(D, r + 1, i, wr * m);
        }
    }
}

// Warp computes the coverage of the 8 pixels of every lane (column lane&15, rows
// (lane>>4)*8 .. +7) of an alpha tile; D must be zero on entry and is left zero.
// Fills are rasterised as (fill, pixel column) work items spread over the lanes, 32 fills
// at a time, so a tile of a few wide fills still keeps the warp busy.
// backdrop + the fills' area sums (fixed point) of the warp's 8 pixels per lane, before the fill rule
// src: the tile's n fills (global memory, or the warp's shared-memory stage).
__device__ __forceinline__ void coverage_raw(const uint2 *src, uint32_t n, int8_t bd, int *D, FillPrep *prep,
                                             int raw[8]) {
    const int lane = threadIdx.x & 31;
    const uint32_t f0 = 0, f1 = n;
    for (uint32_t base = f0; base < f1; base += 32) {
        const uint32_t f = base + lane;
        int items = 0;
        FillPrep fp;
        if (f < f1) {
            const uint2 q = src[f];
            const float x0 = (float)(q.x & 0xffffu) * (1.0f / 256.0f), y0 = (float)(q.x >> 16) * (1.0f / 256.0f);
            const float x1 = (float)(q.y & 0xffffu) * (1.0f / 256.0f), y1 = (float)(q.y >> 16) * (1.0f / 256.0f);
            fp.s = x0 > x1 ? 1.0f : -1.0f;
            fp.xl = fminf(x0, x1);
            fp.xr = fmaxf(x0, x1);
            fp.yl = x0 < x1 ? y0 : y1;
            fp.yr = x0 < x1 ? y1 : y0;
            // xr - xl >= 1/256 (vertical fills are culled when quantised): the fast divide is
            // within 2 ulp, far inside the coverage tolerance
            fp.dydx = __fdividef(fp.yr - fp.yl, fp.xr - fp.xl);
            fp.i0 = max((int)floorf(fp.xl), 0);
            items = max(min((int)ceilf(fp.xr), 16) - fp.i0, 0);
        }
        int incl = items;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        fp.first = incl - items;
        prep[lane] = fp;
        __syncwarp();
        for (int k = lane; k < total; k += 32) {
            // fill of item k: the last fill whose first item is <= k
            int lo = 0, hi = 31;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (prep[mid].first <= k && mid < (int)min(32u, f1 - base)) lo = mid;
                else hi = mid - 1;
            }
            const FillPrep &g = prep[lo];
            raster_column(g, g.i0 + (k - g.first), D);
        }
        __syncwarp();
    }
    const int col = lane & 15, h = lane >> 4;
    int acc[8];
    int run = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int idx = cov_index(h * 8 + k, col);
        run += D[idx];
        D[idx] = 0;  // read and clear: the next tile starts from zero cells
        acc[k] = run;
    }
    const int upper = __shfl_sync(0xffffffffu, run, col);  // rows 0..7 total of this column
    const int base = (h ? upper : 0) + ((int)bd << kCovShift);
#pragma unroll
    for (int k = 0; k < 8; k++) raw[k] = base + acc[k];
}

// The fill rule (fill.comp:133-140): nonzero min(|c|, 1), even-odd 1 - |1 - (c mod 2)|.
__device__ __forceinline__ void coverage_rule(const int raw[8], bool eo, float cov[8]) {
    const float scale = 1.0f / (float)(1 << kCovShift);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int c = raw[k];
        if (!eo) {
            cov[k] = fminf(fabsf((float)c) * scale, 1.0f);
        } else {
            const float t = (float)(c & ((2 << kCovShift) - 1)) * scale;
            cov[k] = __saturatef(1.0f - fabsf(1.0f - t));
        }
    }
}

__device__ __forceinline__ void alpha_coverage(const Batch &b, uint32_t f0, uint32_t f1, int8_t bd, bool eo, int *D,
                                               FillPrep *prep, float cov[8]) {
    int raw[8];
    coverage_raw(b.fills + f0, f1 - f0, bd, D, prep, raw);
    coverage_rule(raw, eo, cov);
}

__device__ __forceinline__ void zero_cells(int *D) {
    const int lane = threadIdx.x & 31;
    for (int k = lane; k < kCovCells; k += 32) D[k] = 0;
    __syncwarp();
}

constexpr int kCompWarps = 1;

// One framebuffer tile: walk the paths spanning its row from the topmost down, test 32
// candidates at a time (one per lane), and visit the visible tiles in order.  A visible tile
// is an alpha tile or a solid tile with a nonzero backdrop (scene_builder.cpp:57-63); the
// walk ends at the first occluding tile - a solid, opaque tile whose fill rule covers it
// (the d3d11 z-buffer rule, propagate.comp:190-205) - so the tiles visited are exactly the
// framebuffer tile's composite list after z-culling (sort.comp:49-83), in reverse order.
// With kFetch, every visible candidate also loads its colour and (alpha tiles) its fill
// range in parallel before the visits, so a visit waits on its fills alone.
// visit(candidate) returns true to stop the walk.
struct Cand {
    uint32_t p, gt, st, flags;  // st: the tile state, with a clipped tile's mask source in bits 9-10
                                // and (kMaskBoth) the draw tile's own backdrop in bits 16-23
    uint32_t f0, f1, color;     // kFetch only (kMaskClip: the clip tile's fills)
    uint32_t gc;                // kMaskClip, kMaskBoth: the clip tile
};

__device__ __forceinline__ uint32_t mask_mode(uint32_t st) { return (st >> 9) & 3u; }

// A clipped draw tile against the clip path's tile at the same coordinates
// (Tiler::prepare_tiles, pathfinder/core/d3d9/tiler.cpp:386-431): culled outside the clip's
// rect or over a blank clip tile; a solid tile over a clip alpha tile takes the clip's mask and
// backdrop; an alpha tile over a clip alpha tile keeps its mask, to be combined with the clip's,
// and its backdrop is zeroed; otherwise unchanged.  Updates c.st (and c.f0/f1, c.gc).
__device__ __forceinline__ void apply_clip(const Batch &b, uint32_t p, int32_t tx, int32_t ty, Cand &c) {
    const uint32_t cp = b.path_clip_rel[p];
    const PathDev C = b.paths[cp];
    if (tx < C.rx0 || tx >= C.rx1 || ty < C.ry0 || ty >= C.ry1) {
        c.st = 0;
        return;
    }
    const uint32_t gc = C.tile_first + (uint32_t)((ty - C.ry0) * (C.rx1 - C.rx0) + (tx - C.rx0));
    const uint32_t cs = b.tile_state[gc];
    const bool ca = (cs & 0x100u) != 0, da = (c.st & 0x100u) != 0;
    const int8_t cbd = (int8_t)(cs & 0xffu), dbd = (int8_t)(c.st & 0xffu);
    if (ca && da) {
        c.st = 0x100u | kMaskBoth << 9 | (uint32_t)(uint8_t)dbd << 16;
        c.gc = gc;
    } else if (ca && dbd != 0) {
        c.st = 0x100u | kMaskClip << 9 | (uint32_t)(uint8_t)cbd;
        c.f0 = gc == C.tile_first ? b.path_fill[cp] : b.tile_fills[gc - 1];
        c.f1 = b.tile_fills[gc];
        c.gc = gc;
    } else if (!ca && cbd == 0) {
        c.st = 0;
    }
}

template <bool kFetch, bool kClip, class Visit>
__device__ __forceinline__ void walk_fb_tile(const Batch &b, uint32_t row, uint32_t fx, uint32_t fy, Visit &&visit,
                                             uint32_t &chunks) {
    const int lane = threadIdx.x & 31;
    const uint32_t k_lo = b.row_first[row], k_hi = b.row_first[row + 1];
    for (uint32_t top = k_hi; top > k_lo; top = top > k_lo + 32 ? top - 32 : k_lo) {
        chunks++;
        const int64_t k = (int64_t)top - 1 - lane;
        Cand c{0, 0, 0, 0, 0, 0, 0, kNone};
        bool vis = false;
        if (k >= (int64_t)k_lo) {
            const uint4 e = b.row_paths[k];
            if (fx >= (e.y & 0xffffu) && fx < (e.y >> 16)) {
                c.p = e.x;
                c.flags = e.w;
                c.gt = e.z + fx;
                c.st = b.tile_state[c.gt];
                if (kClip && (c.flags & kRowClipped)) apply_clip(b, c.p, (int32_t)fx, (int32_t)fy, c);
                vis = c.st != 0;
                if (kFetch && vis) {
                    c.color = b.color[b.path_base + c.p];
                    if ((c.st & 0x100u) && mask_mode(c.st) != kMaskClip) {
                        // the first tile of a path starts the path's block of fills
                        const bool first = (c.flags & 4u) && fx == (e.y & 0xffffu);
                        c.f0 = first ? b.path_fill[c.p] : b.tile_fills[c.gt - 1];
                        c.f1 = b.tile_fills[c.gt];
                    }
                }
            }
        }
        uint32_t mask = __ballot_sync(0xffffffffu, vis);
        while (mask) {
            const int l = __ffs(mask) - 1;
            mask &= mask - 1;
            Cand v;
            v.p = __shfl_sync(0xffffffffu, c.p, l);
            v.gt = __shfl_sync(0xffffffffu, c.gt, l);
            v.st = __shfl_sync(0xffffffffu, c.st, l);
            v.flags = __shfl_sync(0xffffffffu, c.flags, l);
            if (kFetch) {
                v.f0 = __shfl_sync(0xffffffffu, c.f0, l);
                v.f1 = __shfl_sync(0xffffffffu, c.f1, l);
                v.color = __shfl_sync(0xffffffffu, c.color, l);
                if (kClip) v.gc = __shfl_sync(0xffffffffu, c.gc, l);
            }
            if (visit(v)) return;
        }
    }
}

__device__ __forceinline__ bool solid_hidden(bool eo, int8_t bd) { return eo && ((bd < 0 ? -bd : bd) & 1) == 0; }

// First fill of tile gt of path p: the path's block starts at path_fill[p]; every other tile
// starts where the tile before it ends.
__device__ __forceinline__ uint32_t fill_begin(const Batch &b, uint32_t p, uint32_t gt) {
    return gt == b.path_tiles[p] ? b.path_fill[p] : b.tile_fills[gt - 1];
}

// The colour (straight alpha) a gradient gives the pixel centred at (x, y): tile.comp's colour
// texture coordinate (computeTileVaryings, tile.comp:694-724: the half-float transform times
// the pixel centre), filterRadialGradient (tile.comp:319-347) for radial gradients, then a
// linearly filtered fetch of the 256-texel ramp (clamped, or repeated for PF_WRAP_REPEAT).
__device__ __forceinline__ float4 gradient_color(const Batch &b, uint32_t g, float x, float y) {
    const float4 *m = b.grad_meta + 4 * g;
    const float4 m0 = m[0], m1 = m[1], m3 = m[3];
    const uint32_t type = __float_as_uint(m3.x);
    const bool repeat = __float_as_uint(m3.y) == PF_WRAP_REPEAT;
    float u;
    if (type == PF_PAINT_LINEAR) {
        u = m0.x * x + m0.z * y + m1.x;
    } else {
        const float4 m2 = m[2];
        const float cx = m0.x * x + m0.z * y + m1.x, cy = m0.y * x + m0.w * y + m1.y;
        const float dpx = cx - m1.z, dpy = cy - m1.w, dcx = m2.x, dcy = m2.y;
        const float r0 = m2.z, dr = m2.w - r0;
        const float a = dcx * dcx + dcy * dcy - dr * dr;
        const float bb = dpx * dcx + dpy * dcy + r0 * dr;
        const float c = dpx * dpx + dpy * dpy - r0 * r0;
        const float disc = bb * bb - a * c;
        if (!(disc > 0.0f)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // no real t (or the shader's 0)
        const float sq = sqrtf(disc);
        float t0 = (sq + bb) / a, t1 = (-sq + bb) / a;
        if (t0 > t1) {
            const float tmp = t0;
            t0 = t1;
            t1 = tmp;
        }
        u = t0 >= 0.0f ? t0 : t1;
    }
    if (!isfinite(u)) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (repeat) u -= floorf(u);
    const float s = u * 256.0f - 0.5f, f0 = floorf(s), f = s - f0;
    int i0 = (int)fmaxf(fminf(f0, 1e9f), -1e9f), i1 = i0 + 1;
    if (repeat) {
        i0 &= 255;
        i1 &= 255;
    } else {
        i0 = min(max(i0, 0), 255);
        i1 = min(max(i1, 0), 255);
    }
    const uint32_t *ramp = b.grad_ramp + 256 * (size_t)g;
    const uint32_t p0 = __ldg(ramp + i0), p1 = __ldg(ramp + i1);
    const float inv = 1.0f / 255.0f;
    float4 o;
    o.x = ((float)(p0 & 0xffu) + ((float)(p1 & 0xffu) - (float)(p0 & 0xffu)) * f) * inv;
    o.y = ((float)((p0 >> 8) & 0xffu) + ((float)((p1 >> 8) & 0xffu) - (float)((p0 >> 8) & 0xffu)) * f) * inv;
    o.z = ((float)((p0 >> 16) & 0xffu) + ((float)((p1 >> 16) & 0xffu) - (float)((p0 >> 16) & 0xffu)) * f) * inv;
    o.w = ((float)(p0 >> 24) + ((float)(p1 >> 24) - (float)(p0 >> 24)) * f) * inv;
    return o;
}

// kClip: the batch has clip paths; kPaint: it has gradient paints; kTicket: resident warps
// take tiles by ticket (b.comp_ticket > 0).  Variants of their own, so that code one frame does
// not need costs it no registers.
template <bool kClip, bool kPaint, bool kTicket>
__global__ void __launch_bounds__(kCompWarps * 32, (kPaint ? 20 : kClip ? 24 : 32) / kCompWarps) k_composite(Batch b) {
    __shared__ int cells[kCompWarps][kCovCells];
    __shared__ FillPrep prep[kCompWarps][32];
    __shared__ int park[kCompWarps][8][32];  // kMaskBoth: the clip tile's |coverage|
    // a frame whose leaf lines or fills overran their buffers is redone; nothing to read here
    if (b.status[kStErr] & (kErrOverflowLeaf | kErrOverflowFill)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *D = cells[warp];
    zero_cells(D);  // once: coverage_raw leaves the cells it reads zero
    const int col = lane & 15, h = lane >> 4;
    const float inv255 = 1.0f / 255.0f;
    uint32_t entries = 0, comp_fills = 0, chunks = 0;
    // one framebuffer tile per warp, or (kTicket) warps that stay and take comp_ticket
    // consecutive tiles at a time from a frame-wide ticket counter
    uint32_t next = 0, left = 0;
    for (uint32_t round = 0;; round++) {
        uint32_t fb;
        if (!kTicket) {
            if (round > 0) break;
            fb = blockIdx.x * kCompWarps + warp;
        } else {
            if (left == 0) {
                uint32_t t = 0;
                if (lane == 0) t = atomicAdd(&b.bin_ctl[kCtlCompTicket], b.comp_ticket);
                next = __shfl_sync(0xffffffffu, t, 0);
                left = b.comp_ticket;
            }
            fb = next++;
            left--;
        }
        if (fb >= b.n_fb) break;
        const uint32_t fbg = b.fb_base + fb;
        const uint32_t s = b.fb_scene[fbg];
        const SceneDev &S = b.scenes[s];
        const uint32_t local = fbg - S.fb_first;
        const uint32_t fx = local % S.fbw, fy = local / S.fbw;
        // front to back: acc = sum of T * premultiplied source, T = product of (1 - a) above;
        // the accumulated alpha is 1 - T
        float ar[8], ag[8], ab[8], tr[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            ar[k] = ag[k] = ab[k] = 0.0f;
            tr[k] = 1.0f;
        }
        walk_fb_tile<true, kClip>(b, S.row_first - b.row_base + fy, fx, fy, [&](const Cand &v) -> bool {
            const bool eo = (v.flags & 1u) != 0;
            const int8_t bd = (int8_t)(v.st & 0xffu);
            float cov[8];
            bool stop = false;
            entries++;
            if (!(v.st & 0x100u)) {
                if (solid_hidden(eo, bd)) return false;
#pragma unroll
                for (int k = 0; k < 8; k++) cov[k] = 1.0f;
                stop = (v.flags & 2u) != 0;
            } else {
                // the tile's own mask; kMaskClip (a solid tile over a clip alpha tile): the clip's;
                // kMaskBoth: the clip's mask first, parked, then the tile's own, combined as
                // tile_clip_combine.frag does - min(|draw + its backdrop|, |clip + its backdrop|) -
                // before the draw path's fill rule
                bool both = kClip && mask_mode(v.st) == kMaskBoth, combined = false;
                uint32_t f0 = v.f0, f1 = v.f1;
                int8_t tbd = bd;
                if (both) {
                    const uint32_t cp = b.path_clip_rel[v.p];
                    f0 = fill_begin(b, cp, v.gc);
                    f1 = b.tile_fills[v.gc];
                    tbd = (int8_t)(b.tile_state[v.gc] & 0xffu);
                }
                int raw[8];
                for (;;) {
                    comp_fills += f1 - f0;
                    coverage_raw(b.fills + f0, f1 - f0, tbd, D, prep[warp], raw);
                    __syncwarp();
                    if (!both) break;
#pragma unroll
                    for (int k = 0; k < 8; k++) park[warp][k][lane] = abs(raw[k]);
                    both = false;
                    combined = true;
                    f0 = v.f0;
                    f1 = v.f1;
                    tbd = (int8_t)(v.st >> 16);
                }
                if (combined) {
#pragma unroll
                    for (int k = 0; k < 8; k++) raw[k] = min(abs(raw[k]), park[warp][k][lane]);
                }
                coverage_rule(raw, eo, cov);
            }
            const uint32_t color = v.color;
            float pr = (float)(color & 0xffu) * inv255, pg = (float)((color >> 8) & 0xffu) * inv255,
                  pb = (float)((color >> 16) & 0xffu) * inv255, pa = (float)(color >> 24) * inv255;
            const uint32_t grad = kPaint ? b.path_grad[b.path_base + v.p] : kNone;
            bool opaque = true;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                if (kPaint && grad != kNone) {  // SrcIn over the opaque white base colour
                    const float4 g = gradient_color(b, grad, (float)(fx * 16 + col) + 0.5f,
                                                    (float)(fy * 16 + h * 8 + k) + 0.5f);
                    pr = g.x;
                    pg = g.y;
                    pb = g.z;
                    pa = g.w;
                }
                const float a = pa * cov[k], w = tr[k] * a;
                ar[k] += w * pr;
                ag[k] += w * pg;
                ab[k] += w * pb;
                tr[k] *= 1.0f - a;
                opaque &= tr[k] == 0.0f;
            }
            return stop || __all_sync(0xffffffffu, opaque);
        }, chunks);
        // the scene's image fields in registers before the stores: a store through the image
        // pointer may alias the scene table as far as the compiler knows, and would make it
        // load them again for every pixel
        const uint32_t img_w = S.img_w, img_h = S.img_h, clear = S.clear;
        const bool load_dst = S.load == PF_LOAD_LOAD;
        uchar4 *const img = reinterpret_cast<uchar4 *>(b.image + S.img_offset);
        const uint32_t px = fx * 16 + (uint32_t)col;
        if (px < img_w) {
            float cr = (float)(clear & 0xffu) * inv255, cg = (float)((clear >> 8) & 0xffu) * inv255,
                  cb = (float)((clear >> 16) & 0xffu) * inv255, ca = (float)(clear >> 24) * inv255;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t py = fy * 16 + (uint32_t)(h * 8 + k);
                if (py < img_h) {
                    if (load_dst) {
                        // LOAD_ACTION_LOAD (tile.comp:744-757): start from the pixel already there
                        const uchar4 d = img[(size_t)py * img_w + px];
                        cr = (float)d.x * inv255;
                        cg = (float)d.y * inv255;
                        cb = (float)d.z * inv255;
                        ca = (float)d.w * inv255;
                    }
                    img[(size_t)py * img_w + px] =
                        make_uchar4((unsigned char)__float2uint_rn(__saturatef(ar[k] + tr[k] * cr) * 255.0f),
                                    (unsigned char)__float2uint_rn(__saturatef(ag[k] + tr[k] * cg) * 255.0f),
                                    (unsigned char)__float2uint_rn(__saturatef(ab[k] + tr[k] * cb) * 255.0f),
                                    (unsigned char)__float2uint_rn(__saturatef(1.0f - tr[k] + tr[k] * ca) * 255.0f));
                }
            }
        }
    }
    if (b.counters) {
        // one reduction per block into the frame counters
        __shared__ uint32_t red[kCompWarps][3];
        if (lane == 0) {
            red[warp][0] = entries;
            red[warp][1] = comp_fills;
            red[warp][2] = chunks;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            uint32_t v = 0;
            for (int w = 0; w < kCompWarps; w++) v += red[w][threadIdx.x];
            const int slot = threadIdx.x == 0 ? kStEntries : (threadIdx.x == 1 ? kStListFills : kStWalkChunks);
            if (v) atomicAdd(&b.status[slot], v);
        }
    }
}

// Frame counters: the draw paths' alpha tiles and visible tiles (an alpha tile or a nonzero
// backdrop: the tiles build_tile_batches keeps, core/d3d9/scene_builder.cpp:57-63).  One block
// per path, over its tile states.
__global__ void __launch_bounds__(kThreads) k_tile_counts(Batch b) {
    __shared__ uint32_t red[2][kThreads / 32];
    const uint32_t p = blockIdx.x;
    const PathDev P = b.paths[p];
    uint32_t alpha = 0, visible = 0;
    if (!(P.flags & kPathIsClip)) {
        const uint32_t T = (uint32_t)max(P.rx1 - P.rx0, 0) * (uint32_t)max(P.ry1 - P.ry0, 0);
        for (uint32_t t = threadIdx.x; t < T; t += kThreads) {
            const uint32_t st = b.tile_state[P.tile_first + t];
            alpha += (st >> 8) & 1u;
            visible += (st & 0x1ffu) != 0;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        alpha += __shfl_down_sync(0xffffffffu, alpha, o);
        visible += __shfl_down_sync(0xffffffffu, visible, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = alpha;
        red[1][threadIdx.x >> 5] = visible;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        uint32_t v = 0;
        for (int w = 0; w < kThreads / 32; w++) v += red[threadIdx.x][w];
        if (v) atomicAdd(&b.status[threadIdx.x == 0 ? kStAlphaTiles : kStVisible], v);
    }
}

// Composite lists and z per framebuffer tile for the canonical output (not part of a frame):
// the same walk as k_composite, written back to front.
template <bool kWrite>
__global__ void __launch_bounds__(kCompWarps * 32) k_list_dump(Batch b) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t fb = blockIdx.x * kCompWarps + warp;
    if (fb >= b.n_fb) return;
    const uint32_t fbg = b.fb_base + fb;
    const uint32_t s = b.fb_scene[fbg];
    const SceneDev &S = b.scenes[s];
    const uint32_t local = fbg - S.fb_first;
    const uint32_t fx = local % S.fbw, fy = local / S.fbw;
    uint32_t n = 0, first = 0, count = 0, n_chunks = 0;
    int32_t z = -1;
    if (kWrite) {
        first = b.fb_count[fb];
        count = b.fb_count[fb + 1] - first;
    }
    walk_fb_tile<false, true>(b, S.row_first - b.row_base + fy, fx, fy, [&](const Cand &v) -> bool {
        if (kWrite && lane == 0) b.list[first + count - 1 - n] = v.gt;
        n++;
        const int8_t bd = (int8_t)(v.st & 0xffu);
        if (!(v.st & 0x100u) && (v.flags & 2u) && !solid_hidden((v.flags & 1u) != 0, bd)) {
            z = (int32_t)v.p;
            return true;
        }
        return false;
    }, n_chunks);
    if (lane == 0) {
        if (kWrite) b.z[fb] = z;
        else b.fb_count[fb] = n;
    }
}

// Every tile of the frame after the clip rules, for the canonical output (not part of a frame):
// the state the composite's walk sees - apply_clip, the same function, on each tile of a
// clipped path - and the clip tile whose mask it takes (kNone if none).  state[t] holds the
// int8 backdrop in bits 0-7, the alpha flag in bit 8, the mask source in bits 9-10 and, for
// kMaskBoth, the draw tile's own backdrop in bits 16-23.  One thread per tile.
__global__ void __launch_bounds__(kThreads) k_clip_dump(Batch b, uint32_t n_tiles, uint32_t *state, uint32_t *clip) {
    const uint32_t t = global_tid();
    if (t >= n_tiles) return;
    const uint32_t p = upper_bound(b.path_tiles, b.n_paths + 1, t) - 1;
    Cand c{0, t, b.tile_state[t], 0, 0, 0, 0, kNone};
    if (b.path_clip_rel[p] != kNone && !(b.paths[p].flags & kPathIsClip)) {
        const PathDev P = b.paths[p];
        const uint32_t local = t - P.tile_first, rw = (uint32_t)(P.rx1 - P.rx0);
        apply_clip(b, p, P.rx0 + (int32_t)(local % rw), P.ry0 + (int32_t)(local / rw), c);
        if (mask_mode(c.st) == kMaskOwn) c.gc = kNone;
    }
    state[t] = c.st;
    clip[t] = c.gc;
}

// Coverage of listed alpha tiles after the fill rule (test output; one warp per tile).
__global__ void __launch_bounds__(kCompWarps * 32) k_coverage_dump(Batch b, const uint32_t *tiles, uint32_t n,
                                                                   float *out) {
    __shared__ int cells[kCompWarps][kCovCells];
    __shared__ FillPrep prep[kCompWarps][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t k = blockIdx.x * kCompWarps + warp;
    if (k >= n) return;
    int *D = cells[warp];
    const uint32_t gt = tiles[k];
    const uint32_t p = upper_bound(b.path_tiles, b.n_paths + 1, gt) - 1;
    zero_cells(D);
    float cov[8];
    alpha_coverage(b, fill_begin(b, p, gt), b.tile_fills[gt], (int8_t)(b.tile_state[gt] & 0xffu),
                   (b.paths[p].flags & 1u) != 0, D, prep[warp], cov);
    const int col = lane & 15, h = lane >> 4;
#pragma unroll
    for (int r = 0; r < 8; r++) out[(size_t)k * 256 + (h * 8 + r) * 16 + col] = cov[r];
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers

static std::atomic<uint64_t> g_launches{0};
uint64_t launches() { return g_launches.load(); }
void count_launches(uint32_t n) { g_launches += n; }

#define PF_LAUNCH(...)           \
    do {                         \
        __VA_ARGS__;             \
        count_launches(1);       \
    } while (0)

cudaError_t launch_normalize(const Batch &b, uint2 *path_contours, cudaStream_t st) {
    if (b.n_contours) PF_LAUNCH(k_normalize_contours<<<grid_for(b.n_contours), kThreads, 0, st>>>(b));
    if (b.n_paths) PF_LAUNCH(k_normalize_paths<<<grid_for(b.n_paths), kThreads, 0, st>>>(b, path_contours));
    return cudaGetLastError();
}

cudaError_t launch_path_setup(const Batch &b, const uint2 *path_contours, cudaStream_t st) {
    if (b.n_paths) PF_LAUNCH(k_path_setup<<<grid_for(uint64_t(b.n_paths) * 32), kThreads, 0, st>>>(b, path_contours));
    return cudaGetLastError();
}

cudaError_t launch_path_offsets(const Batch &b, cudaStream_t st) {
    if (b.n_paths) PF_LAUNCH(k_path_offsets<<<grid_for(b.n_paths), kThreads, 0, st>>>(b));
    return cudaGetLastError();
}

cudaError_t launch_contour_segments(const Batch &b, bool write, cudaStream_t st) {
    if (!b.n_contours) return cudaSuccess;
    if (write) PF_LAUNCH(k_contour_segments<true><<<grid_for(b.n_contours), kThreads, 0, st>>>(b));
    else PF_LAUNCH(k_contour_segments<false><<<grid_for(b.n_contours), kThreads, 0, st>>>(b));
    return cudaGetLastError();
}

// The warp-shared flattening runs as many blocks as fit on every SM (they take segments by
// ticket), fewer when the frame has fewer groups of 32 segments than resident warps.
template <bool kExact>
static cudaError_t flatten_pool_blocks(uint64_t *resident) {
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_flatten_pool<kExact>, kPoolWarps * 32, 0);
    *resident = uint64_t(std::max(1, per_sm)) * uint64_t(sms);
    return e;
}

template <bool kExact>
static cudaError_t launch_flatten_pool(const Batch &b, uint32_t n_segs, cudaStream_t st) {
    uint64_t resident = 0;
    if (const cudaError_t e = flatten_pool_blocks<kExact>(&resident)) return e;
    const uint64_t groups = (uint64_t(n_segs) + 31) / 32;
    const uint64_t blocks = std::min<uint64_t>(resident, (groups + kPoolWarps - 1) / kPoolWarps);
    PF_LAUNCH(k_flatten_pool<kExact><<<(unsigned)blocks, kPoolWarps * 32, 0, st>>>(b, n_segs));
    return cudaGetLastError();
}

// Exact frame: the count pass one segment per thread (it stores nothing, so its stack stays in
// L1).  The write pass is shared by the lanes of a warp when the segments bisect deeply enough
// and are many enough to give every resident warp a group of 32; otherwise one segment per
// thread keeps more of them in flight (GB300, exact frames: 512-scene batch, 51 lines per
// segment, 38.28 -> 34.48 ms with the shared pass; 20,000 paths, 25 per segment, 2.28 -> 2.10 ms;
// 150,000 glyphs, 2.3 per segment, 2.29 -> 2.37 ms; 240 paths, 4,062 segments, 0.445 -> 0.453 ms).
constexpr uint64_t kPoolMinLinesPerSeg = 8;

cudaError_t launch_flatten(const Batch &b, uint32_t n_segs, bool write, cudaStream_t st, uint64_t n_lines) {
    if (!n_segs) return cudaSuccess;
    if (write) {
        uint64_t resident = 0;
        if (const cudaError_t e = flatten_pool_blocks<true>(&resident)) return e;
        if (n_lines >= kPoolMinLinesPerSeg * n_segs && n_segs >= resident * kPoolWarps * 32)
            return launch_flatten_pool<true>(b, n_segs, st);
        PF_LAUNCH(k_flatten<true><<<grid_for(n_segs), kThreads, 0, st>>>(b, n_segs));
        return cudaGetLastError();
    }
    PF_LAUNCH(k_flatten<false><<<grid_for(n_segs), kThreads, 0, st>>>(b, n_segs));
    return cudaGetLastError();
}

size_t seg_ctl_bytes() { return (size_t(kSegBlocks) + 1) * kSegBuckets * 4; }

cudaError_t launch_seg_order(const Batch &b, uint32_t n_segs, uint32_t *ctl, cudaStream_t st) {
    if (!n_segs) return cudaSuccess;
    PF_LAUNCH(k_seg_buckets<false><<<kSegBlocks, kThreads, 0, st>>>(b, ctl));
    PF_LAUNCH(k_seg_bucket_totals<<<kSegBuckets, kThreads, 0, st>>>(ctl));
    PF_LAUNCH(k_seg_bucket_starts<<<kSegBuckets, kThreads, 0, st>>>(ctl));
    PF_LAUNCH(k_seg_buckets<true><<<kSegBlocks, kThreads, 0, st>>>(b, ctl));
    return cudaGetLastError();
}

cudaError_t launch_flatten_budget(const Batch &b, uint32_t n_segs, cudaStream_t st) {
    if (!n_segs) return cudaSuccess;
    return launch_flatten_pool<false>(b, n_segs, st);
}

cudaError_t launch_bin_classify(const Batch &b, bool learned, cudaStream_t st) {
    if (b.n_paths) {
        PF_LAUNCH(k_bin_classify<<<grid_for(b.n_paths), kThreads, 0, st>>>(b, learned));
        PF_LAUNCH(k_bin_bucket_starts<<<1, 32, 0, st>>>(b));
        PF_LAUNCH(k_bin_scatter<<<grid_for(b.n_paths), kThreads, 0, st>>>(b));
    }
    return cudaGetLastError();
}

// Grid of a CTA class: as many CTAs as fit on every SM (they take paths by ticket), or
// per_sm_wanted per SM when that is nonzero and fits.
template <int kCls>
static cudaError_t fused_grid(unsigned *grid, uint32_t per_sm_wanted = 0) {
    const size_t smem = size_t(class_words(kCls)) * 4;
    static int configured_device = -1;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (configured_device != dev) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_bin_fused<kCls>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured_device = dev;
    }
    int per_sm = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bin_fused<kCls>, class_threads(kCls), smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(1, per_sm);
    if (per_sm_wanted) per_sm = std::min(per_sm, (int)per_sm_wanted);
    *grid = (unsigned)per_sm * (unsigned)sms;
    return cudaSuccess;
}

template <int kCls>
static cudaError_t launch_fused(const Batch &b, uint32_t per_sm, cudaStream_t st) {
    unsigned grid = 0;
    const cudaError_t e = fused_grid<kCls>(&grid, per_sm);
    if (e != cudaSuccess) return e;
    PF_LAUNCH(k_bin_fused<kCls><<<grid, class_threads(kCls), size_t(class_words(kCls)) * 4, st>>>(b));
    return cudaGetLastError();
}

cudaError_t bin_stage_bytes(const Tuning &t, size_t *bytes) {
    unsigned g0 = 0, g1 = 0, g2 = 0;
    cudaError_t e;
    if ((e = fused_grid<0>(&g0, t.bin_ctas_per_sm[0])) != cudaSuccess) return e;
    if ((e = fused_grid<1>(&g1, t.bin_ctas_per_sm[1])) != cudaSuccess) return e;
    if ((e = fused_grid<2>(&g2, t.bin_ctas_per_sm[2])) != cudaSuccess) return e;
    const size_t s0 = size_t(g0) * class_stage(0), s1 = size_t(g1) * class_stage(1), s2 = size_t(g2) * class_stage(2);
    // concurrent classes each keep their own slice of the stage
    *bytes = 8 * (t.bin_concurrent ? s0 + s1 + s2 : std::max({s0, s1, s2}));
    return cudaSuccess;
}

cudaError_t bin_class_max_ctas(int out[3]) {
    unsigned g[3];
    cudaError_t e;
    if ((e = fused_grid<0>(&g[0])) != cudaSuccess) return e;
    if ((e = fused_grid<1>(&g[1])) != cudaSuccess) return e;
    if ((e = fused_grid<2>(&g[2])) != cudaSuccess) return e;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int c = 0; c < 3; c++) out[c] = (int)(g[c] / (unsigned)sms);
    return cudaSuccess;
}

// Class 3 (zero, count, backdrops and offsets, write; each returns at once when the class is
// empty), then the CTA classes, largest rects first.
cudaError_t launch_bin_paths(const Batch &b, const Tuning &t, const BinStreams *bs, cudaStream_t st) {
    if (!b.n_paths) return cudaSuccess;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    PF_LAUNCH(k_bin_zero_large<<<sms * 2, 256, 0, st>>>(b));
    PF_LAUNCH(k_bin_large<false><<<sms * 8, kThreads, 0, st>>>(b));
    PF_LAUNCH(k_bin_large_prep<<<sms * 2, kPrepThreads, 0, st>>>(b));
    PF_LAUNCH(k_bin_large<true><<<sms * 8, kThreads, 0, st>>>(b));
    cudaError_t e;
    if (!t.bin_concurrent || !bs) {
        if ((e = launch_fused<2>(b, t.bin_ctas_per_sm[2], st)) != cudaSuccess) return e;
        if ((e = launch_fused<1>(b, t.bin_ctas_per_sm[1], st)) != cudaSuccess) return e;
        return launch_fused<0>(b, t.bin_ctas_per_sm[0], st);
    }
    // the three classes at once: classes 1 and 0 on side streams, each with its own slice of
    // the fill stage (the classes' grids follow each other in it), joined back before the
    // composite; the block scheduler fills the SMs a class's tail leaves idle with the others
    unsigned g2 = 0, g1 = 0;
    if ((e = fused_grid<2>(&g2, t.bin_ctas_per_sm[2])) != cudaSuccess) return e;
    if ((e = fused_grid<1>(&g1, t.bin_ctas_per_sm[1])) != cudaSuccess) return e;
    if ((e = cudaEventRecord(bs->fork, st)) != cudaSuccess) return e;
    for (int k = 0; k < 2; k++)
        if ((e = cudaStreamWaitEvent(bs->side[k], bs->fork, 0)) != cudaSuccess) return e;
    Batch b1 = b, b0 = b;
    b1.stage = b.stage ? b.stage + size_t(g2) * class_stage(2) : nullptr;
    b0.stage = b.stage ? b1.stage + size_t(g1) * class_stage(1) : nullptr;
    if ((e = launch_fused<2>(b, t.bin_ctas_per_sm[2], st)) != cudaSuccess) return e;
    if ((e = launch_fused<1>(b1, t.bin_ctas_per_sm[1], bs->side[0])) != cudaSuccess) return e;
    if ((e = launch_fused<0>(b0, t.bin_ctas_per_sm[0], bs->side[1])) != cudaSuccess) return e;
    for (int k = 0; k < 2; k++) {
        if ((e = cudaEventRecord(bs->join[k], bs->side[k])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st, bs->join[k], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_pool_lists(const Batch &b, bool scatter, cudaStream_t st) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (scatter) PF_LAUNCH(k_pool_scatter<<<sms * 2, kThreads, 0, st>>>(b));
    else PF_LAUNCH(k_pool_count<<<sms * 2, kThreads, 0, st>>>(b));
    return cudaGetLastError();
}

// Status words to pinned host memory by a kernel rather than a copy-engine transfer, so a
// frame's readback never queues behind a large device-to-host copy (pf_read_images_async).
__global__ void k_copy_words(uint32_t *dst, const uint32_t *src, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

cudaError_t launch_copy_words(uint32_t *dst, const uint32_t *src, uint32_t n, cudaStream_t st) {
    if (n) PF_LAUNCH(k_copy_words<<<1, 64, 0, st>>>(dst, src, n));
    return cudaGetLastError();
}

// Small device reads (totals, flags, per-scene bounds) into mapped host memory the same way.
__global__ void k_copy_bytes(uint8_t *dst, const uint8_t *src, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

__global__ void k_gather_words(uint32_t *dst, WordSources s) {
    if (threadIdx.x < s.n) dst[threadIdx.x] = *s.p[threadIdx.x];
}

cudaError_t launch_copy_bytes(uint8_t *dst, const uint8_t *src, uint32_t n, cudaStream_t st) {
    if (n) PF_LAUNCH(k_copy_bytes<<<std::min<uint32_t>((n + 255) / 256, 64), 256, 0, st>>>(dst, src, n));
    return cudaGetLastError();
}

cudaError_t launch_gather_words(uint32_t *dst, const WordSources &s, cudaStream_t st) {
    if (s.n) PF_LAUNCH(k_gather_words<<<1, 32, 0, st>>>(dst, s));
    return cudaGetLastError();
}

cudaError_t launch_rows(const Batch &b, bool write, cudaStream_t st) {
    if (!b.n_rows) return cudaSuccess;
    if (write) PF_LAUNCH(k_rows<true><<<b.n_rows, kRowThreads, 0, st>>>(b));
    else PF_LAUNCH(k_rows<false><<<b.n_rows, kRowThreads, 0, st>>>(b));
    return cudaGetLastError();
}

// Grid of the composite: a warp per framebuffer tile, or (ticketed) as many resident blocks as
// fit on every SM.
template <bool kClip, bool kPaint>
static cudaError_t launch_composite_variant(const Batch &b, cudaStream_t st) {
    if (!b.comp_ticket) {
        PF_LAUNCH(k_composite<kClip, kPaint, false><<<grid_for(b.n_fb, kCompWarps), kCompWarps * 32, 0, st>>>(b));
        return cudaGetLastError();
    }
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_composite<kClip, kPaint, true>, kCompWarps * 32, 0);
    if (e != cudaSuccess) return e;
    const unsigned grid =
        std::min<unsigned>(grid_for(b.n_fb, kCompWarps), (unsigned)std::max(per_sm, 1) * (unsigned)sms);
    PF_LAUNCH(k_composite<kClip, kPaint, true><<<grid, kCompWarps * 32, 0, st>>>(b));
    return cudaGetLastError();
}

cudaError_t launch_composite(const Batch &b, cudaStream_t st) {
    if (!b.n_fb) return cudaSuccess;
    if (b.path_clip_cat && b.path_grad) return launch_composite_variant<true, true>(b, st);
    if (b.path_clip_cat) return launch_composite_variant<true, false>(b, st);
    if (b.path_grad) return launch_composite_variant<false, true>(b, st);
    return launch_composite_variant<false, false>(b, st);
}

// One block per scene: its framebuffer tiles get its index.
__global__ void k_fb_scene(const uint32_t *scene_fb_first, uint32_t *fb_scene) {
    const uint32_t s = blockIdx.x, a = scene_fb_first[s], e = scene_fb_first[s + 1];
    for (uint32_t t = a + threadIdx.x; t < e; t += blockDim.x) fb_scene[t] = s;
}

cudaError_t launch_fb_scene(const uint32_t *scene_fb_first, uint32_t n_scenes, uint32_t *fb_scene, cudaStream_t st) {
    if (n_scenes) PF_LAUNCH(k_fb_scene<<<n_scenes, kThreads, 0, st>>>(scene_fb_first, fb_scene));
    return cudaGetLastError();
}

cudaError_t launch_tile_counts(const Batch &b, cudaStream_t st) {
    if (b.n_paths) PF_LAUNCH(k_tile_counts<<<b.n_paths, kThreads, 0, st>>>(b));
    return cudaGetLastError();
}

cudaError_t launch_list_dump(const Batch &b, bool write, cudaStream_t st) {
    if (!b.n_fb) return cudaSuccess;
    if (write) PF_LAUNCH(k_list_dump<true><<<grid_for(b.n_fb, kCompWarps), kCompWarps * 32, 0, st>>>(b));
    else PF_LAUNCH(k_list_dump<false><<<grid_for(b.n_fb, kCompWarps), kCompWarps * 32, 0, st>>>(b));
    return cudaGetLastError();
}

cudaError_t launch_clip_dump(const Batch &b, uint32_t n_tiles, uint32_t *state, uint32_t *clip, cudaStream_t st) {
    if (n_tiles && b.path_clip_cat) PF_LAUNCH(k_clip_dump<<<grid_for(n_tiles), kThreads, 0, st>>>(b, n_tiles, state, clip));
    return cudaGetLastError();
}

cudaError_t launch_coverage_dump(const Batch &b, const uint32_t *tiles, uint32_t n, float *out, cudaStream_t st) {
    if (n) PF_LAUNCH(k_coverage_dump<<<grid_for(n, kCompWarps), kCompWarps * 32, 0, st>>>(b, tiles, n, out));
    return cudaGetLastError();
}

}  // namespace pfc
