// pf_api.cu - host side of the fill pipeline: context, device buffers, stage order,
// and the C-ABI of include/pfcuda.h.
//
// The exact two-pass frame (pf_render) is the reference's count-then-allocate loop
// (RendererD3D11::prepare_tiles, pathfinder/core/d3d11/renderer.cpp:510-616) done with
// exact counts: every stage that appends (segments, leaf lines, fills, composite-list
// entries) first counts on the GPU, the counts are scanned into offsets, the host reads
// the total and grows the buffer, and the second pass writes into place.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/pfcuda.h"
#include "pf_internal.h"

using namespace pfc;

namespace {

constexpr size_t kStageBytes = 64 << 10;  // mapped host staging for small device reads

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes + bytes / 4, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostCanon {
    std::vector<int32_t> rect;
    std::vector<uint64_t> tile_first, col_first;
    std::vector<uint8_t> alpha;
    std::vector<int8_t> backdrop;
    std::vector<uint32_t> fill_count;
    std::vector<uint16_t> fills;
    std::vector<int32_t> col_backdrop;
    std::vector<int32_t> z;
    std::vector<uint64_t> list_first;
    std::vector<uint32_t> list;
    std::vector<uint8_t> mask;
    std::vector<uint64_t> clip;
    std::vector<int8_t> dest_backdrop;
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t flags = 0;
    std::string err;

    // inputs
    DevBuf points, pflags, cstart, pstart, fill_rule, color, scenes, scene_path_first, scene_contour_first,
        scene_fb_first, fb_scene;
    std::vector<SceneDev> h_scenes;
    std::vector<uint32_t> h_scene_fb_first;
    // clip paths: per uploaded path its scene-local clip path (PF_NO_CLIP) and whether it is one;
    // empty when no scene of the batch has clip paths
    DevBuf path_clip, path_is_clip, path_clip_rel;
    std::vector<uint32_t> h_path_clip;
    std::vector<uint8_t> h_path_is_clip;
    // stroked paths: the uploaded outline and what the upload's stroke pass works in
    DevBuf in_points, in_pflags, in_cstart, in_pstart, st_stroke, st_closed, st_dashes, st_scenes, st_cfirst;
    DevBuf dash_pts, dash_cnt, dash_end, dash_points, dash_flags, job_first, jobs, job_pts, st_bounds;
    DevBuf job_units, job_nfwd, job_flags, job_cap1, job_end, units, unit_leaves, st_leaves, leaf_pts;
    DevBuf st_order_ctl, unit_order, dash_order;
    uint32_t stroke_jobs = 0, stroke_dash_points = 0;  // of the last upload with strokes
    // gradient paints: per uploaded path its gradient (kNone: solid), per gradient its paint,
    // sorted stops, ramp and shader metadata; empty when the batch has no gradient
    DevBuf path_grad, grad_paint, grad_stop_range, grad_stops, grad_meta, grad_ramp;
    uint32_t n_grads = 0;
    std::vector<uint32_t> h_grad_sbase;  // the scenes' first stops (kept until the upload's copies end)
    pf_upload_stats ustats{};
    cudaEvent_t sev[8] = {};  // stroke pass timing (stage timing on)
    uint32_t n_scenes = 0, n_paths = 0, n_contours = 0, n_points = 0, n_fb = 0;
    uint64_t image_bytes = 0;
    bool uploaded = false, rendered = false;

    // working buffers
    DevBuf contour_point_first, contour_path, paths, path_tiles, path_cols, contour_segs, path_contours, path_bounds;
    // learned sizer: weights (bf16 used by the kernels, fp32 master + Adam moments for training)
    DevBuf sz_w, sz_master, sz_m, sz_v, sz_grad, sz_loss, sz_feat, sz_target, sz_index, sz_pred;
    DevBuf path_feat, contour_feat, path_pred, path_leaf_first, path_leaf_budget, path_leaf_cursor, path_fill_budget;
    DevBuf bin_list, bin_ctl, path_leaf_range;
    int sz_step = 0;
    bool sz_ready = false;
    float sz_mul = 1.25f, sz_add = 8.0f, sz_pool = 0.10f;
    uint32_t last_paths_over = 0, last_pool_used = 0;
    DevBuf segs, seg_leaves, seg_order, seg_ctl, leaves, pool_path, pool_cnt, pool_idx;
    DevBuf tile_fills, tile_state, col_above, col_final, fills, path_fill, path_cls, bin_stage;
    DevBuf row_first, row_paths, scene_row_first;
    DevBuf z, fb_count, list, image, status, scan_temp;
    DevBuf canon_state, canon_clip;  // clipped frames: tile states after the clip rules (read-back only)
    // host image target (pf_set_host_image): frames composite straight into this host buffer
    uint8_t *host_img = nullptr;      // host address
    uint8_t *host_img_dev = nullptr;  // the same memory as the device addresses it
    size_t host_img_bytes = 0;
    bool host_img_registered = false; // pinned by this context (unpinned when replaced)
    // asynchronous image readback (pf_read_images_async): a device snapshot of the images and
    // its copy to the host on a stream of its own
    DevBuf image_snap;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_done = nullptr, copy_done = nullptr;
    bool copy_pending = false;
    uint32_t *h_status = nullptr;      // pinned
    uint32_t *h_status_dev = nullptr;  // the same memory as the device addresses it
    uint8_t *h_stage = nullptr, *h_stage_dev = nullptr;  // mapped staging for small reads

    // the scene range of the last frame and its totals
    uint32_t r_first = 0, r_count = 0, r_paths = 0, r_contours = 0, r_fb = 0, r_rows = 0;
    uint32_t r_path_base = 0, r_contour_base = 0, r_fb_base = 0, r_row_base = 0;
    uint32_t n_segs = 0, n_tiles = 0, n_cols = 0, n_leaves = 0, n_list = 0, n_row_entries = 0;
    uint64_t n_fills = 0;
    uint64_t fill_hint = 0;  // fills of the largest frame so far: the next frame's starting capacity
    bool lists_dumped = false;
    std::vector<uint32_t> h_scene_row_first;
    uint32_t syncs = 0;

    HostCanon canon;
    struct {
        std::vector<float2> points;
        std::vector<uint8_t> flags, rule;
        std::vector<uint32_t> cstart, pstart;
    } outline;  // pf_read_outline's arrays
    cudaEvent_t ev[8] = {};

    // The learned frame captured as a CUDA graph once it has run with its buffers sized: later
    // frames over the same scenes replay it (one launch, one synchronisation) while the
    // uploaded scenes, the sizer, the flags, the image target and every buffer stay the same.
    cudaGraphExec_t lg_exec = nullptr;
    uint32_t lg_first = 0, lg_count = 0, lg_flags = 0, lg_launches = 0;
    uint32_t lg_status[kStCount] = {};  // the totals the captured frame was sized for
    std::vector<void *> lg_ptrs;        // the buffers it uses, by address
    bool capturing = false;             // recording the graph: no host synchronisation
    bool learned_done = false;          // the last learned frame ran the learned path to the end
    // The graph is recorded on the second learned frame in a row over the same upload, range,
    // flags and buffers (a frame after every upload never replays: recording it would be wasted)
    struct {
        bool valid = false;
        uint64_t epoch = 0;
        uint32_t first = 0, count = 0, flags = 0;
        std::vector<void *> ptrs;
        uint32_t status[kStCount] = {};  // the totals the plain frame sized its buffers for
    } lg_prev;
    int lg_kind = 0;  // the last learned frame: 0 plain, 1 recorded then replayed, 2 replayed

    // pf_render_auto: the device times of the exact and the learned frame over a workload (the
    // scene range and the upload's totals), measured as they run; the faster one runs once both
    // are known
    uint64_t upload_epoch = 0;
    struct {
        uint64_t sig[5] = {~0ull, 0, 0, 0, 0};  // first, count, paths, contours, points of the range
        float exact_ms = -1.0f, learned_ms = -1.0f;  // fastest timed frame of each kind; < 0: none yet
        int exact_runs = 0, learned_runs = 0;    // frames run over the workload (the first is not timed)
        int exact_timed = 0, learned_timed = 0;  // frames timed (kAutoSamples of each decide)
        int last = PF_FRAME_EXACT;     // the frame the last auto call ran
    } au;
    cudaEvent_t au_ev[2] = {};

    // launch parameters (pf_tuning) and the side streams of concurrent binning classes
    Tuning tune;
    BinStreams bs{};
    bool bs_ready = false;
};

thread_local std::string g_last_error;

void drop_graph(Ctx *c);
void forget_learned(Ctx *c);

int fail(Ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    g_last_error = msg;
    return code;
}

int cuda_fail(Ctx *c, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? PF_ERR_OUT_OF_MEMORY : PF_ERR_CUDA, m);
}

#define PF_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);     \
    } while (0)

float view_box_right(float width) {
    // Scene::set_view_box: right = round_up(ceil(right), 16) (pathfinder/core/scene.cpp:175)
    int32_t w = (int32_t)std::ceil(width);
    int32_t rem = std::abs(w) % kTile;
    if (rem != 0) w = w < 0 ? w + rem : w + kTile - rem;
    return (float)w;
}

int validate_scene(Ctx *c, const pf_scene_view *s) {
    if (!s) return fail(c, PF_ERR_INVALID_ARGUMENT, "scene is null");
    if (!(s->width > 0.0f) || !(s->height > 0.0f) || !std::isfinite(s->width) || !std::isfinite(s->height) ||
        s->width > 65536.0f || s->height > 65536.0f)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "canvas size must be finite, positive and at most 65536");
    if (!s->path_start || !s->contour_start)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "path_start and contour_start are required");
    if (s->load_action > PF_LOAD_LOAD) return fail(c, PF_ERR_INVALID_ARGUMENT, "unknown load action");
    if (s->view_box) {
        const float *v = s->view_box;
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(v[k]) || std::fabs(v[k]) > 65536.0f)
                return fail(c, PF_ERR_INVALID_ARGUMENT, "view box coordinates must be finite and within 65536");
        if (!(v[0] <= v[2]) || !(v[1] <= v[3]))
            return fail(c, PF_ERR_INVALID_ARGUMENT, "the view box needs left <= right and top <= bottom");
    }
    if (s->n_paths && (!s->fill_rule || !s->color))
        return fail(c, PF_ERR_INVALID_ARGUMENT, "fill_rule and color are required");
    if (s->n_points && (!s->points || !s->point_flags))
        return fail(c, PF_ERR_INVALID_ARGUMENT, "points and point_flags are required");
    if (s->path_start[0] != 0 || s->path_start[s->n_paths] != s->n_contours)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "path_start must run from 0 to n_contours");
    if (s->contour_start[0] != 0 || s->contour_start[s->n_contours] != s->n_points)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "contour_start must run from 0 to n_points");
    for (uint32_t p = 0; p < s->n_paths; p++)
        if (s->path_start[p] > s->path_start[p + 1])
            return fail(c, PF_ERR_INVALID_ARGUMENT, "path_start must be non-decreasing");
    for (uint32_t k = 0; k < s->n_contours; k++)
        if (s->contour_start[k] > s->contour_start[k + 1])
            return fail(c, PF_ERR_INVALID_ARGUMENT, "contour_start must be non-decreasing");
    for (uint32_t p = 0; s->path_stroke && p < s->n_paths; p++) {
        // StrokeStyle (core/stroke.h:14-27) and the canvas's dash pattern
        const pf_stroke &st = s->path_stroke[p];
        if (!(st.line_width >= 0.0f) || !std::isfinite(st.line_width) || !std::isfinite(st.miter_limit) ||
            st.line_cap > PF_CAP_ROUND || st.line_join > PF_JOIN_ROUND)
            return fail(c, PF_ERR_INVALID_ARGUMENT, "stroke styles need a finite width >= 0, a finite miter "
                                                    "limit and a known cap and join");
        if (st.line_width == 0.0f) continue;
        for (uint32_t i = s->contour_start[s->path_start[p]]; i < s->contour_start[s->path_start[p + 1]]; i++)
            if (!std::isfinite(s->points[2 * i]) || !std::isfinite(s->points[2 * i + 1]))
                return fail(c, PF_ERR_INVALID_ARGUMENT, "a stroked path has a non-finite point");
        if (st.dash_count) {
            if (!s->dashes || uint64_t(st.dash_first) + st.dash_count > s->n_dashes)
                return fail(c, PF_ERR_INVALID_ARGUMENT, "a dash pattern lies outside the dashes array");
            float total = 0.0f;
            for (uint32_t i = 0; i < st.dash_count; i++) {
                const float d = s->dashes[st.dash_first + i];
                if (!(d >= 0.0f) || !std::isfinite(d))
                    return fail(c, PF_ERR_INVALID_ARGUMENT, "dash lengths must be finite and >= 0");
                total += d;
            }
            // an all-zero pattern never advances (the reference loops forever on it)
            if (!(total > 0.0f) || !std::isfinite(total) || !std::isfinite(st.dash_offset))
                return fail(c, PF_ERR_INVALID_ARGUMENT, "a dash pattern needs a finite positive total and phase");
        }
    }
    for (uint32_t p = 0; s->path_paint && p < s->n_paths; p++) {
        // Paint::from_gradient (core/paint/paint.h:87-95)
        const pf_paint &pp = s->path_paint[p];
        if (pp.type > PF_PAINT_RADIAL || pp.wrap > PF_WRAP_REPEAT)
            return fail(c, PF_ERR_INVALID_ARGUMENT, "unknown paint type or wrap mode");
        if (pp.type == PF_PAINT_SOLID) continue;
        if ((pp.stop_count && !s->stops) || uint64_t(pp.stop_first) + pp.stop_count > s->n_stops)
            return fail(c, PF_ERR_INVALID_ARGUMENT, "a gradient's stops lie outside the stops array");
        if (pp.stop_count > 1024) return fail(c, PF_ERR_INVALID_ARGUMENT, "at most 1024 stops per gradient");
        for (uint32_t i = 0; i < pp.stop_count; i++)
            if (!std::isfinite(s->stops[pp.stop_first + i].offset))
                return fail(c, PF_ERR_INVALID_ARGUMENT, "gradient stop offsets must be finite");
        bool finite = true;
        for (float v : pp.line) finite &= std::isfinite(v);
        for (float v : pp.radii) finite &= std::isfinite(v);
        for (float v : pp.transform) finite &= std::isfinite(v);
        if (!finite) return fail(c, PF_ERR_INVALID_ARGUMENT, "gradient geometry must be finite");
    }
    if (s->path_clip || s->path_is_clip) {
        // Scene::push_draw_path / push_clip_path: clip paths come after every draw path, are not
        // clipped themselves, and a draw path names a clip path or none
        if (!s->path_clip || !s->path_is_clip)
            return fail(c, PF_ERR_INVALID_ARGUMENT, "path_clip and path_is_clip go together");
        bool seen_clip = false;
        for (uint32_t p = 0; p < s->n_paths; p++) {
            const uint32_t k = s->path_clip[p];
            if (s->path_is_clip[p]) {
                seen_clip = true;
                if (k != PF_NO_CLIP) return fail(c, PF_ERR_INVALID_ARGUMENT, "a clip path is not clipped");
            } else {
                if (seen_clip) return fail(c, PF_ERR_INVALID_ARGUMENT, "clip paths follow all draw paths");
                if (k != PF_NO_CLIP && (k >= s->n_paths || !s->path_is_clip[k]))
                    return fail(c, PF_ERR_INVALID_ARGUMENT, "path_clip must name a clip path of the scene");
            }
        }
    }
    return PF_OK;
}

// Copy n bytes from host to device, merging with the previous copy when the host
// ranges are contiguous (a batch packed into one host buffer costs one copy per array).
struct CopyPlan {
    struct Op {
        const char *src;
        char *dst;
        size_t n;
    };
    std::vector<Op> ops;
    void add(void *dst, const void *src, size_t n) {
        if (!n) return;
        const char *s = static_cast<const char *>(src);
        char *d = static_cast<char *>(dst);
        if (!ops.empty() && ops.back().src + ops.back().n == s && ops.back().dst + ops.back().n == d) {
            ops.back().n += n;
            return;
        }
        ops.push_back({s, d, n});
    }
    cudaError_t run(cudaStream_t st) {
        for (auto &o : ops) {
            cudaError_t e = cudaMemcpyAsync(o.dst, o.src, o.n, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
};

// Device to host and wait.  Small reads go through a kernel into mapped host memory, not the
// copy engine, so they never queue behind an image copy (pf_read_images_async).
template <class T>
int d2h_wait(Ctx *c, T *host, const void *dev, size_t count) {
    const size_t bytes = count * sizeof(T);
    if (bytes <= kStageBytes) {
        PF_CUDA(launch_copy_bytes(c->h_stage_dev, static_cast<const uint8_t *>(dev), (uint32_t)bytes, c->stream));
        PF_CUDA(cudaStreamSynchronize(c->stream));
        std::memcpy(host, c->h_stage, bytes);
        return PF_OK;
    }
    PF_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

// Single words from device memory, gathered by one kernel into mapped host memory, and wait.
int read_words(Ctx *c, std::initializer_list<const uint32_t *> src, uint32_t *out) {
    WordSources s{};
    for (const uint32_t *p : src) s.p[s.n++] = p;
    PF_CUDA(launch_gather_words(reinterpret_cast<uint32_t *>(c->h_stage_dev), s, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    std::memcpy(out, c->h_stage, s.n * 4);
    return PF_OK;
}

// Stroke-to-fill and dashing of the uploaded scenes (pf_stroke.cu): reads the outline staged
// in the in_* buffers with the input layout in c->h_scenes, writes the fill outline into the
// buffers the frames read and rewrites the scene table for it.  scf: the input's first contour
// per scene.
int stroke_upload(Ctx *c, const pf_scene_view *scenes, uint32_t n, const std::vector<uint32_t> &scf) {
    cudaStream_t st = c->stream;
    const uint32_t N = c->n_paths, C = c->n_contours;
    std::vector<pf_stroke> hs(N);
    std::vector<uint8_t> hc(C, 0);
    std::vector<float> hd;
    bool dashed = false;
    std::memset(hs.data(), 0, hs.size() * sizeof(pf_stroke));
    for (uint32_t i = 0; i < n; i++) {
        const pf_scene_view &s = scenes[i];
        const SceneDev &S = c->h_scenes[i];
        const uint32_t base = (uint32_t)hd.size();
        if (s.path_stroke)
            for (uint32_t p = 0; p < s.n_paths; p++) {
                pf_stroke x = s.path_stroke[p];
                if (!(x.line_width > 0.0f)) x.dash_count = 0;
                x.dash_first += base;
                dashed |= x.line_width > 0.0f && x.dash_count != 0;
                hs[S.path_first + p] = x;
            }
        if (s.dashes && s.n_dashes) hd.insert(hd.end(), s.dashes, s.dashes + s.n_dashes);
        if (s.contour_closed && s.n_contours) std::memcpy(hc.data() + S.contour_first, s.contour_closed, s.n_contours);
    }
    if (hd.empty()) hd.push_back(0.0f);
    PF_CUDA(c->st_stroke.ensure(size_t(N) * sizeof(pf_stroke) + 16));
    PF_CUDA(c->st_closed.ensure(size_t(C) + 16));
    PF_CUDA(c->st_dashes.ensure(hd.size() * 4));
    PF_CUDA(c->st_scenes.ensure(size_t(n) * sizeof(SceneDev)));
    PF_CUDA(c->st_cfirst.ensure((size_t(n) + 1) * 4));
    PF_CUDA(cudaMemcpyAsync(c->st_stroke.p, hs.data(), size_t(N) * sizeof(pf_stroke), cudaMemcpyHostToDevice, st));
    PF_CUDA(cudaMemcpyAsync(c->st_closed.p, hc.data(), C, cudaMemcpyHostToDevice, st));
    PF_CUDA(cudaMemcpyAsync(c->st_dashes.p, hd.data(), hd.size() * 4, cudaMemcpyHostToDevice, st));
    PF_CUDA(cudaMemcpyAsync(c->st_scenes.p, c->h_scenes.data(), size_t(n) * sizeof(SceneDev), cudaMemcpyHostToDevice, st));
    PF_CUDA(cudaMemcpyAsync(c->st_cfirst.p, scf.data(), (size_t(n) + 1) * 4, cudaMemcpyHostToDevice, st));
    PF_CUDA(c->status.ensure(kStCount * 4));
    PF_CUDA(cudaMemsetAsync(c->status.p, 0, kStCount * 4, st));
    uint32_t *status = c->status.as<uint32_t>();
    const bool timing = (c->flags & PF_CONFIG_STAGE_TIMING) != 0;
    if (timing && !c->sev[0])
        for (auto &e : c->sev) PF_CUDA(cudaEventCreate(&e));
    auto mark = [&](int i) -> cudaError_t { return timing ? cudaEventRecord(c->sev[i], st) : cudaSuccess; };
    c->ustats = pf_upload_stats{};
    for (uint32_t p = 0; p < N; p++) {
        c->ustats.stroked_paths += hs[p].line_width > 0.0f;
        c->ustats.dashed_paths += hs[p].line_width > 0.0f && hs[p].dash_count != 0;
    }

    StrokeIn in{};
    in.n_paths = N;
    in.n_scenes = n;
    in.scenes = c->st_scenes.as<SceneDev>();
    in.scene_path_first = c->scene_path_first.as<uint32_t>();
    in.scene_contour_first = c->st_cfirst.as<uint32_t>();
    in.cstart = c->in_cstart.as<uint32_t>();
    in.pstart = c->in_pstart.as<uint32_t>();
    in.points = c->in_points.as<float2>();
    in.flags = c->in_pflags.as<uint8_t>();
    in.closed = c->st_closed.as<uint8_t>();
    in.stroke = c->st_stroke.as<pf_stroke>();
    in.dashes = c->st_dashes.as<float>();
    PF_CUDA(c->dash_pts.ensure((size_t(N) + 1) * 4));
    PF_CUDA(c->dash_cnt.ensure((size_t(N) + 1) * 4));
    PF_CUDA(c->job_first.ensure((size_t(N) + 1) * 4));
    in.dash_pts = c->dash_pts.as<uint32_t>();
    in.dash_cnt = c->dash_cnt.as<uint32_t>();
    in.job_first = c->job_first.as<uint32_t>();
    PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(N + 1)));

    PF_CUDA(c->st_order_ctl.ensure(stroke_order_ctl_bytes()));
    // dashing: counts, offsets, the dashed contours (the dashed paths taken longest first)
    if (dashed) {
        PF_CUDA(mark(0));
        PF_CUDA(c->dash_order.ensure(size_t(N) * 4 + 16));
        PF_CUDA(cudaMemsetAsync(in.dash_pts, 0, size_t(N) * 4, st));
        PF_CUDA(cudaMemsetAsync(in.dash_cnt, 0, size_t(N) * 4, st));
        PF_CUDA(launch_stroke_order(in, 1, c->st_order_ctl.as<uint32_t>(), c->dash_order.as<uint32_t>(), st));
        in.dash_order = c->dash_order.as<uint32_t>();
        in.n_dashed = c->ustats.dashed_paths;
        PF_CUDA(launch_dash(in, false, status, st));
        PF_CUDA(scan_exclusive_u32(in.dash_pts, in.dash_pts, N, in.dash_pts + N, c->scan_temp.p, st, status));
        PF_CUDA(scan_exclusive_u32(in.dash_cnt, in.dash_cnt, N, in.dash_cnt + N, c->scan_temp.p, st, status));
        uint32_t tot[3], w[5];
        PF_CUDA(mark(1));
        if (int e = read_words(c, {in.dash_pts + N, in.dash_cnt + N, status + kStFill64, status + kStFill64 + 1,
                                   status + kStErr}, w))
            return e;
        tot[0] = w[0], tot[1] = w[1], tot[2] = w[4];
        const uint64_t wide = uint64_t(w[2]) | uint64_t(w[3]) << 32;  // the dash points' 64-bit total
        if (tot[2] & kErrStroke)
            return fail(c, PF_ERR_KERNEL_LIMIT, "a dash pattern needs more than 2^22 steps on one path");
        if (tot[2]) return fail(c, PF_ERR_CUDA, "dash pass failed");
        if (wide >= (1ull << 31)) return fail(c, PF_ERR_OVERFLOW, "dashed outline too large (2^31 points)");
        c->stroke_dash_points = tot[0];
        PF_CUDA(c->dash_points.ensure(size_t(tot[0]) * 8 + 16));
        PF_CUDA(c->dash_flags.ensure(size_t(tot[0]) + 16));
        PF_CUDA(c->dash_end.ensure(size_t(tot[1]) * 4 + 16));
        in.dash_points = c->dash_points.as<float2>();
        in.dash_flags = c->dash_flags.as<uint8_t>();
        in.dash_end = c->dash_end.as<uint32_t>();
        PF_CUDA(mark(2));
        PF_CUDA(launch_dash(in, true, status, st));
        PF_CUDA(mark(3));
    }
    // one job per output contour
    float ms_stroke = 0.0f;
    auto span = [&]() -> int {  // after a synchronisation: the device time between marks 4 and 5
        if (!timing) return PF_OK;
        float t = 0.0f;
        PF_CUDA(cudaEventElapsedTime(&t, c->sev[4], c->sev[5]));
        ms_stroke += t;
        return PF_OK;
    };
    auto read_u32 = [&](const uint32_t *dev, uint32_t &v) -> int {
        PF_CUDA(mark(5));
        if (int e = d2h_wait(c, &v, dev, 1)) return e;
        return span();
    };
    PF_CUDA(mark(4));
    PF_CUDA(launch_stroke_jobs(in, false, st));
    PF_CUDA(scan_exclusive_u32(in.job_first, in.job_first, N, in.job_first + N, c->scan_temp.p, st, status));
    uint32_t J = 0;
    if (int e = read_u32(in.job_first + N, J)) return e;
    if (J >= (1u << 31)) return fail(c, PF_ERR_OVERFLOW, "stroked outline too large (2^31 contours)");
    PF_CUDA(c->jobs.ensure(size_t(J) * 16 + 16));
    PF_CUDA(c->job_pts.ensure((size_t(J) + 1) * 4));
    PF_CUDA(c->job_units.ensure((size_t(J) + 1) * 4));
    PF_CUDA(c->job_nfwd.ensure(size_t(J) * 4 + 16));
    PF_CUDA(c->job_flags.ensure(size_t(J) * 4 + 16));
    PF_CUDA(c->job_cap1.ensure(size_t(J) * 4 + 16));
    PF_CUDA(c->job_end.ensure(size_t(J) * 4 + 16));
    PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(J + 1)));
    in.n_jobs = J;
    in.jobs = c->jobs.as<uint4>();
    in.job_pts = c->job_pts.as<uint32_t>();
    in.job_units = c->job_units.as<uint32_t>();
    in.job_nfwd = c->job_nfwd.as<uint32_t>();
    in.job_flags = c->job_flags.as<uint32_t>();
    in.job_cap1 = c->job_cap1.as<uint32_t>();
    in.job_end = c->job_end.as<uint32_t>();
    c->stroke_jobs = J;
    // units: every stroked contour's segments, forward and backward
    PF_CUDA(mark(4));
    PF_CUDA(launch_stroke_jobs(in, true, st));
    PF_CUDA(cudaMemsetAsync(in.job_flags, 0, size_t(J) * 4, st));
    PF_CUDA(launch_units(in, false, st));
    PF_CUDA(scan_exclusive_u32(in.job_units, in.job_units, J, in.job_units + J, c->scan_temp.p, st, status));
    uint32_t U = 0;
    if (int e = read_u32(in.job_units + J, U)) return e;
    if (U >= (1u << 31)) return fail(c, PF_ERR_OVERFLOW, "stroked outline too large (2^31 segments)");
    PF_CUDA(c->units.ensure(size_t(U) * 48 + 16));
    PF_CUDA(c->unit_leaves.ensure((size_t(U) + 1) * 4));
    PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(U + 1)));
    in.n_units = U;
    in.units = c->units.as<float4>();
    in.unit_leaves = c->unit_leaves.as<uint32_t>();
    // leaves: the offset recursion of every unit (units taken most work first)
    PF_CUDA(c->unit_order.ensure(size_t(U) * 4 + 16));
    PF_CUDA(mark(4));
    PF_CUDA(launch_units(in, true, st));
    PF_CUDA(launch_stroke_order(in, 0, c->st_order_ctl.as<uint32_t>(), c->unit_order.as<uint32_t>(), st));
    in.unit_order = c->unit_order.as<uint32_t>();
    PF_CUDA(launch_unit_leaves(in, false, st));
    PF_CUDA(scan_exclusive_u32(in.unit_leaves, in.unit_leaves, U, in.unit_leaves + U, c->scan_temp.p, st, status));
    uint32_t NL = 0;
    if (int e = read_u32(in.unit_leaves + U, NL)) return e;
    if (NL >= (1u << 31)) return fail(c, PF_ERR_OVERFLOW, "stroked outline too large (2^31 offset pieces)");
    PF_CUDA(c->st_leaves.ensure(size_t(NL) * 48 + 16));
    PF_CUDA(c->leaf_pts.ensure((size_t(NL) + 1) * 4));
    PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(NL + 1)));
    in.n_leaves = NL;
    in.leaves = c->st_leaves.as<float4>();
    in.leaf_pts = c->leaf_pts.as<uint32_t>();
    // counts: joins and points per leaf, caps and closing joins per contour, the degenerate
    // contours by the sequential kernel; then the contours' offsets
    PF_CUDA(mark(4));
    PF_CUDA(launch_unit_leaves(in, true, st));
    PF_CUDA(launch_job_ends(in, false, st));
    PF_CUDA(launch_leaf_pts(in, false, st));
    PF_CUDA(launch_stroke(in, false, status, st));
    PF_CUDA(scan_exclusive_u32(in.leaf_pts, in.leaf_pts, NL, in.leaf_pts + NL, c->scan_temp.p, st, status));
    PF_CUDA(launch_job_totals(in, status, st));
    PF_CUDA(scan_exclusive_u32(in.job_pts, in.job_pts, J, in.job_pts + J, c->scan_temp.p, st, status));
    uint32_t tot[2], w[4];
    PF_CUDA(mark(5));
    if (int e = read_words(c, {in.job_pts + J, status + kStFill64 + 2, status + kStFill64 + 3, status + kStErr}, w))
        return e;
    tot[0] = w[0], tot[1] = w[3];
    const uint64_t wide = uint64_t(w[1]) | uint64_t(w[2]) << 32;  // the output points' 64-bit total
    if (int e = span()) return e;
    if (wide >= (1ull << 31)) return fail(c, PF_ERR_OVERFLOW, "stroked outline too large (2^31 points)");
    if (tot[1] & kErrStroke)
        return fail(c, PF_ERR_KERNEL_LIMIT, "stroking hit a limit (a dash pattern over 2^22 steps on one path, "
                                            "or a cap searching back past 64 points)");
    if (tot[1]) return fail(c, PF_ERR_CUDA, "stroke pass failed");
    const uint32_t P = tot[0];
    if (P >= (1u << 31)) return fail(c, PF_ERR_OVERFLOW, "stroked outline too large (2^31 points)");
    PF_CUDA(c->points.ensure(size_t(P) * 8 + 16));
    PF_CUDA(c->pflags.ensure(size_t(P) + 16));
    in.out_points = c->points.as<float2>();
    in.out_flags = c->pflags.as<uint8_t>();
    in.n_out_points = P;
    PF_CUDA(mark(6));
    PF_CUDA(launch_leaf_pts(in, true, st));
    PF_CUDA(launch_job_ends(in, true, st));
    PF_CUDA(launch_stroke(in, true, status, st));
    PF_CUDA(mark(7));
    // the new layout: per scene its first contour and point
    PF_CUDA(c->st_bounds.ensure((size_t(n) + 1) * 8));
    PF_CUDA(launch_scene_bounds(in, c->st_bounds.as<uint32_t>(), st));
    std::vector<uint32_t> bounds(2 * (size_t(n) + 1));
    if (int e = d2h_wait(c, bounds.data(), c->st_bounds.p, bounds.size())) return e;
    std::vector<uint32_t> ocf(n + 1);
    for (uint32_t i = 0; i < n; i++) {
        SceneDev &S = c->h_scenes[i];
        S.contour_first = bounds[2 * i];
        S.contour_end = bounds[2 * i + 2];
        S.point_first = bounds[2 * i + 1];
        S.point_end = bounds[2 * i + 3];
        S.cstart_base = S.contour_first + i;
        ocf[i] = S.contour_first;
    }
    ocf[n] = J;
    c->n_points = P;
    c->n_contours = J;
    PF_CUDA(c->cstart.ensure((size_t(J) + n) * 4 + 16));
    PF_CUDA(cudaMemcpyAsync(c->scenes.p, c->h_scenes.data(), size_t(n) * sizeof(SceneDev), cudaMemcpyHostToDevice, st));
    PF_CUDA(cudaMemcpyAsync(c->scene_contour_first.p, ocf.data(), (size_t(n) + 1) * 4, cudaMemcpyHostToDevice, st));
    PF_CUDA(launch_outline_starts(in, c->scenes.as<SceneDev>(), c->cstart.as<uint32_t>(), c->pstart.as<uint32_t>(),
                                  st));
    c->ustats.stroke_contours = J;
    c->ustats.dash_points = dashed ? c->stroke_dash_points : 0u;
    if (timing) {  // every marked pair brackets work enqueued back to back (no host wait inside)
        PF_CUDA(cudaStreamSynchronize(st));
        float a = 0.0f, b = 0.0f;
        if (dashed) {
            PF_CUDA(cudaEventElapsedTime(&a, c->sev[0], c->sev[1]));
            PF_CUDA(cudaEventElapsedTime(&b, c->sev[2], c->sev[3]));
            c->ustats.ms_dash = a + b;
        }
        PF_CUDA(cudaEventElapsedTime(&b, c->sev[6], c->sev[7]));
        c->ustats.ms_stroke = ms_stroke + b;
    }
    return PF_OK;
}

int upload(Ctx *c, const pf_scene_view *scenes, uint32_t n) {
    if (!scenes || n == 0) return fail(c, PF_ERR_INVALID_ARGUMENT, "no scenes");
    forget_learned(c);
    uint64_t P = 0, C = 0, N = 0, fb = 0, img = 0, cs = 0, ps = 0;
    c->h_scenes.assign(n, SceneDev{});
    c->h_scene_fb_first.assign(n + 1, 0);
    c->h_scene_row_first.assign(n + 1, 0);
    uint64_t rows = 0;
    std::vector<uint32_t> spf(n + 1, 0), scf(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) {
        int st = validate_scene(c, &scenes[i]);
        if (st) return st;
        const pf_scene_view &s = scenes[i];
        SceneDev &S = c->h_scenes[i];
        // the view box (Scene::set_view_box rounds its right edge up to a multiple of 16);
        // framebuffer tiles cover the destination image from (0, 0)
        S.vb_left = s.view_box ? s.view_box[0] : 0.0f;
        S.vb_top = s.view_box ? s.view_box[1] : 0.0f;
        S.vb_right = view_box_right(s.view_box ? s.view_box[2] : s.width);
        S.vb_bottom = s.view_box ? s.view_box[3] : s.height;
        S.load = s.load_action;
        S.fbw = (uint32_t)std::ceil(view_box_right(s.width) / kTile);
        S.fbh = (uint32_t)std::ceil(s.height / kTile);
        S.fb_first = (uint32_t)fb;
        S.img_w = (uint32_t)std::ceil(s.width);
        S.img_h = (uint32_t)std::ceil(s.height);
        S.clear = s.clear_color;
        S.img_offset = img;
        S.path_first = (uint32_t)N;
        S.path_end = (uint32_t)(N + s.n_paths);
        S.contour_first = (uint32_t)C;
        S.contour_end = (uint32_t)(C + s.n_contours);
        S.point_first = (uint32_t)P;
        S.point_end = (uint32_t)(P + s.n_points);
        S.cstart_base = (uint32_t)cs;
        S.pstart_base = (uint32_t)ps;
        spf[i] = (uint32_t)N;
        scf[i] = (uint32_t)C;
        c->h_scene_fb_first[i] = (uint32_t)fb;
        S.row_first = (uint32_t)rows;
        c->h_scene_row_first[i] = (uint32_t)rows;
        rows += S.fbh;
        P += s.n_points;
        C += s.n_contours;
        N += s.n_paths;
        fb += uint64_t(S.fbw) * S.fbh;
        img += uint64_t(S.img_w) * S.img_h * 4;
        img = (img + 255) & ~uint64_t(255);
        cs += s.n_contours + 1;
        ps += s.n_paths + 1;
    }
    spf[n] = (uint32_t)N;
    scf[n] = (uint32_t)C;
    c->h_scene_fb_first[n] = (uint32_t)fb;
    c->h_scene_row_first[n] = (uint32_t)rows;
    if (P >= (1ull << 31) || C >= (1ull << 31) || N >= (1ull << 31) || fb >= (1ull << 31))
        return fail(c, PF_ERR_OVERFLOW, "batch too large (2^31 points, contours, paths or tiles)");
    c->n_scenes = n;
    c->n_points = (uint32_t)P;
    c->n_contours = (uint32_t)C;
    c->n_paths = (uint32_t)N;
    c->n_fb = (uint32_t)fb;
    c->image_bytes = img;

    bool strokes = false;
    for (uint32_t i = 0; i < n && !strokes; i++)
        for (uint32_t p = 0; scenes[i].path_stroke && p < scenes[i].n_paths; p++)
            if (scenes[i].path_stroke[p].line_width > 0.0f) {
                strokes = true;
                break;
            }
    // With stroked paths the uploaded outline lands in the in_* buffers and the stroke pass
    // writes the outline the frames read.
    DevBuf &d_points = strokes ? c->in_points : c->points, &d_pflags = strokes ? c->in_pflags : c->pflags;
    DevBuf &d_cstart = strokes ? c->in_cstart : c->cstart;
    PF_CUDA(d_points.ensure(P * 8 + 16));
    PF_CUDA(d_pflags.ensure(P + 16));
    PF_CUDA(d_cstart.ensure(cs * 4 + 16));
    PF_CUDA(c->pstart.ensure(ps * 4 + 16));
    if (strokes) PF_CUDA(c->in_pstart.ensure(ps * 4 + 16));
    PF_CUDA(c->fill_rule.ensure(N + 16));
    PF_CUDA(c->color.ensure(N * 4 + 16));
    PF_CUDA(c->scenes.ensure(n * sizeof(SceneDev)));
    PF_CUDA(c->scene_path_first.ensure((n + 1) * 4));
    PF_CUDA(c->scene_contour_first.ensure((n + 1) * 4));
    PF_CUDA(c->scene_fb_first.ensure((n + 1) * 4));
    PF_CUDA(c->scene_row_first.ensure((n + 1) * 4));
    {
        // a new image buffer starts transparent, so a first frame with PF_LOAD_LOAD loads zeros
        void *const before = c->image.p;
        PF_CUDA(c->image.ensure(img + 256));
        if (c->image.p != before) PF_CUDA(cudaMemsetAsync(c->image.p, 0, c->image.cap, c->stream));
    }
    bool clips = false;
    for (uint32_t i = 0; i < n; i++) clips |= scenes[i].path_clip != nullptr;
    c->h_path_clip.clear();
    c->h_path_is_clip.clear();
    if (clips) {
        c->h_path_clip.assign(N, PF_NO_CLIP);
        c->h_path_is_clip.assign(N, 0);
        for (uint32_t i = 0; i < n; i++) {
            const pf_scene_view &s = scenes[i];
            if (!s.path_clip) continue;
            const uint32_t b = c->h_scenes[i].path_first;
            std::memcpy(c->h_path_clip.data() + b, s.path_clip, size_t(s.n_paths) * 4);
            std::memcpy(c->h_path_is_clip.data() + b, s.path_is_clip, s.n_paths);
        }
        PF_CUDA(c->path_clip.ensure(N * 4 + 16));
        PF_CUDA(c->path_is_clip.ensure(N + 16));
        PF_CUDA(cudaMemcpyAsync(c->path_clip.p, c->h_path_clip.data(), N * 4, cudaMemcpyHostToDevice, c->stream));
        PF_CUDA(cudaMemcpyAsync(c->path_is_clip.p, c->h_path_is_clip.data(), N, cudaMemcpyHostToDevice, c->stream));
    }

    PF_CUDA(cudaMemcpyAsync(c->scene_path_first.p, spf.data(), (n + 1) * 4, cudaMemcpyHostToDevice, c->stream));
    // gradient paints: the paths' pf_paint records and every scene's stops go to the device as
    // given; the device numbers the gradients, orders each one's stops and builds its ramp and
    // metadata (no host pass over stops, no extra synchronisation)
    c->n_grads = 0;
    {
        uint64_t G = 0, S = 0;
        std::vector<uint32_t> sbase(n + 1, 0);
        bool any = false;
        for (uint32_t i = 0; i < n; i++) {
            const pf_scene_view &s = scenes[i];
            sbase[i] = (uint32_t)S;
            if (!s.path_paint) continue;
            any = true;
            S += s.n_stops;
            for (uint32_t p = 0; p < s.n_paths; p++) G += s.path_paint[p].type != PF_PAINT_SOLID;
        }
        sbase[n] = (uint32_t)S;
        if (any && G) {
            if (S >= (1ull << 31)) return fail(c, PF_ERR_OVERFLOW, "too many gradient stops (2^31)");
            PF_CUDA(c->grad_paint.ensure(size_t(N) * sizeof(pf_paint) + 16));
            PF_CUDA(c->grad_stops.ensure(size_t(S) * sizeof(pf_color_stop) + 16));
            PF_CUDA(c->grad_stop_range.ensure((size_t(n) + 1) * 4 + 4 * (size_t(N) + 1) + 4 * G + 64));
            PF_CUDA(c->path_grad.ensure(size_t(N) * 4 + 16));
            PF_CUDA(c->grad_meta.ensure(G * 64));
            PF_CUDA(c->grad_ramp.ensure(G * 1024));
            CopyPlan pp, ss;
            for (uint32_t i = 0; i < n; i++) {
                const pf_scene_view &s = scenes[i];
                char *dst = c->grad_paint.as<char>() + uint64_t(c->h_scenes[i].path_first) * sizeof(pf_paint);
                if (s.path_paint) pp.add(dst, s.path_paint, uint64_t(s.n_paths) * sizeof(pf_paint));
                else PF_CUDA(cudaMemsetAsync(dst, 0, uint64_t(s.n_paths) * sizeof(pf_paint), c->stream));
                if (s.path_paint && s.n_stops)
                    ss.add(c->grad_stops.as<char>() + uint64_t(sbase[i]) * sizeof(pf_color_stop), s.stops,
                           uint64_t(s.n_stops) * sizeof(pf_color_stop));
            }
            PF_CUDA(pp.run(c->stream));
            PF_CUDA(ss.run(c->stream));
            // grad_stop_range holds the scene stop bases, the per-path gradient flags (scanned)
            // and the gradient -> path map
            uint32_t *bases = c->grad_stop_range.as<uint32_t>();
            uint32_t *flags = bases + (n + 1);
            uint32_t *grad_path = flags + (N + 1);
            c->h_grad_sbase = sbase;
            PF_CUDA(cudaMemcpyAsync(bases, c->h_grad_sbase.data(), (size_t(n) + 1) * 4, cudaMemcpyHostToDevice,
                                    c->stream));
            PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(N + 1)));
            PF_CUDA(c->status.ensure(kStCount * 4));
            PF_CUDA(launch_gradient_index(c->grad_paint.as<pf_paint>(), N, flags, c->path_grad.as<uint32_t>(),
                                          grad_path, c->scan_temp.p, c->status.as<uint32_t>(), c->stream));
            PF_CUDA(launch_gradients(c->grad_paint.as<pf_paint>(), grad_path, c->scene_path_first.as<uint32_t>(),
                                     n, bases, c->grad_stops.as<pf_color_stop>(), (uint32_t)G,
                                     c->grad_meta.as<float4>(), c->grad_ramp.as<uint32_t>(), c->stream));
            c->n_grads = (uint32_t)G;
        }
    }

    // stroke outlines are filled nonzero (Canvas::stroke_path)
    std::vector<uint8_t> rules;
    if (strokes) {
        rules.resize(N);
        for (uint32_t i = 0; i < n; i++) {
            const pf_scene_view &s = scenes[i];
            for (uint32_t p = 0; p < s.n_paths; p++)
                rules[c->h_scenes[i].path_first + p] =
                    s.path_stroke && s.path_stroke[p].line_width > 0.0f ? uint8_t(PF_FILL_NONZERO) : s.fill_rule[p];
        }
    }
    DevBuf &d_pstart = strokes ? c->in_pstart : c->pstart;
    CopyPlan pts, fl, csp, psp, fr, col;
    for (uint32_t i = 0; i < n; i++) {
        const pf_scene_view &s = scenes[i];
        const SceneDev &S = c->h_scenes[i];
        pts.add(d_points.as<char>() + uint64_t(S.point_first) * 8, s.points, uint64_t(s.n_points) * 8);
        fl.add(d_pflags.as<char>() + S.point_first, s.point_flags, s.n_points);
        csp.add(d_cstart.as<char>() + uint64_t(S.cstart_base) * 4, s.contour_start, uint64_t(s.n_contours + 1) * 4);
        psp.add(d_pstart.as<char>() + uint64_t(S.pstart_base) * 4, s.path_start, uint64_t(s.n_paths + 1) * 4);
        fr.add(c->fill_rule.as<char>() + S.path_first, strokes ? rules.data() + S.path_first : s.fill_rule,
               s.n_paths);
        col.add(c->color.as<char>() + uint64_t(S.path_first) * 4, s.color, uint64_t(s.n_paths) * 4);
    }
    for (CopyPlan *cp : {&pts, &fl, &csp, &psp, &fr, &col}) PF_CUDA(cp->run(c->stream));
    PF_CUDA(cudaMemcpyAsync(c->scene_fb_first.p, c->h_scene_fb_first.data(), (n + 1) * 4, cudaMemcpyHostToDevice,
                            c->stream));
    PF_CUDA(c->fb_scene.ensure(size_t(fb) * 4 + 16));
    PF_CUDA(launch_fb_scene(c->scene_fb_first.as<uint32_t>(), n, c->fb_scene.as<uint32_t>(), c->stream));
    PF_CUDA(cudaMemcpyAsync(c->scene_row_first.p, c->h_scene_row_first.data(), (n + 1) * 4, cudaMemcpyHostToDevice,
                            c->stream));
    if (strokes) {
        if (int e = stroke_upload(c, scenes, n, scf)) {
            cudaStreamSynchronize(c->stream);
            c->uploaded = false;
            return e;
        }
    } else {
        c->ustats = pf_upload_stats{};
        PF_CUDA(cudaMemcpyAsync(c->scenes.p, c->h_scenes.data(), n * sizeof(SceneDev), cudaMemcpyHostToDevice,
                                c->stream));
        PF_CUDA(cudaMemcpyAsync(c->scene_contour_first.p, scf.data(), (n + 1) * 4, cudaMemcpyHostToDevice,
                                c->stream));
    }
    // the host arrays are borrowed only for this call
    PF_CUDA(cudaStreamSynchronize(c->stream));
    c->uploaded = true;
    c->rendered = false;
    c->upload_epoch++;
    return PF_OK;
}

Batch make_batch(Ctx *c) {
    Batch b{};
    b.points = c->points.as<float2>();
    b.flags = c->pflags.as<uint8_t>();
    b.contour_start_cat = c->cstart.as<uint32_t>();
    b.path_start_cat = c->pstart.as<uint32_t>();
    b.fill_rule = c->fill_rule.as<uint8_t>();
    b.color = c->color.as<uint32_t>();
    b.scenes = c->scenes.as<SceneDev>();
    b.scene_path_first = c->scene_path_first.as<uint32_t>();
    b.scene_contour_first = c->scene_contour_first.as<uint32_t>();
    b.scene_fb_first = c->scene_fb_first.as<uint32_t>();
    b.fb_scene = c->fb_scene.as<uint32_t>();
    b.scene_row_first = c->scene_row_first.as<uint32_t>();
    const bool clips = !c->h_path_clip.empty();
    b.path_clip_cat = clips ? c->path_clip.as<uint32_t>() : nullptr;
    b.path_is_clip_cat = clips ? c->path_is_clip.as<uint8_t>() : nullptr;
    b.path_clip_rel = clips ? c->path_clip_rel.as<uint32_t>() : nullptr;
    b.path_grad = c->n_grads ? c->path_grad.as<uint32_t>() : nullptr;
    b.grad_meta = c->n_grads ? c->grad_meta.as<float4>() : nullptr;
    b.grad_ramp = c->n_grads ? c->grad_ramp.as<uint32_t>() : nullptr;
    b.n_scenes_all = c->n_scenes;
    b.scene_base = c->r_first;
    b.n_scenes = c->r_count;
    b.path_base = c->r_path_base;
    b.n_paths = c->r_paths;
    b.contour_base = c->r_contour_base;
    b.n_contours = c->r_contours;
    b.fb_base = c->r_fb_base;
    b.row_base = c->r_row_base;
    b.contour_point_first = c->contour_point_first.as<uint32_t>();
    b.contour_path = c->contour_path.as<uint32_t>();
    b.paths = c->paths.as<PathDev>();
    b.path_bounds = c->path_bounds.as<float4>();
    b.path_leaf_first = c->path_leaf_first.as<uint32_t>();
    b.path_leaf_budget = c->path_leaf_budget.as<uint32_t>();
    b.path_leaf_cursor = c->path_leaf_cursor.as<uint32_t>();
    b.leaf_pool_first = 0xffffffffu;  // no spill pool unless a learned frame sets one
    b.leaf_pool_cap = 0;
    b.path_leaf_range = c->path_leaf_range.as<uint2>();
    b.path_contours = c->path_contours.as<uint2>();
    b.bin_list = c->bin_list.as<uint32_t>();
    b.bin_ctl = c->bin_ctl.as<uint32_t>();
    b.path_tiles = c->path_tiles.as<uint32_t>();
    b.path_cols = c->path_cols.as<uint32_t>();
    b.contour_segs = c->contour_segs.as<uint32_t>();
    b.segs = c->segs.as<SegDev>();
    b.seg_cap = (uint32_t)std::min<size_t>(c->segs.cap / sizeof(SegDev), 0xffffffffu);
    b.seg_leaves = c->seg_leaves.as<uint32_t>();
    b.seg_order = c->seg_order.as<uint32_t>();
    b.leaves = c->leaves.as<float4>();
    b.leaf_cap = (uint32_t)std::min<size_t>(c->leaves.cap / 16, 0xffffffffu);
    b.pool_path = nullptr;  // set by a learned frame
    b.pool_cnt = nullptr;
    b.pool_idx = nullptr;
    b.tile_fills = c->tile_fills.as<uint32_t>();
    b.path_fill = c->path_fill.as<uint32_t>();
    b.path_cls = c->path_cls.as<uint8_t>();
    b.tile_state = c->tile_state.as<uint16_t>();
    b.col_above = c->col_above.as<int32_t>();
    b.col_final = c->col_final.as<int32_t>();
    b.fills = c->fills.as<uint2>();
    b.fill_cap = (uint32_t)std::min<size_t>(c->fills.cap / 8, 0xffffffffu);
    b.stage = c->bin_stage.as<uint2>();
    b.row_first = c->row_first.as<uint32_t>();
    b.row_paths = c->row_paths.as<uint4>();
    b.row_cap = (uint32_t)std::min<size_t>(c->row_paths.cap / 16, 0xffffffffu);
    b.n_rows = c->r_rows;
    b.n_fb = c->r_fb;
    b.z = c->z.as<int32_t>();
    b.fb_count = c->fb_count.as<uint32_t>();
    b.list = c->list.as<uint32_t>();
    b.image = c->host_img_dev ? c->host_img_dev : c->image.as<uint8_t>();
    b.status = c->status.as<uint32_t>();
    b.counters = (c->flags & PF_CONFIG_FRAME_COUNTERS) ? 1u : 0u;
    b.long_line = c->tune.long_line;
    b.comp_ticket = c->tune.comp_ticket;
    if (!c->tune.seg_sorted) b.seg_order = nullptr;
    return b;
}

int read_status(Ctx *c) {
    if (c->capturing) return PF_OK;  // the captured frame's totals are already in h_status
    PF_CUDA(launch_copy_words(c->h_status_dev, c->status.as<uint32_t>(), kStCount, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    c->syncs++;
    return PF_OK;
}

int check_kernel_status(Ctx *c) {
    const uint32_t e = c->h_status[kStErr];
    if (e & kErrNonFinite) return fail(c, PF_ERR_INVALID_ARGUMENT, "a point coordinate is NaN or infinite");
    if (e & (kErrDepth | kErrWalk | kErrClip | kErrScanWait)) {
        char m[128];
        std::snprintf(m, sizeof m, "a kernel hit an iteration bound (flags 0x%x)", e);
        return fail(c, PF_ERR_KERNEL_LIMIT, m);
    }
    if (e & (kErrOverflowSeg | kErrOverflowLeaf | kErrOverflowFill | kErrOverflowList))
        return fail(c, PF_ERR_OVERFLOW, "a buffer capacity was exceeded");
    return PF_OK;
}

int scan(Ctx *c, uint32_t *arr, uint32_t n, int slot) {
    PF_CUDA(c->scan_temp.ensure(scan_temp_bytes(n)));
    PF_CUDA(scan_exclusive_u32(arr, arr, n, c->status.as<uint32_t>() + slot, c->scan_temp.p, c->stream,
                               c->status.as<uint32_t>() + kStErr));
    return PF_OK;
}

void record(Ctx *c, int i) {
    if (!(c->flags & PF_CONFIG_STAGE_TIMING)) return;
    // while a graph is recorded, an external record makes the event a node the replay records
    if (c->capturing) cudaEventRecordWithFlags(c->ev[i], c->stream, cudaEventRecordExternal);
    else cudaEventRecord(c->ev[i], c->stream);
}

void set_range(Ctx *c, uint32_t first, uint32_t count) {
    const SceneDev &a = c->h_scenes[first], &e = c->h_scenes[first + count - 1];
    c->r_first = first;
    c->r_count = count;
    c->r_path_base = a.path_first;
    c->r_paths = e.path_end - a.path_first;
    c->r_contour_base = a.contour_first;
    c->r_contours = e.contour_end - a.contour_first;
    c->r_fb_base = a.fb_first;
    c->r_fb = c->h_scene_fb_first[first + count] - a.fb_first;
    c->r_row_base = a.row_first;
    c->r_rows = c->h_scene_row_first[first + count] - a.row_first;
}

int begin_frame(Ctx *c, uint32_t first, uint32_t count) {
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    if (c->host_img && c->host_img_bytes < c->image_bytes)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "the host image buffer is smaller than the batch's images");
    if (count == 0 || first >= c->n_scenes || count > c->n_scenes - first)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "scene range out of bounds");
    c->rendered = false;
    c->lists_dumped = false;
    set_range(c, first, count);
    c->syncs = 0;
    cudaStream_t st = c->stream;
    const uint32_t N = c->r_paths, C = c->r_contours;
    PF_CUDA(c->status.ensure(kStCount * 4));
    PF_CUDA(cudaMemsetAsync(c->status.p, 0, kStCount * 4, st));
    PF_CUDA(c->contour_point_first.ensure((size_t(C) + 1) * 4));
    PF_CUDA(c->contour_path.ensure(size_t(C) * 4 + 4));
    PF_CUDA(c->contour_segs.ensure((size_t(C) + 1) * 4));
    PF_CUDA(c->paths.ensure(size_t(N) * sizeof(PathDev) + 16));
    PF_CUDA(c->path_tiles.ensure((size_t(N) + 1) * 4));
    PF_CUDA(c->path_cols.ensure((size_t(N) + 1) * 4));
    PF_CUDA(c->path_contours.ensure(size_t(N) * 8 + 8));
    PF_CUDA(c->path_bounds.ensure(size_t(N) * 16 + 16));
    PF_CUDA(c->row_first.ensure((size_t(c->r_rows) + 1) * 4));
    PF_CUDA(c->bin_list.ensure(size_t(N) * 20 + 16));
    PF_CUDA(c->path_fill.ensure(size_t(N) * 4 + 16));
    size_t stage_bytes = 0;
    PF_CUDA(bin_stage_bytes(c->tune, &stage_bytes));
    PF_CUDA(c->bin_stage.ensure(stage_bytes));
    PF_CUDA(c->path_cls.ensure(size_t(N) + 16));
    PF_CUDA(c->bin_ctl.ensure(1024));
    PF_CUDA(c->path_leaf_range.ensure(size_t(N) * 8 + 16));
    if (!c->h_path_clip.empty()) PF_CUDA(c->path_clip_rel.ensure(size_t(N) * 4 + 16));
    return PF_OK;
}

// Stage 1: topology, tile rects, segment counts, per-row path counts (and, for a learned
// frame, the sizer's per-path budgets), ending with the frame's first host synchronisation.
int stage_setup(Ctx *c, bool learned) {
    cudaStream_t st = c->stream;
    const uint32_t N = c->r_paths, C = c->r_contours, R = c->r_rows;
    Batch b = make_batch(c);
    PF_CUDA(launch_normalize(b, c->path_contours.as<uint2>(), st));
    PF_CUDA(launch_path_setup(b, c->path_contours.as<uint2>(), st));
    PF_CUDA(cudaMemsetAsync(b.contour_segs + C, 0, 4, st));
    PF_CUDA(cudaMemsetAsync(b.path_tiles + N, 0, 4, st));
    PF_CUDA(cudaMemsetAsync(b.path_cols + N, 0, 4, st));
    PF_CUDA(cudaMemsetAsync(b.row_first + R, 0, 4, st));
    PF_CUDA(launch_contour_segments(b, false, st));
    PF_CUDA(launch_rows(b, false, st));
    if (int e = scan(c, b.contour_segs, C + 1, kStSegs)) return e;
    if (int e = scan(c, b.path_tiles, N + 1, kStTiles)) return e;
    if (int e = scan(c, b.path_cols, N + 1, kStCols)) return e;
    if (int e = scan(c, b.row_first, R + 1, kStRows)) return e;
    PF_CUDA(launch_path_offsets(b, st));
    if (learned) {
        PF_CUDA(c->path_feat.ensure(size_t(N) * kSizerIn * 4 + 16));
        PF_CUDA(c->contour_feat.ensure(size_t(C) * 32 + 32));
        PF_CUDA(c->path_pred.ensure(size_t(N) * kSizerOut * 4 + 16));
        PF_CUDA(c->path_leaf_first.ensure((size_t(N) + 1) * 4));
        PF_CUDA(c->path_leaf_budget.ensure(size_t(N) * 4 + 16));
        PF_CUDA(c->path_leaf_cursor.ensure(size_t(N) * 4 + 16));
        PF_CUDA(c->path_fill_budget.ensure((size_t(N) + 1) * 4));
        b = make_batch(c);
        PF_CUDA(launch_features(b, c->path_contours.as<uint2>(), c->contour_feat.as<float4>(), c->path_feat.as<float>(),
                                st));
        PF_CUDA(launch_mlp_predict(c->sz_w.as<__nv_bfloat16>(), c->path_feat.as<float>(), N, c->path_pred.as<float>(),
                                   st));
        PF_CUDA(launch_budgets(b, c->path_pred.as<float>(), c->sz_mul, c->sz_add, b.path_leaf_first,
                               c->path_fill_budget.as<uint32_t>(), b.path_leaf_cursor, st));
        PF_CUDA(cudaMemcpyAsync(b.path_leaf_budget, b.path_leaf_first, size_t(N) * 4, cudaMemcpyDeviceToDevice, st));
        PF_CUDA(cudaMemsetAsync(b.path_leaf_first + N, 0, 4, st));
        PF_CUDA(cudaMemsetAsync(c->path_fill_budget.as<uint32_t>() + N, 0, 4, st));
        if (int e = scan(c, b.path_leaf_first, N + 1, kStLeafBudget)) return e;
        if (int e = scan(c, c->path_fill_budget.as<uint32_t>(), N + 1, kStFillBudget)) return e;
    }
    if (int e = read_status(c)) return e;
    if (int e = check_kernel_status(c)) return e;
    c->n_segs = c->h_status[kStSegs];
    c->n_tiles = c->h_status[kStTiles];
    c->n_cols = c->h_status[kStCols];
    c->n_row_entries = c->h_status[kStRows];
    PF_CUDA(c->segs.ensure(size_t(c->n_segs) * sizeof(SegDev) + 16));
    PF_CUDA(c->seg_leaves.ensure((size_t(c->n_segs) + 1) * 4));
    PF_CUDA(c->seg_order.ensure(size_t(c->n_segs) * 4 + 16));
    PF_CUDA(c->seg_ctl.ensure(seg_ctl_bytes()));
    PF_CUDA(c->row_paths.ensure(size_t(c->n_row_entries) * 16 + 16));
    const size_t T = c->n_tiles, K = c->n_cols;
    PF_CUDA(c->tile_fills.ensure(T * 4 + 16));
    PF_CUDA(c->tile_state.ensure(T * 2 + 16));
    PF_CUDA(c->col_above.ensure(K * 4 + 4));
    PF_CUDA(c->col_final.ensure(K * 4 + 4));
    return PF_OK;
}

// Binning and composite of a frame whose leaf lines are in place.  The fills buffer starts
// at the largest frame's size (or about three fills per line); a frame that overruns it is
// counted to the exact total, the buffer grows, and binning and composite run again.  Ends
// with the status words read back.
int bin_and_composite(Ctx *c, Batch b, bool learned) {
    cudaStream_t st = c->stream;
    for (int attempt = 0;; attempt++) {
        PF_CUDA(cudaMemsetAsync(b.bin_ctl, 0, 1024, st));
        PF_CUDA(cudaMemsetAsync(b.status + kStFill64, 0, 8, st));
        PF_CUDA(launch_bin_classify(b, learned, st));
        if (c->tune.bin_concurrent && !c->bs_ready) {
            for (auto &s : c->bs.side) PF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            PF_CUDA(cudaEventCreateWithFlags(&c->bs.fork, cudaEventDisableTiming));
            for (auto &e : c->bs.join) PF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            c->bs_ready = true;
        }
        PF_CUDA(launch_bin_paths(b, c->tune, c->bs_ready ? &c->bs : nullptr, st));
        record(c, 3);
        record(c, 4);
        record(c, 5);
        PF_CUDA(launch_composite(b, st));
        record(c, 6);
        if (b.counters) PF_CUDA(launch_tile_counts(b, st));
        if (int e = read_status(c)) return e;
        const uint32_t err = c->h_status[kStErr];
        const uint64_t need = uint64_t(c->h_status[kStFill64]) | uint64_t(c->h_status[kStFill64 + 1]) << 32;
        if (!(err & kErrOverflowFill) || (err & kErrOverflowLeaf)) {
            c->n_fills = need;
            c->fill_hint = std::max(c->fill_hint, need);
            return PF_OK;
        }
        if (attempt > 0 || need >= 0xffffffffull)
            return fail(c, PF_ERR_OVERFLOW, "the frame's fills exceed what one frame can index (2^32)");
        PF_CUDA(c->fills.ensure(need * 8 + 16));
        c->fill_hint = std::max(c->fill_hint, need);
        b.fills = c->fills.as<uint2>();
        b.fill_cap = (uint32_t)std::min<size_t>(c->fills.cap / 8, 0xffffffffu);
        // clear the error word and the composite's counters before the second run
        const uint32_t zero = 0;
        for (int slot : {(int)kStErr, (int)kStListFills, (int)kStEntries, (int)kStWalkChunks, (int)kStAlphaTiles,
                         (int)kStVisible})
            PF_CUDA(cudaMemcpyAsync(b.status + slot, &zero, 4, cudaMemcpyHostToDevice, st));
    }
}

// Statistics of the frame; the status words were read back by bin_and_composite.
int finish_frame(Ctx *c, uint32_t first, uint32_t count, uint64_t launches0, pf_frame_stats *stats) {
    const uint32_t NFB = c->r_fb;
    if (int e = check_kernel_status(c)) return e;
    c->n_list = c->h_status[kStEntries];
    c->rendered = true;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->paths = c->r_paths;
        stats->contours = c->r_contours;
        stats->points = c->h_scenes[first + count - 1].point_end - c->h_scenes[first].point_first;
        stats->segments = c->n_segs;
        stats->microlines = c->n_leaves;
        stats->tiles = c->n_tiles;
        stats->fills = c->n_fills;
        stats->composite_entries = c->n_list;
        stats->framebuffer_tiles = NFB;
        stats->composited_fills = c->h_status[kStListFills];
        // alpha and visible tiles are counted with PF_CONFIG_FRAME_COUNTERS (else 0)
        stats->alpha_tiles = c->h_status[kStAlphaTiles];
        stats->visible_tiles = c->h_status[kStVisible];
        stats->kernel_launches = (uint32_t)(launches() - launches0);
        stats->host_syncs = c->syncs;
        if ((c->flags & PF_CONFIG_STAGE_TIMING) && !c->capturing) {
            float ms[6] = {};
            for (int i = 0; i < 6; i++) cudaEventElapsedTime(&ms[i], c->ev[i], c->ev[i + 1]);
            stats->ms_setup = ms[0];
            stats->ms_flatten = ms[1];
            stats->ms_bin = ms[2];
            stats->ms_propagate = ms[3];
            stats->ms_lists = ms[4];
            stats->ms_composite = ms[5];
            cudaEventElapsedTime(&stats->ms_total, c->ev[0], c->ev[6]);
        }
    }
    return PF_OK;
}

// The exact two-pass frame over uploaded scenes [first, first + count).
int render_exact(Ctx *c, uint32_t first, uint32_t count, pf_frame_stats *stats) {
    if (int e = begin_frame(c, first, count)) return e;
    const uint64_t launches0 = launches();
    cudaStream_t st = c->stream;
    record(c, 0);
    if (int e = stage_setup(c, false)) return e;
    record(c, 1);

    // 2. segments, row lists, leaf counts, leaves
    Batch b = make_batch(c);
    PF_CUDA(launch_contour_segments(b, true, st));
    PF_CUDA(launch_rows(b, true, st));
    if (c->tune.seg_sorted) PF_CUDA(launch_seg_order(b, c->n_segs, c->seg_ctl.as<uint32_t>(), st));
    PF_CUDA(cudaMemsetAsync(b.seg_leaves + c->n_segs, 0, 4, st));
    PF_CUDA(launch_flatten(b, c->n_segs, false, st));
    if (int e = scan(c, b.seg_leaves, c->n_segs + 1, kStLeaves)) return e;
    if (int e = read_status(c)) return e;
    if (int e = check_kernel_status(c)) return e;
    c->n_leaves = c->h_status[kStLeaves];
    PF_CUDA(c->leaves.ensure(size_t(c->n_leaves) * 16 + 16));
    b = make_batch(c);
    PF_CUDA(launch_flatten(b, c->n_segs, true, st, c->n_leaves));
    record(c, 2);

    // 3. binning (one CTA per path: counts, backdrops, fill offsets, fills grouped by tile),
    //    then coverage and the front-to-back composite with the z-cull walk
    PF_CUDA(c->fills.ensure(std::max<uint64_t>(c->fill_hint, uint64_t(c->n_leaves) * 3) * 8 + 16));
    b = make_batch(c);
    if (int e = bin_and_composite(c, b, false)) return e;
    return finish_frame(c, first, count, launches0, stats);
}

// The learned one-pass frame: per-path leaf regions and the fill capacity come from the
// sizer's predictions, so leaf lines are produced once (flattened, stored and counted in the
// same kernel) and the frame synchronises only after set-up.  If a path overruns its leaf
// budget or the fills overrun the capacity, the frame is redone by the exact two-pass method
// (the reference's own recovery, renderer.cpp:540-577, made exact).
int render_learned_frame(Ctx *c, uint32_t first, uint32_t count, pf_frame_stats *stats) {
    c->learned_done = false;
    if (int e = begin_frame(c, first, count)) return e;
    const uint64_t launches0 = launches();
    cudaStream_t st = c->stream;
    record(c, 0);
    if (int e = stage_setup(c, true)) return e;
    // per-path regions, then a shared spill pool sized as a fraction of them
    const uint64_t leaf_regions = c->h_status[kStLeafBudget];
    const uint64_t leaf_pool = uint64_t(double(leaf_regions) * c->sz_pool) + 4096;
    const uint64_t leaf_slots = leaf_regions + leaf_pool;
    const uint64_t fill_pred = uint64_t(c->h_status[kStFillBudget]);
    if (leaf_slots >= 0xffffffffull) return render_exact(c, first, count, stats);
    const uint32_t N = c->r_paths;
    PF_CUDA(c->leaves.ensure(leaf_slots * 16 + 16));
    PF_CUDA(c->pool_path.ensure(leaf_pool * 4 + 16));
    PF_CUDA(c->pool_idx.ensure(leaf_pool * 4 + 16));
    PF_CUDA(c->pool_cnt.ensure((size_t(N) + 2) * 4));
    PF_CUDA(c->fills.ensure(std::min<uint64_t>(std::max(fill_pred, c->fill_hint), 0xfffffffeull) * 8 + 16));
    record(c, 1);

    Batch b = make_batch(c);
    b.leaf_pool_first = (uint32_t)leaf_regions;
    b.leaf_pool_cap = (uint32_t)leaf_pool;
    b.pool_path = c->pool_path.as<uint32_t>();
    b.pool_idx = c->pool_idx.as<uint32_t>();
    PF_CUDA(launch_contour_segments(b, true, st));
    PF_CUDA(launch_rows(b, true, st));
    if (c->tune.seg_sorted) PF_CUDA(launch_seg_order(b, c->n_segs, c->seg_ctl.as<uint32_t>(), st));
    PF_CUDA(launch_flatten_budget(b, c->n_segs, st));
    record(c, 2);
    // the spill pool's lines listed by path, so each path's CTA finds them
    PF_CUDA(cudaMemsetAsync(c->pool_cnt.p, 0, (size_t(N) + 2) * 4, st));
    b.pool_cnt = c->pool_cnt.as<uint32_t>() + 1;
    PF_CUDA(launch_pool_lists(b, false, st));
    if (int e = scan(c, b.pool_cnt, N + 1, kStPoolListed)) return e;
    PF_CUDA(launch_pool_lists(b, true, st));
    if (int e = bin_and_composite(c, b, true)) return e;
    if (c->h_status[kStErr] & kErrOverflowLeaf) {
        // a path overran its leaf region and the pool: redo the frame exactly
        const int e = render_exact(c, first, count, stats);
        if (stats) stats->overflow = 1;
        return e;
    }
    c->n_leaves = c->h_status[kStLeafCount];
    c->last_paths_over = c->h_status[kStPathsOver];
    c->last_pool_used = c->h_status[kStPoolUsed];
    const int e = finish_frame(c, first, count, launches0, stats);
    if (stats) {
        stats->microlines = c->n_leaves;
        stats->overflow = 0;
    }
    c->learned_done = e == PF_OK;
    return e;
}

// The buffers a learned frame uses, by address (a reallocated one invalidates the graph).
std::vector<void *> frame_buffers(const Ctx *c) {
    const DevBuf *bufs[] = {&c->status, &c->contour_point_first, &c->contour_path, &c->paths, &c->path_tiles,
                            &c->path_cols, &c->path_contours, &c->path_bounds, &c->row_first, &c->bin_list,
                            &c->bin_ctl, &c->path_leaf_range, &c->path_fill, &c->path_cls, &c->bin_stage,
                            &c->path_feat, &c->contour_feat, &c->path_pred, &c->path_leaf_first, &c->path_leaf_budget,
                            &c->path_leaf_cursor, &c->path_fill_budget, &c->segs, &c->seg_leaves, &c->seg_order,
                            &c->seg_ctl, &c->row_paths, &c->tile_fills, &c->tile_state, &c->col_above,
                            &c->col_final, &c->leaves, &c->pool_path, &c->pool_idx, &c->pool_cnt, &c->fills,
                            &c->scan_temp, &c->image, &c->sz_w, &c->path_clip_rel};
    std::vector<void *> v;
    for (const DevBuf *d : bufs) v.push_back(d->p);
    v.push_back(c->host_img_dev);
    return v;
}

void drop_graph(Ctx *c) {
    if (c->lg_exec) cudaGraphExecDestroy(c->lg_exec);
    c->lg_exec = nullptr;
}

// The scenes or the sizer changed: no graph, and no plain frame to record one from.
void forget_learned(Ctx *c) {
    drop_graph(c);
    c->lg_prev.valid = false;
}

// Records the learned frame over [first, first + count) as a graph, right after the same frame
// ran with the same buffers.  A failure leaves the plain path in use.
void capture_learned(Ctx *c, uint32_t first, uint32_t count) {
    drop_graph(c);
    uint32_t saved[kStCount];
    std::memcpy(saved, c->h_status, sizeof saved);
    const bool rendered = c->rendered, dumped = c->lists_dumped;
    const uint32_t syncs = c->syncs;
    const uint64_t l0 = launches();
    cudaGraph_t g = nullptr;
    c->capturing = true;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
    int r = PF_ERR_CUDA;
    if (e == cudaSuccess) {
        pf_frame_stats scratch;
        r = render_learned_frame(c, first, count, &scratch);
        e = cudaStreamEndCapture(c->stream, &g);
    }
    c->capturing = false;
    std::memcpy(c->h_status, saved, sizeof saved);
    c->rendered = rendered;
    c->lists_dumped = dumped;
    c->syncs = syncs;
    if (e == cudaSuccess && r == PF_OK && g) e = cudaGraphInstantiate(&c->lg_exec, g, 0);
    else e = cudaErrorUnknown;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (e != cudaSuccess) {
        c->lg_exec = nullptr;
        return;
    }
    c->lg_first = first;
    c->lg_count = count;
    c->lg_flags = c->flags;
    c->lg_launches = (uint32_t)(launches() - l0);
    std::memcpy(c->lg_status, saved, sizeof saved);
    c->lg_ptrs = frame_buffers(c);
}

constexpr int kReplayMiss = -1;

// Replays the captured learned frame; kReplayMiss when it does not apply (or its frame came out
// different from the one it was sized for), and the caller runs the plain frame.
int replay_learned(Ctx *c, uint32_t first, uint32_t count, pf_frame_stats *stats) {
    if (!c->lg_exec || c->lg_first != first || c->lg_count != count || c->lg_flags != c->flags ||
        c->lg_ptrs != frame_buffers(c)) {
        drop_graph(c);
        return kReplayMiss;
    }
    c->rendered = false;
    c->lists_dumped = false;
    set_range(c, first, count);
    c->syncs = 0;
    const uint64_t l0 = launches();
    PF_CUDA(cudaGraphLaunch(c->lg_exec, c->stream));
    if (int e = read_status(c)) return e;
    const uint32_t *h = c->h_status, *want = c->lg_status;
    if (h[kStErr] != 0 || h[kStSegs] != want[kStSegs] || h[kStTiles] != want[kStTiles] ||
        h[kStCols] != want[kStCols] || h[kStRows] != want[kStRows] || h[kStLeafBudget] != want[kStLeafBudget] ||
        h[kStFillBudget] != want[kStFillBudget]) {
        drop_graph(c);
        return kReplayMiss;
    }
    c->n_leaves = h[kStLeafCount];
    c->n_fills = uint64_t(h[kStFill64]) | uint64_t(h[kStFill64 + 1]) << 32;
    c->last_paths_over = h[kStPathsOver];
    c->last_pool_used = h[kStPoolUsed];
    const int e = finish_frame(c, first, count, l0, stats);
    if (stats) {
        stats->microlines = c->n_leaves;
        stats->overflow = 0;
        stats->kernel_launches = c->lg_launches;
    }
    return e;
}

int render_learned(Ctx *c, uint32_t first, uint32_t count, pf_frame_stats *stats) {
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights loaded");
    c->lg_kind = 2;
    int r = replay_learned(c, first, count, stats);
    if (r != kReplayMiss) return r;
    auto &pv = c->lg_prev;
    if (pv.valid && pv.epoch == c->upload_epoch && pv.first == first && pv.count == count && pv.flags == c->flags &&
        pv.ptrs == frame_buffers(c)) {
        // the last frame ran this one plainly with these buffers: record it (with the totals that
        // frame sized the buffers for) and replay it
        std::memcpy(c->h_status, pv.status, sizeof pv.status);
        capture_learned(c, first, count);
        c->lg_kind = 1;
        r = replay_learned(c, first, count, stats);
        if (r != kReplayMiss) return r;
    }
    pv.valid = false;
    pf_frame_stats local;
    pf_frame_stats *st = stats ? stats : &local;
    c->lg_kind = 0;
    const int e = render_learned_frame(c, first, count, st);
    if (e == PF_OK && c->learned_done) {
        pv.valid = true;
        pv.epoch = c->upload_epoch;
        pv.first = first;
        pv.count = count;
        pv.flags = c->flags;
        pv.ptrs = frame_buffers(c);
        std::memcpy(pv.status, c->h_status, sizeof pv.status);
    }
    return e;
}

// A frame between two device events; *ms is its time on the device (the frame ends with a host
// synchronisation, so the events have completed by then).
template <class F>
int timed_frame(Ctx *c, float *ms, F &&frame) {
    if (!c->au_ev[0]) {
        PF_CUDA(cudaEventCreate(&c->au_ev[0]));
        PF_CUDA(cudaEventCreate(&c->au_ev[1]));
    }
    PF_CUDA(cudaEventRecord(c->au_ev[0], c->stream));
    const int e = frame();
    if (e != PF_OK) return e;
    PF_CUDA(cudaEventRecord(c->au_ev[1], c->stream));
    PF_CUDA(cudaEventSynchronize(c->au_ev[1]));
    PF_CUDA(cudaEventElapsedTime(ms, c->au_ev[0], c->au_ev[1]));
    return PF_OK;
}

// Timed frames of each kind before pf_render_auto decides, and the calls that always suffice:
// an untimed first exact frame and two timed ones, then an untimed first learned frame, the one
// that records its graph, and two timed replays.
constexpr int kAutoSamples = 2;
constexpr int kAutoSettle = 2 * kAutoSamples + 3;

void auto_reset(Ctx *c) {
    auto &a = c->au;
    a.exact_ms = a.learned_ms = -1.0f;
    a.exact_runs = a.learned_runs = 0;
    a.exact_timed = a.learned_timed = 0;
}

// The frame the library picks.  With sizer weights it times, on the device, the exact frame and
// the learned frame over the workload - the scene range and the totals of its paths, contours and
// points, so a new upload of scenes of the same size keeps what was measured - and runs the
// faster one once both are known.  Each frame's first run over the workload is not timed (it may
// grow buffers), nor is a learned frame that records its graph (the next one, a replay, is).
// Each kind is timed kAutoSamples times and its fastest frame counts, so one frame slowed by
// something outside it does not decide; a learned frame that had to be redone exactly counts as
// the slower one at once.  Without weights: the exact frame.
int render_auto(Ctx *c, uint32_t first, uint32_t count, pf_frame_stats *stats) {
    auto &a = c->au;
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    if (count == 0 || first >= c->n_scenes || count > c->n_scenes - first)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "scene range out of bounds");
    a.last = PF_FRAME_EXACT;
    if (!c->sz_ready) return render_exact(c, first, count, stats);
    const SceneDev &s0 = c->h_scenes[first], &s1 = c->h_scenes[first + count - 1];
    const uint64_t sig[5] = {first, count, uint64_t(s1.path_end - s0.path_first),
                             uint64_t(s1.contour_end - s0.contour_first), uint64_t(s1.point_end - s0.point_first)};
    if (std::memcmp(sig, a.sig, sizeof sig) != 0) {
        std::memcpy(a.sig, sig, sizeof sig);
        auto_reset(c);
    }
    pf_frame_stats local;
    pf_frame_stats *st = stats ? stats : &local;
    float ms = 0.0f;
    auto keep = [](float &best, int &timed, float v) {
        best = timed == 0 ? v : std::min(best, v);
        timed++;
    };
    if (a.exact_timed < kAutoSamples) {
        const int e = timed_frame(c, &ms, [&] { return render_exact(c, first, count, st); });
        if (e == PF_OK && a.exact_runs++ > 0) keep(a.exact_ms, a.exact_timed, ms);
        return e;
    }
    if (a.learned_timed < kAutoSamples || a.learned_ms < a.exact_ms) {
        a.last = PF_FRAME_LEARNED;
        const int e = timed_frame(c, &ms, [&] { return render_learned(c, first, count, st); });
        if (e != PF_OK) return e;
        if (st->overflow) {  // redone exactly: the exact frame wins
            a.learned_ms = 2.0f * a.exact_ms + 1.0f;
            a.learned_timed = kAutoSamples;
        } else if (a.learned_timed < kAutoSamples && (c->lg_kind == 2 || (c->lg_kind == 0 && a.learned_runs > 0))) {
            keep(a.learned_ms, a.learned_timed, ms);  // a replay, or a plain frame after the first
        }
        a.learned_runs++;
        return e;
    }
    return render_exact(c, first, count, st);
}

template <class T>
int d2h(Ctx *c, std::vector<T> &dst, const void *src, size_t n) {
    dst.resize(n);
    if (n) PF_CUDA(cudaMemcpyAsync(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    return PF_OK;
}

// Composite lists of the last frame (canonical output only): count, scan, write.
int dump_lists(Ctx *c) {
    if (c->lists_dumped) return PF_OK;
    const uint32_t NFB = c->r_fb;
    PF_CUDA(c->z.ensure(size_t(NFB) * 4 + 4));
    PF_CUDA(c->fb_count.ensure((size_t(NFB) + 1) * 4));
    Batch b = make_batch(c);
    PF_CUDA(cudaMemsetAsync(b.fb_count + NFB, 0, 4, c->stream));
    PF_CUDA(launch_list_dump(b, false, c->stream));
    if (int e = scan(c, b.fb_count, NFB + 1, kStList)) return e;
    if (int e = read_status(c)) return e;
    PF_CUDA(c->list.ensure(size_t(c->h_status[kStList]) * 4 + 16));
    b = make_batch(c);
    PF_CUDA(launch_list_dump(b, true, c->stream));
    if (!c->h_path_clip.empty()) {
        // the clip rules as the composite applies them, tile by tile
        PF_CUDA(c->canon_state.ensure(size_t(c->n_tiles) * 4 + 16));
        PF_CUDA(c->canon_clip.ensure(size_t(c->n_tiles) * 4 + 16));
        PF_CUDA(launch_clip_dump(b, c->n_tiles, c->canon_state.as<uint32_t>(), c->canon_clip.as<uint32_t>(),
                                 c->stream));
    }
    PF_CUDA(cudaStreamSynchronize(c->stream));
    c->lists_dumped = true;
    return PF_OK;
}

// Canonical integer output of scene `si` of the last frame.
int read_canon(Ctx *c, uint32_t si, pf_canon *out) {
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    if (si < c->r_first || si >= c->r_first + c->r_count)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "scene was not rendered by the last frame");
    if (int e = dump_lists(c)) return e;
    const SceneDev &S = c->h_scenes[si];
    const uint32_t p0 = S.path_first - c->r_path_base, p1 = S.path_end - c->r_path_base, np = p1 - p0;
    const uint32_t fb0 = S.fb_first - c->r_fb_base;
    std::vector<PathDev> paths;
    std::vector<uint32_t> tf, cf;
    if (int e = d2h(c, paths, c->paths.as<PathDev>() + p0, np)) return e;
    if (int e = d2h(c, tf, c->path_tiles.as<uint32_t>() + p0, np + 1)) return e;
    if (int e = d2h(c, cf, c->path_cols.as<uint32_t>() + p0, np + 1)) return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    const uint32_t t0 = tf[0], t1 = tf[np], k0 = cf[0], k1 = cf[np];
    HostCanon &h = c->canon;
    h.rect.resize(size_t(np) * 4);
    h.tile_first.resize(np + 1);
    h.col_first.resize(np + 1);
    for (uint32_t p = 0; p < np; p++) {
        h.rect[4 * p + 0] = paths[p].rx0;
        h.rect[4 * p + 1] = paths[p].ry0;
        h.rect[4 * p + 2] = paths[p].rx1;
        h.rect[4 * p + 3] = paths[p].ry1;
    }
    for (uint32_t p = 0; p <= np; p++) {
        h.tile_first[p] = tf[p] - t0;
        h.col_first[p] = cf[p] - k0;
    }
    // every path's fills are one block from path_fill[p], grouped by tile; tile_fills[t] is one
    // past the last fill of tile t
    std::vector<uint32_t> tend, pfill, state, clip_tile;
    std::vector<uint16_t> state16;
    const bool clips = !c->h_path_clip.empty();
    if (int e = d2h(c, tend, c->tile_fills.as<uint32_t>() + t0, size_t(t1 - t0))) return e;
    if (int e = d2h(c, pfill, c->path_fill.as<uint32_t>() + p0, np)) return e;
    if (clips) {
        // tile states after the clip rules, as the GPU applied them (k_clip_dump)
        if (int e = d2h(c, state, c->canon_state.as<uint32_t>() + t0, t1 - t0)) return e;
        if (int e = d2h(c, clip_tile, c->canon_clip.as<uint32_t>() + t0, t1 - t0)) return e;
    } else if (int e = d2h(c, state16, c->tile_state.as<uint16_t>() + t0, t1 - t0)) {
        return e;
    }
    if (int e = d2h(c, h.col_backdrop, c->col_final.as<int32_t>() + k0, k1 - k0)) return e;
    if (int e = d2h(c, h.z, c->z.as<int32_t>() + fb0, size_t(S.fbw) * S.fbh)) return e;
    std::vector<uint32_t> fbc;
    if (int e = d2h(c, fbc, c->fb_count.as<uint32_t>() + fb0, size_t(S.fbw) * S.fbh + 1)) return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    const size_t nt = t1 - t0;
    if (!clips) state.assign(state16.begin(), state16.end());
    // gather the paths' blocks in path order (one copy per run of blocks adjacent on the device)
    std::vector<uint64_t> blk(np + 1, 0);
    for (uint32_t p = 0; p < np; p++) {
        const uint32_t a = tf[p] - t0, e = tf[p + 1] - t0;
        blk[p + 1] = blk[p] + (e > a ? tend[e - 1] - pfill[p] : 0u);
    }
    std::vector<uint2> fl(blk[np]);
    for (uint32_t p = 0; p < np;) {
        uint32_t q = p + 1;
        while (q < np && pfill[q] == pfill[q - 1] + (blk[q] - blk[q - 1])) q++;
        if (blk[q] > blk[p])
            PF_CUDA(cudaMemcpyAsync(fl.data() + blk[p], c->fills.as<uint2>() + pfill[p], (blk[q] - blk[p]) * 8,
                                    cudaMemcpyDeviceToHost, c->stream));
        p = q;
    }
    const uint32_t l0 = fbc[0], l1 = fbc[size_t(S.fbw) * S.fbh];
    if (int e = d2h(c, h.list, c->list.as<uint32_t>() + l0, l1 - l0)) return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    // tile t's fills in the gathered numbering: [begin[t], begin[t + 1])
    std::vector<uint64_t> begin(nt + 1);
    for (uint32_t p = 0; p < np; p++)
        for (uint32_t t = tf[p] - t0; t < tf[p + 1] - t0; t++)
            begin[t + 1] = blk[p] + (tend[t] - pfill[p]);
    const uint64_t f0 = 0, f1 = blk[np];

    h.alpha.resize(nt);
    h.backdrop.resize(nt);
    h.fill_count.resize(nt);
    h.fills.resize(size_t(f1 - f0) * 4);
    std::vector<uint64_t> keys;
    for (size_t t = 0; t < nt; t++) {
        const uint64_t a = begin[t] - f0, e = begin[t + 1] - f0;
        h.fill_count[t] = e - a;
        h.alpha[t] = (state[t] >> 8) & 1;
        h.backdrop[t] = (int8_t)(state[t] & 0xff);
        keys.clear();
        for (uint32_t k = a; k < e; k++)
            keys.push_back((uint64_t(fl[k].x & 0xffffu) << 48) | (uint64_t(fl[k].x >> 16) << 32) |
                           (uint64_t(fl[k].y & 0xffffu) << 16) | uint64_t(fl[k].y >> 16));
        std::sort(keys.begin(), keys.end());
        for (uint32_t k = 0; k < e - a; k++) {
            uint16_t *d = &h.fills[4 * (size_t(a) + k)];
            d[0] = uint16_t(keys[k] >> 48);
            d[1] = uint16_t(keys[k] >> 32);
            d[2] = uint16_t(keys[k] >> 16);
            d[3] = uint16_t(keys[k]);
        }
    }
    // clipped draw tiles (Tiler::prepare_tiles, pathfinder/core/d3d9/tiler.cpp:386-431): the
    // mask source, the clip tile and the draw tile's own backdrop, from the states k_clip_dump
    // wrote with the composite's own clip rules
    h.mask.assign(nt, 0);
    h.clip.assign(nt, UINT64_MAX);
    h.dest_backdrop.assign(nt, 0);
    for (size_t t = 0; clips && t < nt; t++) {
        const uint32_t mode = (state[t] >> 9) & 3u;
        h.mask[t] = (uint8_t)mode;
        if (mode != 0) h.clip[t] = uint64_t(clip_tile[t]) - t0;
        if (mode == 2) h.dest_backdrop[t] = (int8_t)((state[t] >> 16) & 0xffu);
    }
    for (auto &z : h.z)
        if (z >= 0) z -= (int32_t)p0;
    h.list_first.resize(fbc.size());
    for (size_t i = 0; i < fbc.size(); i++) h.list_first[i] = fbc[i] - l0;
    for (auto &g : h.list) g -= t0;

    std::memset(out, 0, sizeof(*out));
    out->n_paths = np;
    out->path_rect = h.rect.data();
    out->path_tile_first = h.tile_first.data();
    out->path_column_first = h.col_first.data();
    out->n_tiles = nt;
    out->tile_alpha = h.alpha.data();
    out->tile_backdrop = h.backdrop.data();
    out->tile_fill_count = h.fill_count.data();
    out->n_fills = f1 - f0;
    out->fills = h.fills.data();
    out->n_columns = k1 - k0;
    out->column_backdrop = h.col_backdrop.data();
    out->fb_tiles_x = S.fbw;
    out->fb_tiles_y = S.fbh;
    out->z = h.z.data();
    out->fb_list_first = h.list_first.data();
    out->n_list = l1 - l0;
    out->fb_list = h.list.data();
    out->tile_mask = h.mask.data();
    out->tile_clip = h.clip.data();
    out->tile_dest_backdrop = h.dest_backdrop.data();
    return PF_OK;
}

int read_image(Ctx *c, uint32_t si, uint8_t *rgba, size_t cap) {
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    if (si >= c->n_scenes) return fail(c, PF_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneDev &S = c->h_scenes[si];
    const size_t bytes = size_t(S.img_w) * S.img_h * 4;
    if (!rgba || cap < bytes) return fail(c, PF_ERR_INVALID_ARGUMENT, "image buffer too small");
    if (c->host_img) {
        // the frame already wrote the image into host memory
        if (rgba != c->host_img + S.img_offset) std::memcpy(rgba, c->host_img + S.img_offset, bytes);
        return PF_OK;
    }
    PF_CUDA(cudaMemcpyAsync(rgba, c->image.as<uint8_t>() + S.img_offset, bytes, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

// Unpin a host image target this context pinned.
void drop_host_image(Ctx *c) {
    if (c->host_img_registered) cudaHostUnregister(c->host_img);
    c->host_img = nullptr;
    c->host_img_dev = nullptr;
    c->host_img_bytes = 0;
    c->host_img_registered = false;
}

Ctx *as_ctx(void *p) { return static_cast<Ctx *>(p); }

}  // namespace

extern "C" int pf_image_bytes(void *ctx, uint64_t *bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c || !bytes) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    *bytes = c->image_bytes;
    return PF_OK;
}

extern "C" int pf_image_offset(void *ctx, uint32_t scene, uint64_t *offset) {
    Ctx *c = as_ctx(ctx);
    if (!c || !offset) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (scene >= c->n_scenes) return fail(c, PF_ERR_INVALID_ARGUMENT, "scene index out of range");
    *offset = c->h_scenes[scene].img_offset;
    return PF_OK;
}

extern "C" int pf_read_images(void *ctx, uint8_t *dst, size_t capacity_bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c || !dst) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    if (capacity_bytes < c->image_bytes) return fail(c, PF_ERR_INVALID_ARGUMENT, "image buffer too small");
    if (c->host_img) {
        if (dst != c->host_img) std::memcpy(dst, c->host_img, c->image_bytes);
        return PF_OK;
    }
    PF_CUDA(cudaMemcpyAsync(dst, c->image.p, c->image_bytes, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

// The images of the last frame to host memory without holding up the next frame: a
// device-to-device snapshot on the frame's stream (HBM speed), then the snapshot's copy to dst
// on the context's copy stream, which runs while later uploads and frames proceed.  The next
// snapshot waits, on the device, for the previous copy to have left the snapshot buffer.
extern "C" int pf_read_images_async(void *ctx, uint8_t *dst, size_t capacity_bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c || !dst) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    if (capacity_bytes < c->image_bytes) return fail(c, PF_ERR_INVALID_ARGUMENT, "image buffer too small");
    cudaSetDevice(c->device);
    if (c->host_img) {  // the frame already wrote the images into host memory
        if (dst != c->host_img) {
            PF_CUDA(cudaStreamSynchronize(c->stream));
            std::memcpy(dst, c->host_img, c->image_bytes);
        }
        return PF_OK;
    }
    if (!c->copy_stream) {
        PF_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        PF_CUDA(cudaEventCreateWithFlags(&c->snap_done, cudaEventDisableTiming));
        PF_CUDA(cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming));
    }
    if (c->copy_pending) {
        if (c->image_snap.cap < c->image_bytes || !c->image_snap.p) {
            // the snapshot buffer grows: the copy still reading it must finish first
            PF_CUDA(cudaEventSynchronize(c->copy_done));
            c->copy_pending = false;
        } else {
            PF_CUDA(cudaStreamWaitEvent(c->stream, c->copy_done, 0));
        }
    }
    PF_CUDA(c->image_snap.ensure(c->image_bytes));
    PF_CUDA(cudaMemcpyAsync(c->image_snap.p, c->image.p, c->image_bytes, cudaMemcpyDeviceToDevice, c->stream));
    PF_CUDA(cudaEventRecord(c->snap_done, c->stream));
    PF_CUDA(cudaStreamWaitEvent(c->copy_stream, c->snap_done, 0));
    // in 32 MB pieces: a frame's own small device-to-host reads (its status words) would
    // otherwise queue behind the whole copy on the copy engine
    constexpr size_t kPiece = size_t(32) << 20;
    for (size_t off = 0; off < c->image_bytes; off += kPiece)
        PF_CUDA(cudaMemcpyAsync(dst + off, c->image_snap.as<uint8_t>() + off, std::min(kPiece, c->image_bytes - off),
                                cudaMemcpyDeviceToHost, c->copy_stream));
    PF_CUDA(cudaEventRecord(c->copy_done, c->copy_stream));
    c->copy_pending = true;
    return PF_OK;
}

extern "C" int pf_images_wait(void *ctx) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    if (c->copy_pending) {
        cudaSetDevice(c->device);
        PF_CUDA(cudaEventSynchronize(c->copy_done));
        c->copy_pending = false;
    }
    return PF_OK;
}

// Frames composite straight into host memory over the GPU's coherent link (NVLink-C2C on
// GB300): the pixels cross to the host while the composite runs, and no copy follows the
// frame.  The buffer is pinned and mapped here unless the caller pinned it already (then it
// stays the caller's to unpin).  NULL restores device-resident images.
extern "C" int pf_set_host_image(void *ctx, void *host, size_t bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    PF_CUDA(cudaStreamSynchronize(c->stream));
    drop_host_image(c);
    c->rendered = false;
    if (!host) return PF_OK;
    if (bytes == 0) return fail(c, PF_ERR_INVALID_ARGUMENT, "empty host image buffer");
    bool registered = false;
    cudaPointerAttributes attr{};
    cudaError_t e = cudaPointerGetAttributes(&attr, host);
    if (e != cudaSuccess) cudaGetLastError();
    if (e != cudaSuccess || attr.type != cudaMemoryTypeHost) {
        // pageable memory: pin and map it here
        e = cudaHostRegister(host, bytes, cudaHostRegisterMapped);
        if (e == cudaSuccess) {
            registered = true;
        } else if (e == cudaErrorHostMemoryAlreadyRegistered) {
            cudaGetLastError();
        } else {
            cudaGetLastError();
            return cuda_fail(c, e, "cudaHostRegister(host image)");
        }
    }
    void *dev = nullptr;
    e = cudaHostGetDevicePointer(&dev, host, 0);
    if (e != cudaSuccess) {
        if (registered) cudaHostUnregister(host);
        cudaGetLastError();
        return cuda_fail(c, e, "cudaHostGetDevicePointer(host image)");
    }
    c->host_img = static_cast<uint8_t *>(host);
    c->host_img_dev = static_cast<uint8_t *>(dev);
    c->host_img_bytes = bytes;
    c->host_img_registered = registered;
    return PF_OK;
}

extern "C" {

int pf_abi_version(void) { return PF_ABI_VERSION; }

int pf_device_count(int *count) {
    if (!count) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "count is null");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        return fail(nullptr, PF_ERR_CUDA, cudaGetErrorString(e));
    }
    return PF_OK;
}

int pf_ctx_create(const pf_config *config, void **out) {
    if (!out) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx out pointer is null");
    *out = nullptr;
    Ctx *c = new (std::nothrow) Ctx();
    if (!c) return fail(nullptr, PF_ERR_OUT_OF_MEMORY, "host allocation failed");
    if (config) {
        c->device = config->device;
        c->stream = static_cast<cudaStream_t>(config->stream);
        c->flags = config->flags;
    }
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess && !c->stream) {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        c->own_stream = e == cudaSuccess;
    }
    if (e == cudaSuccess) e = cudaHostAlloc(&c->h_status, kStCount * 4, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&c->h_status_dev), c->h_status, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&c->h_stage, kStageBytes, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&c->h_stage_dev), c->h_stage, 0);
    for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
    if (e == cudaSuccess) e = c->status.ensure(kStCount * 4);
    if (e != cudaSuccess) {
        int st = cuda_fail(nullptr, e, "pf_ctx_create");
        pf_ctx_destroy(c);
        return st;
    }
    *out = c;
    return PF_OK;
}

int pf_ctx_destroy(void *ctx) {
    Ctx *c = as_ctx(ctx);
    if (!c) return PF_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->snap_done) cudaEventDestroy(c->snap_done);
    if (c->copy_done) cudaEventDestroy(c->copy_done);
    forget_learned(c);
    drop_host_image(c);
    DevBuf *bufs[] = {&c->sz_w, &c->sz_master, &c->sz_m, &c->sz_v, &c->sz_grad, &c->sz_loss, &c->sz_feat,
                      &c->sz_target, &c->sz_index, &c->sz_pred, &c->path_feat, &c->contour_feat, &c->path_pred, &c->path_leaf_first,
                      &c->path_leaf_budget, &c->path_leaf_cursor, &c->path_fill_budget, &c->path_bounds,
                      &c->bin_list, &c->bin_ctl, &c->path_leaf_range,
                      &c->points, &c->pflags, &c->cstart, &c->pstart, &c->fill_rule, &c->color, &c->scenes,
                      &c->scene_path_first, &c->scene_contour_first, &c->scene_fb_first, &c->fb_scene, &c->contour_point_first,
                      &c->contour_path, &c->paths, &c->path_tiles, &c->path_cols, &c->contour_segs,
                      &c->path_contours, &c->segs, &c->seg_leaves, &c->seg_order, &c->seg_ctl, &c->leaves, &c->pool_path, &c->pool_cnt,
                      &c->pool_idx, &c->tile_fills, &c->path_fill, &c->path_cls, &c->tile_state, &c->col_above,
                      &c->col_final, &c->fills, &c->bin_stage, &c->row_first,
                      &c->row_paths, &c->scene_row_first, &c->z, &c->fb_count, &c->list, &c->image,
                      &c->status, &c->scan_temp, &c->path_clip, &c->path_is_clip, &c->path_clip_rel,
                      &c->in_points, &c->in_pflags, &c->in_cstart, &c->in_pstart, &c->st_stroke, &c->st_closed,
                      &c->st_dashes, &c->st_scenes, &c->st_cfirst, &c->dash_pts, &c->dash_cnt, &c->dash_end,
                      &c->dash_points, &c->dash_flags, &c->job_first, &c->jobs, &c->job_pts, &c->st_bounds,
                      &c->job_units, &c->job_nfwd, &c->job_flags, &c->job_cap1, &c->job_end, &c->units,
                      &c->unit_leaves, &c->st_leaves, &c->leaf_pts, &c->path_grad, &c->grad_paint, &c->image_snap,
                      &c->grad_stop_range, &c->grad_stops, &c->grad_meta, &c->grad_ramp, &c->st_order_ctl,
                      &c->unit_order, &c->dash_order};
    for (DevBuf *b : bufs) b->release();
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->sev)
        if (e) cudaEventDestroy(e);
    for (auto &e : c->au_ev)
        if (e) cudaEventDestroy(e);
    if (c->bs_ready) {
        for (auto &s : c->bs.side) cudaStreamDestroy(s);
        cudaEventDestroy(c->bs.fork);
        for (auto &e : c->bs.join) cudaEventDestroy(e);
    }
    c->canon_state.release();
    c->canon_clip.release();
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return PF_OK;
}

const char *pf_last_error(void *ctx) {
    Ctx *c = as_ctx(ctx);
    return c ? c->err.c_str() : g_last_error.c_str();
}

int pf_scene_upload(void *ctx, const pf_scene_view *scene) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return upload(c, scene, 1);
}

int pf_scene_upload_batch(void *ctx, const pf_scene_view *scenes, uint32_t n_scenes) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return upload(c, scenes, n_scenes);
}

int pf_render(void *ctx, pf_frame_stats *stats) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return render_exact(c, 0, c->n_scenes, stats);
}

int pf_render_scenes(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return render_exact(c, first_scene, n_scenes, stats);
}

int pf_read_image(void *ctx, uint8_t *rgba, size_t capacity_bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    return read_image(c, 0, rgba, capacity_bytes);
}

int pf_read_image_scene(void *ctx, uint32_t scene, uint8_t *rgba, size_t capacity_bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    return read_image(c, scene, rgba, capacity_bytes);
}

int pf_image_device_ptr(void *ctx, void **rgba, uint32_t *width_px, uint32_t *height_px) {
    Ctx *c = as_ctx(ctx);
    if (!c || !rgba) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    *rgba = (c->host_img_dev ? c->host_img_dev : c->image.as<uint8_t>()) + c->h_scenes[c->r_first].img_offset;
    if (width_px) *width_px = c->h_scenes[c->r_first].img_w;
    if (height_px) *height_px = c->h_scenes[c->r_first].img_h;
    return PF_OK;
}

int pf_write_image(void *ctx, uint32_t scene, const uint8_t *rgba, size_t bytes) {
    Ctx *c = as_ctx(ctx);
    if (!c || !rgba) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    if (scene >= c->n_scenes) return fail(c, PF_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneDev &S = c->h_scenes[scene];
    const size_t need = size_t(S.img_w) * S.img_h * 4;
    if (bytes != need) return fail(c, PF_ERR_INVALID_ARGUMENT, "pf_write_image needs width_px * height_px * 4 bytes");
    PF_CUDA(cudaSetDevice(c->device));
    if (c->host_img) {
        // frames composite into the host image target: the destination lives there
        PF_CUDA(cudaStreamSynchronize(c->stream));
        std::memcpy(c->host_img + S.img_offset, rgba, need);
        return PF_OK;
    }
    PF_CUDA(cudaMemcpyAsync(c->image.as<uint8_t>() + S.img_offset, rgba, need, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

int pf_read_canon(void *ctx, pf_canon *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    return read_canon(c, 0, out);
}

int pf_upload_stats_get(void *ctx, pf_upload_stats *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    *out = c->ustats;
    out->n_points = c->n_points;
    out->n_contours = c->n_contours;
    return PF_OK;
}

int pf_read_outline(void *ctx, uint32_t scene, pf_outline *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    if (scene >= c->n_scenes) return fail(c, PF_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneDev &S = c->h_scenes[scene];
    const uint32_t np = S.path_end - S.path_first, nc = S.contour_end - S.contour_first,
                   npt = S.point_end - S.point_first;
    auto &o = c->outline;
    if (int e = d2h(c, o.points, c->points.as<float2>() + S.point_first, npt)) return e;
    if (int e = d2h(c, o.flags, c->pflags.as<uint8_t>() + S.point_first, npt)) return e;
    if (int e = d2h(c, o.cstart, c->cstart.as<uint32_t>() + S.cstart_base, size_t(nc) + 1)) return e;
    if (int e = d2h(c, o.pstart, c->pstart.as<uint32_t>() + S.pstart_base, size_t(np) + 1)) return e;
    if (int e = d2h(c, o.rule, c->fill_rule.as<uint8_t>() + S.path_first, np)) return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    out->n_points = npt;
    out->n_contours = nc;
    out->n_paths = np;
    out->points = reinterpret_cast<const float *>(o.points.data());
    out->point_flags = o.flags.data();
    out->contour_start = o.cstart.data();
    out->path_start = o.pstart.data();
    out->fill_rule = o.rule.data();
    return PF_OK;
}

int pf_read_canon_scene(void *ctx, uint32_t scene, pf_canon *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    return read_canon(c, scene, out);
}

int pf_draw(void *ctx, const pf_scene_view *scene, uint8_t *rgba, size_t capacity_bytes, pf_frame_stats *stats) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    if (int e = upload(c, scene, 1)) return e;
    if (int e = render_exact(c, 0, 1, stats)) return e;
    return read_image(c, 0, rgba, capacity_bytes);
}

// Coverage after the fill rule of every alpha tile of scene 0, in tile order
// (n_alpha x 256 floats, row-major 16x16).  A test and debugging aid.
int pf_read_coverage(void *ctx, float *out, size_t capacity_floats, uint64_t *n_alpha) {
    Ctx *c = as_ctx(ctx);
    if (!c || !n_alpha) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    const SceneDev &S = c->h_scenes[c->r_first];
    std::vector<uint32_t> tf, tfill;
    if (int e = d2h(c, tf, c->path_tiles.as<uint32_t>() + (S.path_first - c->r_path_base),
                    S.path_end - S.path_first + 1))
        return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    const uint32_t t0 = tf.front(), t1 = tf.back();
    std::vector<uint16_t> state;
    if (int e = d2h(c, state, c->tile_state.as<uint16_t>() + t0, size_t(t1 - t0))) return e;
    PF_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<uint32_t> alpha;
    for (uint32_t t = 0; t < t1 - t0; t++)
        if (state[t] & 0x100u) alpha.push_back(t0 + t);
    *n_alpha = alpha.size();
    if (!out) return PF_OK;
    if (capacity_floats < alpha.size() * 256) return fail(c, PF_ERR_INVALID_ARGUMENT, "coverage buffer too small");
    DevBuf dt, dout;
    PF_CUDA(dt.ensure(alpha.size() * 4 + 4));
    PF_CUDA(dout.ensure(alpha.size() * 1024 + 4));
    PF_CUDA(cudaMemcpyAsync(dt.p, alpha.data(), alpha.size() * 4, cudaMemcpyHostToDevice, c->stream));
    Batch b = make_batch(c);
    PF_CUDA(launch_coverage_dump(b, dt.as<uint32_t>(), (uint32_t)alpha.size(), dout.as<float>(), c->stream));
    PF_CUDA(cudaMemcpyAsync(out, dout.p, alpha.size() * 1024, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    dt.release();
    dout.release();
    return PF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Learned sizer: weights, training, prediction (see pf_sizer.cu).

namespace {

int sizer_alloc(Ctx *c) {
    PF_CUDA(c->sz_w.ensure(kSizerParams * 2 + 16));
    PF_CUDA(c->sz_master.ensure(kSizerParams * 4 + 16));
    PF_CUDA(c->sz_m.ensure(kSizerParams * 4 + 16));
    PF_CUDA(c->sz_v.ensure(kSizerParams * 4 + 16));
    PF_CUDA(c->sz_grad.ensure(kSizerParams * 4 + 16));
    PF_CUDA(c->sz_loss.ensure(16));
    return PF_OK;
}

// fp32 master -> device (master, bf16 copy); Adam moments and gradient cleared
int sizer_upload(Ctx *c, const float *params) {
    if (int e = sizer_alloc(c)) return e;
    std::vector<__nv_bfloat16> w(kSizerParams);
    for (int i = 0; i < kSizerParams; i++) w[i] = __float2bfloat16_rn(params[i]);
    PF_CUDA(cudaMemcpyAsync(c->sz_master.p, params, kSizerParams * 4, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(cudaMemcpyAsync(c->sz_w.p, w.data(), kSizerParams * 2, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(cudaMemsetAsync(c->sz_m.p, 0, kSizerParams * 4, c->stream));
    PF_CUDA(cudaMemsetAsync(c->sz_v.p, 0, kSizerParams * 4, c->stream));
    PF_CUDA(cudaMemsetAsync(c->sz_grad.p, 0, kSizerParams * 4, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    c->sz_step = 0;
    c->sz_ready = true;
    return PF_OK;
}

int upload_dataset(Ctx *c, const float *feat, const float *target, uint32_t n) {
    PF_CUDA(c->sz_feat.ensure(size_t(n) * kSizerIn * 4 + 16));
    PF_CUDA(c->sz_target.ensure(size_t(n) * kSizerOut * 4 + 16));
    PF_CUDA(cudaMemcpyAsync(c->sz_feat.p, feat, size_t(n) * kSizerIn * 4, cudaMemcpyHostToDevice, c->stream));
    if (target)
        PF_CUDA(cudaMemcpyAsync(c->sz_target.p, target, size_t(n) * kSizerOut * 4, cudaMemcpyHostToDevice, c->stream));
    return PF_OK;
}

struct SizerFileHeader {
    char magic[4];     // "PFSZ"
    uint32_t version;  // 1
    uint32_t n_in, hidden, n_out, n_params;
    uint32_t step;
    float budget_mul, budget_add;
    uint32_t reserved[7];
};

}  // namespace

extern "C" {

int pf_sizer_init(void *ctx, uint64_t seed) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    forget_learned(c);
    cudaSetDevice(c->device);
    // He-uniform initialisation from a splitmix64 stream
    std::vector<float> w(kSizerParams, 0.0f);
    uint64_t z = seed;
    auto next = [&]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    };
    const int H = kSizerHidden, I = kSizerIn, O = kSizerOut;
    const int oW1 = 0, oW2 = H * I + H, oW3 = oW2 + H * H + H;
    for (int i = 0; i < H * I; i++) w[oW1 + i] = (float)((next() * 2 - 1) * std::sqrt(6.0 / I));
    for (int i = 0; i < H * H; i++) w[oW2 + i] = (float)((next() * 2 - 1) * std::sqrt(6.0 / H));
    for (int i = 0; i < O * H; i++) w[oW3 + i] = (float)((next() * 2 - 1) * std::sqrt(3.0 / H));
    return sizer_upload(c, w.data());
}

int pf_sizer_param_count(void) { return kSizerParams; }

int pf_sizer_set_params(void *ctx, const float *params, size_t n) {
    Ctx *c = as_ctx(ctx);
    if (!c || !params || n != (size_t)kSizerParams) return fail(c, PF_ERR_INVALID_ARGUMENT, "bad sizer parameters");
    forget_learned(c);
    cudaSetDevice(c->device);
    return sizer_upload(c, params);
}

int pf_sizer_get_params(void *ctx, float *params, size_t n) {
    Ctx *c = as_ctx(ctx);
    if (!c || !params || n != (size_t)kSizerParams) return fail(c, PF_ERR_INVALID_ARGUMENT, "bad sizer parameters");
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    PF_CUDA(cudaMemcpyAsync(params, c->sz_master.p, kSizerParams * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

int pf_sizer_set_margin(void *ctx, float mul, float add, float pool) {
    Ctx *c = as_ctx(ctx);
    if (!c || !(mul > 0.0f) || !(add >= 0.0f) || !(pool >= 0.0f)) return fail(c, PF_ERR_INVALID_ARGUMENT, "bad margin");
    forget_learned(c);
    c->sz_mul = mul;
    c->sz_add = add;
    c->sz_pool = pool;
    return PF_OK;
}

// Budget statistics of the last learned frame: paths that overran their leaf budget and
// leaf slots taken from the spill pool.
int pf_sizer_last_frame(void *ctx, uint32_t *paths_over, uint32_t *pool_used) {
    Ctx *c = as_ctx(ctx);
    if (!c || !paths_over || !pool_used) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    *paths_over = c->last_paths_over;
    *pool_used = c->last_pool_used;
    return PF_OK;
}

int pf_sizer_predict(void *ctx, const float *feat, uint32_t n, float *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || (n && (!feat || !out))) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    cudaSetDevice(c->device);
    if (int e = upload_dataset(c, feat, nullptr, n)) return e;
    PF_CUDA(c->sz_pred.ensure(size_t(n) * kSizerOut * 4 + 16));
    PF_CUDA(launch_mlp_predict(c->sz_w.as<__nv_bfloat16>(), c->sz_feat.as<float>(), n, c->sz_pred.as<float>(),
                               c->stream));
    PF_CUDA(cudaMemcpyAsync(out, c->sz_pred.p, size_t(n) * kSizerOut * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

// Gradient of the mean squared error over (feat, target) at the current weights (bf16
// forward, fp32 accumulation), without updating them.  grad: kSizerParams floats.
int pf_sizer_gradient(void *ctx, const float *feat, const float *target, uint32_t n, float *grad, float *loss) {
    Ctx *c = as_ctx(ctx);
    if (!c || !feat || !target || !grad || n == 0) return fail(c, PF_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    cudaSetDevice(c->device);
    if (int e = upload_dataset(c, feat, target, n)) return e;
    PF_CUDA(cudaMemsetAsync(c->sz_grad.p, 0, kSizerParams * 4, c->stream));
    PF_CUDA(cudaMemsetAsync(c->sz_loss.p, 0, 4, c->stream));
    PF_CUDA(launch_mlp_grad(c->sz_w.as<__nv_bfloat16>(), c->sz_feat.as<float>(), c->sz_target.as<float>(), nullptr,
                            n, c->sz_grad.as<float>(), c->sz_loss.as<float>(), c->stream));
    PF_CUDA(cudaMemcpyAsync(grad, c->sz_grad.p, kSizerParams * 4, cudaMemcpyDeviceToHost, c->stream));
    float l = 0.0f;
    PF_CUDA(cudaMemcpyAsync(&l, c->sz_loss.p, 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaMemsetAsync(c->sz_grad.p, 0, kSizerParams * 4, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    if (loss) *loss = l / (float)(size_t(n) * kSizerOut);
    return PF_OK;
}

// Adam training on the GPU: `epochs` passes over (feat, target) in shuffled mini-batches.
// losses (optional): mean squared error of every epoch.
int pf_sizer_train(void *ctx, const float *feat, const float *target, uint32_t n, uint32_t epochs, uint32_t batch,
                   float lr, uint64_t seed, float *losses) {
    Ctx *c = as_ctx(ctx);
    if (!c || !feat || !target || n == 0 || batch == 0) return fail(c, PF_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    forget_learned(c);
    cudaSetDevice(c->device);
    if (int e = upload_dataset(c, feat, target, n)) return e;
    PF_CUDA(c->sz_index.ensure(size_t(n) * 4 + 16));
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; i++) perm[i] = i;
    uint64_t z = seed ^ 0x5DEECE66Dull;
    for (uint32_t ep = 0; ep < epochs; ep++) {
        for (uint32_t i = n - 1; i > 0; i--) {  // Fisher-Yates with splitmix64
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            x ^= x >> 31;
            std::swap(perm[i], perm[x % (i + 1)]);
        }
        PF_CUDA(cudaMemcpyAsync(c->sz_index.p, perm.data(), size_t(n) * 4, cudaMemcpyHostToDevice, c->stream));
        PF_CUDA(cudaMemsetAsync(c->sz_loss.p, 0, 4, c->stream));
        for (uint32_t off = 0; off < n; off += batch) {
            const uint32_t m = std::min(batch, n - off);
            PF_CUDA(launch_mlp_grad(c->sz_w.as<__nv_bfloat16>(), c->sz_feat.as<float>(), c->sz_target.as<float>(),
                                    c->sz_index.as<uint32_t>() + off, m, c->sz_grad.as<float>(),
                                    c->sz_loss.as<float>(), c->stream));
            PF_CUDA(launch_adam(c->sz_master.as<float>(), c->sz_w.as<__nv_bfloat16>(), c->sz_grad.as<float>(),
                                c->sz_m.as<float>(), c->sz_v.as<float>(), lr, ++c->sz_step, c->stream));
        }
        if (losses) {
            float l = 0.0f;
            PF_CUDA(cudaMemcpyAsync(&l, c->sz_loss.p, 4, cudaMemcpyDeviceToHost, c->stream));
            PF_CUDA(cudaStreamSynchronize(c->stream));
            losses[ep] = l / (float)(size_t(n) * kSizerOut);
        }
    }
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

int pf_sizer_save(void *ctx, const char *path) {
    Ctx *c = as_ctx(ctx);
    if (!c || !path) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    std::vector<float> w(kSizerParams), m(kSizerParams), v(kSizerParams);
    PF_CUDA(cudaMemcpyAsync(w.data(), c->sz_master.p, kSizerParams * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaMemcpyAsync(m.data(), c->sz_m.p, kSizerParams * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaMemcpyAsync(v.data(), c->sz_v.p, kSizerParams * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    SizerFileHeader h{};
    std::memcpy(h.magic, "PFSZ", 4);
    h.version = 1;
    h.n_in = kSizerIn;
    h.hidden = kSizerHidden;
    h.n_out = kSizerOut;
    h.n_params = kSizerParams;
    h.step = (uint32_t)c->sz_step;
    h.budget_mul = c->sz_mul;
    h.budget_add = c->sz_add;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(c, PF_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && std::fwrite(w.data(), 4, w.size(), f) == w.size() &&
              std::fwrite(m.data(), 4, m.size(), f) == m.size() && std::fwrite(v.data(), 4, v.size(), f) == v.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? PF_OK : fail(c, PF_ERR_INVALID_ARGUMENT, std::string("short write to ") + path);
}

int pf_sizer_load(void *ctx, const char *path) {
    Ctx *c = as_ctx(ctx);
    if (!c || !path) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    forget_learned(c);
    cudaSetDevice(c->device);
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(c, PF_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
    SizerFileHeader h{};
    std::vector<float> w(kSizerParams), m(kSizerParams), v(kSizerParams);
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, "PFSZ", 4) == 0 && h.version == 1 &&
              h.n_in == (uint32_t)kSizerIn && h.hidden == (uint32_t)kSizerHidden && h.n_out == (uint32_t)kSizerOut &&
              h.n_params == (uint32_t)kSizerParams && std::fread(w.data(), 4, w.size(), f) == w.size() &&
              std::fread(m.data(), 4, m.size(), f) == m.size() && std::fread(v.data(), 4, v.size(), f) == v.size();
    std::fclose(f);
    if (!ok) return fail(c, PF_ERR_INVALID_ARGUMENT, std::string("not a sizer weight file: ") + path);
    if (int e = sizer_upload(c, w.data())) return e;
    PF_CUDA(cudaMemcpyAsync(c->sz_m.p, m.data(), kSizerParams * 4, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(cudaMemcpyAsync(c->sz_v.p, v.data(), kSizerParams * 4, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    c->sz_step = (int)h.step;
    if (h.budget_mul > 0.0f) c->sz_mul = h.budget_mul;
    if (h.budget_add >= 0.0f) c->sz_add = h.budget_add;
    return PF_OK;
}

// Per-path features of the last frame (n_paths x 12 floats).
int pf_path_features(void *ctx, float *out, size_t capacity_floats) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    const size_t n = c->r_paths;
    if (capacity_floats < n * kSizerIn) return fail(c, PF_ERR_INVALID_ARGUMENT, "buffer too small");
    PF_CUDA(c->path_feat.ensure(n * kSizerIn * 4 + 16));
    Batch b = make_batch(c);
    PF_CUDA(c->contour_feat.ensure(size_t(c->r_contours) * 32 + 32));
    PF_CUDA(launch_features(b, c->path_contours.as<uint2>(), c->contour_feat.as<float4>(), c->path_feat.as<float>(),
                            c->stream));
    PF_CUDA(cudaMemcpyAsync(out, c->path_feat.p, n * kSizerIn * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}

// Exact per-path leaf-line and fill counts of the last exact frame (training labels).
int pf_path_counts(void *ctx, uint32_t *leaves, uint32_t *fills, size_t capacity) {
    Ctx *c = as_ctx(ctx);
    if (!c || !leaves || !fills) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!c->rendered) return fail(c, PF_ERR_NOT_READY, "nothing rendered");
    const size_t n = c->r_paths;
    if (capacity < n) return fail(c, PF_ERR_INVALID_ARGUMENT, "buffer too small");
    DevBuf dl, df;
    PF_CUDA(dl.ensure(n * 4 + 16));
    PF_CUDA(df.ensure(n * 4 + 16));
    Batch b = make_batch(c);
    PF_CUDA(launch_path_counts(b, c->path_contours.as<uint2>(), dl.as<uint32_t>(), df.as<uint32_t>(), c->stream));
    PF_CUDA(cudaMemcpyAsync(leaves, dl.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaMemcpyAsync(fills, df.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    dl.release();
    df.release();
    return PF_OK;
}

// Change the PF_CONFIG_* flags of a context (stage timing, frame counters).
int pf_ctx_set_flags(void *ctx, uint32_t flags) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    c->flags = flags;
    return PF_OK;
}

// The frame's status words (error bits, totals, counters; 16 x u32) of the last frame.
int pf_debug_counters(void *ctx, uint32_t *out, size_t n) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (int e = read_status(c)) return e;
    for (size_t i = 0; i < n && i < (size_t)kStCount; i++) out[i] = c->h_status[i];
    return PF_OK;
}

int pf_render_learned(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return render_learned(c, first_scene, n_scenes, stats);
}

int pf_render_auto(void *ctx, uint32_t first_scene, uint32_t n_scenes, pf_frame_stats *stats) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    cudaSetDevice(c->device);
    return render_auto(c, first_scene, n_scenes, stats);
}

static void tuning_out(const Tuning &t, pf_tuning *o) {
    std::memset(o, 0, sizeof *o);
    for (int k = 0; k < 3; k++) o->bin_ctas_per_sm[k] = t.bin_ctas_per_sm[k];
    o->long_line = t.long_line;
    o->bin_concurrent = t.bin_concurrent;
    o->seg_sorted = t.seg_sorted;
    o->composite_ticket = t.comp_ticket;
}

int pf_tuning_get(void *ctx, pf_tuning *out) {
    Ctx *c = as_ctx(ctx);
    if (!c || !out) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    tuning_out(c->tune, out);
    return PF_OK;
}

int pf_tuning_set(void *ctx, const pf_tuning *t) {
    Ctx *c = as_ctx(ctx);
    if (!c || !t) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (!(t->long_line >= 1.0f && t->long_line <= 4096.0f))
        return fail(c, PF_ERR_INVALID_ARGUMENT, "long_line must lie in [1, 4096]");
    for (uint32_t v : t->bin_ctas_per_sm)
        if (v > 64) return fail(c, PF_ERR_INVALID_ARGUMENT, "bin_ctas_per_sm must lie in [0, 64]");
    if (t->composite_ticket > 4096) return fail(c, PF_ERR_INVALID_ARGUMENT, "composite_ticket must lie in [0, 4096]");
    if (t->bin_concurrent > 1 || t->seg_sorted > 1)
        return fail(c, PF_ERR_INVALID_ARGUMENT, "flags must be 0 or 1");
    cudaSetDevice(c->device);
    PF_CUDA(cudaStreamSynchronize(c->stream));
    Tuning n;
    for (int k = 0; k < 3; k++) n.bin_ctas_per_sm[k] = t->bin_ctas_per_sm[k];
    n.long_line = t->long_line;
    n.bin_concurrent = t->bin_concurrent != 0;
    n.seg_sorted = t->seg_sorted != 0;
    n.comp_ticket = t->composite_ticket;
    c->tune = n;
    forget_learned(c);  // the recorded frame has the old parameters in its launches
    auto_reset(c);
    return PF_OK;
}

int pf_autotune(void *ctx, uint32_t first, uint32_t count, uint32_t frames, pf_tuning *best, float *best_ms,
                float *start_ms) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    if (!c->uploaded) return fail(c, PF_ERR_NOT_READY, "no scene uploaded");
    if (frames == 0 || frames > 100) return fail(c, PF_ERR_INVALID_ARGUMENT, "frames must lie in [1, 100]");
    cudaSetDevice(c->device);
    int max_ctas[3] = {1, 1, 1};
    PF_CUDA(bin_class_max_ctas(max_ctas));
    // the default frame settles first (it times the exact and the learned frame), then each
    // trial: set the parameters, warm up (buffers, the learned frame's graph), time `frames`
    pf_frame_stats st;
    for (int k = 0; k < kAutoSettle; k++)
        if (int e = render_auto(c, first, count, &st)) return e;
    const bool learned = c->sz_ready && c->au.learned_ms >= 0.0f && c->au.learned_ms < c->au.exact_ms;
    auto trial = [&](const pf_tuning &t, float *ms) -> int {
        if (int e = pf_tuning_set(c, &t)) return e;
        std::vector<float> v;
        for (uint32_t k = 0; k < frames + 3; k++) {
            float m = 0.0f;
            const int e = timed_frame(c, &m, [&] {
                return learned ? render_learned(c, first, count, &st) : render_exact(c, first, count, &st);
            });
            if (e) return e;
            if (k >= 3) v.push_back(m);
        }
        std::sort(v.begin(), v.end());
        *ms = v[v.size() / 2];
        return PF_OK;
    };
    pf_tuning cur;
    tuning_out(c->tune, &cur);
    float cur_ms = 0.0f;
    if (int e = trial(cur, &cur_ms)) return e;
    if (start_ms) *start_ms = cur_ms;
    // the candidates of each parameter
    std::vector<std::pair<int, std::vector<float>>> space = {
        {0, {0, 4, 8, 12, 16, 20}},  // bin_ctas_per_sm[0]
        {1, {0, 2, 4, 6, 8}},        // bin_ctas_per_sm[1]
        {2, {0, 1, 2, 3}},            // bin_ctas_per_sm[2]
        {3, {4, 6, 8, 12, 16, 32}},   // long_line
        {4, {0, 1}},                  // bin_concurrent
        {5, {0, 1}},                  // seg_sorted
        {6, {0, 1, 2, 4, 8, 16}},     // composite_ticket
    };
    auto get = [](const pf_tuning &t, int i) -> float {
        return i < 3 ? (float)t.bin_ctas_per_sm[i] : i == 3 ? t.long_line : i == 4 ? (float)t.bin_concurrent
               : i == 5 ? (float)t.seg_sorted : (float)t.composite_ticket;
    };
    auto put = [](pf_tuning &t, int i, float v) {
        if (i < 3) t.bin_ctas_per_sm[i] = (uint32_t)v;
        else if (i == 3) t.long_line = v;
        else if (i == 4) t.bin_concurrent = (uint32_t)v;
        else if (i == 5) t.seg_sorted = (uint32_t)v;
        else t.composite_ticket = (uint32_t)v;
    };
    for (int pass = 0; pass < 3; pass++) {
        bool improved = false;
        for (auto &dim : space) {
            for (float v : dim.second) {
                if (dim.first < 3 && v > (float)max_ctas[dim.first]) continue;
                if (v == get(cur, dim.first)) continue;
                pf_tuning t = cur;
                put(t, dim.first, v);
                float ms = 0.0f;
                if (int e = trial(t, &ms)) return e;
                if (ms < cur_ms * 0.99f) {
                    cur = t;
                    cur_ms = ms;
                    improved = true;
                }
            }
        }
        if (!improved) break;
    }
    if (int e = pf_tuning_set(c, &cur)) return e;
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return PF_OK;
}

int pf_auto_choice(void *ctx, int *last, int *choice, float *exact_ms, float *learned_ms) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    const auto &a = c->au;
    if (last) *last = a.last;
    if (choice)
        *choice = !c->sz_ready ? PF_FRAME_EXACT
                  : (a.exact_timed < kAutoSamples || a.learned_timed < kAutoSamples) ? -1
                  : a.learned_ms < a.exact_ms ? PF_FRAME_LEARNED : PF_FRAME_EXACT;
    if (exact_ms) *exact_ms = a.exact_ms > 0.0f ? a.exact_ms : 0.0f;
    if (learned_ms) *learned_ms = a.learned_ms > 0.0f ? a.learned_ms : 0.0f;
    return PF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Sizer prediction that allocates nothing.
//
// Some callers cannot call cudaMalloc: a render loop that plans the next frame's buffers
// while it must not stall the device (cudaMalloc can synchronise it), or a host whose GPU
// memory belongs to another allocator (an engine's own pool) and may not grow.  For them this
// variant of pf_sizer_predict stages features and predictions in a fixed, file-scope device
// array instead of context buffers.  It needs a context that already holds sizer weights
// (pf_sizer_load / pf_sizer_init, which do allocate, once).  Like pf_sizer_predict it waits
// on the context's stream for its results before it returns.  No counterpart in the reference.
//
// Limit: kNoAllocMaxPaths paths per call (the array is (12 + 2) floats per path, about
// 0.9 MB, and every GPU that loads this library keeps it until the process exits).
// The first call on a device looks up the array's device address (cudaGetSymbolAddress, with
// that device current).  All calls share the array and it keeps the last call's contents;
// nothing in it has to start at zero (each call overwrites the rows it uses).  Calls whose GPU
// work overlaps - from two threads, or on two streams - race on the array: serialise them.

namespace {

constexpr uint32_t kNoAllocMaxPaths = 16384;
static __device__ __align__(256) float g_sizer_noalloc_scratch[kNoAllocMaxPaths * (kSizerIn + kSizerOut)];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
float *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// device address of the scratch array on `device` (looked up once per device)
cudaError_t noalloc_scratch(int device, float **out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sizer_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[device] = static_cast<float *>(p);
    }
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int pf_sizer_predict_noalloc(void *ctx, const float *features, uint32_t n, float *out) {
    Ctx *c = as_ctx(ctx);
    if (!c) return fail(nullptr, PF_ERR_INVALID_ARGUMENT, "ctx is null");
    if (n && (!features || !out)) return fail(c, PF_ERR_INVALID_ARGUMENT, "null argument");
    if (n > kNoAllocMaxPaths) {
        return fail(c, PF_ERR_INVALID_ARGUMENT,
                    "pf_sizer_predict_noalloc: " + std::to_string(n) + " paths exceed its limit of " +
                        std::to_string(kNoAllocMaxPaths) + " per call");
    }
    if (!c->sz_ready) return fail(c, PF_ERR_NOT_READY, "no sizer weights");
    if (n == 0) return PF_OK;
    PF_CUDA(cudaSetDevice(c->device));
    float *scratch = nullptr;
    PF_CUDA(noalloc_scratch(c->device, &scratch));
    float *feat = scratch, *pred = scratch + size_t(kNoAllocMaxPaths) * kSizerIn;
    PF_CUDA(cudaMemcpyAsync(feat, features, size_t(n) * kSizerIn * 4, cudaMemcpyHostToDevice, c->stream));
    PF_CUDA(launch_mlp_predict(c->sz_w.as<__nv_bfloat16>(), feat, n, pred, c->stream));
    PF_CUDA(cudaMemcpyAsync(out, pred, size_t(n) * kSizerOut * 4, cudaMemcpyDeviceToHost, c->stream));
    PF_CUDA(cudaStreamSynchronize(c->stream));
    return PF_OK;
}
